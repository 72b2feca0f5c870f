/*
 * Forced-include prelude used only by oracle/Makefile when it compiles the
 * reference's own C/ sources (read in place) into oracle/_ref/.
 *
 * The reference sizes its static pencil and EMF scratch with a one-letter
 * macro `n` from its parameter.h.  This prelude pulls in the system headers
 * first (so the macro cannot reach them), then supplies the grid-size macros
 * with a larger capacity and defines PARAMETER_H so the shipped header is
 * skipped.  Loops in the reference run to the runtime nx/ny/nz, so any grid
 * up to REF_N per side (and REF_N^3 cells) works.  With REF_FP64 the whole
 * reference is retyped to double, as -Dfloat=double does.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <assert.h>
#define PARAMETER_H
#ifndef REF_N
#define REF_N 256
#endif
#define n REF_N
#define box_nx n
#define box_ny n
#define box_nz n
#define TOTAL_CELL_NUMBER box_nx*box_ny*box_nz
#define nu 5
#define nb 3
#ifdef REF_FP64
#define float double
#endif

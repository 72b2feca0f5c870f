/* File formats around the state (host arrays, reference layout u(5,nx,ny,nz),
 * b(3,nx,ny,nz)); every call returns an MHD_* status of mhd_gb300.h.
 *
 * mhd_write_check_value: the reference's check_value dump
 *   (C/check_value.c:25-66): files C_version_check_{u1..u5,b1..b3}.dat in
 *   `dir` (NULL or "" for the working directory), one "%8.6e" value per line,
 *   i fastest, then j, then k.  (The reference writes them at iteration 50;
 *   the caller chooses when.)
 * mhd_read_init: the reference's init file reader (C/init.c:34-52): 8 values
 *   per cell (u1..u5, b1..b3), cells in i-outer, j, k-inner order.
 * mhd_checkpoint_save / _load / _info: a binary checkpoint with no
 *   counterpart in the reference: a 64-byte header ("MHDGB300", version 1,
 *   element size, nx ny nz, t, step, FNV-1a hash of the payload) followed by
 *   u and b as stored.  _load checks the shape, element size and hash.
 */
#ifndef MHD_IO_H
#define MHD_IO_H

#include "mhd_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

MHD_API int mhd_write_check_value(const void *u, const void *b, int nx, int ny, int nz, int fp64, const char *dir);
MHD_API int mhd_read_init(const char *path, void *u, void *b, int nx, int ny, int nz, int fp64);
MHD_API int mhd_checkpoint_save(const char *path, const void *u, const void *b, int nx, int ny, int nz, int fp64,
                                double t, long long step);
MHD_API int mhd_checkpoint_info(const char *path, int *nx, int *ny, int *nz, int *fp64, double *t, long long *step);
MHD_API int mhd_checkpoint_load(const char *path, void *u, void *b, int nx, int ny, int nz, int fp64, double *t,
                                long long *step);

#ifdef __cplusplus
}
#endif
#endif /* MHD_IO_H */

/*
 * CPU oracle for the relaxing-TVD split MHD step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the arithmetic
 * of the reference's serial path (uelipen/Heterogeneous_MHD, directory C/)
 * so that the GPU library can be checked against it.  Only tests/, the
 * smoke() entry and bench.py's CPU-baseline leg may load the library built
 * from this file; the product never links it.
 *
 * Parity contract: every floating-point operation below is the one the
 * reference performs, in the same order and in the same type.  The reference
 * is C with `float` data, so every double literal (2.0, 0.9, 4.0 ...) promotes
 * the surrounding sub-expression to double; those promotions are written out
 * here as explicit (wide) casts.  Built with -ffp-contract=off this file is
 * bit-identical to the reference's own C/ sources built the same way (pinned
 * by tests/test_oracle_golden.py against oracle/_ref outputs).
 *
 * Compiled twice: -DORC_REAL=float (the reference as shipped) and
 * -DORC_REAL=double (the reference built with -Dfloat=double).
 *
 * Layout (C/array_definition.h:12-13): u(5,nx,ny,nz), b(3,nx,ny,nz),
 * Fortran order, component innermost: ((k*ny+j)*nx+i)*nc+c.
 * Boundaries are periodic everywhere.
 *
 * Pencils are independent inside every operator, so the loops over (j,k)
 * run under OpenMP; each pencil's arithmetic is unchanged, so results do not
 * depend on the thread count.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef ORC_REAL
#define ORC_REAL float
#endif
typedef ORC_REAL real;
typedef double wide; /* type of every sub-expression that meets a double literal */

#define EXPORT __attribute__((visibility("default")))

static inline size_t cell_of(int i, int j, int k, int nx, int ny)
{
    return ((size_t)k * (size_t)ny + (size_t)j) * (size_t)nx + (size_t)i;
}

/* abXYc_matrix2D / abXYc_matrix1D (C/includefunc_spu.h:73-94): L = a*X + b*Y + c,
 * evaluated left to right in float with float coefficients. */
static inline real abxyc(real a, real x, real b, real y, real c)
{
    return a * x + b * y + c;
}

/* Relaxing-speed limiter of C/tvd1.c:71-81 and :97-107 (and of C/tvdb.c:72-76):
 * zero unless a*b > 0, else 2ab/(a+b) evaluated in double (2.0 is a double literal). */
static inline real vanleer(real a, real b)
{
    real r = 0;
    if (a * b > 0)
        r = (real)(2.0 * (wide)a * (wide)b / (wide)(a + b));
    return r;
}

EXPORT int orc_real_size(void) { return (int)sizeof(real); }

EXPORT void orc_set_threads(int nthreads)
{
#ifdef _OPENMP
    if (nthreads > 0)
        omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

EXPORT int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ calcfl */

/* max_3num / max_2num (C/calcfl.c:65-101): strict '>' comparisons. */
static inline real max3(real a, real b, real c)
{
    if (a > b)
        return (a > c) ? a : c;
    return (b > c) ? b : c;
}

/* Per-cell fast speed of C/calcfl.c:44-54.  The cell-centred averages at
 * C/calcfl.c:38-43 are computed by the reference but never used; the speed is
 * built from the face values b(:,i,j,k). */
static inline real cfl_speed(const real *q, const real *f)
{
    const real gamma = (real)(5.0 / 3.0);
    real t1 = (real)fabs((wide)(q[1] / q[0]));
    real t2 = (real)fabs((wide)(q[2] / q[0]));
    real t3 = (real)fabs((wide)(q[3] / q[0]));
    real v = max3(t1, t2, t3);
    real mm = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
    real bb = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
    real ps = (real)(((wide)q[4] - (wide)(mm / q[0]) / 2.0) * ((wide)gamma - 1.0) +
                     (2.0 - (wide)gamma) * (wide)bb / 2.0);
    real p = (real)((wide)ps - (wide)bb / 2.0);
    return (real)((wide)v + sqrt(fabs((wide)bb * 2.0 + (wide)(gamma * p)) / (wide)q[0]));
}

/* calcfl (C/calcfl.c:13-63): returns 1/max_c with c starting at 0 and the
 * running max taken in linear (k,j,i) order with max_2num, so a NaN cell
 * resets the running value.  The serial scan is kept for that reason. */
EXPORT real orc_calcfl(real *u, real *b, int *pnx, int *pny, int *pnz)
{
    const int nx = *pnx, ny = *pny, nz = *pnz;
    real c = 0.0;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                size_t id = cell_of(i, j, k, nx, ny);
                real t = cfl_speed(u + 5 * id, b + 3 * id);
                c = (c > t) ? c : t; /* max_2num(&c,&temp1) */
            }
    return 1 / c;
}

/* ------------------------------------------------------------------ fluidx */

struct fluid_ws {
    real *u, *bc, *v, *tc, *wr, *wl, *fr, *fl, *flux, *u1, *tmp, *dfr, *dfl;
};

static void fluid_ws_alloc(struct fluid_ws *w, int n)
{
    size_t s5 = (size_t)5 * n;
    real *m = (real *)malloc(sizeof(real) * (s5 * 11 + (size_t)3 * n + n));
    w->u = m; m += s5;
    w->v = m; m += s5;
    w->wr = m; m += s5;
    w->wl = m; m += s5;
    w->fr = m; m += s5;
    w->fl = m; m += s5;
    w->flux = m; m += s5;
    w->u1 = m; m += s5;
    w->tmp = m; m += s5;
    w->dfr = m; m += s5;
    w->dfl = m; m += s5;
    w->bc = m; m += (size_t)3 * n;
    w->tc = m;
}

static void fluid_ws_free(struct fluid_ws *w) { free(w->u); }

/* mhdflux + find_max (C/mhdflux.c:9-72). */
static void mhdflux_p(real *v, real *pc, const real *u, const real *bc, int n, real *tc)
{
    const real gamma = (real)(5.0 / 3.0);
    for (int i = 0; i < n; i++) {
        const real *q = u + 5 * i;
        const real *f = bc + 3 * i;
        real vx = q[1] / q[0];
        real mm = q[1] * q[1] + q[2] * q[2] + q[3] * q[3];
        real bb = f[0] * f[0] + f[1] * f[1] + f[2] * f[2];
        real ps = (real)(((wide)q[4] - (wide)(mm / q[0]) / 2.0) * ((wide)gamma - 1.0) +
                         (2.0 - (wide)gamma) * (wide)bb / 2.0);
        real *o = v + 5 * i;
        o[0] = q[1];
        o[1] = q[1] * vx + ps - f[0] * f[0];
        o[2] = q[2] * vx - f[1] * f[0];
        o[3] = q[3] * vx - f[2] * f[0];
        o[4] = (q[4] + ps) * vx - f[0] * (f[0] * q[1] + f[1] * q[2] + f[2] * q[3]) / q[0];
        real p = (real)((wide)ps - (wide)bb / 2.0);
        tc[i] = (real)(fabs((wide)vx) + sqrt(fabs((wide)((bb + gamma * p) / q[0]))));
    }
    real c = 0.0; /* find_max, C/mhdflux.c:61-72 */
    for (int i = 0; i < n; i++)
        if (tc[i] > c)
            c = tc[i];
    *pc = c;
    if (c > 0)
        for (int m = 0; m < 5 * n; m++)
            v[m] = v[m] / c;
}

/* tvd1 (C/tvd1.c:8-118): two-stage relaxing TVD on one pencil, in place. */
static void tvd1_p(real *u, const real *bc, int n, real dt, struct fluid_ws *w)
{
    real c;
    const real one = 1, half = (real)0.5, zero = 0;
    /* stage 1: C/tvd1.c:33-49 */
    mhdflux_p(w->v, &c, u, bc, n, w->tc);
    for (int m = 0; m < 5 * n; m++) {
        w->wr[m] = abxyc(one, u[m], one, w->v[m], zero);
        w->wl[m] = abxyc(one, u[m], -one, w->v[m], zero);
        w->fr[m] = abxyc(c, w->wr[m], zero, w->wr[m], zero);
    }
    for (int i = 0; i < n; i++) {
        int ip = (i + 1) % n;
        for (int q = 0; q < 5; q++) {
            real t = w->wl[5 * ip + q];
            w->fl[5 * i + q] = abxyc(c, t, zero, t, zero);
        }
    }
    for (int m = 0; m < 5 * n; m++)
        w->flux[m] = abxyc(half, w->fr[m], -half, w->fl[m], zero);
    const real hdt = (real)(-1.0 * (wide)dt / 2.0);
    for (int i = 0; i < n; i++) {
        int im = (i + n - 1) % n;
        for (int q = 0; q < 5; q++) {
            real d = abxyc(one, w->flux[5 * i + q], -one, w->flux[5 * im + q], zero);
            w->u1[5 * i + q] = abxyc(one, u[5 * i + q], hdt, d, zero);
        }
    }
    /* stage 2: C/tvd1.c:51-116 */
    mhdflux_p(w->v, &c, w->u1, bc, n, w->tc);
    for (int m = 0; m < 5 * n; m++) {
        w->wr[m] = abxyc(one, w->u1[m], one, w->v[m], zero);
        w->wl[m] = abxyc(one, w->u1[m], -one, w->v[m], zero);
        w->fr[m] = abxyc(c, w->wr[m], zero, w->wr[m], zero);
    }
    for (int i = 0; i < n; i++) {
        int ip = (i + 1) % n, im = (i + n - 1) % n;
        for (int q = 0; q < 5; q++) {
            real dfrp = abxyc(half, w->fr[5 * ip + q], -half, w->fr[5 * i + q], zero);
            real dfrm = abxyc(half, w->fr[5 * i + q], -half, w->fr[5 * im + q], zero);
            w->dfr[5 * i + q] = vanleer(dfrp, dfrm);
        }
    }
    for (int i = 0; i < n; i++) {
        int ip = (i + 1) % n;
        for (int q = 0; q < 5; q++) {
            real t = w->wl[5 * ip + q];
            w->fl[5 * i + q] = abxyc(c, t, zero, t, zero);
        }
    }
    for (int i = 0; i < n; i++) {
        int ip = (i + 1) % n, im = (i + n - 1) % n;
        for (int q = 0; q < 5; q++) {
            real dflp = abxyc(half, w->fl[5 * i + q], -half, w->fl[5 * ip + q], zero);
            real dflm = abxyc(half, w->fl[5 * im + q], -half, w->fl[5 * i + q], zero);
            w->dfl[5 * i + q] = vanleer(dflp, dflm);
        }
    }
    for (int m = 0; m < 5 * n; m++) {
        real t1 = abxyc(one, w->fr[m], -one, w->fl[m], zero);
        real t2 = abxyc(one, w->dfr[m], -one, w->dfl[m], zero);
        w->flux[m] = abxyc(half, t1, half, t2, zero);
    }
    const real mdt = (real)(-1.0 * (wide)dt);
    for (int i = 0; i < n; i++) {
        int im = (i + n - 1) % n;
        for (int q = 0; q < 5; q++)
            w->tmp[5 * i + q] = abxyc(one, w->flux[5 * i + q], -one, w->flux[5 * im + q], zero);
    }
    for (int m = 0; m < 5 * n; m++)
        u[m] = abxyc(one, u[m], mdt, w->tmp[m], zero);
}

/* fluidx (C/fluidx.c:19-102): u <- tvd1(update_u) per x-pencil, with the
 * cell-centred field b3x built from update_b at (j,k), (jp,k), (j,kp). */
EXPORT void orc_fluidx(real *u, real *b, int *pnx, int *pny, int *pnz, real *pdt, real *uu,
                       real *ub, int iter)
{
    const int nx = *pnx, ny = *pny, nz = *pnz;
    const real dt = *pdt;
    (void)b;
    (void)iter;
    if (nx <= 0 || ny <= 0 || nz <= 0)
        return;
#pragma omp parallel
    {
        struct fluid_ws w;
        fluid_ws_alloc(&w, nx);
#pragma omp for collapse(2) schedule(static)
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++) {
                const int jp = (j + 1) % ny, kp = (k + 1) % nz;
                for (int i = 0; i < nx; i++)
                    for (int q = 0; q < 5; q++)
                        w.u[5 * i + q] = uu[cell_of(i, j, k, nx, ny) * 5 + q];
                for (int i = 0; i < nx; i++) {
                    const int ip = (i + 1) % nx;
                    const real *f = ub + cell_of(i, j, k, nx, ny) * 3;
                    real h0 = (real)0.5 * f[0];
                    real h0p = (real)0.5 * ub[cell_of(ip, j, k, nx, ny) * 3 + 0];
                    w.bc[3 * i + 0] = h0 + h0p;
                    w.bc[3 * i + 1] = (real)0.5 * f[1] + ub[cell_of(i, jp, k, nx, ny) * 3 + 1] / 2;
                    w.bc[3 * i + 2] = (real)0.5 * f[2] + ub[cell_of(i, j, kp, nx, ny) * 3 + 2] / 2;
                }
                tvd1_p(w.u, w.bc, nx, dt, &w);
                for (int i = 0; i < nx; i++)
                    for (int q = 0; q < 5; q++)
                        u[cell_of(i, j, k, nx, ny) * 5 + q] = w.u[5 * i + q];
            }
        fluid_ws_free(&w);
    }
}

/* -------------------------------------------------------------- advectbyzx */

struct adv_ws {
    real *vx, *vg, *bx, *flux, *vh, *t2, *f1, *b1;
};

static void adv_ws_alloc(struct adv_ws *w, int n)
{
    real *m = (real *)malloc(sizeof(real) * (size_t)n * 8);
    w->vx = m; m += n;
    w->vg = m; m += n;
    w->bx = m; m += n;
    w->flux = m; m += n;
    w->vh = m; m += n;
    w->t2 = m; m += n;
    w->f1 = m; m += n;
    w->b1 = m;
}

static void adv_ws_free(struct adv_ws *w) { free(w->vx); }

/* tvdb (C/tvdb.c:10-91): 1-D constrained-transport advection of a face
 * field b by the face velocity vg.  On return b holds the advected field and
 * flux the EMF times dt at each i+1/2. */
static void tvdb_p(real *flux, real *b, const real *vg, int n, real dt, struct adv_ws *w)
{
    real *vh = w->vh, *t2 = w->t2, *f1 = w->f1, *b1 = w->b1;
    for (int i = 0; i < n; i++)
        vh[i] = abxyc((real)0.5, vg[i], (real)0.5, vg[(i + 1) % n], (real)0);
    for (int i = 0; i < n; i++)
        t2[i] = b[i] * vg[i];
    for (int i = 0; i < n; i++)
        f1[i] = (vh[i] > 0) ? t2[i] : t2[(i + 1) % n];
    for (int i = 0; i < n; i++)
        b1[i] = (real)((wide)b[i] - (wide)((f1[i] - f1[(i + n - 1) % n]) * dt) / 2.0);
    for (int i = 0; i < n; i++) {
        const int ip = (i + 1) % n, ipp = (ip + 1) % n, im = (i + n - 1) % n;
        real w0, wp, wm;
        if (vh[i] > 0) {
            w0 = vg[i] * b1[i];
            wp = (real)((wide)(vg[ip] * b1[ip] - w0) / 2.0);
            wm = (real)((wide)(w0 - vg[im] * b1[im]) / 2.0);
        } else {
            w0 = vg[ip] * b1[ip];
            wp = (real)((wide)(w0 - vg[ipp] * b1[ipp]) / 2.0);
            wm = (real)((wide)(vg[i] * b1[i] - w0) / 2.0);
        }
        real dw = vanleer(wm, wp);
        flux[i] = (w0 + dw) * dt;
    }
    /* b = b - (flux - cshift(flux,-1)); the shifted copy is taken first. */
    real last = flux[n - 1];
    for (int i = n - 1; i >= 1; i--)
        b[i] = b[i] - (flux[i] - flux[i - 1]);
    b[0] = b[0] - (flux[0] - last);
}

/* One tvdb pencil of advectbyzxA1 (C/advectbyzxA1.c:26-58) or B1
 * (C/advectbyzxB1.c:26-57): face velocity from the two u pencils (pm below,
 * pc current), 1-2-1 smoothing, tvdb on component comp of update_b, then
 * b(comp) <- advected, b(1) -= flux(i-1), tmp <- flux(i-1). */
static void adv_pencil(real *b, real *tmp, const real *uu, const real *ub, size_t pm, size_t pc,
                       int comp, int nx, real dt, struct adv_ws *w)
{
    for (int i = 0; i < nx; i++)
        w->vx[i] = (uu[(pm + i) * 5 + 1] + uu[(pc + i) * 5 + 1]) /
                   (uu[(pm + i) * 5 + 0] + uu[(pc + i) * 5 + 0]);
    for (int i = 0; i < nx; i++) {
        real vm = w->vx[(i + nx - 1) % nx], vp = w->vx[(i + 1) % nx];
        w->vg[i] = (real)(((wide)(vm + vp) + 2.0 * (wide)w->vx[i]) / 4.0);
        w->bx[i] = ub[(pc + i) * 3 + comp];
    }
    tvdb_p(w->flux, w->bx, w->vg, nx, dt, w);
    for (int i = 0; i < nx; i++) {
        real f = w->flux[(i + nx - 1) % nx];
        b[(pc + i) * 3 + comp] = w->bx[i];
        b[(pc + i) * 3 + 0] = b[(pc + i) * 3 + 0] - f;
        tmp[pc + i] = f;
    }
}

/* advectbyzx (C/advectbyzx.c:14-23): A1 -> A2 -> B1 -> B2 with one EMF
 * scratch of nx*ny*nz values (the reference's static advectbyzx_tmp). */
EXPORT void orc_advectbyzx(real *u, real *b, int *pnx, int *pny, int *pnz, real *pdt, real *uu,
                           real *ub)
{
    const int nx = *pnx, ny = *pny, nz = *pnz;
    const real dt = *pdt;
    (void)u;
    if (nx <= 0 || ny <= 0 || nz <= 0)
        return;
    real *tmp = (real *)malloc(sizeof(real) * (size_t)nx * ny * nz);
#pragma omp parallel
    {
        struct adv_ws w;
        adv_ws_alloc(&w, nx);
        /* A1 (C/advectbyzxA1.c:26-60) */
#pragma omp for collapse(2) schedule(static)
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++) {
                int jm = (j + ny - 1) % ny;
                adv_pencil(b, tmp, uu, ub, cell_of(0, jm, k, nx, ny), cell_of(0, j, k, nx, ny), 1, nx,
                           dt, &w);
            }
        /* A2 (C/advectbyzxA2.c:16-26): b(1,i,jm,k) += tmp(i,j,k) */
#pragma omp for collapse(2) schedule(static)
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++) {
                int jm = (j + ny - 1) % ny;
                size_t d = cell_of(0, jm, k, nx, ny), s = cell_of(0, j, k, nx, ny);
                for (int i = 0; i < nx; i++)
                    b[(d + i) * 3] = b[(d + i) * 3] + tmp[s + i];
            }
        /* B1 (C/advectbyzxB1.c:26-59) */
#pragma omp for collapse(2) schedule(static)
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++) {
                int km = (k + nz - 1) % nz;
                adv_pencil(b, tmp, uu, ub, cell_of(0, j, km, nx, ny), cell_of(0, j, k, nx, ny), 2, nx,
                           dt, &w);
            }
        /* B2 (C/advectbyzxB2.c:16-26): b(1,i,j,km) += tmp(i,j,k) */
#pragma omp for collapse(2) schedule(static)
        for (int k = 0; k < nz; k++)
            for (int j = 0; j < ny; j++) {
                int km = (k + nz - 1) % nz;
                size_t d = cell_of(0, j, km, nx, ny), s = cell_of(0, j, k, nx, ny);
                for (int i = 0; i < nx; i++)
                    b[(d + i) * 3] = b[(d + i) * 3] + tmp[s + i];
            }
        adv_ws_free(&w);
    }
    free(tmp);
}

/* --------------------------------------------------------------- transposes */

/* transpose12 (C/transpose12.c:7-47): out dims (ny,nx,nz), out(j,i,k) = in(i,j,k);
 * u components reordered (1,3,2,4,5), b components (2,1,3).  Like the
 * reference, each k-plane is read completely into a temporary before it is
 * written, so u == update_u (in place) is allowed. */
EXPORT void orc_transpose12(real *u, real *b, real *uu, real *ub, int *pnx, int *pny, int *pnz,
                            int iter)
{
    const int nx = *pnx, ny = *pny, nz = *pnz;
    static const int pu[5] = {0, 2, 1, 3, 4}, pb[3] = {1, 0, 2};
    const size_t plane = (size_t)nx * ny;
    (void)iter;
    if (nx <= 0 || ny <= 0 || nz <= 0)
        return;
#pragma omp parallel
    {
        real *tu = (real *)malloc(sizeof(real) * plane * 8), *tb = tu + plane * 5;
#pragma omp for schedule(static)
        for (int k = 0; k < nz; k++) {
            memcpy(tu, uu + (size_t)k * plane * 5, sizeof(real) * plane * 5);
            memcpy(tb, ub + (size_t)k * plane * 3, sizeof(real) * plane * 3);
            for (int j = 0; j < ny; j++)
                for (int i = 0; i < nx; i++) {
                    size_t s = (size_t)j * nx + i, d = cell_of(j, i, k, ny, nx);
                    for (int q = 0; q < 5; q++)
                        u[d * 5 + q] = tu[s * 5 + pu[q]];
                    for (int q = 0; q < 3; q++)
                        b[d * 3 + q] = tb[s * 3 + pb[q]];
                }
        }
        free(tu);
    }
}

/* transpose13 (C/transpose13.c:9-62): only for nx==nz; out dims (nz,ny,nx),
 * out(k,j,i) = in(i,j,k); u components (1,4,3,2,5), b components (3,2,1).
 * Each j-plane is staged in a temporary first (in place allowed).  Any other
 * shape leaves the outputs untouched (the reference only prints). */
EXPORT void orc_transpose13(real *u, real *b, real *uu, real *ub, int *pnx, int *pny, int *pnz)
{
    const int nx = *pnx, ny = *pny, nz = *pnz;
    static const int pu[5] = {0, 3, 2, 1, 4}, pb[3] = {2, 1, 0};
    if (nx != nz) {
        fprintf(stderr, "orc_transpose13: nz<>nx not supported\n");
        return;
    }
    if (nx <= 0 || ny <= 0)
        return;
    const size_t plane = (size_t)nx * nz;
#pragma omp parallel
    {
        real *tu = (real *)malloc(sizeof(real) * plane * 8), *tb = tu + plane * 5;
#pragma omp for schedule(static)
        for (int j = 0; j < ny; j++) {
            for (int k = 0; k < nz; k++)
                for (int i = 0; i < nx; i++) {
                    size_t s = cell_of(i, j, k, nx, ny), t = (size_t)k * nx + i;
                    for (int q = 0; q < 5; q++)
                        tu[t * 5 + q] = uu[s * 5 + pu[q]];
                    for (int q = 0; q < 3; q++)
                        tb[t * 3 + q] = ub[s * 3 + pb[q]];
                }
            for (int k = 0; k < nz; k++)
                for (int i = 0; i < nx; i++) {
                    size_t d = cell_of(k, j, i, nz, ny), t = (size_t)k * nx + i;
                    memcpy(u + d * 5, tu + t * 5, sizeof(real) * 5);
                    memcpy(b + d * 3, tb + t * 3, sizeof(real) * 3);
                }
        }
        free(tu);
    }
}

/* copy_matrix (C/copy_matrix.c:9-38): update_u <- u, update_b <- b. */
EXPORT void orc_copy_matrix(real *u, real *b, int *pnx, int *pny, int *pnz, real *uu, real *ub)
{
    size_t nc = (size_t)(*pnx) * (*pny) * (*pnz);
    if (*pnx <= 0 || *pny <= 0 || *pnz <= 0)
        return;
    memcpy(uu, u, nc * 5 * sizeof(real));
    memcpy(ub, b, nc * 3 * sizeof(real));
}

/* -------------------------------------------------------------- the driver */

/* One or more full Strang steps exactly as the time loop of C/mhd.c:59-124:
 * dt = cfl*calcfl (0.9 in the reference), clamp to (tf-t)/2, t += 2dt, then
 * x(F,A) T12 y(F,A) T13 z(F,A,A,F) T13 y(A,F) T12 x(A,F) with a copy_matrix
 * after every operator and the dimensions permuted as the reference passes
 * them.  On entry update_* must equal u,b (C/mhd.c:50-51 initialises both).
 * Requires ny == nz (transpose13 is called with (ny,nx,nz) and (nz,nx,ny)).
 * Returns the number of steps taken (stops early once t >= tf). */
EXPORT int orc_strang_steps(real *u, real *b, real *uu, real *ub, int nx, int ny, int nz,
                            int nsteps, double cfl, real tf, real *t_io, real *dt_out)
{
    real t = *t_io, dt = 0;
    int s;
    for (s = 0; s < nsteps; s++) {
        if (!(t < tf))
            break;
        dt = (real)(cfl * (wide)orc_calcfl(u, b, &nx, &ny, &nz));
        if (dt > (tf - t) / 2)
            dt = (tf - t) / 2;
        t = t + 2 * dt;
        orc_fluidx(u, b, &nx, &ny, &nz, &dt, uu, ub, s + 1);
        orc_copy_matrix(u, b, &nx, &ny, &nz, uu, ub);
        orc_advectbyzx(u, b, &nx, &ny, &nz, &dt, uu, ub);
        orc_copy_matrix(u, b, &nx, &ny, &nz, uu, ub);
        /* y sweep */
        orc_transpose12(u, b, uu, ub, &nx, &ny, &nz, s + 1);
        orc_copy_matrix(u, b, &ny, &nx, &nz, uu, ub);
        orc_fluidx(u, b, &ny, &nx, &nz, &dt, uu, ub, s + 1);
        orc_copy_matrix(u, b, &ny, &nx, &nz, uu, ub);
        orc_advectbyzx(u, b, &ny, &nx, &nz, &dt, uu, ub);
        orc_copy_matrix(u, b, &ny, &nx, &nz, uu, ub);
        /* z sweep */
        orc_transpose13(u, b, uu, ub, &ny, &nx, &nz);
        orc_copy_matrix(u, b, &nz, &nx, &ny, uu, ub);
        orc_fluidx(u, b, &nz, &nx, &ny, &dt, uu, ub, s + 1);
        orc_copy_matrix(u, b, &nz, &nx, &ny, uu, ub);
        orc_advectbyzx(u, b, &nz, &nx, &ny, &dt, uu, ub);
        orc_copy_matrix(u, b, &nz, &nx, &ny, uu, ub);
        orc_advectbyzx(u, b, &nz, &nx, &ny, &dt, uu, ub);
        orc_copy_matrix(u, b, &nz, &nx, &ny, uu, ub);
        orc_fluidx(u, b, &nz, &nx, &ny, &dt, uu, ub, s + 1);
        orc_copy_matrix(u, b, &nz, &nx, &ny, uu, ub);
        /* back */
        orc_transpose13(u, b, uu, ub, &nz, &nx, &ny);
        orc_copy_matrix(u, b, &ny, &nx, &nz, uu, ub);
        orc_advectbyzx(u, b, &ny, &nx, &nz, &dt, uu, ub);
        orc_copy_matrix(u, b, &ny, &nx, &nz, uu, ub);
        orc_fluidx(u, b, &ny, &nx, &nz, &dt, uu, ub, s + 1);
        orc_copy_matrix(u, b, &ny, &nx, &nz, uu, ub);
        /* x again */
        orc_transpose12(u, b, uu, ub, &ny, &nx, &nz, s + 1);
        orc_copy_matrix(u, b, &nx, &ny, &nz, uu, ub);
        orc_advectbyzx(u, b, &nx, &ny, &nz, &dt, uu, ub);
        orc_copy_matrix(u, b, &nx, &ny, &nz, uu, ub);
        orc_fluidx(u, b, &nx, &ny, &nz, &dt, uu, ub, s + 1);
        orc_copy_matrix(u, b, &nx, &ny, &nz, uu, ub);
    }
    *t_io = t;
    if (dt_out)
        *dt_out = dt;
    return s;
}

/*
 * Seeded initial conditions for the MHD step, written into the reference
 * layout u(5,nx,ny,nz) / b(3,nx,ny,nz) (C/array_definition.h:12).
 *
 * The reference reads its initial state from text files that do not ship
 * (C/init.c:28-52), so these generators stand in for them.  They are host C,
 * built with -ffp-contract=off and use only IEEE add/sub/mul/div/sqrt plus
 * this file's own sin and log series: the same seed gives the same bits on
 * x86-64 and aarch64, so fixtures recorded on one host check runs on the
 * other.
 *
 * Geometry: unit box, cell (i,j,k) centred at ((i+1/2)/nx, ...).  b(1,i,j,k)
 * sits on the x-face at i/nx (the cell-centred Bx is (b1(i)+b1(i+1))/2,
 * C/fluidx.c:71-78); b(2), b(3) likewise on the y- and z-faces.  The energy
 * is E = p/(gamma-1) + rho|v|^2/2 + |B_c|^2/2 with B_c the face average, which
 * is what mhdflux inverts (C/mhdflux.c:28,41).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/mhd_gb300.h"

#define GAMMA_D (5.0 / 3.0)
#define TWO_PI 6.283185307179586476925286766559
#define LN2 0.693147180559945309417232121458

/* ------------------------------------------------------- deterministic math */

/* sin(2*pi*t): reduce t to [0,1), fold to [0,1/8] and evaluate a Taylor
 * series (truncation < 1e-16 on |x| <= pi/4). */
static double sin_series(double x)
{
    double x2 = x * x, term = x, sum = x;
    for (int k = 1; k <= 9; k++) {
        term = -term * x2 / (double)((2 * k) * (2 * k + 1));
        sum = sum + term;
    }
    return sum;
}

static double cos_series(double x)
{
    double x2 = x * x, term = 1.0, sum = 1.0;
    for (int k = 1; k <= 9; k++) {
        term = -term * x2 / (double)((2 * k - 1) * (2 * k));
        sum = sum + term;
    }
    return sum;
}

static double sin_turns(double t)
{
    double r = t - floor(t); /* [0,1) */
    double sgn = 1.0;
    if (r >= 0.5) {
        r = r - 0.5;
        sgn = -1.0;
    }
    if (r > 0.25)
        r = 0.5 - r; /* sin(pi - x) = sin x */
    if (r > 0.125)
        return sgn * cos_series(TWO_PI * (0.25 - r));
    return sgn * sin_series(TWO_PI * r);
}

static double cos_turns(double t) { return sin_turns(t + 0.25); }

/* sin/cos of 2*pi*num/den with the integer part removed exactly. */
static void cis_ratio(long long num, long long den, double *c, double *s)
{
    long long r = num % den;
    if (r < 0)
        r += den;
    double t = (double)r / (double)den;
    *s = sin_turns(t);
    *c = cos_turns(t);
}

static double log_series(double x) /* x > 0 */
{
    int e;
    double m = frexp(x, &e); /* x = m 2^e, m in [0.5,1) */
    if (m < 0.70710678118654752440) {
        m = m * 2.0;
        e -= 1;
    }
    double s = (m - 1.0) / (m + 1.0), s2 = s * s, term = s, sum = s;
    for (int k = 1; k <= 14; k++) {
        term = term * s2;
        sum = sum + term / (double)(2 * k + 1);
    }
    return 2.0 * sum + (double)e * LN2;
}

/* Counter-based generator (splitmix64 finaliser): one 64-bit hash per
 * (seed, stream, counter) so every value is independent of evaluation order. */
static uint64_t mix64(uint64_t z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static double uniform01(uint64_t seed, uint64_t stream, uint64_t ctr) /* (0,1] */
{
    uint64_t h = mix64(mix64(seed ^ (stream * 0xD1B54A32D192ED03ull)) + ctr);
    return ((double)(h >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

static double normal01(uint64_t seed, uint64_t stream, uint64_t ctr) /* Box-Muller */
{
    double u1 = uniform01(seed, stream, 2 * ctr), u2 = uniform01(seed, stream, 2 * ctr + 1);
    return sqrt(-2.0 * log_series(u1)) * cos_turns(u2);
}

static inline void put(void *a, int fp64, size_t idx, double v)
{
    if (fp64)
        ((double *)a)[idx] = v;
    else
        ((float *)a)[idx] = (float)v;
}

static inline double get(const void *a, int fp64, size_t idx)
{
    return fp64 ? ((const double *)a)[idx] : (double)((const float *)a)[idx];
}

static inline size_t cidx(int i, int j, int k, int nx, int ny)
{
    return ((size_t)k * ny + j) * nx + i;
}

/* E from rho, momentum and the face-averaged B read back from b as stored. */
static void fill_energy(void *u, const void *b, int fp64, int nx, int ny, int nz, const double *p_of)
{
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                size_t c = cidx(i, j, k, nx, ny);
                size_t ci = cidx((i + 1) % nx, j, k, nx, ny), cj = cidx(i, (j + 1) % ny, k, nx, ny),
                       ck = cidx(i, j, (k + 1) % nz, nx, ny);
                double bx = 0.5 * (get(b, fp64, 3 * c) + get(b, fp64, 3 * ci));
                double by = 0.5 * (get(b, fp64, 3 * c + 1) + get(b, fp64, 3 * cj + 1));
                double bz = 0.5 * (get(b, fp64, 3 * c + 2) + get(b, fp64, 3 * ck + 2));
                double rho = get(u, fp64, 5 * c);
                double mx = get(u, fp64, 5 * c + 1), my = get(u, fp64, 5 * c + 2),
                       mz = get(u, fp64, 5 * c + 3);
                double e = p_of[0] / (GAMMA_D - 1.0) + (mx * mx + my * my + mz * mz) / (2.0 * rho) +
                           (bx * bx + by * by + bz * bz) / 2.0;
                put(u, fp64, 5 * c + 4, e);
            }
}

/* ---------------------------------------------------- Orszag-Tang-like box */

MHD_API int mhd_init_vortex(void *u, void *b, int nx, int ny, int nz, int fp64, unsigned long long seed,
                            double rho0, double p0, double vscale, double noise, double bscale)
{
    if (!u || !b || nx <= 0 || ny <= 0 || nz <= 0 || !(rho0 > 0) || !(p0 > 0))
        return MHD_ERR_ARG;
    const double b0 = bscale / sqrt(2.0 * TWO_PI); /* 1/sqrt(4 pi) */
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                size_t c = cidx(i, j, k, nx, ny);
                double sy, cy, sx, cx, sz, cz, s2x, c2x;
                cis_ratio(2LL * j + 1, 2LL * ny, &cy, &sy);    /* y centre */
                cis_ratio(2LL * i + 1, 2LL * nx, &cx, &sx);    /* x centre */
                cis_ratio(2LL * k + 1, 2LL * nz, &cz, &sz);    /* z centre */
                cis_ratio(2LL * (2 * i + 1), 2LL * nx, &c2x, &s2x); /* 4 pi x centre */
                double vx = -sy * vscale + noise * normal01(seed, 1, 3 * c + 0);
                double vy = sx * vscale + noise * normal01(seed, 1, 3 * c + 1);
                double vz = 0.1 * sz * vscale + noise * normal01(seed, 1, 3 * c + 2);
                put(u, fp64, 5 * c + 0, rho0);
                put(u, fp64, 5 * c + 1, rho0 * vx);
                put(u, fp64, 5 * c + 2, rho0 * vy);
                put(u, fp64, 5 * c + 3, rho0 * vz);
                /* b1 on the x-face depends on y only, b2 on the y-face on x only:
                 * every face difference vanishes, so div B = 0 exactly. */
                put(b, fp64, 3 * c + 0, -sy * b0);
                put(b, fp64, 3 * c + 1, s2x * b0);
                put(b, fp64, 3 * c + 2, 0.0);
            }
    fill_energy(u, b, fp64, nx, ny, nz, &p0);
    return MHD_OK;
}

/* ------------------------------------------------- decaying turbulence box */

typedef struct {
    int K, W;        /* |k| <= K, W = 2K+1 */
    double *ar, *ai; /* amplitude cube [kz][ky][kx], kz in [0,K], ky,kx in [-K,K] */
} modes_t;

static size_t mode_at(const modes_t *m, int kx, int ky, int kz)
{
    return ((size_t)kz * m->W + (ky + m->K)) * m->W + (kx + m->K);
}

/* Evaluate f(x) = sum_modes 2 Re(A_k exp(2 pi i k.x)) on the grid points
 * x = ((i+sx)/n, (j+sy)/n, (k+sz)/n) with s* in {0, 1/2} given as 2*s*
 * (0 or 1), by three separable passes; writes f into comp of arr (stride nc). */
static void eval_field(const modes_t *m, int n, int hx, int hy, int hz, double scale, void *arr,
                       int fp64, int nc, int comp)
{
    const int K = m->K, W = m->W, KZ = K + 1;
    double *ex = (double *)malloc(sizeof(double) * 2 * W * n);
    double *ey = (double *)malloc(sizeof(double) * 2 * W * n);
    double *ez = (double *)malloc(sizeof(double) * 2 * KZ * n);
    for (int q = -K; q <= K; q++)
        for (int i = 0; i < n; i++) {
            double c, s;
            cis_ratio((long long)q * (2 * i + hx), 2LL * n, &c, &s);
            ex[2 * ((q + K) * n + i)] = c;
            ex[2 * ((q + K) * n + i) + 1] = s;
            cis_ratio((long long)q * (2 * i + hy), 2LL * n, &c, &s);
            ey[2 * ((q + K) * n + i)] = c;
            ey[2 * ((q + K) * n + i) + 1] = s;
        }
    for (int q = 0; q <= K; q++)
        for (int i = 0; i < n; i++) {
            double c, s;
            cis_ratio((long long)q * (2 * i + hz), 2LL * n, &c, &s);
            ez[2 * (q * n + i)] = c;
            ez[2 * (q * n + i) + 1] = s;
        }
    /* S1[kx][ky][z] = sum_kz A e^{i kz z} */
    double *s1 = (double *)calloc((size_t)2 * W * W * n, sizeof(double));
#pragma omp parallel for collapse(2) schedule(static)
    for (int kx = 0; kx < W; kx++)
        for (int ky = 0; ky < W; ky++)
            for (int z = 0; z < n; z++) {
                double re = 0, im = 0;
                for (int kz = 0; kz < KZ; kz++) {
                    size_t a = mode_at(m, kx - K, ky - K, kz);
                    double c = ez[2 * (kz * n + z)], s = ez[2 * (kz * n + z) + 1];
                    re = re + (m->ar[a] * c - m->ai[a] * s);
                    im = im + (m->ar[a] * s + m->ai[a] * c);
                }
                size_t o = ((size_t)kx * W + ky) * n + z;
                s1[2 * o] = re;
                s1[2 * o + 1] = im;
            }
    /* S2[kx][y][z] = sum_ky S1 e^{i ky y} */
    double *s2 = (double *)malloc(sizeof(double) * 2 * (size_t)W * n * n);
#pragma omp parallel for collapse(2) schedule(static)
    for (int kx = 0; kx < W; kx++)
        for (int y = 0; y < n; y++)
            for (int z = 0; z < n; z++) {
                double re = 0, im = 0;
                for (int ky = 0; ky < W; ky++) {
                    size_t a = ((size_t)kx * W + ky) * n + z;
                    double c = ey[2 * (ky * n + y)], s = ey[2 * (ky * n + y) + 1];
                    re = re + (s1[2 * a] * c - s1[2 * a + 1] * s);
                    im = im + (s1[2 * a] * s + s1[2 * a + 1] * c);
                }
                size_t o = ((size_t)kx * n + y) * n + z;
                s2[2 * o] = re;
                s2[2 * o + 1] = im;
            }
    /* f[x][y][z] = 2 Re sum_kx S2 e^{i kx x} */
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < n; z++)
        for (int y = 0; y < n; y++)
            for (int x = 0; x < n; x++) {
                double re = 0;
                for (int kx = 0; kx < W; kx++) {
                    size_t a = ((size_t)kx * n + y) * n + z;
                    double c = ex[2 * (kx * n + x)], s = ex[2 * (kx * n + x) + 1];
                    re = re + (s2[2 * a] * c - s2[2 * a + 1] * s);
                }
                put(arr, fp64, cidx(x, y, z, n, n) * nc + comp, 2.0 * re * scale);
            }
    free(ex);
    free(ey);
    free(ez);
    free(s1);
    free(s2);
}

static int in_half_space(int kx, int ky, int kz)
{
    return kz > 0 || (kz == 0 && (ky > 0 || (ky == 0 && kx > 0)));
}

/* x^(q/4) for integer q by square roots and products only. */
static double pow_quarter(double x, int q)
{
    double r = sqrt(sqrt(x)), acc = 1.0;
    int a = q < 0 ? -q : q;
    for (int t = 0; t < a; t++)
        acc = acc * r;
    return q < 0 ? 1.0 / acc : acc;
}

/* Random Gaussian amplitudes on kmin <= |k| <= kmax (upper half space), with
 * per-mode standard deviation (k^2)^((slope-2)/4), i.e. per-mode power
 * |k|^(slope-2), so the shell-summed spectrum goes as k^slope.  slope must be
 * an integer. */
static void draw_modes(modes_t *m, int comps, int kmin, int kmax, int slope, uint64_t seed,
                       uint64_t stream)
{
    const int qexp = slope - 2; /* (k^2)^((slope-2)/4) = (k^2)^(qexp/4) */
    for (int c = 0; c < comps; c++)
        for (int kz = 0; kz <= m->K; kz++)
            for (int ky = -m->K; ky <= m->K; ky++)
                for (int kx = -m->K; kx <= m->K; kx++) {
                    size_t a = mode_at(m, kx, ky, kz) + (size_t)c * (m->K + 1) * m->W * m->W;
                    int k2 = kx * kx + ky * ky + kz * kz;
                    m->ar[a] = 0;
                    m->ai[a] = 0;
                    if (!in_half_space(kx, ky, kz) || k2 < kmin * kmin || k2 > kmax * kmax)
                        continue;
                    double sd = pow_quarter((double)k2, qexp);
                    m->ar[a] = sd * normal01(seed, stream, 2 * a);
                    m->ai[a] = sd * normal01(seed, stream, 2 * a + 1);
                }
}

MHD_API int mhd_init_turbulence(void *u, void *b, int n, int fp64, unsigned long long seed, double rho0,
                                double p0, double mach, double bx0, double dbrms, int kmin, int kmax)
{
    if (!u || !b || n <= 0 || kmin < 1 || kmax < kmin || 2 * kmax >= n || !(rho0 > 0) || !(p0 > 0))
        return MHD_ERR_ARG;
    const int K = kmax, W = 2 * K + 1;
    const size_t cube = (size_t)(K + 1) * W * W;
    modes_t vm = {K, W, (double *)malloc(sizeof(double) * cube * 3),
                  (double *)malloc(sizeof(double) * cube * 3)};
    modes_t am = {K, W, (double *)malloc(sizeof(double) * cube * 3),
                  (double *)malloc(sizeof(double) * cube * 3)};
    draw_modes(&vm, 3, kmin, kmax, -2, seed, 11);
    draw_modes(&am, 3, kmin, kmax, -3, seed, 13);

    /* Velocity: rms |v| from Parseval (each mode adds 2|A|^2), set to mach*cs. */
    double v2 = 0;
    for (size_t a = 0; a < 3 * cube; a++)
        v2 += 2.0 * (vm.ar[a] * vm.ar[a] + vm.ai[a] * vm.ai[a]);
    const double cs = sqrt(GAMMA_D * p0 / rho0);
    const double vs = (v2 > 0) ? mach * cs / sqrt(v2) : 0.0;

    /* B = curl A on the staggered grid: for mode k the discrete curl is
     * i (s x A) with s_d = 2 n sin(pi k_d / n), evaluated at the face centres.
     * Build the three delta-B amplitude cubes, then set rms |dB| = dbrms. */
    modes_t bm = {K, W, (double *)malloc(sizeof(double) * cube * 3),
                  (double *)malloc(sizeof(double) * cube * 3)};
    double b2 = 0;
    for (int kz = 0; kz <= K; kz++)
        for (int ky = -K; ky <= K; ky++)
            for (int kx = -K; kx <= K; kx++) {
                size_t a = mode_at(&am, kx, ky, kz);
                double sk[3] = {2.0 * n * sin_turns((double)kx / (2.0 * n)),
                                2.0 * n * sin_turns((double)ky / (2.0 * n)),
                                2.0 * n * sin_turns((double)kz / (2.0 * n))};
                double Ar[3], Ai[3];
                for (int c = 0; c < 3; c++) {
                    Ar[c] = am.ar[a + c * cube];
                    Ai[c] = am.ai[a + c * cube];
                }
                for (int c = 0; c < 3; c++) {
                    int c1 = (c + 1) % 3, c2 = (c + 2) % 3;
                    double cr = sk[c1] * Ar[c2] - sk[c2] * Ar[c1]; /* (s x A)_c */
                    double ci = sk[c1] * Ai[c2] - sk[c2] * Ai[c1];
                    bm.ar[a + c * cube] = -ci; /* i (cr + i ci) */
                    bm.ai[a + c * cube] = cr;
                    b2 += 2.0 * (cr * cr + ci * ci);
                }
            }
    const double bs = (b2 > 0) ? dbrms / sqrt(b2) : 0.0;

    modes_t one = {K, W, NULL, NULL};
    for (int c = 0; c < 3; c++) {
        one.ar = vm.ar + c * cube;
        one.ai = vm.ai + c * cube;
        eval_field(&one, n, 1, 1, 1, vs * rho0, u, fp64, 5, 1 + c);
    }
    /* b(1) on x-faces (0,1/2,1/2), b(2) on y-faces, b(3) on z-faces */
    for (int c = 0; c < 3; c++) {
        one.ar = bm.ar + c * cube;
        one.ai = bm.ai + c * cube;
        eval_field(&one, n, c == 0 ? 0 : 1, c == 1 ? 0 : 1, c == 2 ? 0 : 1, bs, b, fp64, 3, c);
    }
    const size_t nc = (size_t)n * n * n;
#pragma omp parallel for schedule(static)
    for (long long c = 0; c < (long long)nc; c++) {
        put(u, fp64, 5 * c, rho0);
        put(b, fp64, 3 * c, get(b, fp64, 3 * c) + bx0);
    }
    fill_energy(u, b, fp64, n, n, n, &p0);
    free(vm.ar);
    free(vm.ai);
    free(am.ar);
    free(am.ai);
    free(bm.ar);
    free(bm.ai);
    return MHD_OK;
}

/* --------------------------------------------------------------- diagnostics */

/* max over cells of |div B| with the staggered stencil
 * sum_d b(d, idx+e_d) - b(d, idx) (periodic). */
MHD_API double mhd_host_divb_max(const void *b, int nx, int ny, int nz, int fp64)
{
    double mx = 0;
#pragma omp parallel for collapse(2) reduction(max : mx) schedule(static)
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                size_t c = cidx(i, j, k, nx, ny);
                double d = (get(b, fp64, 3 * cidx((i + 1) % nx, j, k, nx, ny)) - get(b, fp64, 3 * c)) +
                           (get(b, fp64, 3 * cidx(i, (j + 1) % ny, k, nx, ny) + 1) -
                            get(b, fp64, 3 * c + 1)) +
                           (get(b, fp64, 3 * cidx(i, j, (k + 1) % nz, nx, ny) + 2) -
                            get(b, fp64, 3 * c + 2));
                d = fabs(d);
                if (d > mx)
                    mx = d;
            }
    return mx;
}

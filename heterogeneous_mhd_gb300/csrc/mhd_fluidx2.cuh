// fluidx with C cells per thread (C/fluidx.c:19-102, C/tvd1.c:8-118,
// C/mhdflux.c:9-72).  A CTA stages P consecutive x-pencils of u and the b
// pencils at (j..j+P, k) and (j.., kp) into shared memory with bulk TMA, each
// pencil is owned by T = n/C threads (mhd_pencil.cuh), and the relaxing TVD
// update runs in registers: the two pencil maxima are shuffle reductions and
// the five neighbour exchanges of the stencil are shuffles.  The new u goes
// back through shared memory and one bulk TMA store.
//
// AX = 1, 2: the same sweep along y or z of the untransposed state (the fused
// step's replacement for transpose12/13 + fluidx + transpose back).  The CTA
// owns P = 4 pencils at consecutive x.  Its rows (the P cells at one position
// along the sweep, contiguous in x) arrive by 3-D tensor copies
// (cp.async.bulk.tensor, one per array: u, b, b of plane k+1 and b of the
// pencil after the group), then one pass over shared memory, with a
// bank-conflict-free thread mapping, builds the cell-centred field and a
// second one turns the u rows into the pencil-major layout the engine reads;
// the new pencils go back the same way and leave by one tensor store.  The
// components are seen in the order the transposed call would see them
// (C/transpose12.c:7-47, C/transpose13.c:9-62); the arithmetic is the x
// sweep's.
#pragma once
#include <cuda.h>  // CUtensorMap

#include "mhd_kernels.cuh"
#include "mhd_pencil.cuh"

namespace mhd {

template <int C, int T>
struct Fx2Shape {
    static constexpr int N = C * T;  // cells per pencil
};

// shared memory (elements of R) of the x sweep: su P pencils of 5n, sb P+1
// pencils of 3n, sbk P of 3n, red 32, seam 2*32*10
__host__ __device__ inline size_t fluidx2_smem_elems(int n, int P)
{
    return P * 5 * (size_t)n + (P + 1) * 3 * (size_t)n + P * 3 * (size_t)n + 32 + 2 * 32 * 10;
}

// Tensor maps of one sweep along y or z, encoded by the launcher: u and b of
// the input state with boxes of P cells along x by the whole pencil, b with a
// box of four words (the b of cell x0+P and one word after it) for the pencil
// after the group, u of the output state, and (when asked) the (rho, m) side
// array of the output with boxes of 2P words.
struct SweepMaps {
    CUtensorMap u_in, b_in, bn_in, u_out, w_out;
};

// Sweeps along y and z: P = 4 pencils of n = 4T cells per CTA, n <= 256 (one
// tensor box per array).  Pencil strides of the pencil-major u and field are
// 8 words more than 5n and 3n (both n % 32 == 0 or 8-word aligned), which
// keeps the transposing passes free of bank conflicts.
constexpr int kSweepP = 4;
__host__ __device__ constexpr int sweep_su(int n) { return 5 * n + 8; }
__host__ __device__ constexpr int sweep_sf(int n) { return 3 * n + 8; }

// Shared memory of a sweep along y or z (bytes): staged u rows [n][5P];
// region B: staged b rows [n][3P], b rows of plane k+1 [n][3P] and b rows of
// the next pencil [n][4], which the pencil-major u [P][SU] replaces once the
// field is built; the cell-centred field [P][SF]; red and seam; 128 bytes of
// alignment slack (the tensor copies want 128-byte aligned buffers).
__host__ __device__ inline size_t fluidx_sweep_regb(int n)
{
    const size_t st = (size_t)n * (6 * kSweepP + 4), su = (size_t)kSweepP * sweep_su(n);
    return st > su ? st : su;
}
__host__ __device__ inline size_t fluidx_sweep_smem_bytes(int n)
{
    return ((size_t)n * 5 * kSweepP + fluidx_sweep_regb(n) + (size_t)kSweepP * sweep_sf(n) + 32 + 2 * 32 * 10) *
               sizeof(float) + 128;
}

// The kernel body, for a CTA at block coordinates `blk` of its size class's
// grid (HwBlock in k_fluidx2, VBlock in the work-list launch over several
// classes, mhd_multi.cuh).  `tm` is read by the sweeps along y and z only.
template <typename R, bool EX, int C, int T, int AX, typename B>
__device__ __forceinline__ void fluidx2_body(FluidxArgs a, const SweepMaps* tm, const B& blk)
{
    static_assert(AX == 0 || (sizeof(R) == 4 && C == 4 && T <= 128), "sweeps along y, z: FP32, 4 cells, n <= 512");
    // y/z sweeps: a tensor box holds at most 256 rows, so longer pencils move in NBX boxes of BXR rows
    constexpr int NBX = (C * T + 255) / 256, BXR = C * T / NBX;
    select_box(a, blk.z(), sizeof(CflPart<R>), blk.gx() * blk.gy());
    constexpr int n = C * T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int P = a.P;
    const int np = n * P;
    const int tid = threadIdx.x;
    const int lp = tid / T;  // local pencil
    const Group<R, T> g(tid);
    const int i0 = g.t * C;
    const int j0 = blk.x() * P, k = a.kbeg + blk.y();  // k: plane along z (x sweep)
    const int kp = (k + 1 == a.nz) ? 0 : k + 1;
    const int jn = (j0 + P == a.ny) ? 0 : j0 + P;

    // pencil strides; x sweep: su [P][5n], sb [P+1][3n], sbk [P][3n]; y/z
    // sweeps: the staged rows, su [P][SU] over the staged b, the field sf [P][SF]
    constexpr int SU = AX ? sweep_su(n) : 5 * n, SB = AX ? sweep_sf(n) : 3 * n;
    // the 128-byte aligned start is an offset from smem_raw (not a pointer rebuilt
    // from an integer), so every access below stays a shared-memory access
    const uint32_t pad = (128u - (static_cast<uint32_t>(__cvta_generic_to_shared(smem_raw)) & 127u)) & 127u;
    R* const base = reinterpret_cast<R*>(smem_raw + (AX ? pad : 0u));
    R* const rows_u = base;                                       // y/z: [n][5P]
    R* const su = AX ? base + n * 5 * kSweepP : base;
    R* const sb = AX ? nullptr : su + P * SU;
    R* const sbk = AX ? nullptr : sb + (P + 1) * SB;
    R* const sf = AX ? su + fluidx_sweep_regb(n) : nullptr;      // y/z: [P][SF]
    R* const red = AX ? sf + P * SB : sbk + P * SB;
    R* const seam = red + 32;
    __shared__ uint64_t bar, bar_u;  // bar_u: the u rows of a sweep along y or z

    const R* uu = static_cast<const R*>(a.uu);
    const R* ub = static_cast<const R*>(a.ub);
    const size_t c0 = ((size_t)k * a.ny + j0) * n;
    const size_t cn = ((size_t)k * a.ny + jn) * n;
    const size_t ck = ((size_t)kp * a.ny + j0) * n;
    const R dt = load_dt<R>(a.dt_ptr, a.dt_val);  // read while the tensor copies land

    if constexpr (AX == 0) {
        if (tid == 0) {
            mbar_init(&bar, 1);
            const uint32_t bu = 5u * np * sizeof(R), bg = 3u * np * sizeof(R), b1 = 3u * n * sizeof(R);
            mbar_arrive_expect_tx(&bar, bu + 2 * bg + b1);
            tma_load_1d(su, uu + c0 * 5, bu, &bar);
            tma_load_1d(sb, ub + c0 * 3, bg, &bar);
            tma_load_1d(sb + 3 * np, ub + cn * 3, b1, &bar);
            tma_load_1d(sbk, ub + ck * 3, bg, &bar);
        }
        __syncthreads();
        // a copy that never lands (the wait gave up and set the error bit):
        // the whole CTA leaves before computing on unfilled shared memory
        if (!__syncthreads_and(mbar_wait_bounded(&bar, 0, a.err)))
            return;
    } else {
        // the rows of the group (x0..x0+P-1) along the whole pencil at plane kk,
        // its b rows at plane kn, and the b of cell x0+P (periodic)
        const int x0 = blk.x() * P, kk = a.kbeg + blk.y();
        const int nk = (AX == 1) ? a.nz : a.ny;
        const int kn = (kk + 1 == nk) ? 0 : kk + 1;
        const int xn = (x0 + P == a.nx) ? 0 : x0 + P;
        R* const rows_b = su;                          // [n][3P]
        R* const rows_bk = rows_b + n * 3 * kSweepP;   // [n][3P]
        R* const rows_bn = rows_bk + n * 3 * kSweepP;  // [n][4]
        // two barriers: the b rows (bar) land before the u rows (bar_u), so the
        // field pass runs while u is still arriving
        if (tid == 0) {
            mbar_init(&bar, 1);
            mbar_init(&bar_u, 1);
            mbar_arrive_expect_tx(&bar, (uint32_t)(n * (6 * kSweepP + 4) * sizeof(R)));
            mbar_arrive_expect_tx(&bar_u, (uint32_t)(n * 5 * kSweepP * sizeof(R)));
            // coordinates (x word, y, z): the pencil runs along y (AX 1) or z (AX 2) from 0
            const int y = (AX == 1) ? 0 : kk, z = (AX == 1) ? kk : 0;
            const int yk = (AX == 1) ? 0 : kn, zk = (AX == 1) ? kn : 0;
#pragma unroll
            for (int h = 0; h < NBX; h++) {  // rows h*BXR.. of the pencil
                const int dy = (AX == 1) ? h * BXR : 0, dz = (AX == 1) ? 0 : h * BXR;
                tma_load_3d(rows_b + h * BXR * 3 * kSweepP, &tm->b_in, 3 * x0, y + dy, z + dz, &bar);
                tma_load_3d(rows_bn + h * BXR * 4, &tm->bn_in, 3 * xn, y + dy, z + dz, &bar);
                tma_load_3d(rows_bk + h * BXR * 3 * kSweepP, &tm->b_in, 3 * x0, yk + dy, zk + dz, &bar);
            }
#pragma unroll
            for (int h = 0; h < NBX; h++) {
                const int dy = (AX == 1) ? h * BXR : 0, dz = (AX == 1) ? 0 : h * BXR;
                tma_load_3d(rows_u + h * BXR * 5 * kSweepP, &tm->u_in, 5 * x0, y + dy, z + dz, &bar_u);
            }
        }
        __syncthreads();
        if (!__syncthreads_and(mbar_wait_bounded(&bar, 0, a.err)))
            return;  // a copy never landed (error bit set)
        // Each thread takes the cells e = tid + it * NT (it < IT): cell (e / P, e % P).
        // Every pass issues all of its loads before its stores.
        constexpr int NT = kSweepP * T, IT = n * kSweepP / NT;
        // cell-centred field (C/fluidx.c:71-81) of cell (r, p), seen in the
        // transposed order: b_d averaged with the next row, b_x with the next
        // pencil, b_k with the next plane.  The staged rows are read at a
        // stride of three words, sf is written with a pencil stride of 8
        // (mod 32) words, both without bank conflicts.
        constexpr int B0 = sweep_b<AX>(0), B1 = sweep_b<AX>(1), B2 = sweep_b<AX>(2);
        {
            R fv[IT][6];
#pragma unroll
            for (int it = 0; it < IT; it++) {
                const int e = tid + it * NT, r = e / kSweepP, p = e - r * kSweepP;
                const int rn = (r + 1 == n) ? 0 : r + 1;
                const R* bc = rows_b + r * 3 * kSweepP + 3 * p;
                fv[it][0] = bc[B0];
                fv[it][1] = rows_b[rn * 3 * kSweepP + 3 * p + B0];
                fv[it][2] = bc[B1];
                fv[it][3] = (p + 1 < kSweepP) ? bc[3 + B1] : rows_bn[r * 4 + B1];
                fv[it][4] = bc[B2];
                fv[it][5] = rows_bk[r * 3 * kSweepP + 3 * p + B2];
            }
#pragma unroll
            for (int it = 0; it < IT; it++) {
                const int e = tid + it * NT, r = e / kSweepP, p = e - r * kSweepP;
                R* o = sf + p * SB + 3 * r;
                if constexpr (EX) {
                    o[0] = R(0.5) * fv[it][0] + R(0.5) * fv[it][1];
                    o[1] = R(0.5) * fv[it][2] + fv[it][3] / R(2);
                    o[2] = R(0.5) * fv[it][4] + fv[it][5] / R(2);
                } else {  // the same values: halving is exact
                    o[0] = R(0.5) * (fv[it][0] + fv[it][1]);
                    o[1] = R(0.5) * (fv[it][2] + fv[it][3]);
                    o[2] = R(0.5) * (fv[it][4] + fv[it][5]);
                }
            }
        }
        // the staged b is dead (su takes its place) once every thread is here and u has landed
        if (!__syncthreads_and(mbar_wait_bounded(&bar_u, 0, a.err)))
            return;
        // u rows -> pencil-major, raw component order (stride-5 reads, 8 (mod 32) pencil stride)
        {
            R uv[IT][5];
#pragma unroll
            for (int it = 0; it < IT; it++) {
                const R* src = rows_u + 5 * (tid + it * NT);
#pragma unroll
                for (int c = 0; c < 5; c++)
                    uv[it][c] = src[c];
            }
#pragma unroll
            for (int it = 0; it < IT; it++) {
                const int e = tid + it * NT, r = e / kSweepP, p = e - r * kSweepP;
                R* dst = su + p * SU + 5 * r;
#pragma unroll
                for (int c = 0; c < 5; c++)
                    dst[c] = uv[it][c];
            }
        }
        __syncthreads();
    }

    using W = wide_t<R, EX>;

    // ---- gather this thread's cells.  q and the cell-centred field are read
    // again from shared memory where they are needed later, which keeps them
    // out of the registers across the exchange phases.
    const R* uq = su + (size_t)lp * SU + (size_t)i0 * 5;
    auto load_q = [&](R (&q)[C][5]) {
        R qf[C * 5];
        lds_chunk<R, C * 5>(uq, qf);
#pragma unroll
        for (int m = 0; m < C; m++)
#pragma unroll
            for (int s = 0; s < 5; s++)
                q[m][s] = qf[5 * m + sweep_u<AX>(s)];
    };
    auto load_f = [&](R (&f)[C][3]) {  // C/fluidx.c:71-81: b/2 + b(neighbour face)/2
        if constexpr (AX != 0) {  // built once from the staged rows
            R ff[C * 3];
            lds_chunk<R, C * 3>(sf + (size_t)lp * SB + (size_t)i0 * 3, ff);
#pragma unroll
            for (int m = 0; m < C; m++)
#pragma unroll
                for (int s = 0; s < 3; s++)
                    f[m][s] = ff[3 * m + s];
            return;
        }
        R bjf[C * 3], bpf[C * 3], bkf[C * 3];
        const R* bj = sb + (size_t)lp * SB;
        lds_chunk<R, C * 3>(bj + 3 * i0, bjf);
        lds_chunk<R, C * 3>(sb + (size_t)(lp + 1) * SB + (size_t)i0 * 3, bpf);
        lds_chunk<R, C * 3>(sbk + (size_t)lp * SB + (size_t)i0 * 3, bkf);
        const int inext = (i0 + C == n) ? 0 : i0 + C;
        constexpr int B0 = sweep_b<AX>(0), B1 = sweep_b<AX>(1), B2 = sweep_b<AX>(2);
        const R b1next = bj[3 * inext + B0];
#pragma unroll
        for (int m = 0; m < C; m++) {
            const R b0n = (m + 1 < C) ? bjf[3 * (m + 1) + B0] : b1next;
            if constexpr (EX) {
                f[m][0] = R(0.5) * bjf[3 * m + B0] + R(0.5) * b0n;
                f[m][1] = R(0.5) * bjf[3 * m + B1] + bpf[3 * m + B1] / R(2);
                f[m][2] = R(0.5) * bjf[3 * m + B2] + bkf[3 * m + B2] / R(2);
            } else {  // the same values: halving is exact
                f[m][0] = R(0.5) * (bjf[3 * m + B0] + b0n);
                f[m][1] = R(0.5) * (bjf[3 * m + B1] + bpf[3 * m + B1]);
                f[m][2] = R(0.5) * (bjf[3 * m + B2] + bkf[3 * m + B2]);
            }
        }
    };
    R q[C][5], f[C][3];
    load_q(q);
    load_f(f);

    // ---- stage 1 (C/tvd1.c:33-49)
    R fr[C][5], gl[C][5];  // fr = c*wr, gl = c*wl (so fl(i) = gl(i+1))
    {
        R v[C][5], cmax = R(0);
#pragma unroll
        for (int m = 0; m < C; m++) {
            R ci;
            cell_flux<R, EX>(q[m], f[m], v[m], ci);
            cmax = fmax(cmax, ci);
        }
        const R c = g.max(cmax, red);
#pragma unroll
        for (int m = 0; m < C; m++) {
            if constexpr (EX) {
                scale_flux<R, EX>(v[m], c);
#pragma unroll
                for (int s = 0; s < 5; s++) {
                    fr[m][s] = scale0<R, EX>(c, lin<R, EX>(R(1), q[m][s], R(1), v[m][s]));
                    gl[m][s] = scale0<R, EX>(c, lin<R, EX>(R(1), q[m][s], R(-1), v[m][s]));
                }
            } else {
                // c*(u +- v/c) = c*u +- v.  c == 0 only when every cell of the pencil has zero
                // velocity and zero magnetosonic speed, where the fluxes v vanish too.
#pragma unroll
                for (int s = 0; s < 5; s++) {
                    fr[m][s] = fma(c, q[m][s], v[m][s]);
                    gl[m][s] = fma(c, q[m][s], -v[m][s]);
                }
            }
        }
    }
    R u1[C][5];
    {
        // FAST keeps the flux undivided (2 flux: the half is exact) and puts the
        // factor into the step: q + (hdt/2)(F(i) - F(i-1)) is the same value.
        R gnext[5], flux[C][5];
        g.template shift<5>(gl[0], gnext, +1, seam, 0);
#pragma unroll
        for (int m = 0; m < C; m++)
#pragma unroll
            for (int s = 0; s < 5; s++) {
                const R gn = (m + 1 < C) ? gl[m + 1][s] : gnext[s];
                if constexpr (EX)
                    flux[m][s] = lin<R, EX>(R(0.5), fr[m][s], R(-0.5), gn);
                else
                    flux[m][s] = fr[m][s] - gn;
            }
        R fprev[5];
        g.template shift<5>(flux[C - 1], fprev, -1, seam, 1);
        const R hdt = EX ? R(W(-1.0) * W(dt) / W(2.0)) : R(-0.25) * dt;
#pragma unroll
        for (int m = 0; m < C; m++)
#pragma unroll
            for (int s = 0; s < 5; s++)
                u1[m][s] = lin<R, EX>(R(1), q[m][s], hdt,
                                      lin<R, EX>(R(1), flux[m][s], R(-1), (m > 0) ? flux[m - 1][s] : fprev[s]));
    }

    // ---- stage 2 (C/tvd1.c:51-116)
    {
        R v[C][5], cmax = R(0);
        load_f(f);
#pragma unroll
        for (int m = 0; m < C; m++) {
            R ci;
            cell_flux<R, EX>(u1[m], f[m], v[m], ci);
            cmax = fmax(cmax, ci);
        }
        const R c = g.max(cmax, red + 16);
#pragma unroll
        for (int m = 0; m < C; m++) {
            if constexpr (EX) {
                scale_flux<R, EX>(v[m], c);
#pragma unroll
                for (int s = 0; s < 5; s++) {
                    fr[m][s] = scale0<R, EX>(c, lin<R, EX>(R(1), u1[m][s], R(1), v[m][s]));
                    gl[m][s] = scale0<R, EX>(c, lin<R, EX>(R(1), u1[m][s], R(-1), v[m][s]));
                }
            } else {
#pragma unroll
                for (int s = 0; s < 5; s++) {
                    fr[m][s] = fma(c, u1[m][s], v[m][s]);
                    gl[m][s] = fma(c, u1[m][s], -v[m][s]);
                }
            }
        }
    }
    R flux[C][5];
    {
        R xs[10], xr[10];
        // left neighbour's last fr, right neighbour's first gl (fl(i) = gl(i+1))
        R frp[5], gln[5];
        g.template shift<5>(fr[C - 1], frp, -1, seam, 0);
        g.template shift<5>(gl[0], gln, +1, seam, 1);
        // dfrm(i), dflm(i); FAST keeps them undivided (2 dfrm, 2 dflm: the halves
        // are exact, and the limiter below absorbs the factor)
        R dm[C][5], dl[C][5];
#pragma unroll
        for (int m = 0; m < C; m++)
#pragma unroll
            for (int s = 0; s < 5; s++) {
                const R frm = (m > 0) ? fr[m - 1][s] : frp[s], gln1 = (m + 1 < C) ? gl[m + 1][s] : gln[s];
                if constexpr (EX) {
                    dm[m][s] = lin<R, EX>(R(0.5), fr[m][s], R(-0.5), frm);
                    dl[m][s] = lin<R, EX>(R(0.5), gl[m][s], R(-0.5), gln1);
                } else {
                    dm[m][s] = fr[m][s] - frm;
                    dl[m][s] = gl[m][s] - gln1;
                }
            }
#pragma unroll
        for (int s = 0; s < 5; s++) {
            xs[s] = dm[0][s];
            xs[5 + s] = dl[0][s];
        }
        g.template shift<10>(xs, xr, +1, seam, 0);  // dfrp(i) = dfrm(i+1), dflp(i) = dflm(i+1)
#pragma unroll
        for (int m = 0; m < C; m++)
#pragma unroll
            for (int s = 0; s < 5; s++) {
                const R dmn = (m + 1 < C) ? dm[m + 1][s] : xr[s];
                const R dln = (m + 1 < C) ? dl[m + 1][s] : xr[5 + s];
                R dfr, dfl;
                if constexpr (EX) {
                    dfr = vanleer<R, EX>(dmn, dm[m][s]);
                    dfl = vanleer<R, EX>(dln, dl[m][s]);
                } else {
                    // branch-free: the quotient is computed for every cell and selected.
                    // With a = A/2, b = B/2: 2ab / (a + b) = AB / (A + B), and every
                    // factor dropped is a power of two, so the value is the halved form's.
                    const R pr = dmn * dm[m][s], pl = dln * dl[m][s];
                    const R qr = fast_div(pr, dmn + dm[m][s]), ql = fast_div(pl, dln + dl[m][s]);
                    dfr = (pr > R(0)) ? qr : R(0);
                    dfl = (pl > R(0)) ? ql : R(0);
                }
                const R gn = (m + 1 < C) ? gl[m + 1][s] : gln[s];
                if constexpr (EX)
                    flux[m][s] = lin<R, EX>(R(0.5), lin<R, EX>(R(1), fr[m][s], R(-1), gn), R(0.5),
                                            lin<R, EX>(R(1), dfr, R(-1), dfl));
                else  // undivided (2 flux), the half goes into the step below
                    flux[m][s] = (fr[m][s] - gn) + (dfr - dfl);
            }
    }
    {
        R fprev[5];
        g.template shift<5>(flux[C - 1], fprev, -1, seam, 1);
        const R mdt = EX ? R(W(-1.0) * W(dt)) : R(-0.5) * dt;
        R of[C * 5];
        load_q(q);
#pragma unroll
        for (int m = 0; m < C; m++)
#pragma unroll
            for (int s = 0; s < 5; s++) {
                q[m][s] = lin<R, EX>(R(1), q[m][s], mdt,
                                     lin<R, EX>(R(1), flux[m][s], R(-1), (m > 0) ? flux[m - 1][s] : fprev[s]));
                of[5 * m + sweep_u<AX>(s)] = q[m][s];
            }
        // own cells: no other thread reads them after the gather
        sts_chunk<R, C * 5>(su + (size_t)lp * SU + (size_t)i0 * 5, of);
        // the two values the next advectbyzx reads (rho, m_x), 8 bytes per cell
        if constexpr (AX == 0 && sizeof(R) == 4) {
            if (a.w_out) {
                float wv[2 * C];
#pragma unroll
                for (int m = 0; m < C; m++) {
                    wv[2 * m] = q[m][0];
                    wv[2 * m + 1] = q[m][1];
                }
                stg_chunk<float, 2 * C>(static_cast<float*>(a.w_out) + 2 * (c0 + (size_t)lp * n + i0), wv);
            }
        }
    }

    // ---- optional calcfl epilogue on the new state (face b at (j,k)); x sweep only
    if (AX == 0 && a.cfl_part) {
        const R* bj = sb + (size_t)lp * SB + (size_t)i0 * 3;
        R m = R(0);
        int ln = -1;
#pragma unroll
        for (int mm = 0; mm < C; mm++) {
            const R fc[3] = {bj[3 * mm], bj[3 * mm + 1], bj[3 * mm + 2]};
            const R sp = cfl_speed<R, EX>(q[mm], fc);
            if (sp != sp)
                ln = (int)(c0 + lp * n + i0 + mm);
            else
                m = fmax(m, sp);
        }
        m = warp_max<R>(m);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            ln = max(ln, __shfl_xor_sync(kFull, ln, o));
        __syncthreads();  // red is reused below
        int* rn = reinterpret_cast<int*>(seam);
        if ((tid & 31) == 0) {
            red[tid >> 5] = m;
            rn[tid >> 5] = ln;
        }
        __syncthreads();
        if (tid == 0) {
            R cm = R(0);
            int lnan = -1;
            for (int s = 0; s < (int)(blockDim.x >> 5); s++) {
                cm = fmax(cm, red[s]);
                lnan = max(lnan, rn[s]);
            }
            CflPart<R>* part = static_cast<CflPart<R>*>(a.cfl_part) + ((size_t)k * blk.gx() + blk.x());
            part->cmax = cm;
            part->last_nan = lnan;
        }
    }

    // ---- write the new pencils
    if constexpr (AX == 0) {
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            tma_store_1d(static_cast<R*>(a.u_out) + c0 * 5, su, 5u * np * sizeof(R));
            tma_store_commit();
            tma_store_wait_read();  // the CTA may leave once its buffers are read
        }
    } else {
        // pencil-major -> rows (the mapping of the gather, reversed), then one
        // tensor store.  With a side array: rho and the momentum the next
        // advectbyzx sweeps with (w_comp) of every cell too, as rows of the
        // x-major side array (8 bytes per cell) in the dead field buffer, and a
        // second tensor store.
        __syncthreads();
        R* const rows_w = sf;  // [n][2P]
        const int wc = a.w_out ? a.w_comp : 0;
        constexpr int NT = kSweepP * T, IT = n * kSweepP / NT;
        R uv[IT][5];
#pragma unroll
        for (int it = 0; it < IT; it++) {
            const int e = tid + it * NT, r = e / kSweepP, p = e - r * kSweepP;
            const R* src = su + p * SU + 5 * r;
#pragma unroll
            for (int c = 0; c < 5; c++)
                uv[it][c] = src[c];
        }
#pragma unroll
        for (int it = 0; it < IT; it++) {
            const int e = tid + it * NT;
            R* dst = rows_u + 5 * e;
#pragma unroll
            for (int c = 0; c < 5; c++)
                dst[c] = uv[it][c];
            if (wc) {
                rows_w[2 * e] = uv[it][0];
                rows_w[2 * e + 1] = (wc == 1) ? uv[it][1] : ((wc == 2) ? uv[it][2] : uv[it][3]);
            }
        }
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            const int x0 = blk.x() * P, kk = a.kbeg + blk.y();
#pragma unroll
            for (int h = 0; h < NBX; h++) {
                const int py = (AX == 1) ? h * BXR : kk, pz = (AX == 1) ? kk : h * BXR;
                tma_store_3d(&tm->u_out, 5 * x0, py, pz, rows_u + h * BXR * 5 * kSweepP);
                if (wc)
                    tma_store_3d(&tm->w_out, 2 * x0, py, pz, rows_w + h * BXR * 2 * kSweepP);
            }
            tma_store_commit();
            tma_store_wait_read();  // the CTA may leave once its buffers are read
        }
    }
}

template <typename R, bool EX, int C, int T, int AX = 0>
__global__ void __launch_bounds__(AX ? kSweepP * T : 256, AX ? (T <= 64 ? 3 : 1) : 0)
    k_fluidx2(FluidxArgs a, const __grid_constant__ SweepMaps tm)
{
    fluidx2_body<R, EX, C, T, AX>(a, &tm, HwBlock{});
}

}  // namespace mhd

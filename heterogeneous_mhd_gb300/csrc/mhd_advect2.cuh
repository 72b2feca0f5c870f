// advectbyzx with C cells per thread (C/advectbyzx.c:14-23, A1
// C/advectbyzxA1.c:18-63, A2 C/advectbyzxA2.c:9-28, B1 C/advectbyzxB1.c:19-62,
// B2 C/advectbyzxB2.c:9-28, tvdb C/tvdb.c:10-91).
//
// A CTA owns P consecutive pencils (j0..j0+P-1, k) and computes 3P+1 tvdb
// rows: A rows for pencils j0..j0+P at plane k (b(2) advected with the face
// velocity of pencils j-1, j) and B rows for pencils j0..j0+P-1 at planes k
// and k+1 (b(3) with pencils k-1, k).  Every row is owned by T = n/C threads
// holding C consecutive cells; the tvdb stencil moves between threads by
// shuffles.  The per-cell EMFs of the neighbour rows meet in shared memory and
// the A-row threads of each owned pencil apply the float updates in the order
// of A1, A2, B1, B2:
//   b1_out = (((b1 - FA(j,k)) + FA(j+1,k)) - FB(j,k)) + FB(j,k+1).
#pragma once
#include "mhd_kernels.cuh"
#include "mhd_pencil.cuh"

namespace mhd {

// Per-cell steps of tvdb, shared by every advectbyzx kernel.  EXACT: the
// reference's expressions (compiled without contraction).  FAST: every
// rounding is explicit (__fadd_rn, __fmul_rn and __fmaf_rn are never
// contracted), so all kernels compute the same bits whatever the compiler
// does around the calls.
__device__ __forceinline__ float r_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double r_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float r_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double r_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float r_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double r_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float r_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double r_fma(double a, double b, double c) { return __fma_rn(a, b, c); }

// Raw face velocity (C/advectbyzxA1.c:34, C/advectbyzxB1.c:34) from m_x and
// rho of the pencil below (m) and the current one (c).
template <typename R, bool EX>
__device__ __forceinline__ R tvdb_face(R mm, R mc, R rm, R rc)
{
    if constexpr (EX)
        return (mm + mc) / (rm + rc);
    else
        return fast_div(r_add(mm, mc), r_add(rm, rc));
}

// 1-2-1 smoothing of the face velocity (C/advectbyzxA1.c:36-41): vm, v, vp at i-1, i, i+1.
template <typename R, bool EX>
__device__ __forceinline__ R tvdb_smooth(R vm, R v, R vp)
{
    using W = wide_t<R, EX>;
    if constexpr (EX)
        return R((W(vm + vp) + W(2.0) * W(v)) / W(4.0));
    else
        return r_mul(r_fma(R(2), v, r_add(vm, vp)), R(0.25));
}

// b vg (C/tvdb.c:31-34), vg b1 (C/tvdb.c:55-60)
template <typename R, bool EX>
__device__ __forceinline__ R tvdb_prod(R x, R y)
{
    if constexpr (EX)
        return x * y;
    else
        return r_mul(x, y);
}

// vh = (vg(i) + vg(i+1)) / 2 in the abXYc form (C/tvdb.c:25-29)
template <typename R, bool EX>
__device__ __forceinline__ R tvdb_vh(R vg, R vgn)
{
    if constexpr (EX)
        return lin<R, EX>(R(0.5), vg, R(0.5), vgn);
    else
        return r_fma(R(0.5), vg, r_mul(R(0.5), vgn));
}

// Half step b1 = b - (f1(i) - f1(i-1)) dt / 2 (C/tvdb.c:41-47).
template <typename R, bool EX>
__device__ __forceinline__ R tvdb_half(R bv, R f1, R fm, R dt)
{
    using W = wide_t<R, EX>;
    if constexpr (EX)
        return R(W(bv) - W((f1 - fm) * dt) / W(2.0));
    else  // dt / 2 is loop-invariant: one fused multiply-add per cell
        return r_fma(r_sub(fm, f1), r_mul(dt, R(0.5)), bv);
}

// Limited upwind flux times dt at i+1/2 (C/tvdb.c:54-78) from vb = vg b1 at
// i-1, i, i+1, i+2 and the sign of vh(i).
template <typename R, bool EX>
__device__ __forceinline__ R tvdb_flux(R vbm, R vb0, R vbp, R vbpp, R vh, R dt)
{
    if constexpr (EX) {
        using W = wide_t<R, EX>;
        R w, wp, wm;
        if (vh > R(0)) {
            w = vb0;
            wp = R(W(vbp - w) / W(2.0));
            wm = R(W(w - vbm) / W(2.0));
        } else {
            w = vbp;
            wp = R(W(w - vbpp) / W(2.0));
            wm = R(W(vb0 - w) / W(2.0));
        }
        const R dw = vanleer<R, EX>(wm, wp);
        return (w + dw) * dt;
    } else {
        // The same differences with the operands selected (no branch), and the
        // limiter on the undivided differences: with wm = dm/2, wp = dp/2,
        // 2 wm wp / (wm + wp) = dm dp / (dm + dp).
        const bool up = vh > R(0);
        const R w = up ? vb0 : vbp;
        const R dp = r_sub(vbp, up ? vb0 : vbpp);
        const R dm = r_sub(vb0, up ? vbm : vbp);
        const R p = r_mul(dm, dp);
        const R dw = (p > R(0)) ? fast_div(p, r_add(dm, dp)) : R(0);
        return r_mul(r_add(w, dw), dt);
    }
}

// Advected field b - (flux(i) - flux(i-1)) (C/tvdb.c:79-88)
template <typename R, bool EX>
__device__ __forceinline__ R tvdb_new(R bv, R flux, R fm)
{
    if constexpr (EX)
        return bv - (flux - fm);
    else
        return r_sub(bv, r_sub(flux, fm));
}

// One tvdb row held by T threads with C cells each: from the raw face
// velocity vr (C/advectbyzxA1.c:31-35) and the advected field bv, the 1-2-1
// smoothing (C/advectbyzxA1.c:36-41) and tvdb (C/tvdb.c:10-91).  Returns
// F(i) = flux(i-1) (the EMF times dt used by the CT update) and the advected
// field.  Seven neighbour exchanges; for T > 32 each is one block barrier.
template <typename R, bool EX, int C, int T, bool NM>
__device__ __forceinline__ void tvdb_row(const Group<R, T, NM>& g, const R (&vr)[C], const R (&bv)[C], R dt, R* seam,
                                         R (&F)[C], R (&bnew)[C])
{
    // ---- 1-2-1 smoothing (C/advectbyzxA1.c:36-41)
    R vg[C];
    {
        R l[1], rr[1], x0[1] = {vr[C - 1]}, x1[1] = {vr[0]};
        g.template shift<1>(x0, l, -1, seam, 0);
        g.template shift<1>(x1, rr, +1, seam, 1);
#pragma unroll
        for (int m = 0; m < C; m++) {
            const R vm = (m > 0) ? vr[m - 1] : l[0];
            const R vp = (m + 1 < C) ? vr[m + 1] : rr[0];
            vg[m] = tvdb_smooth<R, EX>(vm, vr[m], vp);
        }
    }
    // ---- tvdb half step (C/tvdb.c:25-52)
    R vh[C], b1[C];
    {
        R t2[C];
#pragma unroll
        for (int m = 0; m < C; m++)
            t2[m] = tvdb_prod<R, EX>(bv[m], vg[m]);
        R xs[2] = {vg[0], t2[0]}, xr[2];
        g.template shift<2>(xs, xr, +1, seam, 0);
        R f1[C];
#pragma unroll
        for (int m = 0; m < C; m++) {
            const R vgn = (m + 1 < C) ? vg[m + 1] : xr[0];
            const R t2n = (m + 1 < C) ? t2[m + 1] : xr[1];
            vh[m] = tvdb_vh<R, EX>(vg[m], vgn);
            f1[m] = (vh[m] > R(0)) ? t2[m] : t2n;
        }
        R fl[1], fx[1] = {f1[C - 1]};
        g.template shift<1>(fx, fl, -1, seam, 1);
#pragma unroll
        for (int m = 0; m < C; m++) {
            const R fm = (m > 0) ? f1[m - 1] : fl[0];
            b1[m] = tvdb_half<R, EX>(bv[m], f1[m], fm, dt);
        }
    }
    // ---- limited upwind flux (C/tvdb.c:54-78)
    R flux[C];
    {
        R vb[C];
#pragma unroll
        for (int m = 0; m < C; m++)
            vb[m] = tvdb_prod<R, EX>(vg[m], b1[m]);
        R l[1], x0[1] = {vb[C - 1]};
        g.template shift<1>(x0, l, -1, seam, 0);
        R xs[2] = {vb[0], vb[1 < C ? 1 : 0]}, xr[2];
        g.template shift<2>(xs, xr, +1, seam, 1);
        // right neighbour's first two values; for C == 1 the second is two threads away
#pragma unroll
        for (int m = 0; m < C; m++) {
            const R vbm = (m > 0) ? vb[m - 1] : l[0];
            const R vbp = (m + 1 < C) ? vb[m + 1] : xr[0];
            const R vbpp = (m + 2 < C) ? vb[m + 2] : ((m + 2 == C) ? xr[0] : xr[1]);
            flux[m] = tvdb_flux<R, EX>(vbm, vb[m], vbp, vbpp, vh[m], dt);
        }
    }
    // ---- b - (flux - flux(i-1)) (C/tvdb.c:79-88) and F(i) = flux(i-1)
    {
        R l[1], x0[1] = {flux[C - 1]};
        g.template shift<1>(x0, l, -1, seam, 0);
#pragma unroll
        for (int m = 0; m < C; m++) {
            F[m] = (m > 0) ? flux[m - 1] : l[0];
            bnew[m] = tvdb_new<R, EX>(bv[m], flux[m], F[m]);
        }
    }
}

__host__ __device__ inline int advect2_rows(int P) { return 3 * P + 1; }

// rows padded so that rows*T is a whole number of warps
__host__ __device__ inline int advect2_threads(int P, int T)
{
    const int t = advect2_rows(P) * T;
    return ((t + 31) / 32) * 32;
}

// shared memory (elements of R): FX [rows][n] + BN of the B rows at k [P][n] + seam
__host__ __device__ inline size_t advect2_smem_elems(int n, int P)
{
    return (size_t)(advect2_rows(P) + P) * n + 2 * 32 * kSeamVals;
}

template <typename R, bool EX, int C, int T>
__global__ void __launch_bounds__(512) k_advect2(AdvectArgs a)
{
    select_box(a, blockIdx.z);
    using W = wide_t<R, EX>;
    constexpr int n = C * T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int P = a.P;
    const int NR = advect2_rows(P);
    const int tid = threadIdx.x;
    const Group<R, T> g(tid);
    int r = tid / T;
    const bool live = r < NR;  // padding rows compute row 0 again and write nothing
    if (!live)
        r = 0;
    const int i0 = g.t * C;
    const int ny = a.ny, nz = a.nz;
    const int j0 = blockIdx.x * P, k = blockIdx.y;
    const int kp = (k + 1 == nz) ? 0 : k + 1;

    R* FXs = reinterpret_cast<R*>(smem_raw);  // [NR][n]: F(i) = flux(i-1) of each row
    R* BNs = FXs + (size_t)NR * n;            // [P][n]: advected b(3) of the B rows at k
    R* seam = BNs + (size_t)P * n;

    const R* uu = static_cast<const R*>(a.uu);
    const R* ub = static_cast<const R*>(a.ub);
    const R dt = load_dt<R>(a.dt_ptr, a.dt_val);

    // the two u pencils and the advected component of this row
    size_t pm, pc;
    int comp;
    if (r <= P) {
        int j = j0 + r;
        if (j >= ny)
            j -= ny;
        const int jm = (j == 0) ? ny - 1 : j - 1;
        pm = ((size_t)k * ny + jm) * n;
        pc = ((size_t)k * ny + j) * n;
        comp = 1;
    } else {
        const int r2 = r - (P + 1);
        const int p = (r2 < P) ? r2 : r2 - P;
        const int kk = (r2 < P) ? k : kp;
        const int kkm = (kk == 0) ? nz - 1 : kk - 1;
        pm = ((size_t)kkm * ny + j0 + p) * n;
        pc = ((size_t)kk * ny + j0 + p) * n;
        comp = 2;
    }

    // ---- raw face velocity (C/advectbyzxA1.c:31-35) and the advected field
    R vr[C], bv[C], b1own[C];
    {
        R um[C * 5], uc[C * 5], bb[C * 3];
        ldg_chunk<R, C * 5>(uu + (pm + i0) * 5, um);
        ldg_chunk<R, C * 5>(uu + (pc + i0) * 5, uc);
        ldg_chunk<R, C * 3>(ub + (pc + i0) * 3, bb);
#pragma unroll
        for (int m = 0; m < C; m++) {
            const R num = um[5 * m + 1] + uc[5 * m + 1], den = um[5 * m] + uc[5 * m];
            if constexpr (EX)
                vr[m] = num / den;
            else
                vr[m] = fast_div(num, den);
            bv[m] = (comp == 1) ? bb[3 * m + 1] : bb[3 * m + 2];
            b1own[m] = bb[3 * m];
        }
    }
    R bnew[C], F[C];
    tvdb_row<R, EX, C, T>(g, vr, bv, dt, seam, F, bnew);
    if (live) {
        R* fx = FXs + (size_t)r * n + i0;
#pragma unroll
        for (int m = 0; m < C; m++)
            fx[m] = F[m];
        if (r > P && r <= 2 * P) {
            R* bn = BNs + (size_t)(r - P - 1) * n + i0;
#pragma unroll
            for (int m = 0; m < C; m++)
                bn[m] = bnew[m];
        }
    }
    __syncthreads();
    // ---- A1/A2/B1/B2 combine by the A-row threads of the owned pencils
    if (live && r < P) {
        const size_t cell0 = pc + i0;  // pencil (j0+r, k)
        const R* b1s = static_cast<const R*>(a.b1_src);
        if (b1s != ub) {
            R bb[C * 3];
            ldg_chunk<R, C * 3>(b1s + cell0 * 3, bb);
#pragma unroll
            for (int m = 0; m < C; m++)
                b1own[m] = bb[3 * m];
        }
        R out[C * 3];
        const R* fa1 = FXs + (size_t)(r + 1) * n + i0;
        const R* fb = FXs + (size_t)(P + 1 + r) * n + i0;
        const R* fbp = FXs + (size_t)(2 * P + 1 + r) * n + i0;
        const R* b3 = BNs + (size_t)r * n + i0;
#pragma unroll
        for (int m = 0; m < C; m++) {
            R x = b1own[m];
            x = x - F[m];
            x = x + fa1[m];
            x = x - fb[m];
            x = x + fbp[m];
            out[3 * m] = x;
            out[3 * m + 1] = bnew[m];
            out[3 * m + 2] = b3[m];
        }
        stg_chunk<R, C * 3>(static_cast<R*>(a.b_out) + cell0 * 3, out);
    }
}

}  // namespace mhd

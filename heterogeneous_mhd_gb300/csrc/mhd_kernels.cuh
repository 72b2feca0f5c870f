// sm_103a kernels of the relaxing-TVD split MHD step.
//
// Layout (C/array_definition.h:12): u(5,nx,ny,nz), b(3,nx,ny,nz), component
// innermost, so one x-pencil of u is one contiguous run of 5*nx values and a
// group of P consecutive pencils (j0..j0+P-1 at fixed k) is one contiguous run
// of 5*nx*P values.  Every kernel works on x-pencils, as the reference does.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "mhd_math.cuh"
#include "mhd_ptx.cuh"

namespace mhd {

// ------------------------------------------------------------------ params

// Batched launches: the boxes of one size class lie at a fixed byte stride
// from each other in every array, and the box index is blockIdx.z (for the
// transposes blockIdx.z / their own z extent).  Zero strides = one box.
struct BoxStrides {
    size_t u = 0;   // bytes between the u arrays of consecutive boxes
    size_t b = 0;   // bytes between the b arrays
    size_t dt = 0;  // bytes between the device clocks (dt) of consecutive boxes
    size_t w = 0;   // bytes between the (rho, m_x) side arrays
    int count = 1;  // boxes in the launch (the launchers' grid z extent)
};

// size classes in one work-list launch (mhd_multi.cuh)
constexpr int kMaxSegs = 8;

template <typename P>
__device__ __forceinline__ P* box_ptr(P* p, size_t stride, int box)
{
    using C = typename std::conditional<std::is_const<P>::value, const char, char>::type;
    return p ? reinterpret_cast<P*>(reinterpret_cast<C*>(p) + stride * (size_t)box) : p;
}

struct FluidxArgs {
    void* u_out;          // u <- sweep(update_u)
    const void* uu;       // update_u
    const void* ub;       // update_b
    int nx, ny, nz;
    int P;                // pencils per CTA along j (ny % P == 0)
    int use_tma;          // stage pencils with bulk TMA (alignment checked on the host)
    double dt_val;        // dt when dt_ptr == nullptr
    const void* dt_ptr;   // device dt (type R) written by the CFL finalize kernel
    void* cfl_part;       // optional fused calcfl epilogue: per-CTA partials (CflPart<R>)
    int* err;
    BoxStrides bs;
    int axis;             // sweep axis of the untransposed state: 0 x (the drop-in call), 1 y, 2 z
    void* w_out;          // optional (FP32): (rho, m) of the new state, 2 values per cell, x-major:
                          // m = m_x on the x sweep, on the y/z sweeps the momentum component w_comp
    int w_comp;           // y/z sweeps: raw component of u written with rho (1 m_x, 2 m_y, 3 m_z)
    int kbeg, kcount;     // planes along z to update: kbeg .. kbeg+kcount-1 (kcount 0: all); the
                          // neighbours of the range's edge planes are read as usual (periodic box)
};

struct AdvectArgs {
    void* b_out;          // b(2), b(3) <- advected, b(1) <- CT update of b1_src
    const void* b1_src;   // where b(1) is read from (the reference reads b in place)
    const void* uu;       // update_u
    const void* ub;       // update_b
    int nx, ny, nz;
    int P;                // output pencils per CTA along j (ny % P == 0)
    double dt_val;
    const void* dt_ptr;
    int* err;
    int K;                // planes per CTA along k for the marching kernel (nz % K == 0)
    BoxStrides bs;
    int axis;             // sweep axis of the untransposed state: 0 x (the drop-in call), 1 y, 2 z
    const void* w;        // optional (FP32): (rho, m_d) of update_u, 2 values per cell, x-major, m_d the
                          // momentum along the sweep (the fluidx before wrote it)
    int kbeg, kcount;     // planes along z to update (kcount 0: all), as in FluidxArgs
};

struct TransposeArgs {
    void* u_out;
    void* b_out;
    const void* uu;
    const void* ub;
    int nx, ny, nz;
    int axis;             // 1: x<->y (transpose12), 2: x<->z (transpose13, nx == nz)
    BoxStrides bs;
    void* w_out;          // optional (FP32 tiled kernel): (rho, m_x) of the output, 2 values per cell
    int* err = nullptr;   // optional: the bulk-TMA tile kernel sets DEVERR_TIMEOUT here when a copy never lands
};

// Coordinates of a CTA in the grid of its size class.  HwBlock reads the
// hardware registers (a launch over one class); VBlock holds the coordinates
// that a work-list launch over several classes (mhd_multi.cuh) derived from
// the CTA's position in it.  Kernel bodies take either, so the one-class
// kernels compile to the same code as before.
struct HwBlock {
    __device__ __forceinline__ int x() const { return (int)blockIdx.x; }
    __device__ __forceinline__ int y() const { return (int)blockIdx.y; }
    __device__ __forceinline__ int z() const { return (int)blockIdx.z; }
    __device__ __forceinline__ int gx() const { return (int)gridDim.x; }
    __device__ __forceinline__ int gy() const { return (int)gridDim.y; }
};

struct VBlock {
    int bx, by, bz, ngx, ngy;
    __device__ __forceinline__ int x() const { return bx; }
    __device__ __forceinline__ int y() const { return by; }
    __device__ __forceinline__ int z() const { return bz; }
    __device__ __forceinline__ int gx() const { return ngx; }
    __device__ __forceinline__ int gy() const { return ngy; }
};

// Offset every array of a launch to box `box` (the per-CTA partials of the
// CFL epilogue too: `ctas` partials per box, one per CTA of a box's grid).
__device__ __forceinline__ void select_box(FluidxArgs& a, int box, size_t part_bytes, int ctas)
{
    a.u_out = box_ptr(a.u_out, a.bs.u, box);
    a.uu = box_ptr(a.uu, a.bs.u, box);
    a.ub = box_ptr(a.ub, a.bs.b, box);
    a.dt_ptr = box_ptr(a.dt_ptr, a.bs.dt, box);
    a.cfl_part = box_ptr(a.cfl_part, part_bytes * (size_t)ctas, box);
    a.w_out = box_ptr(a.w_out, a.bs.w, box);
}

__device__ __forceinline__ void select_box(AdvectArgs& a, int box)
{
    a.b_out = box_ptr(a.b_out, a.bs.b, box);
    a.b1_src = box_ptr(a.b1_src, a.bs.b, box);
    a.uu = box_ptr(a.uu, a.bs.u, box);
    a.ub = box_ptr(a.ub, a.bs.b, box);
    a.dt_ptr = box_ptr(a.dt_ptr, a.bs.dt, box);
    a.w = box_ptr(a.w, a.bs.w, box);
}

__device__ __forceinline__ void select_box(TransposeArgs& a, int box)
{
    a.u_out = box_ptr(a.u_out, a.bs.u, box);
    a.b_out = box_ptr(a.b_out, a.bs.b, box);
    a.uu = box_ptr(a.uu, a.bs.u, box);
    a.ub = box_ptr(a.ub, a.bs.b, box);
    a.w_out = box_ptr(a.w_out, a.bs.w, box);
}

template <typename R>
struct CflPart {          // one per CTA of a CFL reduction
    R cmax;               // max over the CTA's non-NaN speeds (>= 0)
    int last_nan;         // largest linear index of a NaN speed in the CTA, or -1
    int pad;
};

struct CflFinalizeArgs {
    const void* part;     // CflPart<R>[nparts]
    int nparts;
    const void* u;        // state, for the rescan after a NaN cell
    const void* b;
    int nx, ny, nz;
    double cfl;           // dt = cfl * (1/c) in double, as C/mhd.c:62 does with 0.9
    int advance;          // 1: clamp dt to (tf-t)/2 and advance t (the time loop)
    void* clock;          // R[4]: t, tf, dt, 1/c
    long long* nsteps;    // incremented when advance
    int* err;
    BoxStrides bs;        // batched: u, b and clock strides; nparts is per box
    void* scratch;        // optional (one box): room for kCflReduceCtas CflPart<R> of a first-level reduction
};

// ------------------------------------------------------------- reductions

template <typename R>
__device__ __forceinline__ R warp_max(R x)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}

// Max over the n cells of the caller's pencil, starting from 0 and skipping
// NaN (find_max, C/mhdflux.c:61-72).  Contains one __syncthreads; red must not
// be read by a previous call that is not separated by another barrier.
template <typename R>
__device__ __forceinline__ R pencil_max(R x, R* red, int n, int lp)
{
    if ((n & 31) == 0) {
        R m = warp_max(x);
        const int w = threadIdx.x >> 5;
        if ((threadIdx.x & 31) == 0)
            red[w] = m;
        __syncthreads();
        const int wpp = n >> 5, w0 = lp * wpp;
        R c = R(0);
        for (int s = 0; s < wpp; s++)
            c = fmax(c, red[w0 + s]);
        return c;
    }
    red[threadIdx.x] = x;
    __syncthreads();
    R c = R(0);
    const R* row = red + lp * n;
    for (int s = 0; s < n; s++)
        c = fmax(c, row[s]);
    return c;
}

// --------------------------------------------------------------- staging

// Copy `count` elements global -> shared cooperatively (fallback when the
// bulk-TMA alignment rules do not hold).
template <typename R>
__device__ __forceinline__ void coop_copy(R* dst, const R* src, size_t count)
{
    for (size_t e = threadIdx.x; e < count; e += blockDim.x)
        dst[e] = src[e];
}

template <typename R>
__device__ __forceinline__ R load_dt(const void* dt_ptr, double dt_val)
{
    return dt_ptr ? *static_cast<const R*>(dt_ptr) : R(dt_val);
}

// ----------------------------------------------------------------- fluidx

// Shared memory (elements of R) used by k_fluidx for n cells and P pencils.
__host__ __device__ inline int fluidx_threads(int n, int P) { return ((n * P + 31) / 32) * 32; }

__host__ __device__ inline size_t fluidx_smem_elems(int n, int P)
{
    // su 5nP, sb 3n(P+1), sbk 3nP, xa 10nP, xb 10nP, red max(threads, 64)
    size_t np = (size_t)n * P;
    size_t th = (size_t)fluidx_threads(n, P);
    size_t red = th > 64 ? th : 64;
    return 5 * np + 3 * (np + n) + 3 * np + 20 * np + red;
}

// fluidx (C/fluidx.c:19-102) with tvd1 (C/tvd1.c:8-118) and mhdflux
// (C/mhdflux.c:9-72).  One thread per cell, P whole pencils per CTA (the
// relaxing speed c is a max over the whole pencil, taken twice).  The
// pencils of u and b are staged into shared memory with bulk TMA; the
// neighbour stencil is exchanged through shared memory between barriers.
// Optionally (cfl_part != nullptr) the epilogue evaluates calcfl's per-cell
// speed on the new u and the face b, and writes one partial max per CTA.
template <typename R, bool EX>
__global__ void __launch_bounds__(512) k_fluidx(FluidxArgs a)
{
    select_box(a, blockIdx.z, sizeof(CflPart<R>), gridDim.x * gridDim.y);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = a.nx, P = a.P;
    const int np = n * P;
    const int t = threadIdx.x;
    // The block is rounded up to whole warps; the extra threads shadow cell 0
    // (so warp-wide shuffles see full warps) and never write.
    const bool act = t < np;
    const int tt = act ? t : 0;
    const int lp = tt / n, i = tt - lp * n;
    const int j0 = blockIdx.x * P, k = blockIdx.y;
    const int kp = (k + 1 == a.nz) ? 0 : k + 1;
    const int jn = (j0 + P == a.ny) ? 0 : j0 + P;

    R* su = reinterpret_cast<R*>(smem_raw);
    R* sb = su + 5 * np;           // rows j0..j0+P-1 and jn at plane k
    R* sbk = sb + 3 * (np + n);    // rows j0..j0+P-1 at plane kp
    R* xa = sbk + 3 * np;          // exchange buffer A (10 per cell)
    R* xb = xa + 10 * np;          // exchange buffer B (10 per cell)
    R* red = xb + 10 * np;
    __shared__ uint64_t bar;

    const R* uu = static_cast<const R*>(a.uu);
    const R* ub = static_cast<const R*>(a.ub);
    const size_t c0 = ((size_t)k * a.ny + j0) * n;   // first cell of the group
    const size_t cn = ((size_t)k * a.ny + jn) * n;   // pencil after the group
    const size_t ck = ((size_t)kp * a.ny + j0) * n;  // group at kp

    if (a.use_tma) {
        if (t == 0) {
            mbar_init(&bar, 1);
            const uint32_t bu = 5u * np * sizeof(R), bg = 3u * np * sizeof(R), b1 = 3u * n * sizeof(R);
            mbar_arrive_expect_tx(&bar, bu + 2 * bg + b1);
            tma_load_1d(su, uu + c0 * 5, bu, &bar);
            tma_load_1d(sb, ub + c0 * 3, bg, &bar);
            tma_load_1d(sb + 3 * np, ub + cn * 3, b1, &bar);
            tma_load_1d(sbk, ub + ck * 3, bg, &bar);
        }
        __syncthreads();
        if (!__syncthreads_and(mbar_wait_bounded(&bar, 0, a.err)))
            return;  // the copy never landed (error bit set): leave before computing on it
    } else {
        coop_copy(su, uu + c0 * 5, (size_t)5 * np);
        coop_copy(sb, ub + c0 * 3, (size_t)3 * np);
        coop_copy(sb + 3 * np, ub + cn * 3, (size_t)3 * n);
        coop_copy(sbk, ub + ck * 3, (size_t)3 * np);
        __syncthreads();
    }

    const R dt = load_dt<R>(a.dt_ptr, a.dt_val);
    const int ip = (i + 1 == n) ? 0 : i + 1;
    const int im = (i == 0) ? n - 1 : i - 1;
    const int me = lp * n + i, mep = lp * n + ip, mem = lp * n + im;

    R q[5], f[3];
#pragma unroll
    for (int c = 0; c < 5; c++)
        q[c] = su[5 * me + c];
    {   // cell-centred B (C/fluidx.c:71-81): b/2 + b(neighbour face)/2
        const R* bj = sb + 3 * lp * n;
        const R* bjp = sb + 3 * (lp + 1) * n;
        const R* bkp = sbk + 3 * lp * n;
        const R h0 = R(0.5) * bj[3 * i], h0p = R(0.5) * bj[3 * ip];
        f[0] = h0 + h0p;
        f[1] = R(0.5) * bj[3 * i + 1] + bjp[3 * i + 1] / R(2);
        f[2] = R(0.5) * bj[3 * i + 2] + bkp[3 * i + 2] / R(2);
    }

    // ---- stage 1 (C/tvd1.c:33-49)
    R v[5], ci, fr[5], flux[5], u1[5];
    cell_flux<R, EX>(q, f, v, ci);
    R c = pencil_max<R>(ci, red, n, lp);
    scale_flux<R, EX>(v, c);
#pragma unroll
    for (int s = 0; s < 5; s++) {
        const R wr = lin<R, EX>(R(1), q[s], R(1), v[s]);
        const R wl = lin<R, EX>(R(1), q[s], R(-1), v[s]);
        fr[s] = scale0<R, EX>(c, wr);
        if (act)
            xa[5 * me + s] = scale0<R, EX>(c, wl);  // fl(i-1) = c*wl(i)
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < 5; s++) {
        flux[s] = lin<R, EX>(R(0.5), fr[s], R(-0.5), xa[5 * mep + s]);
        if (act)
            xb[5 * me + s] = flux[s];
    }
    __syncthreads();
    {
        using W = wide_t<R, EX>;
        const R hdt = R(W(-1.0) * W(dt) / W(2.0));
#pragma unroll
        for (int s = 0; s < 5; s++)
            u1[s] = lin<R, EX>(R(1), q[s], hdt, lin<R, EX>(R(1), flux[s], R(-1), xb[5 * mem + s]));
    }

    // ---- stage 2 (C/tvd1.c:51-116)
    cell_flux<R, EX>(u1, f, v, ci);
    c = pencil_max<R>(ci, red, n, lp);
    scale_flux<R, EX>(v, c);
    R g[5];
#pragma unroll
    for (int s = 0; s < 5; s++) {
        const R wr = lin<R, EX>(R(1), u1[s], R(1), v[s]);
        const R wl = lin<R, EX>(R(1), u1[s], R(-1), v[s]);
        fr[s] = scale0<R, EX>(c, wr);
        g[s] = scale0<R, EX>(c, wl);
        if (act) {
            xa[5 * me + s] = fr[s];
            xa[5 * (np + me) + s] = g[s];
        }
    }
    __syncthreads();
    R gp[5];
#pragma unroll
    for (int s = 0; s < 5; s++) {
        gp[s] = xa[5 * (np + mep) + s];                                   // fl(i) = g(i+1)
        const R dfrm = lin<R, EX>(R(0.5), fr[s], R(-0.5), xa[5 * mem + s]);
        const R dflm = lin<R, EX>(R(0.5), g[s], R(-0.5), gp[s]);
        if (act) {
            xb[5 * me + s] = dfrm;
            xb[5 * (np + me) + s] = dflm;
        }
    }
    __syncthreads();
#pragma unroll
    for (int s = 0; s < 5; s++) {
        // dfrp(i) = dfrm(i+1), dflp(i) = dflm(i+1)
        const R dfr = vanleer<R, EX>(xb[5 * mep + s], xb[5 * me + s]);
        const R dfl = vanleer<R, EX>(xb[5 * (np + mep) + s], xb[5 * (np + me) + s]);
        const R t1 = lin<R, EX>(R(1), fr[s], R(-1), gp[s]);
        const R t2 = lin<R, EX>(R(1), dfr, R(-1), dfl);
        flux[s] = lin<R, EX>(R(0.5), t1, R(0.5), t2);
        if (act)
            xa[5 * me + s] = flux[s];
    }
    __syncthreads();
    {
        using W = wide_t<R, EX>;
        const R mdt = R(W(-1.0) * W(dt));
#pragma unroll
        for (int s = 0; s < 5; s++) {
            const R un = lin<R, EX>(R(1), q[s], mdt, lin<R, EX>(R(1), flux[s], R(-1), xa[5 * mem + s]));
            q[s] = un;
            if (act)
                su[5 * me + s] = un;  // own slot: no other thread reads su after staging
        }
    }

    // ---- optional calcfl epilogue on the new state
    if (a.cfl_part) {
        const R* bj = sb + 3 * lp * n;
        const R fc[3] = {bj[3 * i], bj[3 * i + 1], bj[3 * i + 2]};
        const R sp = act ? cfl_speed<R, EX>(q, fc) : R(0);
        const bool isn = (sp != sp);
        R m = warp_max<R>(isn ? R(0) : sp);
        int ln = isn ? (int)(c0 + me) : -1;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            ln = max(ln, __shfl_xor_sync(0xffffffffu, ln, o));
        R* rm = red;                       // reuse: last read of red was before 3 barriers
        int* rn = reinterpret_cast<int*>(red + 32);
        const int w = t >> 5;
        if ((t & 31) == 0) {
            rm[w] = m;
            rn[w] = ln;
        }
        __syncthreads();
        if (t == 0) {
            R cm = R(0);
            int lnan = -1;
            for (int s = 0; s < (int)((blockDim.x + 31) >> 5); s++) {
                cm = fmax(cm, rm[s]);
                lnan = max(lnan, rn[s]);
            }
            CflPart<R>* part = static_cast<CflPart<R>*>(a.cfl_part) + (blockIdx.y * gridDim.x + blockIdx.x);
            part->cmax = cm;
            part->last_nan = lnan;
        }
    }

    // ---- write the new u pencils
    R* uo = static_cast<R*>(a.u_out);
    if (a.use_tma) {
        fence_proxy_async_smem();
        __syncthreads();
        if (t == 0) {
            tma_store_1d(uo + c0 * 5, su, 5u * np * sizeof(R));
            tma_store_commit();
            tma_store_wait_all();
        }
    } else {
        __syncthreads();
        for (size_t e = t; e < (size_t)5 * np; e += blockDim.x)
            uo[c0 * 5 + e] = su[e];
    }
}

// ------------------------------------------------------------- advectbyzx

// Rows of tvdb work per CTA: A rows for pencils j0..j0+P (P+1), B rows for
// (j0..j0+P-1, k) and (j0..j0+P-1, kp) (2P).
__host__ __device__ inline int advect_rows(int P) { return 3 * P + 1; }

__host__ __device__ inline size_t advect_smem_elems(int n, int P)
{
    return (size_t)7 * advect_rows(P) * n;  // VR/BN, VG, BV, T2/VB, F1, FX, VH
}

// advectbyzx (C/advectbyzx.c:14-23) = A1 (C/advectbyzxA1.c:18-63), A2
// (C/advectbyzxA2.c:9-28), B1 (C/advectbyzxB1.c:19-62), B2
// (C/advectbyzxB2.c:9-28) with tvdb (C/tvdb.c:10-91), fused into one pass:
//   b1_out(i,j,k) = (((b1 - FA(i,j,k)) + FA(i,j+1,k)) - FB(i,j,k)) + FB(i,j,k+1)
// (the order in which A1, A2, B1, B2 apply their float updates), where
// F*(i,j,k) is tvdb's flux at i-1 for pencil (j,k).  A CTA owns P pencils
// along j and recomputes the neighbour tvdb rows it needs (j0+P for A, kp for
// B) instead of exchanging EMFs through global scratch.
template <typename R, bool EX>
__global__ void __launch_bounds__(512) k_advect(AdvectArgs a)
{
    select_box(a, blockIdx.z);
    using W = wide_t<R, EX>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = a.nx, P = a.P;
    const int NR = advect_rows(P);
    const int items = NR * n;
    const int j0 = blockIdx.x * P, k = blockIdx.y;
    const int ny = a.ny, nz = a.nz;
    const int km = (k == 0) ? nz - 1 : k - 1;
    const int kp = (k + 1 == nz) ? 0 : k + 1;

    R* VR = reinterpret_cast<R*>(smem_raw);  // raw face velocity, later the advected b
    R* VG = VR + items;                      // smoothed face velocity
    R* BV = VG + items;                      // the advected component before the update
    R* T2 = BV + items;                      // b*vg, later vg*b1
    R* F1 = T2 + items;                      // half-step flux
    R* FX = F1 + items;                      // tvdb flux (EMF*dt at i+1/2)
    R* VH = FX + items;                      // vh

    const R* uu = static_cast<const R*>(a.uu);
    const R* ub = static_cast<const R*>(a.ub);
    const R dt = load_dt<R>(a.dt_ptr, a.dt_val);

    // Row r -> (pencil below pm, pencil pc, advected component).
    auto row_cells = [&](int r, size_t& pm, size_t& pc, int& comp) {
        if (r <= P) {  // A row: pencil j = j0+r, neighbour jm = j-1, advects b(2)
            int j = j0 + r;
            if (j >= ny) j -= ny;
            int jm = (j == 0) ? ny - 1 : j - 1;
            pm = ((size_t)k * ny + jm) * n;
            pc = ((size_t)k * ny + j) * n;
            comp = 1;
        } else {       // B row: (j0+p, kk) with kk = k or kp, neighbour kk-1, advects b(3)
            int r2 = r - (P + 1);
            int p = (r2 < P) ? r2 : r2 - P;
            int kk = (r2 < P) ? k : kp;
            int kkm = (kk == 0) ? nz - 1 : kk - 1;
            pm = ((size_t)kkm * ny + j0 + p) * n;
            pc = ((size_t)kk * ny + j0 + p) * n;
            comp = 2;
        }
    };

    // Phase 1: raw face velocity (C/advectbyzxA1.c:31-35) and the b component.
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int r = it / n, i = it - r * n;
        size_t pm, pc;
        int comp;
        row_cells(r, pm, pc, comp);
        const R* um = uu + (pm + i) * 5;
        const R* uc = uu + (pc + i) * 5;
        VR[it] = (um[1] + uc[1]) / (um[0] + uc[0]);
        BV[it] = ub[(pc + i) * 3 + comp];
    }
    __syncthreads();
    // Phase 2: 1-2-1 smoothing (C/advectbyzxA1.c:37-41), b*vg (C/tvdb.c:31-34).
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int r = it / n, i = it - r * n;
        const int ip = (i + 1 == n) ? 0 : i + 1, im = (i == 0) ? n - 1 : i - 1;
        const R* row = VR + r * n;
        R vg;
        if constexpr (EX)
            vg = R((W(row[im] + row[ip]) + W(2.0) * W(row[i])) / W(4.0));
        else
            vg = ((row[im] + row[ip]) + R(2) * row[i]) * R(0.25);
        VG[it] = vg;
        T2[it] = BV[it] * vg;
    }
    __syncthreads();
    // Phase 3: vh and the upwind half-step flux (C/tvdb.c:25-46).
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int r = it / n, i = it - r * n;
        const int ip = (i + 1 == n) ? 0 : i + 1;
        const R vh = lin<R, EX>(R(0.5), VG[it], R(0.5), VG[r * n + ip]);
        VH[it] = vh;
        F1[it] = (vh > R(0)) ? T2[it] : T2[r * n + ip];
    }
    __syncthreads();
    // Phase 4: half step b1 (C/tvdb.c:47-52), then vg*b1.
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int r = it / n, i = it - r * n;
        const int im = (i == 0) ? n - 1 : i - 1;
        R b1;
        if constexpr (EX)
            b1 = R(W(BV[it]) - W((F1[it] - F1[r * n + im]) * dt) / W(2.0));
        else
            b1 = BV[it] - (F1[it] - F1[r * n + im]) * dt * R(0.5);
        T2[it] = VG[it] * b1;
    }
    __syncthreads();
    // Phase 5: limited upwind flux (C/tvdb.c:54-78).
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int r = it / n, i = it - r * n;
        const int ip = (i + 1 == n) ? 0 : i + 1;
        const int ipp = (ip + 1 == n) ? 0 : ip + 1;
        const int im = (i == 0) ? n - 1 : i - 1;
        const R* vb = T2 + r * n;
        R w, wp, wm;
        if (VH[it] > R(0)) {
            w = vb[i];
            wp = R(W(vb[ip] - w) / W(2.0));
            wm = R(W(w - vb[im]) / W(2.0));
        } else {
            w = vb[ip];
            wp = R(W(w - vb[ipp]) / W(2.0));
            wm = R(W(vb[i] - w) / W(2.0));
        }
        const R dw = vanleer<R, EX>(wm, wp);
        FX[it] = (w + dw) * dt;
    }
    __syncthreads();
    // Phase 6: b - (flux - flux(i-1)) (C/tvdb.c:79-88) into VR.
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int r = it / n, i = it - r * n;
        const int im = (i == 0) ? n - 1 : i - 1;
        VR[it] = BV[it] - (FX[it] - FX[r * n + im]);
    }
    __syncthreads();
    // Phase 7: combine A1/A2/B1/B2 for the P owned pencils and write b.
    const R* b1s = static_cast<const R*>(a.b1_src);
    R* bo = static_cast<R*>(a.b_out);
    for (int it = threadIdx.x; it < P * n; it += blockDim.x) {
        const int p = it / n, i = it - p * n;
        const int im = (i == 0) ? n - 1 : i - 1;
        const size_t cell = ((size_t)k * ny + j0 + p) * n + i;
        const R fa = FX[p * n + im], fa1 = FX[(p + 1) * n + im];
        const R fb = FX[(P + 1 + p) * n + im], fbp = FX[(2 * P + 1 + p) * n + im];
        R b1 = b1s[cell * 3];
        b1 = b1 - fa;
        b1 = b1 + fa1;
        b1 = b1 - fb;
        b1 = b1 + fbp;
        const R b2 = VR[p * n + i];
        const R b3 = VR[(P + 1 + p) * n + i];
        bo[cell * 3 + 0] = b1;
        bo[cell * 3 + 1] = b2;
        bo[cell * 3 + 2] = b3;
    }
    (void)km;
}

// -------------------------------------------------------------- transposes

// Component permutations: transpose12 takes u components (1,3,2,4,5) and b
// components (2,1,3) (C/transpose12.c:22-29); transpose13 takes u (1,4,3,2,5)
// and b (3,2,1) (C/transpose13.c:24-31).  Written as selects so no lookup
// table lands in local memory.
template <int AXIS>
__host__ __device__ __forceinline__ int perm_u(int c)
{
    if (AXIS == 1)
        return (c == 1) ? 2 : (c == 2) ? 1 : c;
    return (c == 1) ? 3 : (c == 3) ? 1 : c;
}
template <int AXIS>
__host__ __device__ __forceinline__ int perm_b(int c)
{
    if (AXIS == 1)
        return (c < 2) ? 1 - c : c;
    return 2 - c;
}

// Transpose tile edge in cells: 32 for float, 16 for double (static shared
// memory stays under 48 KB).
template <typename R>
struct TTile {
    static constexpr int E = (sizeof(R) == 4) ? 32 : 16;
};

// transpose12 (C/transpose12.c:7-47) and transpose13 (C/transpose13.c:9-62):
// out(a, ., i) = in(i, ., a) with the component permutation of each.  A CTA
// moves a 32x32 tile of cells through shared memory so both the reads (rows
// of x) and the writes (rows of the swapped axis) are contiguous.  Tiles at
// the edges of grids that are not multiples of 32 are partial.
//
// The body stages into su [kTT][kTT*5+1] and sb [kTT][kTT*3+1] and takes the
// CTA's block coordinates `blk` (HwBlock and static arrays in k_transpose,
// VBlock and dynamic shared memory in the work-list launch over several size
// classes, mhd_multi.cuh).  With w_out (FP32) it also writes the first two
// components of the output cells, the (rho, m_x) side array.
template <typename R>
__host__ __device__ constexpr size_t transpose_smem_bytes()
{
    return (size_t)TTile<R>::E * (TTile<R>::E * 8 + 2) * sizeof(R);
}

template <typename R, typename B>
__device__ __forceinline__ void transpose_body(TransposeArgs a, R* su, R* sb, const B& blk)
{
    constexpr int kTT = TTile<R>::E;
    constexpr int SU = kTT * 5 + 1, SB = kTT * 3 + 1;  // padded row strides
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int na = (a.axis == 1) ? ny : nz;  // extent of the swapped axis
    const int nbz = (a.axis == 1) ? nz : ny;  // extent of the untouched axis
    const int i0 = blk.x() * kTT, a0 = blk.y() * kTT, z = blk.z() % nbz;
    select_box(a, blk.z() / nbz);
    const int ti = min(kTT, nx - i0), ta = min(kTT, na - a0);
    const R* uu = static_cast<const R*>(a.uu);
    const R* ub = static_cast<const R*>(a.ub);
    R* uo = static_cast<R*>(a.u_out);
    R* bo = static_cast<R*>(a.b_out);
    R* wo = static_cast<R*>(a.w_out);

    // input cell (i, a, z) for axis 1 is (i, j=a, k=z); for axis 2 it is (i, j=z, k=a)
    const size_t rstride = (a.axis == 1) ? (size_t)nx : (size_t)nx * ny;  // cells between rows of a
    const size_t cin0 = (a.axis == 1) ? (((size_t)z * ny + a0) * nx + i0) : (((size_t)a0 * ny + z) * nx + i0);
    for (int e = threadIdx.x; e < ta * ti * 5; e += blockDim.x) {
        const int r = e / (ti * 5), c = e - r * (ti * 5);
        su[r * SU + c] = uu[(cin0 + r * rstride) * 5 + c];
    }
    for (int e = threadIdx.x; e < ta * ti * 3; e += blockDim.x) {
        const int r = e / (ti * 3), c = e - r * (ti * 3);
        sb[r * SB + c] = ub[(cin0 + r * rstride) * 3 + c];
    }
    __syncthreads();
    // output: axis 1 -> dims (ny,nx,nz), cell (a, i, z); axis 2 -> dims (nz,ny,nx), cell (a, z, i)
    for (int r = 0; r < ti; r++) {
        const int iv = i0 + r;
        const size_t cout = (a.axis == 1) ? (((size_t)z * nx + iv) * ny + a0)
                                          : (((size_t)iv * ny + z) * nz + a0);
        for (int e = threadIdx.x; e < ta * 5; e += blockDim.x) {
            const int aa = e / 5, c = e - aa * 5;
            const int src = (a.axis == 1) ? perm_u<1>(c) : perm_u<2>(c);
            uo[cout * 5 + e] = su[aa * SU + r * 5 + src];
        }
        for (int e = threadIdx.x; e < ta * 3; e += blockDim.x) {
            const int aa = e / 3, c = e - aa * 3;
            const int src = (a.axis == 1) ? perm_b<1>(c) : perm_b<2>(c);
            bo[cout * 3 + e] = sb[aa * SB + r * 3 + src];
        }
        if (wo) {
            for (int e = threadIdx.x; e < ta * 2; e += blockDim.x) {
                const int aa = e / 2, c = e - aa * 2;
                const int src = (a.axis == 1) ? perm_u<1>(c) : perm_u<2>(c);
                wo[cout * 2 + e] = su[aa * SU + r * 5 + src];
            }
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(256) k_transpose(TransposeArgs a)
{
    constexpr int kTT = TTile<R>::E;
    __shared__ R su[kTT * (kTT * 5 + 1)];
    __shared__ R sb[kTT * (kTT * 3 + 1)];
    transpose_body<R>(a, su, sb, HwBlock{});
}

// copy_matrix (C/copy_matrix.c:9-38) as a vectorised device copy.
static __global__ void __launch_bounds__(256) k_copy16(const uint4* __restrict__ src, uint4* __restrict__ dst, size_t n16)
{
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n16; e += (size_t)gridDim.x * blockDim.x)
        dst[e] = src[e];
}

static __global__ void __launch_bounds__(256) k_copy4(const float* __restrict__ src, float* __restrict__ dst, size_t n4)
{
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n4; e += (size_t)gridDim.x * blockDim.x)
        dst[e] = src[e];
}

// ------------------------------------------------------------------ calcfl

// calcfl (C/calcfl.c:13-63), first pass: per-CTA max of the per-cell speed
// over a contiguous range of cells (blockDim cells per CTA) and the last NaN
// index in the range (cell0 + the index in the range: the index in the box).
template <typename R, bool EX>
__global__ void __launch_bounds__(256) k_calcfl(const R* __restrict__ u, const R* __restrict__ b, size_t ncell,
                                                size_t cell0, CflPart<R>* part, BoxStrides bs)
{
    __shared__ R rm[8];
    __shared__ int rn[8];
    // batched: box blockIdx.y, its partials after those of the boxes before it
    u = box_ptr(u, bs.u, blockIdx.y);
    b = box_ptr(b, bs.b, blockIdx.y);
    part += (size_t)blockIdx.y * gridDim.x;
    const size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    R sp = R(0);
    bool isn = false;
    if (cell < ncell) {
        R q[5], f[3];
#pragma unroll
        for (int c = 0; c < 5; c++)
            q[c] = u[cell * 5 + c];
#pragma unroll
        for (int c = 0; c < 3; c++)
            f[c] = b[cell * 3 + c];
        sp = cfl_speed<R, EX>(q, f);
        isn = (sp != sp);
    }
    R m = warp_max<R>(isn ? R(0) : sp);
    int ln = isn ? (int)(cell0 + cell) : -1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        ln = max(ln, __shfl_xor_sync(0xffffffffu, ln, o));
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        rm[w] = m;
        rn[w] = ln;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        R cm = R(0);
        int lnan = -1;
        for (int s = 0; s < (int)(blockDim.x >> 5); s++) {
            cm = fmax(cm, rm[s]);
            lnan = max(lnan, rn[s]);
        }
        part[blockIdx.x].cmax = cm;
        part[blockIdx.x].last_nan = lnan;
    }
}

// Second pass (one CTA): combine the partials.  Without NaN, c = max(0, all);
// after a NaN at linear index L the reference's running max_2num restarts, so
// c = max over cells after L (NaN if L is the last cell).  Then 1/c, and in
// the time loop dt = cfl*(1/c) (double product as C/mhd.c:62), dt clamped to
// (tf-t)/2 and t += 2dt (C/mhd.c:63-64).
// First level of the CFL reduction over many partials: CTA g takes the
// contiguous range g of the partials and writes their max speed and largest
// NaN index (both order-free, so the result is the one-CTA reduction's).
// One CTA reading 65536 partials is bound by its own L1 sector throughput.
template <typename R>
__global__ void __launch_bounds__(256) k_cfl_reduce(const CflPart<R>* __restrict__ part, int nparts,
                                                    CflPart<R>* __restrict__ out)
{
    __shared__ R rm[8];
    __shared__ int rn[8];
    const int per = (nparts + (int)gridDim.x - 1) / (int)gridDim.x;
    const int s0 = (int)blockIdx.x * per, s1 = min(nparts, s0 + per);
    R m = R(0);
    int ln = -1;
    for (int s = s0 + (int)threadIdx.x; s < s1; s += blockDim.x) {
        m = fmax(m, part[s].cmax);
        ln = max(ln, part[s].last_nan);
    }
    m = warp_max<R>(m);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        ln = max(ln, __shfl_xor_sync(0xffffffffu, ln, o));
    if ((threadIdx.x & 31) == 0) {
        rm[threadIdx.x >> 5] = m;
        rn[threadIdx.x >> 5] = ln;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) {
            m = fmax(m, rm[w]);
            ln = max(ln, rn[w]);
        }
        out[blockIdx.x].cmax = m;
        out[blockIdx.x].last_nan = ln;
        out[blockIdx.x].pad = 0;
    }
}

// The kernel body for the CTA of box blk.x() (HwBlock in k_cfl_finalize,
// VBlock in the work-list launch over several size classes, mhd_multi.cuh).
template <typename R, bool EX, typename B>
__device__ __forceinline__ void cfl_finalize_body(CflFinalizeArgs a, const B& blk)
{
    using W = wide_t<R, EX>;
    __shared__ R rm[32];
    __shared__ int rn[32];
    // batched: one CTA per box (blk.x()), each with its own partials, state and clock
    const int box = blk.x();
    a.u = box_ptr(a.u, a.bs.u, box);
    a.b = box_ptr(a.b, a.bs.b, box);
    a.clock = box_ptr(a.clock, a.bs.dt, box);
    if (box != 0)
        a.nsteps = nullptr;
    const CflPart<R>* part = static_cast<const CflPart<R>*>(a.part) + (size_t)box * a.nparts;
    R m = R(0);
    int ln = -1;
    for (int s = threadIdx.x; s < a.nparts; s += blockDim.x) {
        m = fmax(m, part[s].cmax);
        ln = max(ln, part[s].last_nan);
    }
    m = warp_max<R>(m);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        ln = max(ln, __shfl_xor_sync(0xffffffffu, ln, o));
    if ((threadIdx.x & 31) == 0) {
        rm[threadIdx.x >> 5] = m;
        rn[threadIdx.x >> 5] = ln;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int nw = (blockDim.x + 31) >> 5;
        m = (threadIdx.x < nw) ? rm[threadIdx.x] : R(0);
        ln = (threadIdx.x < nw) ? rn[threadIdx.x] : -1;
        m = warp_max<R>(m);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            ln = max(ln, __shfl_xor_sync(0xffffffffu, ln, o));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        rm[0] = m;
        rn[0] = ln;
    }
    __syncthreads();
    R c = rm[0];
    const int lnan = rn[0];
    const size_t ncell = (size_t)a.nx * a.ny * a.nz;
    if (lnan >= 0) {
        // Rare path: rescan the cells after the last NaN.
        const R* u = static_cast<const R*>(a.u);
        const R* b = static_cast<const R*>(a.b);
        R mm = R(0);
        bool any = false;
        for (size_t cell = (size_t)lnan + 1 + threadIdx.x; cell < ncell; cell += blockDim.x) {
            R q[5], f[3];
            for (int s = 0; s < 5; s++)
                q[s] = u[cell * 5 + s];
            for (int s = 0; s < 3; s++)
                f[s] = b[cell * 3 + s];
            const R sp = cfl_speed<R, EX>(q, f);
            if (sp == sp) mm = fmax(mm, sp);
            any = true;
        }
        // cells after L exist iff L < ncell-1; a NaN among them cannot occur (L is the last)
        __syncthreads();
        mm = warp_max<R>(mm);
        if ((threadIdx.x & 31) == 0)
            rm[threadIdx.x >> 5] = mm;
        __syncthreads();
        if (threadIdx.x == 0) {
            R r = R(0);
            for (int s = 0; s < (int)((blockDim.x + 31) >> 5); s++)
                r = fmax(r, rm[s]);
            rm[0] = r;
        }
        __syncthreads();
        (void)any;
        if ((size_t)lnan + 1 >= ncell)
            c = R(NAN);
        else
            c = rm[0];
        if (threadIdx.x == 0 && a.err)
            atomicOr(a.err, DEVERR_NONFINITE);
    }
    if (threadIdx.x == 0) {
        R* clk = static_cast<R*>(a.clock);
        const R inv = R(1) / c;
        clk[3] = inv;
        if (a.advance) {
            R dt = R(W(a.cfl) * W(inv));
            const R t = clk[0], tf = clk[1];
            if (dt > (tf - t) / R(2))
                dt = (tf - t) / R(2);
            clk[2] = dt;
            clk[0] = t + R(2) * dt;
            if (a.nsteps)
                *a.nsteps += 1;
        }
    }
}

template <typename R, bool EX>
__global__ void __launch_bounds__(1024) k_cfl_finalize(CflFinalizeArgs a)
{
    cfl_finalize_body<R, EX>(a, HwBlock{});
}

// Max |div B| (staggered stencil, periodic): per-CTA partial maxima.
template <typename R>
__global__ void __launch_bounds__(256) k_divb(const R* __restrict__ b, int nx, int ny, int nz, double* part)
{
    __shared__ double rm[8];
    const size_t ncell = (size_t)nx * ny * nz;
    const size_t cell = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    double d = 0;
    if (cell < ncell) {
        const int i = (int)(cell % nx);
        const int j = (int)((cell / nx) % ny);
        const int k = (int)(cell / ((size_t)nx * ny));
        const size_t ci = ((size_t)k * ny + j) * nx + ((i + 1 == nx) ? 0 : i + 1);
        const size_t cj = ((size_t)k * ny + ((j + 1 == ny) ? 0 : j + 1)) * nx + i;
        const size_t ck = ((size_t)((k + 1 == nz) ? 0 : k + 1) * ny + j) * nx + i;
        d = ((double)b[ci * 3] - (double)b[cell * 3]) + ((double)b[cj * 3 + 1] - (double)b[cell * 3 + 1]) +
            ((double)b[ck * 3 + 2] - (double)b[cell * 3 + 2]);
        d = fabs(d);
    }
    d = warp_max<double>(d);
    if ((threadIdx.x & 31) == 0)
        rm[threadIdx.x >> 5] = d;
    __syncthreads();
    if (threadIdx.x == 0) {
        double m = 0;
        for (int s = 0; s < (int)(blockDim.x >> 5); s++)
            m = fmax(m, rm[s]);
        part[blockIdx.x] = m;
    }
}

}  // namespace mhd

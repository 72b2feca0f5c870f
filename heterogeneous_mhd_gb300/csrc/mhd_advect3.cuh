// advectbyzx marching along k (C/advectbyzx.c:14-23 with A1/A2/B1/B2 and
// tvdb, C/advectbyzxA1.c:18-63 ... C/tvdb.c:10-91).
//
// A CTA owns J consecutive pencils (j0..j0+J-1) and K consecutive planes
// (k0..k0+K-1).  Marching k, it keeps a ring of NS plane slabs in shared
// memory: u pencils j0-1..j0+J and b pencils j0..j0+J of one plane, one bulk
// TMA copy per pencil.  With three slots the slab of plane k+2 is requested
// at the start of step k; with two it is requested as soon as step k has read
// plane k.  At step k the CTA computes
//   * J+1 A rows at plane k   (b(2) advected with the face velocity of j-1, j),
//   * J   B rows at plane k+1 (b(3) advected with the face velocity of k, k+1),
// one row per thread group of T = n/C threads, and combines for each owned
// pencil (the order of the float updates of A1, A2, B1, B2)
//   b1_out = (((b1 - FA(j,k)) + FA(j+1,k)) - FB(j,k)) + FB(j,k+1)
// with FB(.,k) and the advected b(3) of plane k kept from the previous step.
// Every input pencil is read from global memory once per CTA and every B row
// is computed once (one extra plane of B rows per K planes).  With C = 4 the
// 20-word thread chunks are read without bank conflicts.
//
// AX = 1, 2: the same operator along y or z of the untransposed state (the
// fused step): pencils along the sweep axis, j = x, k = z (AX = 1) or y
// (AX = 2).  A plane slab is gathered from its rows (the J+2 cells at
// consecutive x, contiguous in HBM) word by word over consecutive threads
// into the same pencil-major layout (pencil stride padded by kSweepPad) by
// 4-byte cp.async, with the components seen in the transposed order; the
// combined b pencils are staged in shared memory and written back as rows.
#pragma once
#include "mhd_advect2.cuh"

namespace mhd {

__host__ __device__ inline int advect3_rows(int J) { return 2 * J + 1; }

__host__ __device__ inline int advect3_threads(int J, int T)
{
    const int t = advect3_rows(J) * T;
    return ((t + 31) / 32) * 32;
}

// shared memory in floats: NS u slabs, NS b slabs, FA[J+1][n], FB[2][J][n],
// B3[2][J][n], seam, and for the y/z sweeps the output rows [J][n][3]; plus
// the mbarriers (in the static part)
// (uc: floats per cell of a staged u pencil: 5, or 2 for the (rho, m_x) side
// array of the fluidx before)
__host__ __device__ inline size_t advect3_smem_floats(int J, int n, int NS, int ax = 0, int uc = 5)
{
    const size_t pad = ax ? kSweepPad : 0;
    const size_t uslab = (size_t)(J + 2) * (n * uc + pad), bslab = (size_t)(J + 1) * (n * 3 + pad);
    return NS * uslab + NS * bslab + (size_t)(J + 1) * n + (size_t)4 * J * n + 2 * 32 * kSeamVals +
           (ax ? (size_t)J * (3 * n + pad) : 0);
}

// WU (x sweep only): the u slabs hold the (rho, m_x) side array a.w written
// by the fluidx before (8 instead of 20 bytes per cell of HBM traffic and of
// shared memory).
template <bool EX, int C, int T, int NS, int AX = 0, bool WU = false>
__global__ void __launch_bounds__(384) k_advect3(AdvectArgs a)
{
    select_box(a, blockIdx.z);
    using R = float;
    constexpr int n = C * T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint64_t bar[NS];
    const int J = a.P, K = a.K;
    const int NR = advect3_rows(J);
    const int tid = threadIdx.x;
    const Group<R, T> g(tid);
    int r = tid / T;
    const bool live = r < NR;
    if (!live)
        r = 0;
    // sizes of the j and k axes (j = y, k = z for the x sweep; j = x otherwise)
    const int ny = (AX == 0) ? a.ny : a.nx, nz = (AX == 0) ? a.nz : (AX == 1 ? a.nz : a.ny);
    const int j0 = blockIdx.x * J, k0 = blockIdx.y * K;
    const R dt = load_dt<R>(a.dt_ptr, a.dt_val);

    static_assert(!WU || AX == 0, "the side array is written by the x-sweep fluidx");
    constexpr int UC = WU ? 2 : 5;  // floats per cell of a staged u pencil
    constexpr int UROW = n * UC + (AX ? kSweepPad : 0), BROW = n * 3 + (AX ? kSweepPad : 0);  // pencil strides
    const size_t uslab = (size_t)(J + 2) * UROW, bslab = (size_t)(J + 1) * BROW;
    float* U = reinterpret_cast<float*>(smem_raw);  // [NS][J+2][n*5]
    float* B = U + NS * uslab;                        // [NS][J+1][n*3]
    float* FA = B + NS * bslab;                       // [J+1][n]
    float* FB = FA + (size_t)(J + 1) * n;             // [2][J][n]
    float* B3 = FB + (size_t)2 * J * n;               // [2][J][n]
    float* seam = B3 + (size_t)2 * J * n;
    float* SO = seam + 2 * 32 * kSeamVals;            // [J][BROW] output pencils (AX != 0)

    const float* uu = static_cast<const float*>(a.uu);
    const float* ub = static_cast<const float*>(a.ub);
    const float* usrc = WU ? static_cast<const float*>(a.w) : uu;  // what the u slabs hold

    // ---- slab loads: plane p into ring slot s (one mbarrier per slot),
    // issued by warp 0: lane 0 registers the bytes, one lane per pencil copies.
    auto load_plane = [&](int p, int s) {
        const int pp = ((p % nz) + nz) % nz;
        if constexpr (AX == 0) {
            if (tid < 32) {
                if (tid == 0)
                    mbar_arrive_expect_tx(&bar[s], (uint32_t)((J + 2) * n * UC * 4 + (J + 1) * n * 12));
                __syncwarp();
                for (int row = tid; row < J + 2; row += 32) {
                    int j = j0 - 1 + row;
                    j = (j < 0) ? j + ny : (j >= ny ? j - ny : j);
                    const size_t cell = ((size_t)pp * ny + j) * n;
                    tma_load_1d(U + s * uslab + (size_t)row * UROW, usrc + cell * UC, n * UC * 4, &bar[s]);
                }
                for (int row = tid; row < J + 1; row += 32) {
                    int j = j0 + row;
                    j = (j >= ny) ? j - ny : j;
                    const size_t cell = ((size_t)pp * ny + j) * n;
                    tma_load_1d(B + s * bslab + (size_t)row * BROW, ub + cell * 3, n * 12, &bar[s]);
                }
            }
        } else {
            // rows of u at x0-1..x0+J and of b at x0..x0+J (x periodic) of plane pp
            const size_t rs = (AX == 1) ? (size_t)a.nx : (size_t)a.nx * a.ny;
            const float* u0 = uu + sweep_cell<AX>(0, 0, pp, a.nx, a.ny) * 5;
            const float* b0 = ub + sweep_cell<AX>(0, 0, pp, a.nx, a.ny) * 3;
            auto ucol = [&](int p) { int x = j0 - 1 + p; return (x < 0) ? x + ny : (x >= ny ? x - ny : x); };
            auto bcol = [&](int p) { int x = j0 + p; return (x >= ny) ? x - ny : x; };
            gather_tile<5>(U + s * uslab, UROW, u0, rs * 5, J + 2, n, ucol, tid, blockDim.x);
            gather_tile<3>(B + s * bslab, BROW, b0, rs * 3, J + 1, n, bcol, tid, blockDim.x);
            cp_async_commit();
        }
    };
    // wait for the slab of a plane; `later` = planes requested after it (0 or 1)
    auto wait_plane = [&](int p, int later) {
        if constexpr (AX == 0) {
            mbar_wait_bounded(&bar[(p - k0 + 1) % NS], (uint32_t)(((p - k0 + 1) / NS) & 1), a.err);
        } else {
            if (later)
                cp_async_wait<1>();
            else
                cp_async_wait<0>();
            __syncthreads();
        }
    };
    // ring slot and mbarrier parity of plane p (slot 0 gets k0-1, k0-1+NS, ...)
    auto slot_of = [&](int p) { return (p - k0 + 1) % NS; };
    auto parity_of = [&](int p) { return (uint32_t)(((p - k0 + 1) / NS) & 1); };

    // this thread's chunk of u pencil `row` (0 = j0-1) / b pencil `row` (0 = j0) in slot s
    auto u_chunk = [&](int s, int row, float (&out)[C * UC]) {
        lds_chunk<float, C * UC>(U + s * uslab + (size_t)row * UROW + g.t * C * UC, out);
    };
    auto b_chunk = [&](int s, int row, float (&out)[C * 3]) {
        lds_chunk<float, C * 3>(B + s * bslab + (size_t)row * BROW + g.t * C * 3, out);
    };
    // raw face velocity between two u chunks (C/advectbyzxA1.c:34, C/advectbyzxB1.c:34)
    constexpr int UM = sweep_u<AX>(1), BD = sweep_b<AX>(0), BJ = sweep_b<AX>(1), BK = sweep_b<AX>(2);
    auto face_v = [&](const float (&um)[C * UC], const float (&uc)[C * UC], float (&vr)[C]) {
#pragma unroll
        for (int m = 0; m < C; m++) {
            if constexpr (WU)
                vr[m] = tvdb_face<float, EX>(um[2 * m + 1], uc[2 * m + 1], um[2 * m], uc[2 * m]);
            else
                vr[m] = tvdb_face<float, EX>(um[5 * m + UM], uc[5 * m + UM], um[5 * m], uc[5 * m]);
        }
    };

    if (AX == 0 && tid == 0)
        for (int s = 0; s < NS; s++)
            mbar_init(&bar[s], 1);
    __syncthreads();
    load_plane(k0 - 1, slot_of(k0 - 1));
    load_plane(k0, slot_of(k0));
    if (NS >= 3)
        load_plane(k0 + 1, slot_of(k0 + 1));
    wait_plane(k0 - 1, 1);
    wait_plane(k0, NS >= 3 ? 1 : 0);

    // ---- prologue: B rows of plane k0 (FB and advected b(3) of the first step)
    const bool brow = live && r > J;  // B-row groups: pencil j0 + (r-J-1)
    const int bp = r - J - 1;
    {
        const int sm = slot_of(k0 - 1), sc = slot_of(k0);
        float um[C * UC], uc[C * UC], bb[C * 3], vr[C], bv[C], F[C], bn[C];
        const int prow = brow ? bp + 1 : 1;  // u row of pencil j0+bp
        u_chunk(sm, prow, um);
        u_chunk(sc, prow, uc);
        b_chunk(sc, brow ? bp : 0, bb);
        face_v(um, uc, vr);
#pragma unroll
        for (int m = 0; m < C; m++)
            bv[m] = bb[3 * m + BK];
        tvdb_row<R, EX, C, T>(g, vr, bv, dt, seam, F, bn);
        if (brow) {
            const int pb = k0 & 1;
            sts_chunk<float, C>(FB + ((size_t)pb * J + bp) * n + g.t * C, F);  // one 16-byte store per row
            sts_chunk<float, C>(B3 + ((size_t)pb * J + bp) * n + g.t * C, bn);
        }
    }
    __syncthreads();
    if (NS == 2) {  // plane k0-1 is no longer needed
        fence_proxy_async_smem();
        load_plane(k0 + 1, slot_of(k0 + 1));
    }

    const float* b1s = static_cast<const float*>(a.b1_src);
    float* bo = static_cast<float*>(a.b_out);
    for (int k = k0; k < k0 + K; k++) {
        const int sk = slot_of(k), sk1 = slot_of(k + 1);
        if (NS >= 3 && k + 2 <= k0 + K) {  // plane k-1's slot is free
            fence_proxy_async_smem();
            load_plane(k + 2, slot_of(k + 2));
        }
        wait_plane(k + 1, (NS >= 3 && k + 2 <= k0 + K) ? 1 : 0);
        // ---- rows: A at plane k (r <= J), B at plane k+1 (r > J)
        float F[C], bn[C], b1own[C];
        {
            float um[C * UC], uc[C * UC], bb[C * 3], vr[C], bv[C];
            if (r <= J) {
                u_chunk(sk, r, um);      // pencil j0+r-1
                u_chunk(sk, r + 1, uc);  // pencil j0+r
                b_chunk(sk, r, bb);
            } else {
                u_chunk(sk, bp + 1, um);   // plane k
                u_chunk(sk1, bp + 1, uc);  // plane k+1
                b_chunk(sk1, bp, bb);
            }
            face_v(um, uc, vr);
#pragma unroll
            for (int m = 0; m < C; m++) {
                bv[m] = (r <= J) ? bb[3 * m + BJ] : bb[3 * m + BK];
                b1own[m] = bb[3 * m + BD];
            }
            tvdb_row<R, EX, C, T>(g, vr, bv, dt, seam, F, bn);
        }
        const int pk = k & 1, pk1 = (k + 1) & 1;
        if (live) {
            float* w = (r <= J) ? FA + (size_t)r * n + g.t * C : FB + ((size_t)pk1 * J + bp) * n + g.t * C;
            sts_chunk<float, C>(w, F);
        }
        __syncthreads();
        if (NS == 2 && k + 2 <= k0 + K) {  // plane k has been read: refill its slot
            fence_proxy_async_smem();
            load_plane(k + 2, sk);
        }
        // ---- combine and store the owned pencils (A-row groups 0..J-1)
        if (live && r < J) {
            const size_t cell0 = ((size_t)(k % nz) * ny + j0 + r) * n + g.t * C;
            if (AX == 0 && b1s != ub) {
                float b1c[C * 3];
                ldg_chunk<float, C * 3>(b1s + cell0 * 3, b1c);
#pragma unroll
                for (int m = 0; m < C; m++)
                    b1own[m] = b1c[3 * m];
            }
            float fa1[C], fb[C], fbp[C], b3[C];  // 16-byte loads: no bank conflicts for C = 4
            lds_chunk<float, C>(FA + (size_t)(r + 1) * n + g.t * C, fa1);
            lds_chunk<float, C>(FB + ((size_t)pk * J + r) * n + g.t * C, fb);
            lds_chunk<float, C>(FB + ((size_t)pk1 * J + r) * n + g.t * C, fbp);
            lds_chunk<float, C>(B3 + ((size_t)pk * J + r) * n + g.t * C, b3);
            float out[C * 3];
#pragma unroll
            for (int m = 0; m < C; m++) {
                float x = b1own[m];
                x = x - F[m];
                x = x + fa1[m];
                x = x - fb[m];
                x = x + fbp[m];
                out[3 * m + BD] = x;
                out[3 * m + BJ] = bn[m];
                out[3 * m + BK] = b3[m];
            }
            if constexpr (AX == 0)
                stg_chunk<float, C * 3>(bo + cell0 * 3, out);
            else
                sts_chunk<float, C * 3>(SO + (size_t)r * BROW + (size_t)g.t * C * 3, out);
        }
        if constexpr (AX != 0) {  // the J combined pencils back as rows of consecutive x
            __syncthreads();
            const size_t rs = (AX == 1) ? (size_t)a.nx : (size_t)a.nx * a.ny;
            scatter_tile<3>(bo + sweep_cell<AX>(0, j0, k % nz, a.nx, a.ny) * 3, rs * 3, SO, BROW, J, n, tid,
                            blockDim.x);
        }
        // the B rows' advected b(3) of plane k+1, for the next step
        if (brow)
            sts_chunk<float, C>(B3 + ((size_t)pk1 * J + bp) * n + g.t * C, bn);
        __syncthreads();
    }
}

}  // namespace mhd

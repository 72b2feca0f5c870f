// advectbyzx along y or z of the untransposed state (C/advectbyzx.c:14-23
// with A1 C/advectbyzxA1.c:18-63, A2 C/advectbyzxA2.c:9-28, B1
// C/advectbyzxB1.c:19-62, B2 C/advectbyzxB2.c:9-28 and tvdb C/tvdb.c:10-91):
// the fused step's replacement for transpose + advectbyzx + transpose back.
//
// The call that the transposed state would see has pencils along the sweep
// axis d (AX = 1: y, AX = 2: z), its "j" neighbour along x and its "k"
// neighbour along the remaining axis (AX = 1: z, AX = 2: y), with the
// components in the transposed order (u: rho, m_d, m_j, m_k, E; b: b_d, b_j,
// b_k; C/transpose12.c:7-47, C/transpose13.c:9-62).  Here the lanes of a warp
// are 32 consecutive x positions, so every staged row -- 32 cells along x at
// one position of the walk and one plane -- is one contiguous run of the
// x-major state (640 bytes of u, 384 of b): no gather and no transpose.
//
// The rest is the x-walking kernel's (mhd_advect4.cuh): every thread owns the
// A row (b_j advected with the face velocity of pencils x-1, x) and the B row
// (b_k with planes k-1, k) of its pencil and walks them along the sweep axis
// in chunks of four positions with the stencil in registers (XRow); warp w <
// KT owns plane k0+w, warp KT the B rows of plane k0+KT and, in lanes < KT,
// the A rows of pencil x0+32.  Per chunk the neighbouring EMFs meet (FA of
// pencil x+1 by a shuffle or from warp KT, FB of plane k+1 through shared
// memory) and warp w < KT applies the float updates in the order of A1, A2,
// B1, B2: b_d = (((b_d - FA(j,k)) + FA(j+1,k)) - FB(j,k)) + FB(j,k+1).
//
// Staging: per chunk and plane, four rows of u (cells x0..x0+31 by 16-byte
// cp.async of whole records, plus rho and m_d of the halo cells x0-1 and
// x0+32 by 4-byte cp.async) and of b (x0..x0+31, plus the halo x0+32), into
// a ring of NS buffers.  A lane reads rho and m_d of its cell at a stride of
// five words and its b at a stride of three: no bank conflicts.  The CTAs
// are persistent, with the x-walking kernel's work split (whole tiles in
// rounds, then the leftover tiles split along the walk).
#pragma once
#include <type_traits>

#include "mhd_advect4.cuh"
#include "mhd_pencil.cuh"

namespace mhd {

constexpr int kA5J = 32;                 // pencils (consecutive x) per tile: the lanes
constexpr int kA5UIN = 4;                // first float of the 32 staged u records of a row
constexpr int kA5UHR = kA5UIN + 5 * 32;  // rho, m_d of the right halo cell x0+32
constexpr int kA5UROW = kA5UHR + 4;      // staged u row (left halo rho, m_d, 2 pad | 32 records | right halo)
constexpr int kA5BHR = 3 * 32;           // b of the right halo cell x0+32
constexpr int kA5BROW = kA5BHR + 4;      // staged b row (32 records | halo + 1 pad)

// With the side array (WU): a staged u row holds (rho, m_d) only: left halo
// rho, m_d, 2 pad | 32 pairs | right halo rho, m_d, 2 pad
constexpr int kA5WIN = 4;                 // first float of the 32 staged pairs
constexpr int kA5WHR = kA5WIN + 2 * 32;   // rho, m_d of the right halo cell x0+32
constexpr int kA5WROW = kA5WHR + 4;

__host__ __device__ inline int advect5_threads(int KT) { return (KT + 1) * 32; }

__host__ __device__ inline size_t advect5_smem_bytes(int KT, int NS, bool wu = false)
{
    const size_t buf = (size_t)(KT + 2) * kA4X * (wu ? kA5WROW : kA5UROW) + (size_t)(KT + 1) * kA4X * kA5BROW;
    return (NS * buf + 4 * ((size_t)(KT + 1) * 32 + KT)) * sizeof(float);
}

// WU: the u rows come from the (rho, m_d) side array a.w that the fluidx
// before wrote (8 instead of 20 bytes per cell staged and read)
template <bool EX, int KT, int NS, int AX, bool WU = false>
__global__ void __launch_bounds__((KT + 1) * 32, advect4_min_ctas(KT, NS)) k_advect5(AdvectArgs a)
{
    static_assert(AX == 1 || AX == 2, "sweeps along y or z");
    static_assert(NS == 2 || NS == 3, "two or three chunk buffers");
    select_box(a, blockIdx.z);
    constexpr int NW = KT + 1;
    // staged u row: first record, right halo, length, floats per record (rho at 0)
    constexpr int UIN = WU ? kA5WIN : kA5UIN, UHR = WU ? kA5WHR : kA5UHR, UROW = WU ? kA5WROW : kA5UROW;
    constexpr int REC = WU ? 2 : 5, UPR = WU ? 16 : 40;       // floats per record, 16-byte pieces per row
    constexpr int PU = kA4X * UROW, PB = kA4X * kA5BROW;      // one staged plane (four rows)
    constexpr int UBUF = (KT + 2) * PU, BBUF = (KT + 1) * PB;
    constexpr int MD = WU ? 1 : sweep_u<AX>(1);                          // the sweep momentum in a record
    constexpr int CD = sweep_b<AX>(0), CJ = sweep_b<AX>(1), CK = sweep_b<AX>(2);
    extern __shared__ __align__(16) float a5_smem[];
    float* Us = a5_smem;                                      // [NS][KT+2][4][UROW]
    float* Bs = Us + NS * UBUF;                               // [NS][KT+1][4][kA5BROW]
    float4* FBx = reinterpret_cast<float4*>(Bs + NS * BBUF);  // [KT+1][32]
    float4* FAx = FBx + NW * 32;                              // [KT]

    // offsets in floats fit 32 bits: the planner takes boxes of fewer than 2^31 / 5 cells
    const int nx = a.nx, ny = a.ny;
    const int n = (AX == 1) ? a.ny : a.nz;    // positions along the walk (pencil length)
    const int nk = (AX == 1) ? a.nz : a.ny;   // planes
    const int di = (AX == 1) ? nx : nx * ny;  // cells between walk positions
    const int dk = (AX == 1) ? nx * ny : nx;  // cells between planes
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const bool bw = (w == KT);
    const float dt = load_dt<float>(a.dt_ptr, a.dt_val);
    const float* uu = static_cast<const float*>(WU ? a.w : a.uu);  // what the u rows hold
    const float* ub = static_cast<const float*>(a.ub);
    const float* b1s = static_cast<const float*>(a.b1_src);
    float* bo = static_cast<float*>(a.b_out);
    const bool b1_staged = (b1s == ub);

    // this thread's rows: staged offsets of rho and m_d of the A row's lower
    // (x-1) and current cell, and of the B row's lower (k-1) and current cell
    const int ka = bw ? (lane < KT ? lane : 0) : w;  // plane in the tile of the A row
    int rAm, mAm, rAc, mAc, rBm, mBm, rBc, mBc, bA, bB;
    if (!bw) {
        rAc = (w + 1) * PU + UIN + REC * lane;
        rAm = (w + 1) * PU + (lane ? UIN + REC * (lane - 1) : 0);
        mAm = rAm + (lane ? MD : 1);
        rBm = w * PU + UIN + REC * lane;
        rBc = rAc;
        bA = bB = w * PB + 3 * lane;
    } else {
        rAm = (ka + 1) * PU + UIN + REC * 31;
        mAm = rAm + MD;
        rAc = (ka + 1) * PU + UHR;
        rBm = KT * PU + UIN + REC * lane;
        rBc = (KT + 1) * PU + UIN + REC * lane;
        bA = ka * PB + kA5BHR;
        bB = KT * PB + 3 * lane;
    }
    mAc = (!bw) ? rAc + MD : rAc + 1;
    mBm = rBm + MD;
    mBc = rBc + MD;

    // copy assignments of this lane inside one staged plane: 16-byte pieces
    // p = lane + 32 q of the four rows (u: 40 per row, or 16 of the side
    // array; b: 24 per row) and one 4-byte halo word (u: lanes 0..15, b: lanes
    // 0..11); source offsets in floats from the plane's first row at x0
    // (recomputed per chunk: a few integer operations, which keeps them out of
    // the registers)
    auto uq = [&](int q, int& d, int& src) {
        const int p = lane + 32 * q, r = p / UPR, pc = p - UPR * r;
        d = r * UROW + UIN + 4 * pc;
        src = r * di * REC + 4 * pc;
    };
    auto bq = [&](int q, int& d, int& src) {
        const int p = lane + 32 * q, r = p / 24, pc = p - 24 * r;
        d = r * kA5BROW + 4 * pc;
        src = r * di * 3 + 4 * pc;
    };
    auto kwrap = [&](int k) { return (k < 0) ? k + nk : (k >= nk ? k - nk : k); };

    // Work split (as the x-walking kernel): whole tiles in rounds, then the
    // tiles left over split along the walk.
    const int NC = n / kA4X, tj = nx / kA5J, tk = nk / KT;
    const int ntiles = tj * tk, P = (int)gridDim.x, full = ntiles / P;
    const long long rest = (long long)(ntiles - full * P) * NC;
    long long ws = rest * blockIdx.x / P;
    const long long wend = rest * (blockIdx.x + 1) / P;

    for (int round = 0;; round++) {
        int tile, c0, c1;
        if (round < full) {
            tile = (int)blockIdx.x + round * P;
            c0 = 0;
            c1 = NC;
        } else {
            if (ws >= wend)
                break;
            const long long u = ws / NC;
            c0 = (int)(ws - u * NC);
            c1 = (int)((wend - ws < (long long)(NC - c0)) ? (c0 + (wend - ws)) : NC);
            ws += c1 - c0;
            tile = full * P + (int)u;
        }
        const int x0 = (tile % tj) * kA5J, k0 = (tile / tj) * KT;
        const int xl = (x0 == 0) ? nx - 1 : x0 - 1, xh = (x0 + kA5J == nx) ? 0 : x0 + kA5J;
        // halo words of this lane (u: row r, left/right, rho/m_d; b: row r, component)
        const int uh_r = (lane >> 2) & 3, uh_side = (lane >> 1) & 1, uh_word = lane & 1;
        const int uhd = uh_r * UROW + (uh_side ? UHR : 0) + uh_word;
        const int uhs = uh_r * di * REC + ((uh_side ? xh : xl) - x0) * REC + (uh_word ? MD : 0);
        const int bh_r = lane / 3, bh_c = lane - 3 * bh_r;
        const int bhd = bh_r * kA5BROW + kA5BHR + bh_c;
        const int bhs = bh_r * di * 3 + (xh - x0) * 3 + bh_c;
        const int kbu0 = kwrap(k0 + w - 1) * dk + x0;  // staged u plane w
        const int kbu1 = kwrap(k0 + KT) * dk + x0;     // staged u plane KT+1 (warp 0)
        const int kbb = kwrap(k0 + w) * dk + x0;       // staged b plane w

        // virtual chunk v (c0-1 .. c1, periodic) into ring buffer s
        auto load_chunk = [&](int v, int s) {
            const int xr = (v < 0) ? v + NC : (v >= NC ? v - NC : v);
            const int row0 = kA4X * xr * di;
            float* ud = Us + s * UBUF + w * PU;
            const float* us = uu + (row0 + kbu0) * REC;
#pragma unroll
            for (int q = 0; q < 4 * UPR / 32; q++) {
                int d, src;
                uq(q, d, src);
                cp_async16(ud + d, us + src);
            }
            if (lane < 16)
                cp_async4(ud + uhd, us + uhs);
            if (w == 0) {  // the last staged u plane (k0 + KT)
                float* ud1 = Us + s * UBUF + (KT + 1) * PU;
                const float* us1 = uu + (row0 + kbu1) * REC;
#pragma unroll
                for (int q = 0; q < 4 * UPR / 32; q++) {
                    int d, src;
                    uq(q, d, src);
                    cp_async16(ud1 + d, us1 + src);
                }
                if (lane < 16)
                    cp_async4(ud1 + uhd, us1 + uhs);
            }
            float* bd = Bs + s * BBUF + w * PB;
            const float* bsrc = ub + (row0 + kbb) * 3;
#pragma unroll
            for (int q = 0; q < 3; q++) {
                int d, src;
                bq(q, d, src);
                cp_async16(bd + d, bsrc + src);
            }
            if (lane < 12)
                cp_async4(bd + bhd, bsrc + bhs);
        };

        const int nv = c1 - c0 + 2;
        __syncthreads();  // the previous segment no longer reads the buffers
#pragma unroll
        for (int i = 0; i < NS - 1; i++) {
            if (i < nv)
                load_chunk(c0 - 1 + i, i);
            cp_async_commit();
        }
        XRow<EX> RA, RB;
        RA.reset();
        RB.reset();
        float bdp[4] = {0.f, 0.f, 0.f, 0.f};  // b_d of the chunk before the one read
        // global cell of warp w's pencil at walk position 0
        const int cellw = (k0 + w) * dk + x0 + lane;
        auto chunk = [&](int i, auto sbuf) {
            constexpr int S = decltype(sbuf)::value;
            cp_async_wait<NS - 2>();
            __syncthreads();  // chunk i has landed everywhere; chunk i-1's buffer is free
            if (i + NS - 1 < nv)
                load_chunk(c0 - 1 + i + NS - 1, (S + NS - 1) % NS);
            cp_async_commit();
            const float* U = Us + S * UBUF;
            const float* Bv = Bs + S * BBUF;
            float vxA[4], vxB[4], bvA[4], bvB[4], bd1[4];
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const float* Ur = U + r * UROW;
                const float* Br = Bv + r * kA5BROW;
                const float rc = Ur[rAc], mc = Ur[mAc];
                vxA[r] = tvdb_face<float, EX>(Ur[mAm], mc, Ur[rAm], rc);
                vxB[r] = tvdb_face<float, EX>(Ur[mBm], Ur[mBc], Ur[rBm], Ur[rBc]);
                bvA[r] = Br[bA + CJ];
                bvB[r] = Br[bB + CK];
                bd1[r] = Br[bA + CD];  // warp KT: unused
            }
            float FA[4], BNA[4], FB[4], BNB[4];
            RA.step(vxA, bvA, dt, FA, BNA);
            RB.step(vxB, bvB, dt, FB, BNB);
            if (i >= 2) {  // the chunk before the one read (c0 + i - 2) is complete
                FBx[w * 32 + lane] = make_float4(FB[0], FB[1], FB[2], FB[3]);
                if (bw && lane < KT)
                    FAx[lane] = make_float4(FA[0], FA[1], FA[2], FA[3]);
                __syncthreads();
                if (!bw) {
                    float fan[4];
#pragma unroll
                    for (int m = 0; m < 4; m++)
                        fan[m] = __shfl_down_sync(kFull, FA[m], 1);
                    if (lane == 31) {
                        const float4 t = FAx[w];
                        fan[0] = t.x, fan[1] = t.y, fan[2] = t.z, fan[3] = t.w;
                    }
                    const float4 fbn = FBx[(w + 1) * 32 + lane];
                    const float fbv[4] = {fbn.x, fbn.y, fbn.z, fbn.w};
                    const int pos0 = kA4X * (c0 + i - 2);
#pragma unroll
                    for (int m = 0; m < 4; m++) {
                        const int cell = cellw + (pos0 + m) * di;
                        float x = b1_staged ? bdp[m] : b1s[cell * 3 + CD];
                        x = x - FA[m];
                        x = x + fan[m];
                        x = x - FB[m];
                        x = x + fbv[m];
                        float* o = bo + cell * 3;
                        o[CD] = x;
                        o[CJ] = BNA[m];
                        o[CK] = BNB[m];
                    }
                }
            }
#pragma unroll
            for (int m = 0; m < 4; m++)
                bdp[m] = bd1[m];
        };
        // unrolled by the ring depth: every buffer offset is a constant
        using S0 = std::integral_constant<int, 0>;
        using S1 = std::integral_constant<int, 1>;
        using S2 = std::integral_constant<int, (NS > 2 ? 2 : 0)>;
        int i = 0;
        for (; i + NS <= nv; i += NS) {
            chunk(i, S0{});
            chunk(i + 1, S1{});
            if constexpr (NS == 3)
                chunk(i + 2, S2{});
        }
        if (i < nv)
            chunk(i, S0{});
        if (NS == 3 && i + 1 < nv)
            chunk(i + 1, S1{});
    }
    cp_async_wait<0>();
}

}  // namespace mhd

// advectbyzx of the x sweep with one warp per pencil (C/advectbyzx.c:14-23
// with A1 C/advectbyzxA1.c:18-63, A2 C/advectbyzxA2.c:9-28, B1
// C/advectbyzxB1.c:19-62, B2 C/advectbyzxB2.c:9-28 and tvdb C/tvdb.c:10-91),
// FP32, reading (rho, m_x) from the side array the fluidx before it wrote.
//
// A CTA owns J consecutive pencils j0..j0+J-1 and K consecutive planes and
// marches along k.  Warp w < J owns pencil j = j0+w: its 32 lanes hold the
// C = n/32 consecutive cells of the tvdb rows (the stencil crosses lanes by
// shuffles only, so no row needs a CTA barrier), and at plane k the warp
// computes
//   * the A row (j, k): b(2) advected with the face velocity of pencils j-1, j,
//   * the B row (j, k+1): b(3) advected with the face velocity of planes k, k+1,
// then combines pencil (j, k) in the order of the float updates of A1, A2, B1,
// B2:  b1_out = (((b1 - FA(j,k)) + FA(j+1,k)) - FB(j,k)) + FB(j,k+1),
// with FB(j,k) and the advected b(3) of plane k carried in registers from the
// previous plane.  Warp J computes the A row of pencil j0+J, whose EMF the
// last owned pencil needs; the A rows' EMFs meet through shared memory, one
// CTA barrier per plane.
//
// Every plane is staged once: the side-array pencils j0-1..j0+J and the b
// pencils j0..j0+J of plane k+1 arrive by bulk TMA copies into a ring of two
// slots while plane k is computed, and a warp reads everything it needs from
// plane k+1 during step k (the B row's upper plane, the next A row's face
// velocity, and b(1), b(2) of the next plane, kept in registers), so a slot
// is free again after one step.  The output pencil is written from
// registers (16-byte stores for C = 4, 8; 3 C words apart for C = 3, so
// 4-byte stores there).
//
// SW: the side-array pencils arrive by 2-D tensor copies whose rows are the
// lanes' C cells (8 C bytes) with the shared-memory swizzle of that row
// width (64 B: 16-byte chunk c of row l at c ^ ((l >> 1) & 3); 32 B: at
// c ^ ((l >> 2) & 1)), so the lanes of a quarter warp read distinct banks;
// read in place, 64-byte rows put four lanes on the same banks.
#pragma once
#include <cuda.h>  // CUtensorMap

#include "mhd_advect2.cuh"

namespace mhd {

__host__ __device__ inline int advect6_threads(int J) { return (J + 1) * 32; }

// shared memory in bytes of n-cell pencils: two slots of J+2 side-array
// pencils (8 B/cell) and J+1 b pencils (12 B/cell), and two buffers of J+1
// EMF rows (4 B/cell)
__host__ __device__ inline size_t advect6_smem_bytes(int n, int J)
{
    return (size_t)n * (2 * 8 * (J + 2) + 2 * 12 * (J + 1) + 2 * 4 * (J + 1)) + 1024;  // + alignment slack
}

__host__ __device__ constexpr int advect6_min_ctas(int J) { return J <= 2 ? 5 : (J <= 4 ? 3 : 2); }

// The kernel body for a CTA at block coordinates `blk` of its size class's
// grid (HwBlock in k_advect6, VBlock in the work-list launch over several
// classes, mhd_multi.cuh).  T = 32: a pencil of 32 C cells per warp.  T = 16
// (short pencils of a work-list launch, 16 C cells): lanes 16..31 of a warp
// repeat the work of lanes 0..15 on the same pencil (the group shuffles stay
// inside each half) and store nothing.
template <bool EX, int C, int J, bool SW, int T, typename B>
__device__ __forceinline__ void advect6_body(AdvectArgs a, const CUtensorMap& wmap, const B& blk)
{
    static_assert(!SW || C == 4 || C == 8, "swizzled rows of 32 or 64 bytes");
    static_assert(T == 32 || (T == 16 && !SW), "16 or 32 cell lanes per warp");
    select_box(a, blk.z());
    constexpr int n = C * T;
    constexpr int UR = 2 * n, BR = 3 * n;  // floats of one staged pencil
    constexpr int USL = (J + 2) * UR, BSL = (J + 1) * BR;
    extern __shared__ __align__(16) unsigned char a6_raw[];
    // 1024-byte aligned start (the swizzle pattern is one of shared-memory
    // address bits), as an offset from the shared array
    const uint32_t pad = (1024u - (static_cast<uint32_t>(__cvta_generic_to_shared(a6_raw)) & 1023u)) & 1023u;
    float* const a6_smem = reinterpret_cast<float*>(a6_raw + pad);
    float* const Us = a6_smem;         // [2][J+2][UR]: side-array pencils j0-1 .. j0+J
    float* const Bs = Us + 2 * USL;    // [2][J+1][BR]: b pencils j0 .. j0+J
    float* const FAx = Bs + 2 * BSL;   // [2][J+1][n]: EMFs of the A rows
    __shared__ uint64_t full[2];

    const int ny = a.ny, nz = a.nz, K = a.K;
    const int j0 = blk.x() * J, k0 = a.kbeg + blk.y() * K;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const bool halo = (w == J);
    const Group<float, T> g(tid);
    const int cl = g.t;               // the lane's place along the pencil (lane, for T = 32)
    const bool owner = (lane < T);    // lanes that write shared and global memory
    const float dt = load_dt<float>(a.dt_ptr, a.dt_val);
    const float* ws = static_cast<const float*>(a.w);
    const float* ub = static_cast<const float*>(a.ub);
    float* bo = static_cast<float*>(a.b_out);
    constexpr int BD = 0, BJ = 1, BK = 2;  // b(1), b(2), b(3)

    // ring slot and mbarrier parity of plane p (plane k0-1 is slot 0, phase 0)
    auto slot_of = [&](int p) { return (p - k0 + 1) & 1; };
    auto parity_of = [&](int p) { return (uint32_t)(((p - k0 + 1) >> 1) & 1); };
    auto wrapk = [&](int p) { return (p < 0) ? p + nz : (p >= nz ? p - nz : p); };
    // plane p into its slot: warp 0, one lane per pencil copy
    auto issue = [&](int p) {
        const int s = slot_of(p), pp = wrapk(p);
        if (lane == 0)
            mbar_arrive_expect_tx(&full[s], (uint32_t)(((J + 2) * UR + (J + 1) * BR) * 4));
        __syncwarp();
        for (int r = lane; r < 2 * J + 3; r += 32) {
            if (r < J + 2) {
                int j = j0 - 1 + r;
                j = (j < 0) ? j + ny : (j >= ny ? j - ny : j);
                if constexpr (SW)  // rows of C cells: 32 per pencil; the boxes' side arrays are contiguous
                    tma_load_2d(Us + s * USL + r * UR, &wmap, 0, ((blk.z() * nz + pp) * ny + j) * 32,
                                &full[s]);
                else
                    tma_load_1d(Us + s * USL + r * UR, ws + ((size_t)pp * ny + j) * UR, UR * 4, &full[s]);
            } else {
                int j = j0 + (r - J - 2);
                j = (j >= ny) ? j - ny : j;
                tma_load_1d(Bs + s * BSL + (r - J - 2) * BR, ub + ((size_t)pp * ny + j) * BR, BR * 4, &full[s]);
            }
        }
    };
    auto wait_plane = [&](int p) { mbar_wait_bounded(&full[slot_of(p)], parity_of(p), a.err); };
    // this lane's C cells of side-array pencil r (0 = j0-1) / b pencil r (0 = j0) of a slot
    auto u_read = [&](int s, int r, float (&rho)[C], float (&mx)[C]) {
        float t[2 * C];
        const float* row = Us + s * USL + r * UR + cl * 2 * C;
        if constexpr (SW) {
            const int x = (C == 8) ? ((cl >> 1) & 3) : ((cl >> 2) & 1);
#pragma unroll
            for (int q = 0; q < C / 2; q++) {
                const float4 v = *reinterpret_cast<const float4*>(row + 4 * (q ^ x));
                t[4 * q] = v.x;
                t[4 * q + 1] = v.y;
                t[4 * q + 2] = v.z;
                t[4 * q + 3] = v.w;
            }
        } else {
            lds_chunk<float, 2 * C>(row, t);
        }
#pragma unroll
        for (int m = 0; m < C; m++) {
            rho[m] = t[2 * m];
            mx[m] = t[2 * m + 1];
        }
    };
    auto b_read = [&](int s, int r, float (&bb)[3 * C]) { lds_chunk<float, 3 * C>(Bs + s * BSL + r * BR + cl * 3 * C, bb); };
    // face velocity between a lower and a current pencil (C/advectbyzxA1.c:34, C/advectbyzxB1.c:34)
    auto face = [&](const float (&rl)[C], const float (&ml)[C], const float (&rc)[C], const float (&mc)[C],
                    float (&v)[C]) {
#pragma unroll
        for (int m = 0; m < C; m++)
            v[m] = tvdb_face<float, EX>(ml[m], mc[m], rl[m], rc[m]);
    };

    if (tid == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
    }
    __syncthreads();
    if (w == 0) {
        issue(k0 - 1);
        issue(k0);
    }

    // ---- prologue: carries for plane k0
    // warp w < J: A row (j, k0) inputs, b(1) of (j, k0), u(j, k0), and the B row (j, k0)
    // warp J: A row (j0+J, k0) inputs
    float vA[C], b2c[C], b1c[C], rB[C], mB[C], FBc[C], b3c[C];
    {
        wait_plane(k0 - 1);
        wait_plane(k0);
        const int sm = slot_of(k0 - 1), sc = slot_of(k0);
        const int r = halo ? J : w;  // side-array row of the lower A pencil (j-1)
        float rl[C], ml[C], rc[C], mc[C], bb[3 * C];
        u_read(sc, r, rl, ml);
        u_read(sc, r + 1, rc, mc);
        face(rl, ml, rc, mc, vA);
        b_read(sc, r, bb);
#pragma unroll
        for (int m = 0; m < C; m++) {
            b2c[m] = bb[3 * m + BJ];
            b1c[m] = bb[3 * m + BD];
            rB[m] = rc[m];
            mB[m] = mc[m];
        }
        if (!halo) {  // warp-uniform: the halo warp has no B rows
            float rp[C], mp[C], vB[C], b3[C];
            u_read(sm, r + 1, rp, mp);
            face(rp, mp, rc, mc, vB);
#pragma unroll
            for (int m = 0; m < C; m++)
                b3[m] = bb[3 * m + BK];
            tvdb_row<float, EX, C, T>(g, vB, b3, dt, nullptr, FBc, b3c);
        }
    }
    __syncthreads();  // slots of planes k0-1 and k0 are free
    if (w == 0) {
        fence_proxy_async_smem();
        if (k0 + 1 <= k0 + K)
            issue(k0 + 1);
        if (k0 + 2 <= k0 + K)
            issue(k0 + 2);
    }

    for (int k = k0; k < k0 + K; k++) {
        const int s = slot_of(k + 1);
        float* const fax = FAx + ((k - k0) & 1) * (J + 1) * n;
        // ---- A row (j, k) from the carried inputs
        float FA[C], bA[C];
        tvdb_row<float, EX, C, T>(g, vA, b2c, dt, nullptr, FA, bA);
        if (owner)
            sts_chunk<float, C>(fax + w * n + cl * C, FA);
        // ---- plane k+1: B row (j, k+1) and the next A row's inputs
        wait_plane(k + 1);
        const int r = halo ? J : w;
        float rc[C], mc[C], bb[3 * C];
        u_read(s, r + 1, rc, mc);
        b_read(s, r, bb);
        float FBn[C], b3n[C];
        if (!halo) {
            float vB[C], b3[C];
            face(rB, mB, rc, mc, vB);
#pragma unroll
            for (int m = 0; m < C; m++)
                b3[m] = bb[3 * m + BK];
            tvdb_row<float, EX, C, T>(g, vB, b3, dt, nullptr, FBn, b3n);
        }
        {
            float rl[C], ml[C];
            u_read(s, r, rl, ml);
            face(rl, ml, rc, mc, vA);
        }
        __syncthreads();  // the A rows' EMFs of plane k are in; plane k+1's slot is read
        if (w == 0 && k + 3 <= k0 + K) {
            fence_proxy_async_smem();
            issue(k + 3);  // the slot of plane k+1
        }
        // ---- combine and store pencil (j, k)
        if (!halo) {
            float fa1[C];
            lds_chunk<float, C>(fax + (w + 1) * n + cl * C, fa1);
            float out[3 * C];
#pragma unroll
            for (int m = 0; m < C; m++) {
                float x = b1c[m];
                x = x - FA[m];
                x = x + fa1[m];
                x = x - FBc[m];
                x = x + FBn[m];
                out[3 * m + BD] = x;
                out[3 * m + BJ] = bA[m];
                out[3 * m + BK] = b3c[m];
            }
            const size_t cell0 = ((size_t)(k % nz) * ny + j0 + w) * n + cl * C;
            if (owner)
                stg_chunk<float, 3 * C>(bo + cell0 * 3, out);
        }
        // ---- carries for plane k+1
#pragma unroll
        for (int m = 0; m < C; m++) {
            b2c[m] = bb[3 * m + BJ];
            b1c[m] = bb[3 * m + BD];
            rB[m] = rc[m];
            mB[m] = mc[m];
            FBc[m] = FBn[m];
            b3c[m] = b3n[m];
        }
    }
}

template <bool EX, int C, int J, bool SW = false>
__global__ void __launch_bounds__((J + 1) * 32, advect6_min_ctas(J))
    k_advect6(AdvectArgs a, const __grid_constant__ CUtensorMap wmap)
{
    advect6_body<EX, C, J, SW, 32>(a, wmap, HwBlock{});
}

}  // namespace mhd

// transpose12 (C/transpose12.c:7-47) / transpose13 (C/transpose13.c:9-62) for
// full E x E-cell tiles (E = 32, or 16 for grids whose edges are multiples of
// 16 but not of 32), staged by bulk TMA.
//
// A CTA requests all 2E rows of its tile (E u rows of 20E bytes and E b rows
// of 12E bytes) at once with bulk copies into padded shared-memory rows,
// so a whole tile per CTA is in flight instead of what registers can hold.
// Each warp then writes whole output rows (E/8 of them): lane l writes floats
// l, l+32, ... of a row, whose (cell, component) source offsets are fixed per
// lane and computed once.  With w_out it also writes the first two
// components of the output cells (rho and the new m_x) as the side array the
// next advectbyzx reads.
#pragma once
#include "mhd_kernels.cuh"

namespace mhd {

constexpr int kT3 = 32;
constexpr int kT3U = 168;  // u row stride (words): 672 bytes, a multiple of 16
constexpr int kT3B = 100;  // b row stride (words): 400 bytes

// Row strides (words, multiples of four: 16-byte aligned rows) and shared
// memory (bytes) of an E x E tile.
template <int E>
struct T3Tile {
    static_assert(E == 32 || E == 16, "tiles of 32 or 16 cells");
    static constexpr int SU = (E == 32) ? kT3U : 5 * E + 4;  // 168 / 84
    static constexpr int SB = (E == 32) ? kT3B : 3 * E + 4;  // 100 / 52
    static constexpr size_t kSmem = (size_t)E * (SU + SB) * sizeof(float);
};

// shared memory of one 32-cell tile (bytes): u rows, b rows (16-byte aligned)
constexpr size_t kT3SmemBytes = T3Tile<32>::kSmem;

// The kernel body for a CTA at block coordinates `blk` of its size class's
// grid, staging into su [E][SU] and sb [E][SB] (16-byte aligned): HwBlock
// and static arrays in k_transpose3, VBlock and dynamic shared memory in the
// work-list launch over several classes (mhd_multi.cuh).
template <int AXIS, int E, typename B>
__device__ __forceinline__ void transpose3_body(TransposeArgs a, float* __restrict__ su, float* __restrict__ sb,
                                                const B& blk)
{
    constexpr int SU = T3Tile<E>::SU, SB = T3Tile<E>::SB;
    // per lane: floats l + 32q of an output row, q < QU (u), QB (b), QW (side array)
    constexpr int QU = (5 * E + 31) / 32, QB = (3 * E + 31) / 32, QW = (2 * E + 31) / 32;
    __shared__ uint64_t bar;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int nbz = (AXIS == 1) ? nz : ny;  // extent of the untouched axis
    const int i0 = blk.x() * E, a0 = blk.y() * E, z = blk.z() % nbz;
    select_box(a, blk.z() / nbz);
    const float* uu = static_cast<const float*>(a.uu);
    const float* ub = static_cast<const float*>(a.ub);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    // input row r: cells i0..i0+E-1 at swapped-axis index a0+r
    const size_t rstride = (AXIS == 1) ? (size_t)nx : (size_t)nx * ny;
    const size_t cin0 = (AXIS == 1) ? (((size_t)z * ny + a0) * nx + i0) : (((size_t)a0 * ny + z) * nx + i0);
    if (tid == 0)
        mbar_init(&bar, 1);
    __syncthreads();
    if (warp == 0) {
        if (lane == 0)
            mbar_arrive_expect_tx(&bar, E * E * (20 + 12));
        __syncwarp();
        if (lane < E) {
            const size_t c = cin0 + lane * rstride;
            tma_load_1d(su + lane * SU, uu + c * 5, E * 20, &bar);
            tma_load_1d(sb + lane * SB, ub + c * 3, E * 12, &bar);
        }
    }
    // per-lane source offsets inside a transposed row: output float f = l + 32q
    // is component c of output cell aa = f / 5, read from tile row aa (floats
    // past the row's end, for E = 16, are not written)
    int su_off[QU], sb_off[QB], sw_off[QW];
#pragma unroll
    for (int q = 0; q < QU; q++) {
        const int f = lane + 32 * q, aa = f / 5, c = f - 5 * aa;
        su_off[q] = (f < 5 * E) ? aa * SU + perm_u<AXIS>(c) : 0;
    }
#pragma unroll
    for (int q = 0; q < QW; q++) {  // side array: components 0, 1 of the output cells
        const int f = lane + 32 * q, aa = f / 2, c = f - 2 * aa;
        sw_off[q] = (f < 2 * E) ? aa * SU + perm_u<AXIS>(c) : 0;
    }
#pragma unroll
    for (int q = 0; q < QB; q++) {
        const int f = lane + 32 * q, aa = f / 3, c = f - 3 * aa;
        sb_off[q] = (f < 3 * E) ? aa * SB + perm_b<AXIS>(c) : 0;
    }
    // a copy that never lands (the wait gave up and set the error bit): the
    // whole CTA leaves before writing from unfilled shared memory
    if (!__syncthreads_and(mbar_wait_bounded(&bar, 0, a.err)))
        return;

    float* uo = static_cast<float*>(a.u_out);
    float* bo = static_cast<float*>(a.b_out);
    float* wo = static_cast<float*>(a.w_out);
#pragma unroll
    for (int s = 0; s < E / 8; s++) {
        const int i = warp + 8 * s;  // output row: position i0+i of the other axis
        const size_t cout = (AXIS == 1) ? (((size_t)z * nx + i0 + i) * ny + a0) : (((size_t)(i0 + i) * ny + z) * nz + a0);
        float* urow = uo + cout * 5;
        float* brow = bo + cout * 3;
#pragma unroll
        for (int q = 0; q < QU; q++)
            if (32 * (q + 1) <= 5 * E || lane + 32 * q < 5 * E)
                urow[lane + 32 * q] = su[su_off[q] + 5 * i];
#pragma unroll
        for (int q = 0; q < QB; q++)
            if (32 * (q + 1) <= 3 * E || lane + 32 * q < 3 * E)
                brow[lane + 32 * q] = sb[sb_off[q] + 3 * i];
        if (wo) {
#pragma unroll
            for (int q = 0; q < QW; q++)
                if (32 * (q + 1) <= 2 * E || lane + 32 * q < 2 * E)
                    wo[cout * 2 + lane + 32 * q] = su[sw_off[q] + 5 * i];
        }
    }
}

template <int AXIS, int E = kT3>
__global__ void __launch_bounds__(256) k_transpose3(TransposeArgs a)
{
    __shared__ __align__(16) float su[E * T3Tile<E>::SU];
    __shared__ __align__(16) float sb[E * T3Tile<E>::SB];
    transpose3_body<AXIS, E>(a, su, sb, HwBlock{});
}

}  // namespace mhd

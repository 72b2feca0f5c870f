// transpose12 (C/transpose12.c:7-47) / transpose13 (C/transpose13.c:9-62) for
// full 32x32-cell tiles, staged by bulk TMA.
//
// A CTA requests all 64 rows of its tile (32 u rows of 640 bytes and 32 b
// rows of 384 bytes) at once with bulk copies into padded shared-memory rows,
// so a whole tile per CTA is in flight instead of what registers can hold.
// Each warp then writes whole output rows: lane l writes floats l, l+32, ...
// of a row, whose (cell, component) source offsets are fixed per lane and
// computed once.  With w_out it also writes the first two components of the
// output cells (rho and the new m_x) as the side array the next advectbyzx
// reads.
#pragma once
#include "mhd_kernels.cuh"

namespace mhd {

constexpr int kT3 = 32;
constexpr int kT3U = 168;  // u row stride (words): 672 bytes, a multiple of 16
constexpr int kT3B = 100;  // b row stride (words): 400 bytes

// shared memory of one tile (bytes): u rows, b rows (16-byte aligned)
constexpr size_t kT3SmemBytes = (size_t)kT3 * (kT3U + kT3B) * sizeof(float);

// The kernel body for a CTA at block coordinates `blk` of its size class's
// grid, staging into su [kT3][kT3U] and sb [kT3][kT3B] (16-byte aligned):
// HwBlock and static arrays in k_transpose3, VBlock and dynamic shared memory
// in the work-list launch over several classes (mhd_multi.cuh).
template <int AXIS, typename B>
__device__ __forceinline__ void transpose3_body(TransposeArgs a, float* __restrict__ su, float* __restrict__ sb,
                                                const B& blk)
{
    __shared__ uint64_t bar;
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int nbz = (AXIS == 1) ? nz : ny;  // extent of the untouched axis
    const int i0 = blk.x() * kT3, a0 = blk.y() * kT3, z = blk.z() % nbz;
    select_box(a, blk.z() / nbz);
    const float* uu = static_cast<const float*>(a.uu);
    const float* ub = static_cast<const float*>(a.ub);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    // input row r: cells i0..i0+31 at swapped-axis index a0+r
    const size_t rstride = (AXIS == 1) ? (size_t)nx : (size_t)nx * ny;
    const size_t cin0 = (AXIS == 1) ? (((size_t)z * ny + a0) * nx + i0) : (((size_t)a0 * ny + z) * nx + i0);
    if (tid == 0)
        mbar_init(&bar, 1);
    __syncthreads();
    if (warp == 0) {
        if (lane == 0)
            mbar_arrive_expect_tx(&bar, kT3 * kT3 * (20 + 12));
        __syncwarp();
        const size_t c = cin0 + lane * rstride;
        tma_load_1d(su + lane * kT3U, uu + c * 5, kT3 * 20, &bar);
        tma_load_1d(sb + lane * kT3B, ub + c * 3, kT3 * 12, &bar);
    }
    // per-lane source offsets inside a transposed row: output float f = l + 32q
    // is component c of output cell aa = f / 5, read from tile row aa
    int su_off[5], sb_off[3], sw_off[2];
#pragma unroll
    for (int q = 0; q < 5; q++) {
        const int f = lane + 32 * q, aa = f / 5, c = f - 5 * aa;
        su_off[q] = aa * kT3U + perm_u<AXIS>(c);
    }
#pragma unroll
    for (int q = 0; q < 2; q++) {  // side array: components 0, 1 of the output cells
        const int f = lane + 32 * q, aa = f / 2, c = f - 2 * aa;
        sw_off[q] = aa * kT3U + perm_u<AXIS>(c);
    }
#pragma unroll
    for (int q = 0; q < 3; q++) {
        const int f = lane + 32 * q, aa = f / 3, c = f - 3 * aa;
        sb_off[q] = aa * kT3B + perm_b<AXIS>(c);
    }
    mbar_wait_bounded(&bar, 0, nullptr);

    float* uo = static_cast<float*>(a.u_out);
    float* bo = static_cast<float*>(a.b_out);
    float* wo = static_cast<float*>(a.w_out);
#pragma unroll
    for (int s = 0; s < kT3 / 8; s++) {
        const int i = warp + 8 * s;  // output row: position i0+i of the other axis
        const size_t cout = (AXIS == 1) ? (((size_t)z * nx + i0 + i) * ny + a0) : (((size_t)(i0 + i) * ny + z) * nz + a0);
        float* urow = uo + cout * 5;
        float* brow = bo + cout * 3;
#pragma unroll
        for (int q = 0; q < 5; q++)
            urow[lane + 32 * q] = su[su_off[q] + 5 * i];
#pragma unroll
        for (int q = 0; q < 3; q++)
            brow[lane + 32 * q] = sb[sb_off[q] + 3 * i];
        if (wo) {
#pragma unroll
            for (int q = 0; q < 2; q++)
                wo[cout * 2 + lane + 32 * q] = su[sw_off[q] + 5 * i];
        }
    }
}

template <int AXIS>
__global__ void __launch_bounds__(256) k_transpose3(TransposeArgs a)
{
    __shared__ __align__(16) float su[kT3 * kT3U];
    __shared__ __align__(16) float sb[kT3 * kT3B];
    transpose3_body<AXIS>(a, su, sb, HwBlock{});
}

}  // namespace mhd

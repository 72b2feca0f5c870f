// transpose12 (C/transpose12.c:7-47) / transpose13 (C/transpose13.c:9-62) for
// full 32x32-cell tiles.  A CTA moves one tile through shared memory: each
// thread issues 32 independent coalesced loads (one 128-byte line per warp
// instruction), the tile rows are padded to a stride of 5 (mod 32) words so
// the permuted reads of the write phase spread over the banks, and every
// warp store writes 32 consecutive floats of an output row.
#pragma once
#include "mhd_kernels.cuh"

namespace mhd {

constexpr int kT2 = 32;            // tile edge (cells)
constexpr int kT2U = kT2 * 5 + 5;  // padded u row (words), = 5 mod 32
constexpr int kT2B = kT2 * 3 + 3;  // padded b row (words), = 3 mod 32

template <int AXIS>
__global__ void __launch_bounds__(256, 4) k_transpose2(TransposeArgs a)
{
    __shared__ float su[kT2 * kT2U];
    __shared__ float sb[kT2 * kT2B];
    const int nx = a.nx, ny = a.ny, nz = a.nz;
    const int nbz = (AXIS == 1) ? nz : ny;  // extent of the untouched axis
    const int i0 = blockIdx.x * kT2, a0 = blockIdx.y * kT2, z = blockIdx.z % nbz;
    select_box(a, blockIdx.z / nbz);
    const float* uu = static_cast<const float*>(a.uu);
    const float* ub = static_cast<const float*>(a.ub);
    float* uo = static_cast<float*>(a.u_out);
    float* bo = static_cast<float*>(a.b_out);
    const int tid = threadIdx.x;

    // input row r of the tile: cells (i0 .. i0+31) at swapped-axis index a0+r
    const size_t rstride = (AXIS == 1) ? (size_t)nx : (size_t)nx * ny;
    const size_t cin0 = (AXIS == 1) ? (((size_t)z * ny + a0) * nx + i0) : (((size_t)a0 * ny + z) * nx + i0);
#pragma unroll 5
    for (int s = 0; s < kT2 * kT2 * 5 / 256; s++) {
        const int e = tid + 256 * s;  // 0 .. 5119
        const int rr = e / (kT2 * 5), c = e - rr * (kT2 * 5);
        su[rr * kT2U + c] = __ldg(uu + (cin0 + rr * rstride) * 5 + c);
    }
#pragma unroll 4
    for (int s = 0; s < kT2 * kT2 * 3 / 256; s++) {
        const int e = tid + 256 * s;
        const int rr = e / (kT2 * 3), c = e - rr * (kT2 * 3);
        sb[rr * kT2B + c] = __ldg(ub + (cin0 + rr * rstride) * 3 + c);
    }
    __syncthreads();
    // output row i: out cells (a0 .. a0+31) at position i0+i of the other axis
#pragma unroll 5
    for (int s = 0; s < kT2 * kT2 * 5 / 256; s++) {
        const int e = tid + 256 * s;
        const int i = e / (kT2 * 5), f = e - i * (kT2 * 5);
        const int aa = f / 5, c = f - aa * 5;
        const int src = perm_u<AXIS>(c);
        const size_t cout = (AXIS == 1) ? (((size_t)z * nx + i0 + i) * ny + a0) : (((size_t)(i0 + i) * ny + z) * nz + a0);
        uo[cout * 5 + f] = su[aa * kT2U + i * 5 + src];
    }
#pragma unroll 4
    for (int s = 0; s < kT2 * kT2 * 3 / 256; s++) {
        const int e = tid + 256 * s;
        const int i = e / (kT2 * 3), f = e - i * (kT2 * 3);
        const int aa = f / 3, c = f - aa * 3;
        const int src = perm_b<AXIS>(c);
        const size_t cout = (AXIS == 1) ? (((size_t)z * nx + i0 + i) * ny + a0) : (((size_t)(i0 + i) * ny + z) * nz + a0);
        bo[cout * 3 + f] = sb[aa * kT2B + i * 3 + src];
    }
}

}  // namespace mhd

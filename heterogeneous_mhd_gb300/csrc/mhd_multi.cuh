// Work-list launches over several size classes of cubes (the batched boxes).
//
// A batch holds boxes of a few edges (size classes); the boxes of one class
// lie at a fixed stride from each other (BoxStrides).  Instead of one launch
// per class and operator, one launch covers every class: its CTAs are laid
// out segment after segment (the classes in launch order, largest first), and
// a CTA finds its segment, then its block coordinates in that class's own
// grid (VBlock), and runs the class's kernel body with them.  The bodies are
// those of the one-class kernels (fluidx2_body, advect6_body,
// transpose3_body / transpose_body, cfl_finalize_body), so every box gets
// the same arithmetic as in a one-box step, bit for bit.  All segments of a
// launch share its block size: 64 threads for fluidx (P = 64 / T pencils per
// CTA), 96 for advectbyzx (J = 2 pencils), 256 for the transposes, 1024 for
// the CFL finalize.  The class's C/mhd.c:62-118 operator sequence is
// unchanged; only the grouping of CTAs into launches differs.
#pragma once
#include <cuda.h>  // CUtensorMap

#include "mhd_advect6.cuh"
#include "mhd_fluidx2.cuh"
#include "mhd_transpose3.cuh"

namespace mhd {

constexpr int kMultiFxThreads = 64;
constexpr int kMultiAdJ = 2;       // pencils per advectbyzx CTA (96 threads)

// One class of a work-list launch: its first CTA in the launch, the x and y
// extents of its own grid (z: the rest, boxes included) and its kernel kind.
struct SegGrid {
    int begin, gx, gy, kind;
};

struct FluidxMulti {
    SegGrid g[kMaxSegs];
    FluidxArgs a[kMaxSegs];
    int nseg;
};

struct AdvectMulti {
    CUtensorMap wmap[kMaxSegs];  // side-array rows of the swizzled kinds (first: 64-byte aligned)
    SegGrid g[kMaxSegs];
    AdvectArgs a[kMaxSegs];
    int nseg;
};

struct TransposeMulti {
    SegGrid g[kMaxSegs];
    TransposeArgs a[kMaxSegs];
    int nseg;
};

struct FinalizeMulti {
    SegGrid g[kMaxSegs];
    CflFinalizeArgs a[kMaxSegs];
    int nseg;
};

// Kinds: fluidx (C cells per thread, T threads per pencil) and advectbyzx
// (C cells per lane, T lanes per pencil) of the classes a work-list launch
// takes, edges 32, 48, 64, 96 and 128.
enum MultiFxKind : int { MFX_4_8 = 0, MFX_3_16, MFX_4_16, MFX_3_32, MFX_4_32, MFX_COUNT };
enum MultiAdKind : int { MAD_2_16 = 0, MAD_3_16, MAD_2_32, MAD_3_32, MAD_4_32, MAD_COUNT };

__host__ __device__ inline int multi_kind_of_edge(int n)
{
    switch (n) {
    case 32: return 0;
    case 48: return 1;
    case 64: return 2;
    case 96: return 3;
    case 128: return 4;
    }
    return -1;
}

// threads per pencil of the fluidx kind of edge n (P = 64 / T pencils per CTA)
__host__ __device__ inline int multi_fx_threads(int n)
{
    switch (multi_kind_of_edge(n)) {
    case MFX_4_8: return 8;
    case MFX_3_16: return 16;
    case MFX_4_16: return 16;
    case MFX_3_32: return 32;
    case MFX_4_32: return 32;
    }
    return 0;
}

// the segment of this CTA (segments in launch order, at most kMaxSegs) and
// its block coordinates in that segment's grid
__device__ __forceinline__ int multi_seg(const SegGrid* g, int nseg)
{
    const int b = (int)blockIdx.x;
    int s = 0;
#pragma unroll
    for (int t = 1; t < kMaxSegs; t++)
        if (t < nseg && b >= g[t].begin)
            s = t;
    return s;
}

__device__ __forceinline__ VBlock multi_block(const SegGrid& g)
{
    const int l = (int)blockIdx.x - g.begin;
    const int t = l / g.gx;
    VBlock v;
    v.bx = l - t * g.gx;
    v.by = t % g.gy;
    v.bz = t / g.gy;
    v.ngx = g.gx;
    v.ngy = g.gy;
    return v;
}

template <typename R, bool EX>
__global__ void __launch_bounds__(kMultiFxThreads) k_fluidx2_multi(const __grid_constant__ FluidxMulti m)
{
    const int s = multi_seg(m.g, m.nseg);
    const VBlock blk = multi_block(m.g[s]);
    switch (m.g[s].kind) {
    case MFX_4_8: fluidx2_body<R, EX, 4, 8, 0>(m.a[s], nullptr, blk); break;
    case MFX_3_16: fluidx2_body<R, EX, 3, 16, 0>(m.a[s], nullptr, blk); break;
    case MFX_4_16: fluidx2_body<R, EX, 4, 16, 0>(m.a[s], nullptr, blk); break;
    case MFX_3_32: fluidx2_body<R, EX, 3, 32, 0>(m.a[s], nullptr, blk); break;
    case MFX_4_32: fluidx2_body<R, EX, 4, 32, 0>(m.a[s], nullptr, blk); break;
    }
}

// The bound of six CTAs per SM makes ptxas allocate 96 registers, as for the
// 4-cell kind alone, so six CTAs of three warps fit on an SM (registers are
// allocated per sub-partition: five warps of 96 registers each); without it
// the union of the kinds took 109 registers and five CTAs (18.85 against
// 18.53 ms per step for 61 boxes of 128^3).
template <bool EX>
__global__ void __launch_bounds__((kMultiAdJ + 1) * 32, 6)
    k_advect6_multi(const __grid_constant__ AdvectMulti m)
{
    const int s = multi_seg(m.g, m.nseg);
    const VBlock blk = multi_block(m.g[s]);
    const CUtensorMap& wm = m.wmap[s];
    switch (m.g[s].kind) {
    case MAD_2_16: advect6_body<EX, 2, kMultiAdJ, false, 16>(m.a[s], wm, blk); break;
    case MAD_3_16: advect6_body<EX, 3, kMultiAdJ, false, 16>(m.a[s], wm, blk); break;
    case MAD_2_32: advect6_body<EX, 2, kMultiAdJ, false, 32>(m.a[s], wm, blk); break;
    case MAD_3_32: advect6_body<EX, 3, kMultiAdJ, false, 32>(m.a[s], wm, blk); break;
    case MAD_4_32: advect6_body<EX, 4, kMultiAdJ, true, 32>(m.a[s], wm, blk); break;
    }
}

// kind 0: bulk-TMA tiles of 32 cells (edges that are multiples of 32), 2: of
// 16 cells (multiples of 16), 1: the general tile kernel (partial tiles); all
// with the side-array output
constexpr size_t kMultiTransposeSmem =
    kT3SmemBytes > transpose_smem_bytes<float>() ? kT3SmemBytes : transpose_smem_bytes<float>();

// Six CTAs per SM, as the tiled kernel alone: 40 registers (48 without the
// bound, which fit five CTAs; the shared memory of a tile allows six).
template <int AXIS>
__global__ void __launch_bounds__(256, 6) k_transpose_multi(const __grid_constant__ TransposeMulti m)
{
    extern __shared__ __align__(16) unsigned char tmul_raw[];
    float* const sm = reinterpret_cast<float*>(tmul_raw);
    const int s = multi_seg(m.g, m.nseg);
    const VBlock blk = multi_block(m.g[s]);
    if (m.g[s].kind == 0)
        transpose3_body<AXIS, 32>(m.a[s], sm, sm + 32 * T3Tile<32>::SU, blk);
    else if (m.g[s].kind == 2)
        transpose3_body<AXIS, 16>(m.a[s], sm, sm + 16 * T3Tile<16>::SU, blk);
    else
        transpose_body<float>(m.a[s], sm, sm + TTile<float>::E * (TTile<float>::E * 5 + 1), blk);
}

template <typename R, bool EX>
__global__ void __launch_bounds__(1024) k_cfl_finalize_multi(const __grid_constant__ FinalizeMulti m)
{
    const int s = multi_seg(m.g, m.nseg);
    cfl_finalize_body<R, EX>(m.a[s], multi_block(m.g[s]));
}

}  // namespace mhd

// Host-side view of the kernel sets.  Each set is one (precision, arithmetic
// policy) instantiation of the kernels in mhd_kernels.cuh; the FAST set is
// compiled with FMA contraction, the EXACT sets with --fmad=false.
#pragma once
#include <cstddef>
#include <cuda_runtime.h>

#include "mhd_kernels.cuh"

namespace mhd {

struct KernelSet {
    int elem;  // sizeof(R)
    int exact; // reproduces the reference bit for bit
    cudaError_t (*fluidx)(const FluidxArgs&, cudaStream_t);
    cudaError_t (*advect)(const AdvectArgs&, cudaStream_t);
    cudaError_t (*transpose)(const TransposeArgs&, cudaStream_t);
    // first CFL pass over ncell cells, the first of which is cell cell0 of the
    // box (NaN cells are reported by their index in the box); returns the
    // number of partials written
    cudaError_t (*calcfl)(const void* u, const void* b, size_t ncell, size_t cell0, void* part, int* nparts,
                          const BoxStrides& bs, cudaStream_t);
    cudaError_t (*cfl_finalize)(const CflFinalizeArgs&, cudaStream_t);
    cudaError_t (*divb)(const void* b, int nx, int ny, int nz, double* part, int* nparts, cudaStream_t);
    size_t part_bytes; // sizeof(CflPart<R>)
    // number of CTAs (= CFL partials of the epilogue) of a fluidx launch
    int (*fluidx_parts)(int nx, int ny, int nz, int aligned);
    // nonzero if the sweeps along y and z of the fused step have kernels for this grid
    int (*fused_ok)(int nx, int ny, int nz);
    // nonzero if the x-sweep fluidx of this grid writes the (rho, m_x) side array (FluidxArgs::w_out)
    int (*fluidx_writes_w)(int nx, int ny, int nz, int aligned);
    // nonzero if the transpose (axis 1 or 2) of this grid writes it (TransposeArgs::w_out)
    int (*transpose_writes_w)(int axis, int nx, int ny, int nz);
    // nonzero if the fused step's fluidx sweep along `axis` (1: y) writes it
    int (*sweep_writes_w)(int axis, int nx, int ny, int nz);
    // nonzero if the fused step's last three operators (the y-sweep fluidx,
    // the x-sweep advectbyzx with the side array and the x-sweep fluidx) take
    // ranges of kcount planes along z (FluidxArgs/AdvectArgs::kbeg, kcount)
    int (*tail_slabs_ok)(int nx, int ny, int nz, int kcount);
    // nonzero if a batch size class of `boxes` cubes of edge n uses the (rho, m_x)
    // side array: its x-sweep advectbyzx is the warp-per-pencil kernel, which
    // reads it (the boxes' arrays one after the other)
    int (*batch_side_ok)(int n, int boxes);
    // Work-list launches over several size classes of cubes (mhd_multi.cuh):
    // nonzero if a class of edge n can join one (FP32, edges 32, 48, 64, 96,
    // 128), the CFL partials per box its fluidx writes, and one launch of an
    // operator over `nseg` classes (one argument set per class, launch order).
    int (*multi_ok)(int n);
    int (*multi_fluidx_parts)(int n);
    cudaError_t (*fluidx_multi)(const FluidxArgs* a, int nseg, cudaStream_t);
    cudaError_t (*advect_multi)(const AdvectArgs* a, int nseg, cudaStream_t);
    cudaError_t (*transpose_multi)(const TransposeArgs* a, int nseg, cudaStream_t);
    cudaError_t (*finalize_multi)(const CflFinalizeArgs* a, int nseg, cudaStream_t);
};

const KernelSet* kernels_f32_fast();
const KernelSet* kernels_f32_exact();
const KernelSet* kernels_f64_exact();

// CFL finalize of one box: with more partials than kCflReduceMin a first
// kernel of up to kCflReduceCtas CTAs reduces them into CflFinalizeArgs::scratch.
constexpr int kCflReduceMin = 4096;
constexpr int kCflReduceCtas = 128;

// Pencils per CTA along j for fluidx / advectbyzx (a divisor of ny).
int fluidx_pencils(int nx, int ny);
int advect_pencils(int nx, int ny);

cudaError_t launch_copy(const void* src, void* dst, size_t bytes, cudaStream_t s);

// Launch-shape knobs set by mhd_tune_set (0 = the planner's own choice).
enum TuneKey : int {
    TUNE_FLUIDX_THREADS = 0,  // threads per CTA of the register-resident fluidx (64/128/256)
    TUNE_ADVECT_C,            // cells per thread of the marching advectbyzx (4 or 8)
    TUNE_ADVECT_SLOTS,        // plane-slab ring depth (2 or 3)
    TUNE_ADVECT_J,            // pencils per CTA along j
    TUNE_ADVECT_K,            // planes per CTA along k
    TUNE_FLUIDX_C,            // cells per thread of the register-resident fluidx (4, or 8: one warp per pencil)
    TUNE_ADVECT_KERNEL,       // advectbyzx of the x sweep: 3 marching along k, 4 walking along x
    TUNE_ADVECT_XK,           // planes per CTA of the x-walking advectbyzx (2, 4 or 8)
    TUNE_SWEEP_KERNEL,        // advectbyzx of the fused step's y/z sweeps: 5 walking (default), 3 marching
    TUNE_SWEEP_K,             // planes per CTA of the sweep-walking advectbyzx (2, 4 or 8)
    TUNE_SWEEP_SLOTS,         // chunk buffers of the sweep-walking advectbyzx (2 or 3)
    TUNE_COUNT
};
int tune_value(int key);
long long tune_generation();  // bumped by every change (captured graphs are rebuilt)
int tune_index(const char* key);  // the TuneKey of a knob name, -1 if unknown
// Sets a knob without bumping the generation and returns its previous value:
// for a caller that applies its own values around its own launches (the
// batch's per-class shapes) and owns the graphs they are captured into.
int tune_swap(int key, int value);

}  // namespace mhd

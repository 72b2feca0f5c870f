// Allocation-free CFL reduction: mhd_calcfl_noalloc.
//
// The regular calcfl entry points (calcfl, mhd_op_calcfl) reduce through a
// per-context scratch buffer that the library allocates with cudaMalloc on
// first use.  Some callers cannot have the library allocate device memory at
// all: code that runs while a stream is being captured into a CUDA graph
// (cudaMalloc is not allowed inside a capture), hosts that give every byte of
// device memory to their own pool and forbid foreign allocations, and
// real-time loops that must not take the allocator's locks or synchronise the
// device.  This entry point serves them: its scratch is a file-scope
// __device__ array that exists from the moment the library is loaded on a
// device until the process exits, so a call never allocates or frees.
//
// Limits and rules (also in include/mhd_gb300.h):
//   * at most kMaxCells = 65536 partials x 2048 cells = 134,217,728 cells
//     (512^3); larger grids are rejected with MHD_ERR_UNSUPPORTED;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture;
//   * all calls share the one array: calls that overlap on the GPU (different
//     streams without ordering) race and may return each other's result.
#include <cstdio>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/mhd_gb300.h"
#include "mhd_kernels.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kCellsPerBlock = 2048;  // 8 cells per thread
constexpr int kMaxParts = 65536;      // partials held by the static scratch (768 KB)
constexpr long long kMaxCells = (long long)kMaxParts * kCellsPerBlock;

// The scratch: one partial (max speed, last NaN index) per CTA of the first
// pass.  Every call writes all the partials it later reads, so nothing has to
// start at zero and the contents left by the previous call are never used.
__device__ __align__(256) mhd::CflPart<float> g_noalloc_parts[kMaxParts];

std::mutex g_mu;
constexpr int kMaxDevices = 64;
mhd::CflPart<float>* g_parts_addr[kMaxDevices] = {};

// First pass: CTA p reduces cells [p*2048, (p+1)*2048) with the fast-path
// per-cell speed of calcfl (C/calcfl.c:44-54).
__global__ void __launch_bounds__(kThreads) k_cfl_static_parts(const float* __restrict__ u, const float* __restrict__ b,
                                                              size_t ncell, mhd::CflPart<float>* part)
{
    __shared__ float rm[kThreads / 32];
    __shared__ int rn[kThreads / 32];
    const size_t base = (size_t)blockIdx.x * kCellsPerBlock;
    float m = 0.0f;
    int ln = -1;
    for (int s = 0; s < kCellsPerBlock / kThreads; s++) {
        const size_t cell = base + threadIdx.x + (size_t)s * kThreads;
        if (cell < ncell) {
            float q[5], f[3];
#pragma unroll
            for (int c = 0; c < 5; c++)
                q[c] = u[cell * 5 + c];
#pragma unroll
            for (int c = 0; c < 3; c++)
                f[c] = b[cell * 3 + c];
            const float sp = mhd::cfl_speed<float, false>(q, f);
            if (sp != sp)
                ln = max(ln, (int)cell);
            else
                m = fmaxf(m, sp);
        }
    }
    m = mhd::warp_max<float>(m);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        ln = max(ln, __shfl_xor_sync(0xffffffffu, ln, o));
    if ((threadIdx.x & 31) == 0) {
        rm[threadIdx.x >> 5] = m;
        rn[threadIdx.x >> 5] = ln;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float cm = 0.0f;
        int lnan = -1;
        for (int w = 0; w < kThreads / 32; w++) {
            cm = fmaxf(cm, rm[w]);
            lnan = max(lnan, rn[w]);
        }
        part[blockIdx.x].cmax = cm;
        part[blockIdx.x].last_nan = lnan;
    }
}

// Second pass (one CTA): max over the partials; after a NaN cell at linear
// index L the reference's running max restarts (C/calcfl.c:55, max_2num), so
// the result is the max over the cells after L (NaN when L is the last cell).
__global__ void __launch_bounds__(1024) k_cfl_static_final(const mhd::CflPart<float>* part, int nparts,
                                                          const float* __restrict__ u, const float* __restrict__ b,
                                                          size_t ncell, float* out)
{
    __shared__ float rm[32];
    __shared__ int rn[32];
    float m = 0.0f;
    int ln = -1;
    for (int s = threadIdx.x; s < nparts; s += blockDim.x) {
        m = fmaxf(m, part[s].cmax);
        ln = max(ln, part[s].last_nan);
    }
    m = mhd::warp_max<float>(m);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        ln = max(ln, __shfl_xor_sync(0xffffffffu, ln, o));
    if ((threadIdx.x & 31) == 0) {
        rm[threadIdx.x >> 5] = m;
        rn[threadIdx.x >> 5] = ln;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float cm = 0.0f;
        int lnan = -1;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            cm = fmaxf(cm, rm[w]);
            lnan = max(lnan, rn[w]);
        }
        rm[0] = cm;
        rn[0] = lnan;
    }
    __syncthreads();
    float c = rm[0];
    const int lnan = rn[0];
    if (lnan >= 0) {  // rare: rescan the cells after the last NaN
        float mm = 0.0f;
        for (size_t cell = (size_t)lnan + 1 + threadIdx.x; cell < ncell; cell += blockDim.x) {
            float q[5], f[3];
            for (int k = 0; k < 5; k++)
                q[k] = u[cell * 5 + k];
            for (int k = 0; k < 3; k++)
                f[k] = b[cell * 3 + k];
            const float sp = mhd::cfl_speed<float, false>(q, f);
            if (sp == sp)
                mm = fmaxf(mm, sp);
        }
        mm = mhd::warp_max<float>(mm);
        __syncthreads();
        if ((threadIdx.x & 31) == 0)
            rm[threadIdx.x >> 5] = mm;
        __syncthreads();
        if (threadIdx.x == 0) {
            float r = 0.0f;
            for (int w = 0; w < (int)(blockDim.x >> 5); w++)
                r = fmaxf(r, rm[w]);
            rm[0] = r;
        }
        __syncthreads();
        c = ((size_t)lnan + 1 >= ncell) ? NAN : rm[0];
    }
    if (threadIdx.x == 0)
        *out = 1.0f / c;
}

// Device address of the scratch for the current device, looked up once.
int scratch_for_current_device(mhd::CflPart<float>** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return MHD_ERR_CUDA;
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_parts_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_parts);
        if (e != cudaSuccess || !p)
            return MHD_ERR_CUDA;
        g_parts_addr[dev] = static_cast<mhd::CflPart<float>*>(p);
    }
    *out = g_parts_addr[dev];
    return MHD_OK;
}

}  // namespace

extern "C" MHD_API int mhd_calcfl_noalloc(const float* u, const float* b, int nx, int ny, int nz, float* inv_cmax,
                                          void* stream)
{
    if (!u || !b || !inv_cmax || nx <= 0 || ny <= 0 || nz <= 0)
        return MHD_ERR_ARG;
    const long long ncell = (long long)nx * ny * nz;
    if (ncell > kMaxCells) {
        fprintf(stderr, "mhd_calcfl_noalloc: %lld cells exceed the static scratch limit of %lld cells\n", ncell,
                kMaxCells);
        return MHD_ERR_UNSUPPORTED;
    }
    mhd::CflPart<float>* parts = nullptr;
    const int st = scratch_for_current_device(&parts);
    if (st != MHD_OK)
        return st;
    const int nparts = (int)((ncell + kCellsPerBlock - 1) / kCellsPerBlock);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_cfl_static_parts<<<nparts, kThreads, 0, s>>>(u, b, (size_t)ncell, parts);
    k_cfl_static_final<<<1, 1024, 0, s>>>(parts, nparts, u, b, (size_t)ncell, inv_cmax);
    return (cudaGetLastError() == cudaSuccess) ? MHD_OK : MHD_ERR_CUDA;
}

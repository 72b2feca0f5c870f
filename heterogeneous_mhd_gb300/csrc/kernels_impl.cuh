// Launcher bodies shared by the kernel-set translation units.  Included once
// per unit with MHD_SET_NAME, MHD_REAL and MHD_EXACT defined.
#include "mhd_launch.h"

namespace mhd {
namespace MHD_SET_NAME {

using R = MHD_REAL;
constexpr bool EX = MHD_EXACT;

static cudaError_t fluidx(const FluidxArgs& a, cudaStream_t s)
{
    static bool attr = false;
    const size_t smem = fluidx_smem_elems(a.nx, a.P) * sizeof(R);
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_fluidx<R, EX>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (e != cudaSuccess)
            return e;
        attr = true;
    }
    dim3 grid(a.ny / a.P, a.nz);
    k_fluidx<R, EX><<<grid, fluidx_threads(a.nx, a.P), smem, s>>>(a);
    return cudaGetLastError();
}

static cudaError_t advect(const AdvectArgs& a, cudaStream_t s)
{
    static bool attr = false;
    const size_t smem = advect_smem_elems(a.nx, a.P) * sizeof(R);
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(k_advect<R, EX>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        if (e != cudaSuccess)
            return e;
        attr = true;
    }
    int threads = ((a.nx * a.P + 31) / 32) * 32;
    if (threads > 512)
        threads = 512;
    if (threads < 128)
        threads = 128;
    dim3 grid(a.ny / a.P, a.nz);
    k_advect<R, EX><<<grid, threads, smem, s>>>(a);
    return cudaGetLastError();
}

static cudaError_t transpose(const TransposeArgs& a, cudaStream_t s)
{
    constexpr int T = TTile<R>::E;
    const int na = (a.axis == 1) ? a.ny : a.nz;
    const int nb = (a.axis == 1) ? a.nz : a.ny;
    dim3 grid((a.nx + T - 1) / T, (na + T - 1) / T, nb);
    k_transpose<R><<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

static cudaError_t calcfl(const void* u, const void* b, size_t ncell, void* part, int* nparts, cudaStream_t s)
{
    const int blocks = (int)((ncell + 255) / 256);
    *nparts = blocks;
    k_calcfl<R, EX><<<blocks, 256, 0, s>>>(static_cast<const R*>(u), static_cast<const R*>(b), ncell,
                                           static_cast<CflPart<R>*>(part));
    return cudaGetLastError();
}

static cudaError_t cfl_finalize(const CflFinalizeArgs& a, cudaStream_t s)
{
    k_cfl_finalize<R, EX><<<1, 1024, 0, s>>>(a);
    return cudaGetLastError();
}

static cudaError_t divb(const void* b, int nx, int ny, int nz, double* part, int* nparts, cudaStream_t s)
{
    const size_t ncell = (size_t)nx * ny * nz;
    const int blocks = (int)((ncell + 255) / 256);
    *nparts = blocks;
    k_divb<R><<<blocks, 256, 0, s>>>(static_cast<const R*>(b), nx, ny, nz, part);
    return cudaGetLastError();
}

static const KernelSet kSet = {(int)sizeof(R), EX ? 1 : 0, fluidx, advect, transpose, calcfl, cfl_finalize, divb,
                               sizeof(CflPart<R>)};

}  // namespace MHD_SET_NAME
}  // namespace mhd

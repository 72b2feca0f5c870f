// FP32 kernels with FMA contraction (the production path).
#define MHD_SET_NAME set_f32_fast
#define MHD_REAL float
#define MHD_EXACT false
#include "kernels_impl.cuh"

namespace mhd {

const KernelSet* kernels_f32_fast() { return &set_f32_fast::kSet; }

static int pick_pencils(int nx, int ny, int target)
{
    int best = 1;
    for (int p = 1; p <= ny; p++)
        if (ny % p == 0 && (long long)p * nx <= target)
            best = p;
    return best;
}

int fluidx_pencils(int nx, int ny) { return pick_pencils(nx, ny, nx >= 256 ? nx : 256); }
int advect_pencils(int nx, int ny) { return pick_pencils(nx, ny, nx >= 256 ? nx : 256); }

cudaError_t launch_copy(const void* src, void* dst, size_t bytes, cudaStream_t s)
{
    if (bytes == 0)
        return cudaSuccess;
    const bool al16 = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) == 0;
    if (al16 && bytes % 16 == 0) {
        size_t n16 = bytes / 16;
        int blocks = (int)((n16 + 255) / 256);
        if (blocks > 152 * 16)
            blocks = 152 * 16;
        k_copy16<<<blocks, 256, 0, s>>>(static_cast<const uint4*>(src), static_cast<uint4*>(dst), n16);
    } else {
        size_t n4 = bytes / 4;
        int blocks = (int)((n4 + 255) / 256);
        if (blocks > 152 * 16)
            blocks = 152 * 16;
        k_copy4<<<blocks, 256, 0, s>>>(static_cast<const float*>(src), static_cast<float*>(dst), n4);
    }
    return cudaGetLastError();
}

}  // namespace mhd

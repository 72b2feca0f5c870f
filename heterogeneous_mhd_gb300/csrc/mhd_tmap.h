// Host-side encoding of TMA tensor maps (cuTensorMapEncodeTiled), reached
// through the runtime's driver entry point so that the library needs no link
// against libcuda.  Used by the launchers of the fused step's sweeps along y
// and z, whose tensor maps describe the x-major state as a 3-D array of
// floats: (words of one x line, y, z).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

namespace mhd {

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline EncodeTiledFn encode_tiled_fn()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// A 3-D float tensor map over `base` with extents (w words, ny, nz), rows of
// w words (w * 4 bytes a multiple of 16) and a box of (bw, by, bz) elements.
inline cudaError_t encode_map_3d(CUtensorMap* map, const void* base, uint64_t w, uint64_t ny, uint64_t nz,
                                 uint32_t bw, uint32_t by, uint32_t bz)
{
    const EncodeTiledFn fn = encode_tiled_fn();
    if (!fn)
        return cudaErrorNotSupported;
    const cuuint64_t dims[3] = {w, ny, nz};
    const cuuint64_t strides[2] = {w * sizeof(float), w * ny * sizeof(float)};
    const cuuint32_t box[3] = {bw, by, bz};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return (r == CUDA_SUCCESS) ? cudaSuccess : cudaErrorInvalidValue;
}

// A 2-D float tensor map over `rows` rows of w words each (w * 4 bytes a
// multiple of 16), a box of (w, by) elements, with the given shared-memory
// swizzle: the 16-byte chunk c of a row lands at chunk c ^ (address bits
// 7.. of the row) in shared memory, which spreads the rows' chunks over the
// banks when consecutive rows are read by consecutive lanes.
inline cudaError_t encode_map_2d(CUtensorMap* map, const void* base, uint64_t w, uint64_t rows, uint32_t by,
                                 CUtensorMapSwizzle swizzle)
{
    const EncodeTiledFn fn = encode_tiled_fn();
    if (!fn)
        return cudaErrorNotSupported;
    const cuuint64_t dims[2] = {w, rows};
    const cuuint64_t strides[1] = {w * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)w, by};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return (r == CUDA_SUCCESS) ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace mhd

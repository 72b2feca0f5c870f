// Kernels that reproduce the reference's arithmetic bit for bit: compiled
// with --fmad=false (no contraction) and IEEE division and square root.
// FP32 is the reference as shipped; FP64 is the reference built with
// -Dfloat=double.
#define MHD_SET_NAME set_f32_exact
#define MHD_REAL float
#define MHD_EXACT true
#include "kernels_impl.cuh"
#undef MHD_SET_NAME
#undef MHD_REAL
#undef MHD_EXACT

#define MHD_SET_NAME set_f64_exact
#define MHD_REAL double
#define MHD_EXACT true
#include "kernels_impl.cuh"

namespace mhd {
const KernelSet* kernels_f32_exact() { return &set_f32_exact::kSet; }
const KernelSet* kernels_f64_exact() { return &set_f64_exact::kSet; }
}  // namespace mhd

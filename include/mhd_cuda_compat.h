/* The reference's CUDA-side entry points (Cuda/cuda_subroutine.h:4-12), as
 * thin compatibility names over libmhd_gb300's kernels.  All arrays are
 * device arrays; the int* nx/ny/nz arguments are the reference's device
 * copies of the dimensions (unused) and h_nx/h_ny/h_nz its host copies
 * (used).  The arithmetic is that of the reference's C path (C/), which its
 * own Cuda/ port departs from; MHD_GB300_MODE=exact selects the kernels that
 * reproduce it bit for bit.  Each call returns when its work is done; the
 * status of the last call is mhd_last_error().
 *
 *   cuda_cfl          *h_dt = 1/max speed (also copied to dt on the device)
 *   cuda_fluidx       u <- fluidx(u, b) in place, dt read on the device
 *   cuda_advectbyzx   b <- advectbyzx(u, b) in place; temp is not used
 *   cuda_transpose12  (ut, bt) <- transpose12(u, b), then (u, b) <- (ut, bt)
 *   cuda_transpose13  (ut, bt) <- transpose13(u, b), then (u, b) <- (ut, bt);
 *                     nx == nz, or the degenerate nz == 1 / nx == 1 boxes
 *                     (Cuda/cuda_transpose13.cu:27-42)
 */
#ifndef MHD_CUDA_COMPAT_H
#define MHD_CUDA_COMPAT_H

#include "mhd_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

MHD_API void cuda_cfl(float *cfl_u, float *cfl_b, int *cfl_nx, int *cfl_ny, int *cfl_nz, float *cfl_dt,
                      float *cfl_c, int *h_cfl_nx, int *h_cfl_ny, int *h_cfl_nz, float *h_cfl_dt);
MHD_API void cuda_fluidx(float *flu_u, float *flu_b, int *flu_nx, int *flu_ny, int *flu_nz, float *flu_dt,
                         int *h_fluidx_nx, int *h_fluidx_ny, int *h_fluidx_nz);
MHD_API void cuda_advectbyzx(float *adv_u, float *adv_b, int *adv_nx, int *adv_ny, int *adv_nz, float *adv_dt,
                             float *adv_temp, int *h_adv_nx, int *h_adv_ny, int *h_adv_nz);
MHD_API void cuda_transpose12(float *t12_ut, float *t12_bt, float *t12_u, float *t12_b, int *t12_nx, int *t12_ny,
                              int *t12_nz, int *h_t12_nx, int *h_t12_ny, int *h_t12_nz);
MHD_API void cuda_transpose13(float *t13_ut, float *t13_bt, float *t13_u, float *t13_b, int *t13_nx, int *t13_ny,
                              int *t13_nz, int *h_t13_nx, int *h_t13_ny, int *h_t13_nz);

#ifdef __cplusplus
}
#endif
#endif /* MHD_CUDA_COMPAT_H */

/* Learned closure for the coarse solver: C ABI of its GPU kernels.
 *
 * No counterpart in the reference, which has no learned model.  The closure
 * is a periodic 3-D convolution net on the coarse state (8 input channels:
 * rho, mx, my, mz, E and the cell-centred B; hidden layers of 32 channels
 * with 3^3 kernels and GELU; a 1^3 head with 8 outputs: 5 fluid corrections
 * and 3 edge EMFs).  Its B correction is the curl of the predicted EMF on the
 * staggered grid, so div B is unchanged.
 *
 * All pointers are device pointers; every call is queued on `stream` (a
 * cudaStream_t, NULL for the default stream) and returns an MHD_* status of
 * mhd_gb300.h.  Tensors of a batch of nb periodic boxes of edge n (a multiple
 * of 8) are [nb][n][n][n][C] with the channels innermost, BF16 unless noted.
 * Weights are FP32 masters [cout][taps][cin] packed by mhd_cl_pack into the
 * BF16 layouts the convolution kernels read.
 */
#ifndef MHD_CLOSURE_H
#define MHD_CLOSURE_H

#include "mhd_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* convolution kinds (implicit GEMM on the BF16 tensor cores, FP32 accumulation) */
#define MHD_CL_FWD_IN 0     /* 16 (8 used) -> 32, 3^3, y = GELU(z) BF16, zsave = z BF16 */
#define MHD_CL_FWD_HID 1    /* 32 -> 32, 3^3, y = GELU(z), zsave = z */
#define MHD_CL_FWD_HEAD 2   /* 32 -> 8, 1^3, y = z FP32 */
#define MHD_CL_DGRAD_HEAD 3 /* d out (16, 8 used) -> d z of the last hidden layer: times GELU'(zprev) */
#define MHD_CL_DGRAD_HID 4  /* d z (32) -> d z of the previous layer (32): times GELU'(zprev) */

/* weight-gradient kinds: dW[co][tap][ci] (FP32) from the layer input a and d z */
#define MHD_CL_WG_IN 0      /* a: 16 channels, d z: 32, 3^3 -> dW [32][27][8] */
#define MHD_CL_WG_HID 1     /* a: 32, d z: 32, 3^3 -> dW [32][27][32] */
#define MHD_CL_WG_HEAD 2    /* a: 32, d out: 16 (8 used), 1^3 -> dW [8][1][32] */

MHD_API int mhd_cl_conv(int kind, const void *x, const void *w, const float *bias, void *y, void *zsave,
                        const void *zprev, int nb, int n, void *stream);
/* The 3^3 kinds (FWD_IN, FWD_HID, DGRAD_HID) run on tcgen05 (TMEM accumulators) when n is a multiple
 * of 16, on mma.sync otherwise; mhd_cl_use_tcgen05(0) forces mma.sync everywhere, (1) selects the
 * warp-specialised tcgen05 kernel (the default), (2) the two-buffer tcgen05 kernel with one loop for
 * all warps (returns the previous setting).  mhd_cl_device_errors returns (and clears) the tcgen05
 * kernels' timeout bits. */
MHD_API int mhd_cl_use_tcgen05(int enable);
MHD_API int mhd_cl_device_errors(void);
/* bytes of FP32 scratch that mhd_cl_wgrad needs (-1 for a bad argument) */
MHD_API long long mhd_cl_wgrad_scratch(int kind, int nb, int n);
MHD_API int mhd_cl_wgrad(int kind, const void *a, const void *dz, float *scratch, float *dw, int nb, int n,
                         void *stream);
/* out[c] = sum over count rows of x[.][c] for c < nout (bias gradients); scratch: 256 * channels floats */
MHD_API int mhd_cl_colsum(const void *x, int channels, long long count, int nout, float *scratch, float *out,
                          void *stream);
/* loss: out FP32 [nb,n^3,8], target BF16 [nb,n^3,8] (5 fluid, 3 face residual targets, normalised);
 * writes d loss/d out as BF16 [nb,n^3,16] (channels 8..15 zero) and *loss = sum of squared residuals
 * (the loss is that over 8 nb n^3).  rb_scratch: 3 nb n^3 floats, loss_scratch: 512 floats. */
MHD_API int mhd_cl_loss(const float *out, const void *target, void *dout, float *rb_scratch, float *loss_scratch,
                        float *loss, int nb, int n, void *stream);
/* net input of one box from its state: raw FP32 [n^3][8] and/or standardised BF16 [n^3][16] */
MHD_API int mhd_cl_features(const float *u, const float *b, int n, const float *mean, const float *inv_std,
                            float *raw, void *x, void *stream);
MHD_API int mhd_cl_normalize(const float *x, int channels, long long count, const float *mean,
                             const float *inv_std, void *y, int out_channels, void *stream);
/* sums[c] += sum x[.][c], sums[channels + c] += sum x[.][c]^2 (FP64; zero them first) */
MHD_API int mhd_cl_moments(const float *x, int channels, long long count, double *sums, void *stream);
/* box filter of a fine FP32 state by `factor`: cell means and means of the fine faces of each coarse face */
MHD_API int mhd_cl_filter(const float *u_fine, const float *b_fine, int n_fine, int factor, float *u_coarse,
                          float *b_coarse, void *stream);
/* d[n^3][8] = (ua - ub, ba - bb) */
MHD_API int mhd_cl_diff(const float *ua, const float *ba, const float *ub, const float *bb, int n, float *d,
                        void *stream);
/* correction step on one box: u += a oscale (out[0..4] - its box mean), b += a bscale (-curl E),
 * E = out[5..7] (removing the means conserves mass, momentum and energy), for a = 1, else 1/2, else
 * 1/4: the first candidate with rho > 0 and p > 0 in every cell and a total energy that moves by at
 * most ecap of itself is committed; if none is, the state is left as it is and *fallbacks is
 * incremented.  All on the device (no host synchronisation).  dt (device, may be NULL): the
 * half step of the step just taken (the clock's dt, mhd_clock_ptr); nothing is done when it is not
 * above dt_min (an empty step of a run already at its final time).
 * u_tmp, b_tmp: candidate buffers; flags: 4 ints; esum: 8 doubles. */
MHD_API int mhd_cl_apply(float *u, float *b, const float *out, int n, const float *oscale, float bscale,
                         float *u_tmp, float *b_tmp, int *flags, double *esum, float ecap,
                         long long *fallbacks, const float *dt, float dt_min, void *stream);
/* AdamW with decoupled weight decay, bias-corrected moments (step >= 1) */
MHD_API int mhd_cl_adamw(float *p, const float *g, float *m, float *v, long long count, int step, float lr,
                         float beta1, float beta2, float eps, float wd, void *stream);
/* master W[cout_real][taps][cin_real] -> forward BF16 [cout_pad][taps][cin_pad] and data-gradient BF16
 * [cin_pad][taps][cout_pad] with the taps flipped; either output may be NULL */
MHD_API int mhd_cl_pack(const float *w, int cout_real, int cin_real, int taps, int cout_pad, int cin_pad,
                        void *w_fwd, void *w_dgrad, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* MHD_CLOSURE_H */

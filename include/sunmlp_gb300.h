/* ---------------------------------------------------------------------------
 * sunmlp_gb300.h -- the learned Newton predictor of the batched BDF
 * integrator: a 129 -> 64 -> 64 -> 64 multilayer perceptron (ReLU hidden
 * layers) with BF16 weights and activations and FP32 accumulation, trained
 * and evaluated by this library's own sm_103a kernels.  No counterpart in the
 * reference (CVODE always starts Newton from the BDF predictor,
 * src/cvode/cvode_nls.c:256-310).
 *
 * Input (SUNMLP_IN features, padded with zeros to SUNMLP_IN_PAD):
 *   x[i]        i < 64   log10(|y_pred,i| + 1e-12)/12 + 1  (species i < n, else 0)
 *   x[64]                log10(gamma)/10, gamma = h * l1 of the Newton matrix
 *   x[65+i]     i < 64   log10(1 + gamma * lambda_i)/10, lambda_i the local
 *                        first-order consumption rate of species i at y_pred
 * Output o[i], i < n: the Newton corrector y_n - y_pred in error-weight units
 * (o_i = ycor_i * ewt_i); the integrator starts Newton from ycor_i = o_i / ewt_i
 * when that initial residual is smaller than the predictor's, else from 0.
 *
 * Parameters (FP32 master copy, this order): W1[144][64], b1[64],
 * W2[64][64], b2[64], W3[64][64], b3[64]  (W[k][j]: input k -> unit j).
 * ------------------------------------------------------------------------- */
#ifndef SUNMLP_GB300_H
#define SUNMLP_GB300_H

#include <stdint.h>

#include "sundials_gb300_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SUNMLP_IN       129
#define SUNMLP_IN_PAD   144
#define SUNMLP_HID      64
#define SUNMLP_OUT      64
#define SUNMLP_NPARAMS  (144 * 64 + 64 + 64 * 64 + 64 + 64 * 64 + 64)
#define SUNMLP_TILE     128 /* training rows per thread block */

typedef struct SUNMLP_GB300_* SUNMLP_GB300;

/* Weights He-initialised from a SplitMix64 stream of `seed`, biases zero,
 * Adam moments zero.  All work on the given cudaStream_t (NULL: legacy). */
SUNGB300_EXPORT SUNMLP_GB300 SUNMLP_GB300_Create(uint64_t seed, void* cuda_stream);
SUNGB300_EXPORT void SUNMLP_GB300_Free(SUNMLP_GB300 m);
/* Host copies of the FP32 master parameters (SUNMLP_NPARAMS floats). */
SUNGB300_EXPORT SUNErrCode SUNMLP_GB300_SetParams(SUNMLP_GB300 m, const float* host);
SUNGB300_EXPORT SUNErrCode SUNMLP_GB300_GetParams(SUNMLP_GB300 m, float* host);
/* Device pointers of the BF16 weight copy (W1, W2, W3 back to back) and of
 * the FP32 biases (b1, b2, b3), as the integrator reads them. */
SUNGB300_EXPORT const uint16_t* SUNMLP_GB300_DeviceWeights(SUNMLP_GB300 m);
SUNGB300_EXPORT const float* SUNMLP_GB300_DeviceBiases(SUNMLP_GB300 m);

/* Inference on `rows` feature rows (device BF16, row stride SUNMLP_IN_PAD):
 * out (device FP32, rows x 64), one warp per row, the integrator's arithmetic. */
SUNGB300_EXPORT SUNErrCode SUNMLP_GB300_Forward(SUNMLP_GB300 m, int64_t rows,
                                               const uint16_t* d_x, float* d_out);
/* Mean-squared-error loss over rows x 64 outputs against d_t (device FP32)
 * and its gradient w.r.t. the parameters (d_grad: device, SUNMLP_NPARAMS
 * floats, FP32 master layout), by the tensor-core training kernels.  rows
 * must be a multiple of SUNMLP_TILE.  *loss is written on the host. */
SUNGB300_EXPORT SUNErrCode SUNMLP_GB300_Gradients(SUNMLP_GB300 m, int64_t rows,
                                                 const uint16_t* d_x, const float* d_t,
                                                 float* d_grad, float* loss);
/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on that gradient; the
 * BF16 copy is refreshed.  *loss (host, may be NULL) gets the batch loss. */
SUNGB300_EXPORT SUNErrCode SUNMLP_GB300_TrainStep(SUNMLP_GB300 m, int64_t rows,
                                                 const uint16_t* d_x, const float* d_t,
                                                 float lr, float* loss);

#ifdef __cplusplus
}
#endif

#endif /* SUNMLP_GB300_H */

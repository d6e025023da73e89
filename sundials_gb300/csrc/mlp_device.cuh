// mlp_device.cuh -- device pieces of the learned Newton predictor shared by
// the integrator (inference inside the persistent BDF kernel), the batched
// inference kernel and the training kernels: feature transforms, parameter
// layout and the warp-per-row forward pass (BF16 weights and activations,
// FP32 accumulation on the CUDA cores: one input row is a matrix-vector
// product, which tensor cores cannot speed up).
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace gb300mlp {

constexpr int IN = 129, INP = 144, HID = 64, OUT = 64;
// BF16 weight copy: W1 | W2 | W3, each row-major W[k][j]
constexpr int WB_W1 = 0, WB_W2 = INP * HID, WB_W3 = INP * HID + HID * HID;
constexpr int WB_TOTAL = INP * HID + 2 * HID * HID;
// FP32 biases: b1 | b2 | b3
constexpr int BB_B1 = 0, BB_B2 = HID, BB_B3 = 2 * HID;
// FP32 master parameters: W1, b1, W2, b2, W3, b3
constexpr int P_W1 = 0, P_B1 = INP * HID, P_W2 = P_B1 + HID, P_B2 = P_W2 + HID * HID;
constexpr int P_W3 = P_B2 + HID, P_B3 = P_W3 + HID * OUT, P_TOTAL = P_B3 + OUT;

__device__ __forceinline__ float bf16_round(float v)
{
  return __bfloat162float(__float2bfloat16_rn(v));
}

// Feature transforms (FP32: the features only steer a guess).
__device__ __forceinline__ float feat_y(double y)
{
  return log10f(fabsf((float)y) + 1e-12f) * (1.0f / 12.0f) + 1.0f;
}
__device__ __forceinline__ float feat_gamma(double g) { return log10f((float)g) * 0.1f; }
__device__ __forceinline__ float feat_rate(double gl) { return log10f(1.0f + (float)gl) * 0.1f; }

// The network on one row, by one warp.  xr[c] holds the BF16-rounded feature
// x[32c + lane] (zero at and past SUNMLP_IN); on return o0 / o1 are outputs
// 2*lane and 2*lane + 1.  Hidden activations are rounded to BF16 as in
// training.
__device__ __forceinline__ void warp_forward(const uint16_t* __restrict__ Wb,
                                             const float* __restrict__ Bb, const float (&xr)[5],
                                             int lane, float& o0, float& o1)
{
  const __nv_bfloat162* W = reinterpret_cast<const __nv_bfloat162*>(Wb);
  float a0 = Bb[BB_B1 + 2 * lane], a1 = Bb[BB_B1 + 2 * lane + 1];
#pragma unroll
  for (int c = 0; c < 5; ++c)
  {
    const int kmax = (c == 4) ? INP - 128 : 32;
    for (int kk = 0; kk < kmax; ++kk)
    {
      const float xk  = __shfl_sync(0xffffffffu, xr[c], kk);
      const float2 wv = __bfloat1622float2(W[(WB_W1 / 2) + (32 * c + kk) * 32 + lane]);
      a0              = fmaf(xk, wv.x, a0);
      a1              = fmaf(xk, wv.y, a1);
    }
  }
  float h0 = bf16_round(fmaxf(a0, 0.0f)), h1 = bf16_round(fmaxf(a1, 0.0f));
  a0 = Bb[BB_B2 + 2 * lane];
  a1 = Bb[BB_B2 + 2 * lane + 1];
  for (int k = 0; k < HID; ++k)
  {
    const float xk  = __shfl_sync(0xffffffffu, (k & 1) ? h1 : h0, k >> 1);
    const float2 wv = __bfloat1622float2(W[(WB_W2 / 2) + k * 32 + lane]);
    a0              = fmaf(xk, wv.x, a0);
    a1              = fmaf(xk, wv.y, a1);
  }
  h0 = bf16_round(fmaxf(a0, 0.0f));
  h1 = bf16_round(fmaxf(a1, 0.0f));
  a0 = Bb[BB_B3 + 2 * lane];
  a1 = Bb[BB_B3 + 2 * lane + 1];
  for (int k = 0; k < HID; ++k)
  {
    const float xk  = __shfl_sync(0xffffffffu, (k & 1) ? h1 : h0, k >> 1);
    const float2 wv = __bfloat1622float2(W[(WB_W3 / 2) + k * 32 + lane]);
    a0              = fmaf(xk, wv.x, a0);
    a1              = fmaf(xk, wv.y, a1);
  }
  o0 = a0;
  o1 = a1;
}

}  // namespace gb300mlp

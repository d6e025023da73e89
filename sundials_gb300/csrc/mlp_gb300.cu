// mlp_gb300.cu -- training and batched inference of the learned Newton
// predictor (include/sunmlp_gb300.h).
//
// Training step = two kernels:
//  * k_mlp_tile: one 128-thread block per 128 rows runs the forward pass,
//    the MSE loss and the whole backward pass with every operand in shared
//    memory (BF16 features, activations, gradients and weights), all GEMMs on
//    the tensor cores (mma.sync m16n8k16, BF16 inputs, FP32 accumulation),
//    and writes its weight / bias gradient partials and loss partial;
//  * k_mlp_reduce: sums the partials in block order (deterministic, no float
//    atomics) and either stores the gradient or applies one Adam step to the
//    FP32 master parameters and refreshes their BF16 copy.
// The layer widths (64) are too small for tcgen05's 128-row tiles to pay:
// a whole training step is a few microseconds of tensor work.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "../../include/sunmlp_gb300.h"
#include "gb300_common.cuh"
#include "mlp_device.cuh"

using namespace gb300;
using namespace gb300mlp;

static_assert(P_TOTAL == SUNMLP_NPARAMS, "parameter layout");
static_assert(INP == SUNMLP_IN_PAD && IN == SUNMLP_IN, "input width");

struct SUNMLP_GB300_
{
  cudaStream_t stream;
  float* master;     // P_TOTAL
  float* adam_m;     // P_TOTAL
  float* adam_v;     // P_TOTAL
  uint16_t* wb;      // WB_TOTAL (BF16 weights)
  float* bias;       // 3 * 64
  float* partials;   // [blocks][P_TOTAL + 1] (last: loss)
  int64_t part_blocks;
  float* grad;       // P_TOTAL scratch for TrainStep
  float* h_loss;     // pinned
  float* d_loss;
  long step;
};

namespace {

constexpr int TR   = SUNMLP_TILE;  // rows per block
constexpr int TW   = 4;            // warps per block
constexpr int SX   = INP + 8;      // smem row strides (elements), conflict-avoiding
constexpr int SH   = HID + 8;
constexpr int SO   = HID + 4;      // fp32 dO stride

struct TileSmem
{
  __nv_bfloat16 x[TR * SX];
  __nv_bfloat16 h1[TR * SH], h2[TR * SH], g1[TR * SH], g2[TR * SH];
  __nv_bfloat16 w1[INP * SH], w2[HID * SH], w3[HID * SH];
  float dof[TR * SO];
  float bias[3 * HID];
  float red[TW];
};

__device__ __forceinline__ uint32_t ld32(const __nv_bfloat16* p)
{
  return *reinterpret_cast<const uint32_t*>(p);
}
__device__ __forceinline__ uint32_t pack2(const __nv_bfloat16* lo, const __nv_bfloat16* hi)
{
  return (uint32_t)__bfloat16_as_ushort(*lo) | ((uint32_t)__bfloat16_as_ushort(*hi) << 16);
}

__device__ __forceinline__ void mma16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2,
                                         uint32_t a3, uint32_t b0, uint32_t b1)
{
  asm volatile(
    "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
    "{%8,%9}, {%0,%1,%2,%3};\n"
    : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
    : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Fragment loads for A (16 x 16) and B (16 x 8) of mma.m16n8k16, from shared
// memory holding the logical matrix either as stored (row-major, element
// [r][c] at p[r*ld + c]) or transposed (element [r][c] at p[c*ld + r]).
struct Frag
{
  int g, t;  // lane / 4, lane % 4
};
__device__ __forceinline__ void load_a(const __nv_bfloat16* p, int ld, bool trans, int m0, int k0,
                                       Frag f, uint32_t (&a)[4])
{
  const int r0 = m0 + f.g, r1 = r0 + 8, c0 = k0 + 2 * f.t, c1 = c0 + 8;
  if (!trans)
  {
    a[0] = ld32(p + r0 * ld + c0);
    a[1] = ld32(p + r1 * ld + c0);
    a[2] = ld32(p + r0 * ld + c1);
    a[3] = ld32(p + r1 * ld + c1);
  }
  else
  {
    a[0] = pack2(p + c0 * ld + r0, p + (c0 + 1) * ld + r0);
    a[1] = pack2(p + c0 * ld + r1, p + (c0 + 1) * ld + r1);
    a[2] = pack2(p + c1 * ld + r0, p + (c1 + 1) * ld + r0);
    a[3] = pack2(p + c1 * ld + r1, p + (c1 + 1) * ld + r1);
  }
}
__device__ __forceinline__ void load_b(const __nv_bfloat16* p, int ld, bool trans, int k0, int n0,
                                       Frag f, uint32_t (&b)[2])
{
  const int n = n0 + f.g, k = k0 + 2 * f.t;
  if (!trans)
  {
    b[0] = pack2(p + k * ld + n, p + (k + 1) * ld + n);
    b[1] = pack2(p + (k + 8) * ld + n, p + (k + 9) * ld + n);
  }
  else
  {
    b[0] = ld32(p + n * ld + k);
    b[1] = ld32(p + n * ld + k + 8);
  }
}

// acc[MT][8][4] += A[m0.., 0..K) * B[0..K, 0..64) for MT 16-row tiles.
template <int MT>
__device__ __forceinline__ void gemm_rows(float (&acc)[MT][8][4], const __nv_bfloat16* A, int lda,
                                          bool ta, const int (&m0)[MT], const __nv_bfloat16* B,
                                          int ldb, bool tb, int K, Frag f)
{
  for (int k0 = 0; k0 < K; k0 += 16)
  {
    uint32_t a[MT][4];
#pragma unroll
    for (int i = 0; i < MT; ++i) load_a(A, lda, ta, m0[i], k0, f, a[i]);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
    {
      uint32_t b[2];
      load_b(B, ldb, tb, k0, nt * 8, f, b);
#pragma unroll
      for (int i = 0; i < MT; ++i) mma16816(acc[i][nt], a[i][0], a[i][1], a[i][2], a[i][3], b[0], b[1]);
    }
  }
}

template <int MT>
__device__ __forceinline__ void zero(float (&acc)[MT][8][4])
{
#pragma unroll
  for (int i = 0; i < MT; ++i)
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e) acc[i][nt][e] = 0.0f;
}

// Hidden-layer epilogue: out[r][c] = bf16(relu(acc + bias[c])).
template <int MT>
__device__ __forceinline__ void store_relu(const float (&acc)[MT][8][4], const int (&m0)[MT],
                                           const float* bias, __nv_bfloat16* out, Frag f)
{
#pragma unroll
  for (int i = 0; i < MT; ++i)
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e)
      {
        const int r = m0[i] + f.g + (e >> 1) * 8, c = nt * 8 + 2 * f.t + (e & 1);
        out[r * SH + c] = __float2bfloat16_rn(fmaxf(acc[i][nt][e] + bias[c], 0.0f));
      }
}

// Backward epilogue: out[r][c] = bf16(acc * (act[r][c] > 0)).
template <int MT>
__device__ __forceinline__ void store_masked(const float (&acc)[MT][8][4], const int (&m0)[MT],
                                             const __nv_bfloat16* act, __nv_bfloat16* out, Frag f)
{
#pragma unroll
  for (int i = 0; i < MT; ++i)
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e)
      {
        const int r = m0[i] + f.g + (e >> 1) * 8, c = nt * 8 + 2 * f.t + (e & 1);
        const bool on = __bfloat162float(act[r * SH + c]) > 0.0f;
        out[r * SH + c] = __float2bfloat16_rn(on ? acc[i][nt][e] : 0.0f);
      }
}

// Weight-gradient tile rows m0.. of an (M x 64) gradient: write to gout[m][c].
template <int MT>
__device__ __forceinline__ void store_grad(const float (&acc)[MT][8][4], const int (&m0)[MT],
                                           float* gout, Frag f)
{
#pragma unroll
  for (int i = 0; i < MT; ++i)
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e)
      {
        const int r = m0[i] + f.g + (e >> 1) * 8, c = nt * 8 + 2 * f.t + (e & 1);
        gout[r * HID + c] = acc[i][nt][e];
      }
}

__device__ __forceinline__ void copy_weights(__nv_bfloat16* dst, const uint16_t* src, int rows)
{
  for (int e = threadIdx.x; e < rows * HID; e += blockDim.x)
  {
    const int r = e / HID, c = e - r * HID;
    dst[r * SH + c] = __ushort_as_bfloat16(src[e]);
  }
}

__global__ void __launch_bounds__(TR)
  k_mlp_tile(const uint16_t* __restrict__ X, const float* __restrict__ T,
             const uint16_t* __restrict__ Wb, const float* __restrict__ Bb, float scale,
             float* __restrict__ partials)
{
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TileSmem& S    = *reinterpret_cast<TileSmem*>(smem_raw);
  const int tid  = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const Frag f   = {lane >> 2, lane & 3};
  const int64_t row0 = (int64_t)blockIdx.x * TR;
  float* out     = partials + (size_t)blockIdx.x * (P_TOTAL + 1);

  // ---- stage the tile's features, the weights and the biases
  for (int e = tid; e < TR * INP; e += TR)
  {
    const int r = e / INP, c = e - r * INP;
    S.x[r * SX + c] = __ushort_as_bfloat16(X[(row0 + r) * INP + c]);
  }
  copy_weights(S.w1, Wb + WB_W1, INP);
  copy_weights(S.w2, Wb + WB_W2, HID);
  copy_weights(S.w3, Wb + WB_W3, HID);
  for (int e = tid; e < 3 * HID; e += TR) S.bias[e] = Bb[e];
  __syncthreads();

  // ---- forward: each warp its own 32 rows (two 16-row tiles)
  const int rows[2] = {warp * 32, warp * 32 + 16};
  float acc[2][8][4];
  zero(acc);
  gemm_rows<2>(acc, S.x, SX, false, rows, S.w1, SH, false, INP, f);
  store_relu<2>(acc, rows, S.bias + BB_B1, S.h1, f);
  __syncwarp();
  zero(acc);
  gemm_rows<2>(acc, S.h1, SH, false, rows, S.w2, SH, false, HID, f);
  store_relu<2>(acc, rows, S.bias + BB_B2, S.h2, f);
  __syncwarp();
  zero(acc);
  gemm_rows<2>(acc, S.h2, SH, false, rows, S.w3, SH, false, HID, f);
  // output, loss and dL/dO = scale * (O - T)   (scale = 2 / (rows * 64))
  float lsum = 0.0f;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int e = 0; e < 4; ++e)
      {
        const int r = rows[i] + f.g + (e >> 1) * 8, c = nt * 8 + 2 * f.t + (e & 1);
        const float o  = acc[i][nt][e] + S.bias[BB_B3 + c];
        const float d  = o - T[(row0 + r) * OUT + c];
        lsum           = fmaf(d, d, lsum);
        const float gd = scale * d;
        S.dof[r * SO + c] = gd;
        S.g1[r * SH + c]  = __float2bfloat16_rn(gd);
      }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
  if (lane == 0) S.red[warp] = lsum;
  __syncthreads();

  // ---- backward
  const int wrow[1] = {warp * 16};  // this warp's 16 rows of a 64-row weight gradient
  float gacc[1][8][4];
  // dW3 = H2^T dO
  zero(gacc);
  gemm_rows<1>(gacc, S.h2, SH, true, wrow, S.g1, SH, false, TR, f);
  store_grad<1>(gacc, wrow, out + P_W3, f);
  // db3 = column sums of dO (FP32)
  if (tid < OUT)
  {
    float s = 0.0f;
    for (int r = 0; r < TR; ++r) s += S.dof[r * SO + tid];
    out[P_B3 + tid] = s;
  }
  // dH2 = (dO W3^T) masked by relu'
  zero(acc);
  gemm_rows<2>(acc, S.g1, SH, false, rows, S.w3, SH, true, HID, f);
  store_masked<2>(acc, rows, S.h2, S.g2, f);
  __syncthreads();
  // dW2 = H1^T dH2, db2
  zero(gacc);
  gemm_rows<1>(gacc, S.h1, SH, true, wrow, S.g2, SH, false, TR, f);
  store_grad<1>(gacc, wrow, out + P_W2, f);
  if (tid < HID)
  {
    float s = 0.0f;
    for (int r = 0; r < TR; ++r) s += __bfloat162float(S.g2[r * SH + tid]);
    out[P_B2 + tid] = s;
  }
  // dH1 = (dH2 W2^T) masked by relu'   (into g1: dO is no longer read)
  zero(acc);
  gemm_rows<2>(acc, S.g2, SH, false, rows, S.w2, SH, true, HID, f);
  __syncthreads();
  store_masked<2>(acc, rows, S.h1, S.g1, f);
  __syncthreads();
  // dW1 = X^T dH1 (144 rows: 9 tiles over 4 warps), db1
  {
    const int m0a[1] = {warp * 16};
    zero(gacc);
    gemm_rows<1>(gacc, S.x, SX, true, m0a, S.g1, SH, false, TR, f);
    store_grad<1>(gacc, m0a, out + P_W1, f);
    const int m0b[1] = {(warp + 4) * 16};
    zero(gacc);
    gemm_rows<1>(gacc, S.x, SX, true, m0b, S.g1, SH, false, TR, f);
    store_grad<1>(gacc, m0b, out + P_W1, f);
    if (warp == 0)
    {
      const int m0c[1] = {8 * 16};
      zero(gacc);
      gemm_rows<1>(gacc, S.x, SX, true, m0c, S.g1, SH, false, TR, f);
      store_grad<1>(gacc, m0c, out + P_W1, f);
    }
  }
  if (tid < HID)
  {
    float s = 0.0f;
    for (int r = 0; r < TR; ++r) s += __bfloat162float(S.g1[r * SH + tid]);
    out[P_B1 + tid] = s;
  }
  if (tid == 0) out[P_TOTAL] = ((S.red[0] + S.red[1]) + S.red[2]) + S.red[3];
}

// Sum the per-block partials in block order; then either store the gradient
// (adam == 0) or apply Adam and refresh the BF16 copy.
__global__ void __launch_bounds__(256)
  k_mlp_reduce(const float* __restrict__ partials, int blocks, float* grad, float* loss,
               int adam, float* master, float* am, float* av, uint16_t* wb, float* bias,
               float lr, float bc1, float bc2)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > P_TOTAL) return;
  float g = 0.0f;
  for (int b = 0; b < blocks; ++b) g += partials[(size_t)b * (P_TOTAL + 1) + p];
  if (p == P_TOTAL)
  {
    *loss = g;
    return;
  }
  if (!adam)
  {
    grad[p] = g;
    return;
  }
  const float m = 0.9f * am[p] + 0.1f * g;
  const float v = 0.999f * av[p] + 0.001f * g * g;
  am[p]         = m;
  av[p]         = v;
  const float w = master[p] - lr * (m / bc1) / (sqrtf(v / bc2) + 1e-8f);
  master[p]     = w;
  int wi = -1, bi = -1;
  if (p < P_B1) wi = WB_W1 + p;
  else if (p < P_W2) bi = BB_B1 + (p - P_B1);
  else if (p < P_B2) wi = WB_W2 + (p - P_W2);
  else if (p < P_W3) bi = BB_B2 + (p - P_B2);
  else if (p < P_B3) wi = WB_W3 + (p - P_W3);
  else bi = BB_B3 + (p - P_B3);
  if (wi >= 0) wb[wi] = __bfloat16_as_ushort(__float2bfloat16_rn(w));
  else bias[bi] = w;
}

// One warp per row: the integrator's forward pass.
__global__ void __launch_bounds__(256)
  k_mlp_forward(int64_t rows, const uint16_t* __restrict__ X, const uint16_t* __restrict__ Wb,
                const float* __restrict__ Bb, float* __restrict__ out)
{
  const int lane    = threadIdx.x & 31;
  const int64_t r   = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (r >= rows) return;
  float xr[5];
#pragma unroll
  for (int c = 0; c < 5; ++c)
  {
    const int k = 32 * c + lane;
    xr[c]       = k < INP ? __bfloat162float(__ushort_as_bfloat16(X[r * INP + k])) : 0.0f;
  }
  float o0, o1;
  warp_forward(Wb, Bb, xr, lane, o0, o1);
  out[r * OUT + 2 * lane]     = o0;
  out[r * OUT + 2 * lane + 1] = o1;
}

// Master parameters -> BF16 weight copy and FP32 biases.
__global__ void k_mlp_publish(const float* __restrict__ master, uint16_t* wb, float* bias)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P_TOTAL) return;
  const float w = master[p];
  if (p < P_B1) wb[WB_W1 + p] = __bfloat16_as_ushort(__float2bfloat16_rn(w));
  else if (p < P_W2) bias[BB_B1 + p - P_B1] = w;
  else if (p < P_B2) wb[WB_W2 + p - P_W2] = __bfloat16_as_ushort(__float2bfloat16_rn(w));
  else if (p < P_W3) bias[BB_B2 + p - P_B2] = w;
  else if (p < P_B3) wb[WB_W3 + p - P_W3] = __bfloat16_as_ushort(__float2bfloat16_rn(w));
  else bias[BB_B3 + p - P_B3] = w;
}

uint64_t splitmix64(uint64_t& s)
{
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z          = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z          = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
double unit_uniform(uint64_t& s) { return ((splitmix64(s) >> 11) + 0.5) * 0x1.0p-53; }

bool ensure_partials(SUNMLP_GB300 m, int64_t blocks)
{
  if (blocks <= m->part_blocks) return true;
  if (m->partials) cudaFree(m->partials);
  m->partials    = nullptr;
  m->part_blocks = 0;
  if (!check_cuda(cudaMalloc(&m->partials, sizeof(float) * (size_t)blocks * (P_TOTAL + 1)),
                  "MLP partials cudaMalloc"))
    return false;
  m->part_blocks = blocks;
  return true;
}

SUNErrCode run_tiles(SUNMLP_GB300 m, int64_t rows, const uint16_t* d_x, const float* d_t)
{
  if (rows <= 0 || rows % TR != 0)
  {
    set_error(SUN_ERR_ARG_OUTOFRANGE, "SUNMLP_GB300: rows must be a positive multiple of 128");
    return SUN_ERR_ARG_OUTOFRANGE;
  }
  const int64_t blocks = rows / TR;
  if (!ensure_partials(m, blocks)) return SUN_ERR_MEM_FAIL;
  static bool attr_set = false;
  if (!attr_set)
  {
    if (!check_cuda(cudaFuncSetAttribute(k_mlp_tile, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(TileSmem)),
                    "MLP smem attribute"))
      return SUN_ERR_EXT_FAIL;
    attr_set = true;
  }
  const float scale = 2.0f / ((float)rows * (float)OUT);
  k_mlp_tile<<<(unsigned)blocks, TR, sizeof(TileSmem), m->stream>>>(d_x, d_t, m->wb, m->bias,
                                                                    scale, m->partials);
  count_launch();
  return check_cuda(cudaGetLastError(), "k_mlp_tile launch") ? SUN_SUCCESS : SUN_ERR_EXT_FAIL;
}

}  // namespace

extern "C" {

SUNMLP_GB300 SUNMLP_GB300_Create(uint64_t seed, void* cuda_stream)
{
  SUNMLP_GB300 m = (SUNMLP_GB300)calloc(1, sizeof(*m));
  m->stream      = (cudaStream_t)cuda_stream;
  const size_t pb = sizeof(float) * P_TOTAL;
  bool ok = check_cuda(cudaMalloc(&m->master, pb), "MLP cudaMalloc") &&
            check_cuda(cudaMalloc(&m->adam_m, pb), "MLP cudaMalloc") &&
            check_cuda(cudaMalloc(&m->adam_v, pb), "MLP cudaMalloc") &&
            check_cuda(cudaMalloc(&m->grad, pb), "MLP cudaMalloc") &&
            check_cuda(cudaMalloc(&m->wb, sizeof(uint16_t) * WB_TOTAL), "MLP cudaMalloc") &&
            check_cuda(cudaMalloc(&m->bias, sizeof(float) * 3 * HID), "MLP cudaMalloc") &&
            check_cuda(cudaHostAlloc(&m->h_loss, sizeof(float), cudaHostAllocMapped),
                       "MLP cudaHostAlloc") &&
            check_cuda(cudaHostGetDevicePointer(&m->d_loss, m->h_loss, 0), "MLP mapped pointer");
  if (!ok)
  {
    SUNMLP_GB300_Free(m);
    return nullptr;
  }
  // He initialisation: W ~ N(0, 2 / fan_in) by Box-Muller on a SplitMix64 stream
  std::vector<float> h(P_TOTAL, 0.0f);
  uint64_t s = seed;
  auto fill = [&](int off, int fan_in, int count) {
    const double sd = sqrt(2.0 / fan_in);
    for (int i = 0; i < count; i += 2)
    {
      double u1 = unit_uniform(s), u2 = unit_uniform(s);
      double r = sqrt(-2.0 * log(u1)), a = 6.283185307179586 * u2;
      h[off + i] = (float)(sd * r * cos(a));
      if (i + 1 < count) h[off + i + 1] = (float)(sd * r * sin(a));
    }
  };
  fill(P_W1, IN, INP * HID);
  for (int k = IN; k < INP; ++k)
    for (int j = 0; j < HID; ++j) h[P_W1 + k * HID + j] = 0.0f;  // padding inputs
  fill(P_W2, HID, HID * HID);
  fill(P_W3, HID, HID * OUT);
  if (SUNMLP_GB300_SetParams(m, h.data()) != SUN_SUCCESS)
  {
    SUNMLP_GB300_Free(m);
    return nullptr;
  }
  return m;
}

void SUNMLP_GB300_Free(SUNMLP_GB300 m)
{
  if (!m) return;
  cudaFree(m->master);
  cudaFree(m->adam_m);
  cudaFree(m->adam_v);
  cudaFree(m->grad);
  cudaFree(m->wb);
  cudaFree(m->bias);
  if (m->partials) cudaFree(m->partials);
  if (m->h_loss) cudaFreeHost(m->h_loss);
  free(m);
}

SUNErrCode SUNMLP_GB300_SetParams(SUNMLP_GB300 m, const float* host)
{
  const size_t pb = sizeof(float) * P_TOTAL;
  if (!check_cuda(cudaMemcpyAsync(m->master, host, pb, cudaMemcpyHostToDevice, m->stream),
                  "MLP params upload") ||
      !check_cuda(cudaMemsetAsync(m->adam_m, 0, pb, m->stream), "MLP memset") ||
      !check_cuda(cudaMemsetAsync(m->adam_v, 0, pb, m->stream), "MLP memset"))
    return SUN_ERR_EXT_FAIL;
  m->step = 0;
  k_mlp_publish<<<(P_TOTAL + 255) / 256, 256, 0, m->stream>>>(m->master, m->wb, m->bias);
  count_launch();
  return check_cuda(cudaStreamSynchronize(m->stream), "MLP publish") ? SUN_SUCCESS
                                                                      : SUN_ERR_EXT_FAIL;
}

SUNErrCode SUNMLP_GB300_GetParams(SUNMLP_GB300 m, float* host)
{
  return check_cuda(cudaMemcpyAsync(host, m->master, sizeof(float) * P_TOTAL,
                                    cudaMemcpyDeviceToHost, m->stream),
                    "MLP params download") &&
             check_cuda(cudaStreamSynchronize(m->stream), "MLP sync")
           ? SUN_SUCCESS
           : SUN_ERR_EXT_FAIL;
}

const uint16_t* SUNMLP_GB300_DeviceWeights(SUNMLP_GB300 m) { return m ? m->wb : nullptr; }
const float* SUNMLP_GB300_DeviceBiases(SUNMLP_GB300 m) { return m ? m->bias : nullptr; }

SUNErrCode SUNMLP_GB300_Forward(SUNMLP_GB300 m, int64_t rows, const uint16_t* d_x, float* d_out)
{
  if (rows <= 0) return SUN_SUCCESS;
  const int64_t threads = rows * 32;
  k_mlp_forward<<<(unsigned)((threads + 255) / 256), 256, 0, m->stream>>>(rows, d_x, m->wb,
                                                                          m->bias, d_out);
  count_launch();
  return check_cuda(cudaGetLastError(), "k_mlp_forward launch") ? SUN_SUCCESS : SUN_ERR_EXT_FAIL;
}

SUNErrCode SUNMLP_GB300_Gradients(SUNMLP_GB300 m, int64_t rows, const uint16_t* d_x,
                                  const float* d_t, float* d_grad, float* loss)
{
  SUNErrCode e = run_tiles(m, rows, d_x, d_t);
  if (e != SUN_SUCCESS) return e;
  k_mlp_reduce<<<(P_TOTAL + 1 + 255) / 256, 256, 0, m->stream>>>(
    m->partials, (int)(rows / TR), d_grad, m->d_loss, 0, nullptr, nullptr, nullptr, nullptr,
    nullptr, 0.0f, 1.0f, 1.0f);
  count_launch();
  if (!check_cuda(cudaStreamSynchronize(m->stream), "MLP gradients")) return SUN_ERR_EXT_FAIL;
  if (loss) *loss = *m->h_loss / ((float)rows * (float)OUT);
  return SUN_SUCCESS;
}

SUNErrCode SUNMLP_GB300_TrainStep(SUNMLP_GB300 m, int64_t rows, const uint16_t* d_x,
                                  const float* d_t, float lr, float* loss)
{
  SUNErrCode e = run_tiles(m, rows, d_x, d_t);
  if (e != SUN_SUCCESS) return e;
  m->step++;
  const float bc1 = 1.0f - powf(0.9f, (float)m->step);
  const float bc2 = 1.0f - powf(0.999f, (float)m->step);
  k_mlp_reduce<<<(P_TOTAL + 1 + 255) / 256, 256, 0, m->stream>>>(
    m->partials, (int)(rows / TR), m->grad, m->d_loss, 1, m->master, m->adam_m, m->adam_v, m->wb,
    m->bias, lr, bc1, bc2);
  count_launch();
  if (!check_cuda(cudaGetLastError(), "k_mlp_reduce launch")) return SUN_ERR_EXT_FAIL;
  if (loss)
  {
    if (!check_cuda(cudaStreamSynchronize(m->stream), "MLP step")) return SUN_ERR_EXT_FAIL;
    *loss = *m->h_loss / ((float)rows * (float)OUT);
  }
  return SUN_SUCCESS;
}

}  // extern "C"

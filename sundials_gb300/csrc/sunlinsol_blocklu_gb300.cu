// sunlinsol_blocklu_gb300.cu -- block-diagonal SUNMatrix (ragged dense blocks
// in HBM) and the direct SUNLinearSolver that factors / solves every block in
// batched kernels.  Compiled with -fmad=false: the FP64 path performs the
// reference's GETRF / GETRS / ScaleAddI / Matvec operation for operation, so
// each block is bit-identical to SUNMATRIX_DENSE + SUNLINSOL_DENSE
// (src/sundials/sundials_dense.c:85-193, src/sunmatrix/dense/
// sunmatrix_dense.c:265-330).  The MIXED path uses explicit fmaf / fma.
//
// Work mapping: blocks of at most 8 rows are handled one per thread (their
// LU lives in thread-local memory); larger blocks one per warp, lanes over
// rows, trailing updates spread over all lanes.
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/nvector_gb300.h"
#include "../../include/sunlinsol_blocklu_gb300.h"
#include "gb300_common.cuh"

using namespace gb300;

namespace {

constexpr int kSmall = 8;   // blocks up to this size: one thread per block
constexpr int kMaxBlk = 64; // largest block

struct BDContent
{
  int64_t nblocks, N, nnz;
  int maxn;
  int64_t* h_off;
  int64_t* h_boff;
  int64_t* d_off;
  int64_t* d_boff;
  double* d_data;
  int32_t* d_small;  // ids of blocks with n <= kSmall
  int32_t* d_large;  // ids of the others
  int64_t nsmall, nlarge;
  cudaStream_t stream;
};

inline BDContent* BD(SUNMatrix A) { return (BDContent*)A->content; }

__device__ __forceinline__ long long abs_key(double v)
{
  return __double_as_longlong(v) & 0x7fffffffffffffffLL;
}
__device__ __forceinline__ long long abs_key(float v)
{
  return (long long)(__float_as_int(v) & 0x7fffffff);
}

// ------------------------------------------------------------ matrix kernels
__global__ void k_bd_scaleaddi(double c, double* data, const int64_t* off, const int64_t* boff,
                               int64_t nblocks)
{
  const int lane  = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t W = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t b = w; b < nblocks; b += W)
  {
    const int n = (int)(off[b + 1] - off[b]);
    double* a   = data + boff[b];
    for (int e = lane; e < n * n; e += 32)
    {
      double v = a[e] * c;
      if ((e / n) == (e % n)) v = v + 1.0;
      a[e] = v;
    }
  }
}

__global__ void k_bd_scaleadd(double c, double* a, const double* b, int64_t nnz)
{
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nnz;
       e += (int64_t)gridDim.x * blockDim.x)
    a[e] = c * a[e] + b[e];
}

// y = A x per block: y_i = sum_j A_ij x_j, j ascending (SUNMatMatvec_Dense)
__global__ void k_bd_matvec(const double* data, const int64_t* off, const int64_t* boff,
                            int64_t nblocks, const double* x, double* y)
{
  const int lane  = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t W = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t b = w; b < nblocks; b += W)
  {
    const int n       = (int)(off[b + 1] - off[b]);
    const double* a   = data + boff[b];
    const double* xb  = x + off[b];
    double* yb        = y + off[b];
    for (int i = lane; i < n; i += 32)
    {
      double acc = 0.0;
      for (int j = 0; j < n; j++) acc = acc + a[j * n + i] * xb[j];
      yb[i] = acc;
    }
  }
}

// ------------------------------------------------------------ LU (FP64)
// One thread per small block: SUNDlsMat_denseGETRF on a local copy.
__global__ void k_bd_getrf_small(double* data, const int64_t* off, const int64_t* boff,
                                 const int32_t* ids, int64_t count, int32_t* piv,
                                 unsigned long long* flag)
{
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += (int64_t)gridDim.x * blockDim.x)
  {
    const int64_t b = ids[t];
    const int n     = (int)(off[b + 1] - off[b]);
    double* g       = data + boff[b];
    double a[kSmall * kSmall];
    for (int e = 0; e < n * n; e++) a[e] = g[e];
    int fail = 0;
    for (int k = 0; k < n && !fail; k++)
    {
      double* ck = a + k * n;
      int l      = k;
      for (int i = k + 1; i < n; i++)
        if (fabs(ck[i]) > fabs(ck[l])) l = i;
      piv[off[b] + k] = l;
      if (ck[l] == 0.0)
      {
        fail = k + 1;
        break;
      }
      if (l != k)
        for (int i = 0; i < n; i++)
        {
          double tmp   = a[i * n + l];
          a[i * n + l] = a[i * n + k];
          a[i * n + k] = tmp;
        }
      double mult = 1.0 / ck[k];
      for (int i = k + 1; i < n; i++) ck[i] *= mult;
      for (int j = k + 1; j < n; j++)
      {
        double* cj  = a + j * n;
        double a_kj = cj[k];
        if (a_kj != 0.0)
          for (int i = k + 1; i < n; i++) cj[i] -= a_kj * ck[i];
      }
    }
    for (int e = 0; e < n * n; e++) g[e] = a[e];
    if (fail) atomicMin(flag, (unsigned long long)(off[b] + fail));
  }
}

// One warp per large block, in place in global memory.
__global__ void k_bd_getrf_warp(double* data, const int64_t* off, const int64_t* boff,
                                const int32_t* ids, int64_t count, int32_t* piv,
                                unsigned long long* flag)
{
  const int lane  = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t W = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = w; t < count; t += W)
  {
    const int64_t b = ids[t];
    const int n     = (int)(off[b + 1] - off[b]);
    double* a       = data + boff[b];
    for (int k = 0; k < n; k++)
    {
      double* ck   = a + k * n;
      long long bk = -1;
      int bi       = n;
      for (int i = k + lane; i < n; i += 32)
      {
        long long v = abs_key(ck[i]);
        if (v > bk)
        {
          bk = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
      {
        long long ov = __shfl_xor_sync(0xffffffffu, bk, o);
        int oi       = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bk || (ov == bk && oi < bi))
        {
          bk = ov;
          bi = oi;
        }
      }
      const int l = bi;
      if (lane == 0) piv[off[b] + k] = l;
      if (bk == 0)
      {
        if (lane == 0) atomicMin(flag, (unsigned long long)(off[b] + k + 1));
        break;
      }
      if (l != k)
        for (int j = lane; j < n; j += 32)
        {
          double tmp   = a[j * n + l];
          a[j * n + l] = a[j * n + k];
          a[j * n + k] = tmp;
        }
      __syncwarp();
      const double mult = 1.0 / ck[k];
      for (int i = k + 1 + lane; i < n; i += 32) ck[i] *= mult;
      __syncwarp();
      const int rows = n - k - 1;
      const int tot  = rows * rows;
      for (int e = lane; e < tot; e += 32)
      {
        const int j = k + 1 + e / rows, i = k + 1 + e % rows;
        const double akj = a[j * n + k];
        if (akj != 0.0) a[j * n + i] -= akj * ck[i];
      }
      __syncwarp();
    }
  }
}

// SUNDlsMat_denseGETRS: x (holding b) <- A^{-1} b, one thread per small block.
__global__ void k_bd_getrs_small(const double* data, const int64_t* off, const int64_t* boff,
                                 const int32_t* ids, int64_t count, const int32_t* piv,
                                 double* x)
{
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < count;
       t += (int64_t)gridDim.x * blockDim.x)
  {
    const int64_t b = ids[t];
    const int n     = (int)(off[b + 1] - off[b]);
    const double* a = data + boff[b];
    double* xb      = x + off[b];
    double v[kSmall];
    for (int i = 0; i < n; i++) v[i] = xb[i];
    for (int k = 0; k < n; k++)
    {
      const int pk = piv[off[b] + k];
      if (pk != k)
      {
        double tmp = v[k];
        v[k]       = v[pk];
        v[pk]      = tmp;
      }
    }
    for (int k = 0; k < n - 1; k++)
      for (int i = k + 1; i < n; i++) v[i] -= a[k * n + i] * v[k];
    for (int k = n - 1; k > 0; k--)
    {
      v[k] /= a[k * n + k];
      for (int i = 0; i < k; i++) v[i] -= a[k * n + i] * v[k];
    }
    v[0] /= a[0];
    for (int i = 0; i < n; i++) xb[i] = v[i];
  }
}

__global__ void k_bd_getrs_warp(const double* data, const int64_t* off, const int64_t* boff,
                                const int32_t* ids, int64_t count, const int32_t* piv, double* x)
{
  const int lane  = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t W = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = w; t < count; t += W)
  {
    const int64_t b = ids[t];
    const int n     = (int)(off[b + 1] - off[b]);
    const double* a = data + boff[b];
    double* xb      = x + off[b];
    double b0 = lane < n ? xb[lane] : 0.0, b1 = lane + 32 < n ? xb[lane + 32] : 0.0;
    for (int k = 0; k < n; k++)
    {
      const int pk = piv[off[b] + k];
      if (pk != k)
      {
        double vk = __shfl_sync(0xffffffffu, k < 32 ? b0 : b1, k & 31);
        double vp = __shfl_sync(0xffffffffu, pk < 32 ? b0 : b1, pk & 31);
        if (lane == (k & 31)) { if (k < 32) b0 = vp; else b1 = vp; }
        if (lane == (pk & 31)) { if (pk < 32) b0 = vk; else b1 = vk; }
      }
    }
    for (int k = 0; k < n - 1; k++)
    {
      const double bk = __shfl_sync(0xffffffffu, k < 32 ? b0 : b1, k & 31);
      if (lane > k && lane < n) b0 -= a[k * n + lane] * bk;
      if (lane + 32 > k && lane + 32 < n) b1 -= a[k * n + lane + 32] * bk;
    }
    for (int k = n - 1; k > 0; k--)
    {
      if (lane == (k & 31))
      {
        if (k < 32) b0 /= a[k * n + k];
        else b1 /= a[k * n + k];
      }
      const double bk = __shfl_sync(0xffffffffu, k < 32 ? b0 : b1, k & 31);
      if (lane < k) b0 -= a[k * n + lane] * bk;
      if (lane + 32 < k) b1 -= a[k * n + lane + 32] * bk;
    }
    if (lane == 0) b0 /= a[0];
    if (lane < n) xb[lane] = b0;
    if (lane + 32 < n) xb[lane + 32] = b1;
  }
}

// ------------------------------------------------------------ MIXED path
// FP32 inverse of each block by Gauss-Jordan with partial pivoting (one warp
// per block, any size <= 64), written to inv (boff layout).
__global__ void k_bd_inv32(const double* data, const int64_t* off, const int64_t* boff,
                           int64_t nblocks, float* inv, uint8_t* fb_mark)
{
  const int lane  = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t W = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t b = w; b < nblocks; b += W)
  {
    const int n     = (int)(off[b + 1] - off[b]);
    const double* g = data + boff[b];
    float* a        = inv + boff[b];
    int perm[kMaxBlk];
    for (int e = lane; e < n * n; e += 32) a[e] = (float)g[e];
    __syncwarp();
    bool failed = false;
    for (int k = 0; k < n; k++)
    {
      float* ck    = a + k * n;
      long long bk = -1;
      int bi       = n;
      for (int i = k + lane; i < n; i += 32)
      {
        long long v = abs_key(ck[i]);
        if (v > bk)
        {
          bk = v;
          bi = i;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
      {
        long long ov = __shfl_xor_sync(0xffffffffu, bk, o);
        int oi       = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bk || (ov == bk && oi < bi))
        {
          bk = ov;
          bi = oi;
        }
      }
      if (bk == 0)
      {  // singular in FP32: the block is factored in FP64 instead
        if (lane == 0) fb_mark[b] = 1;
        failed = true;
        break;
      }
      const int l = bi;
      perm[k]     = l;
      if (l != k)
        for (int j = lane; j < n; j += 32)
        {
          float tmp    = a[j * n + l];
          a[j * n + l] = a[j * n + k];
          a[j * n + k] = tmp;
        }
      __syncwarp();
      const float rp = 1.f / ck[k];
      const int i0 = lane, i1 = lane + 32;
      const float f0 = i0 < n ? ck[i0] : 0.f, f1 = i1 < n ? ck[i1] : 0.f;
      __syncwarp();
      for (int j = lane; j < n; j += 32) a[j * n + k] = (j == k ? 1.f : a[j * n + k]) * rp;
      __syncwarp();
      const bool own0 = i0 < n && i0 != k, own1 = i1 < n && i1 != k;
      for (int j = 0; j < n; j++)
      {
        const float rk = a[j * n + k];
        const bool pc  = j == k;
        if (own0) a[j * n + i0] = pc ? -f0 * rp : fmaf(-f0, rk, a[j * n + i0]);
        if (own1) a[j * n + i1] = pc ? -f1 * rp : fmaf(-f1, rk, a[j * n + i1]);
      }
      __syncwarp();
    }
    if (failed) continue;
    for (int k = n - 1; k >= 0; k--)
    {
      const int p = perm[k];
      if (p != k)
        for (int i = lane; i < n; i += 32)
        {
          float tmp    = a[k * n + i];
          a[k * n + i] = a[p * n + i];
          a[p * n + i] = tmp;
        }
      __syncwarp();
    }
  }
}

// Quality probe of each FP32 inverse X: d = v - X (A v) for v = (1, 1, ...)
// and v = (1, -1, 1, ...), A v in FP64.  One refinement sweep contracts the
// error by about |I - X A|; blocks where |d|_inf > 1/4 (ill-conditioned
// beyond FP32, |A| |A^-1| u32 >~ 1) -- or where the FP32 elimination met a
// zero pivot -- are listed for an FP64 LU (the reference's GETRF/GETRS).
__global__ void k_bd_probe32(const double* data, const float* inv, const int64_t* off,
                             const int64_t* boff, int64_t nblocks, uint8_t* fb_mark,
                             int32_t* fb_ids, unsigned* fb_count)
{
  const int lane  = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t W = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t b = w; b < nblocks; b += W)
  {
    bool bad = fb_mark[b] != 0;
    if (!bad)
    {
      const int n     = (int)(off[b + 1] - off[b]);
      const double* A = data + boff[b];
      const float* V  = inv + boff[b];
      double worst    = 0.0;
      for (int alt = 0; alt < 2; alt++)
      {
        // t = A v (rows lane, lane + 32)
        double t0 = 0.0, t1 = 0.0;
        for (int j = 0; j < n; j++)
        {
          const double vj = (alt && (j & 1)) ? -1.0 : 1.0;
          if (lane < n) t0 = fma(A[j * n + lane], vj, t0);
          if (lane + 32 < n) t1 = fma(A[j * n + lane + 32], vj, t1);
        }
        const float c0 = (float)t0, c1 = (float)t1;
        float u0 = 0.f, u1 = 0.f;
        for (int j = 0; j < n; j++)
        {
          const float tj = __shfl_sync(0xffffffffu, j < 32 ? c0 : c1, j & 31);
          if (lane < n) u0 = fmaf(V[j * n + lane], tj, u0);
          if (lane + 32 < n) u1 = fmaf(V[j * n + lane + 32], tj, u1);
        }
        const double v0 = (alt && (lane & 1)) ? -1.0 : 1.0;
        const double v1 = (alt && ((lane + 32) & 1)) ? -1.0 : 1.0;
        double d = 0.0;
        if (lane < n) d = fabs(v0 - (double)u0);
        if (lane + 32 < n) d = fmax(d, fabs(v1 - (double)u1));
        if (!(d <= 0.25)) d = 1.0e300;  // NaN or too large
        worst = fmax(worst, d);
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) worst = fmax(worst, __shfl_xor_sync(0xffffffffu, worst, o));
      bad = worst > 0.25;
      if (bad && lane == 0) fb_mark[b] = 1;
    }
    if (bad && lane == 0) fb_ids[atomicAdd(fb_count, 1u)] = (int32_t)b;
  }
}

// Copy the listed blocks of A into lu (same layout) for their FP64 LU.
__global__ void k_bd_copy_blocks(const double* data, const int64_t* off, const int64_t* boff,
                                 const int32_t* ids, int64_t count, double* lu)
{
  const int lane  = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t W = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t t = w; t < count; t += W)
  {
    const int64_t b = ids[t];
    const int n     = (int)(off[b + 1] - off[b]);
    for (int e = lane; e < n * n; e += 32) lu[boff[b] + e] = data[boff[b] + e];
  }
}

// x = inv b (FP32), r = b - A x (FP64), x += inv r (FP32 apply); x holds b.
// Blocks marked for the FP64 fallback are left to k_bd_getrs_warp.
__global__ void k_bd_solve_mixed(const double* data, const float* inv, const int64_t* off,
                                 const int64_t* boff, int64_t nblocks, const uint8_t* fb_mark,
                                 double* x)
{
  const int lane  = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t W = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t b = w; b < nblocks; b += W)
  {
    if (fb_mark[b]) continue;
    const int n     = (int)(off[b + 1] - off[b]);
    const double* A = data + boff[b];
    const float* V  = inv + boff[b];
    double* xb      = x + off[b];
    const double b0 = lane < n ? xb[lane] : 0.0, b1 = lane + 32 < n ? xb[lane + 32] : 0.0;
    float s0 = 0.f, s1 = 0.f;
    const float c0 = (float)b0, c1 = (float)b1;
    for (int j = 0; j < n; j++)
    {
      const float bj = __shfl_sync(0xffffffffu, j < 32 ? c0 : c1, j & 31);
      if (lane < n) s0 = fmaf(V[j * n + lane], bj, s0);
      if (lane + 32 < n) s1 = fmaf(V[j * n + lane + 32], bj, s1);
    }
    double x0 = s0, x1 = s1, r0 = 0.0, r1 = 0.0;
    for (int j = 0; j < n; j++)
    {
      const double xj = __shfl_sync(0xffffffffu, j < 32 ? x0 : x1, j & 31);
      if (lane < n) r0 = fma(A[j * n + lane], xj, r0);
      if (lane + 32 < n) r1 = fma(A[j * n + lane + 32], xj, r1);
    }
    const float d0 = (float)(b0 - r0), d1 = (float)(b1 - r1);
    float e0 = 0.f, e1 = 0.f;
    for (int j = 0; j < n; j++)
    {
      const float dj = __shfl_sync(0xffffffffu, j < 32 ? d0 : d1, j & 31);
      if (lane < n) e0 = fmaf(V[j * n + lane], dj, e0);
      if (lane + 32 < n) e1 = fmaf(V[j * n + lane + 32], dj, e1);
    }
    if (lane < n) xb[lane] = x0 + (double)e0;
    if (lane + 32 < n) xb[lane + 32] = x1 + (double)e1;
  }
}

int warp_grid(int64_t units)
{
  int64_t need = (units * 32 + kBlock - 1) / kBlock;
  int64_t cap  = (int64_t)num_sms() * 16;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}
int thread_grid(int64_t units)
{
  int64_t need = (units + kBlock - 1) / kBlock;
  int64_t cap  = (int64_t)num_sms() * 16;
  if (need < 1) need = 1;
  return (int)(need < cap ? need : cap);
}

void fill_mat_ops(SUNMatrix_Ops ops);

template <class T>
T* dalloc(size_t count)
{
  T* p = nullptr;
  if (!check_cuda(cudaMalloc(&p, sizeof(T) * (count ? count : 1)), "cudaMalloc(blockdiag)"))
    return nullptr;
  return p;
}

SUNMatrix new_matrix(int64_t nblocks, const int64_t* off, cudaStream_t stream, SUNContext ctx)
{
  SUNMatrix A = (SUNMatrix)calloc(1, sizeof(*A));
  A->ops      = (SUNMatrix_Ops)calloc(1, sizeof(*A->ops));
  fill_mat_ops(A->ops);
  A->sunctx      = ctx;
  BDContent* c   = (BDContent*)calloc(1, sizeof(BDContent));
  A->content     = c;
  c->nblocks     = nblocks;
  c->stream      = stream;
  c->h_off       = (int64_t*)malloc(sizeof(int64_t) * (nblocks + 1));
  c->h_boff      = (int64_t*)malloc(sizeof(int64_t) * (nblocks + 1));
  std::vector<int32_t> small, large;
  c->h_off[0] = c->h_boff[0] = 0;
  c->maxn = 0;
  for (int64_t b = 0; b < nblocks; b++)
  {
    const int64_t n = off[b + 1] - off[b];
    c->h_off[b + 1]  = off[b + 1];
    c->h_boff[b + 1] = c->h_boff[b] + n * n;
    c->maxn          = std::max<int>(c->maxn, (int)n);
    (n <= kSmall ? small : large).push_back((int32_t)b);
  }
  c->N       = off[nblocks];
  c->nnz     = c->h_boff[nblocks];
  c->nsmall  = (int64_t)small.size();
  c->nlarge  = (int64_t)large.size();
  c->d_off   = dalloc<int64_t>(nblocks + 1);
  c->d_boff  = dalloc<int64_t>(nblocks + 1);
  c->d_data  = dalloc<double>(c->nnz);
  c->d_small = dalloc<int32_t>(small.size());
  c->d_large = dalloc<int32_t>(large.size());
  cudaMemcpy(c->d_off, c->h_off, sizeof(int64_t) * (nblocks + 1), cudaMemcpyHostToDevice);
  cudaMemcpy(c->d_boff, c->h_boff, sizeof(int64_t) * (nblocks + 1), cudaMemcpyHostToDevice);
  if (!small.empty())
    cudaMemcpy(c->d_small, small.data(), sizeof(int32_t) * small.size(), cudaMemcpyHostToDevice);
  if (!large.empty())
    cudaMemcpy(c->d_large, large.data(), sizeof(int32_t) * large.size(), cudaMemcpyHostToDevice);
  cudaMemset(c->d_data, 0, sizeof(double) * (c->nnz ? c->nnz : 1));
  return A;
}

// ------------------------------------------------------------ solver content
struct LSContent
{
  int precision;
  int32_t* d_piv;                 // [N]
  float* d_inv;                   // [nnz] (MIXED)
  uint8_t* d_fb_mark;             // [nblocks] (MIXED): block factored in FP64
  int32_t* d_fb_ids;              // [nblocks] (MIXED): those blocks
  unsigned* d_fb_count;           // (MIXED)
  unsigned* h_fb_count;           // pinned
  double* d_lu64;                 // [nnz] (MIXED, allocated on first use): their FP64 LU
  int64_t fb_count, nblocks;
  unsigned long long* d_flag;     // first zero pivot: global column + 1
  unsigned long long* h_flag;     // pinned
  sunindextype last_flag;
  cudaStream_t stream;
  int64_t N, nnz;
};
inline LSContent* LS(SUNLinearSolver S) { return (LSContent*)S->content; }

}  // namespace

extern "C" {

// ------------------------------------------------------------ matrix API
SUNMatrix SUNMatrix_BlockDiag_GB300(sunindextype nblocks, const sunindextype* off, SUNContext ctx)
{
  if (nblocks < 1 || !off || off[0] != 0) return nullptr;
  for (sunindextype b = 0; b < nblocks; b++)
  {
    const sunindextype n = off[b + 1] - off[b];
    if (n < 1 || n > kMaxBlk)
    {
      set_error(SUN_ERR_ARG_OUTOFRANGE, "SUNMatrix_BlockDiag_GB300: block size outside 1..64");
      return nullptr;
    }
  }
  return new_matrix(nblocks, off, (cudaStream_t)0, ctx);
}

sunindextype SUNMatrix_BlockDiag_GB300_NumBlocks(SUNMatrix A) { return BD(A)->nblocks; }
sunindextype SUNMatrix_BlockDiag_GB300_Rows(SUNMatrix A) { return BD(A)->N; }
sunindextype SUNMatrix_BlockDiag_GB300_NNZ(SUNMatrix A) { return BD(A)->nnz; }
sunrealtype* SUNMatrix_BlockDiag_GB300_Data(SUNMatrix A) { return BD(A)->d_data; }
sunrealtype* SUNMatrix_BlockDiag_GB300_BlockData(SUNMatrix A, sunindextype b)
{
  return BD(A)->d_data + BD(A)->h_boff[b];
}

SUNErrCode SUNMatrix_BlockDiag_GB300_CopyToDevice(SUNMatrix A, const sunrealtype* h)
{
  BDContent* c = BD(A);
  return check_cuda(cudaMemcpy(c->d_data, h, sizeof(double) * c->nnz, cudaMemcpyHostToDevice),
                    "BlockDiag CopyToDevice")
           ? SUN_SUCCESS
           : SUN_ERR_EXT_FAIL;
}

SUNErrCode SUNMatrix_BlockDiag_GB300_CopyFromDevice(SUNMatrix A, sunrealtype* h)
{
  BDContent* c = BD(A);
  cudaStreamSynchronize(c->stream);
  return check_cuda(cudaMemcpy(h, c->d_data, sizeof(double) * c->nnz, cudaMemcpyDeviceToHost),
                    "BlockDiag CopyFromDevice")
           ? SUN_SUCCESS
           : SUN_ERR_EXT_FAIL;
}

SUNMatrix_ID SUNMatGetID_BlockDiag_GB300(SUNMatrix) { return SUNMATRIX_CUSTOM; }

SUNMatrix SUNMatClone_BlockDiag_GB300(SUNMatrix A)
{
  BDContent* c = BD(A);
  return new_matrix(c->nblocks, c->h_off, c->stream, A->sunctx);
}

void SUNMatDestroy_BlockDiag_GB300(SUNMatrix A)
{
  if (!A) return;
  BDContent* c = BD(A);
  if (c)
  {
    cudaStreamSynchronize(c->stream);
    cudaFree(c->d_off);
    cudaFree(c->d_boff);
    cudaFree(c->d_data);
    cudaFree(c->d_small);
    cudaFree(c->d_large);
    free(c->h_off);
    free(c->h_boff);
    free(c);
  }
  free(A->ops);
  free(A);
}

SUNErrCode SUNMatZero_BlockDiag_GB300(SUNMatrix A)
{
  BDContent* c = BD(A);
  return check_cuda(cudaMemsetAsync(c->d_data, 0, sizeof(double) * c->nnz, c->stream),
                    "BlockDiag Zero")
           ? SUN_SUCCESS
           : SUN_ERR_EXT_FAIL;
}

SUNErrCode SUNMatCopy_BlockDiag_GB300(SUNMatrix A, SUNMatrix B)
{
  BDContent *a = BD(A), *b = BD(B);
  if (a->nnz != b->nnz || a->nblocks != b->nblocks) return SUN_ERR_ARG_INCOMPATIBLE;
  return check_cuda(cudaMemcpyAsync(b->d_data, a->d_data, sizeof(double) * a->nnz,
                                    cudaMemcpyDeviceToDevice, a->stream),
                    "BlockDiag Copy")
           ? SUN_SUCCESS
           : SUN_ERR_EXT_FAIL;
}

SUNErrCode SUNMatScaleAdd_BlockDiag_GB300(sunrealtype cc, SUNMatrix A, SUNMatrix B)
{
  BDContent *a = BD(A), *b = BD(B);
  if (a->nnz != b->nnz) return SUN_ERR_ARG_INCOMPATIBLE;
  k_bd_scaleadd<<<thread_grid(a->nnz), kBlock, 0, a->stream>>>(cc, a->d_data, b->d_data, a->nnz);
  count_launch();
  return check_cuda(cudaGetLastError(), "k_bd_scaleadd") ? SUN_SUCCESS : SUN_ERR_EXT_FAIL;
}

SUNErrCode SUNMatScaleAddI_BlockDiag_GB300(sunrealtype cc, SUNMatrix A)
{
  BDContent* a = BD(A);
  k_bd_scaleaddi<<<warp_grid(a->nblocks), kBlock, 0, a->stream>>>(cc, a->d_data, a->d_off,
                                                                   a->d_boff, a->nblocks);
  count_launch();
  return check_cuda(cudaGetLastError(), "k_bd_scaleaddi") ? SUN_SUCCESS : SUN_ERR_EXT_FAIL;
}

SUNErrCode SUNMatMatvec_BlockDiag_GB300(SUNMatrix A, N_Vector x, N_Vector y)
{
  BDContent* a = BD(A);
  if (N_VGetLength_GB300(x) != a->N || N_VGetLength_GB300(y) != a->N)
    return SUN_ERR_ARG_INCOMPATIBLE;
  k_bd_matvec<<<warp_grid(a->nblocks), kBlock, 0, (cudaStream_t)N_VGetStream_GB300(y)>>>(
    a->d_data, a->d_off, a->d_boff, a->nblocks, N_VGetDeviceArrayPointer_GB300(x),
    N_VGetDeviceArrayPointer_GB300(y));
  count_launch();
  return check_cuda(cudaGetLastError(), "k_bd_matvec") ? SUN_SUCCESS : SUN_ERR_EXT_FAIL;
}

static SUNErrCode SUNMatMatvecSetup_BlockDiag_GB300(SUNMatrix) { return SUN_SUCCESS; }
static SUNErrCode SUNMatSpace_BlockDiag_GB300(SUNMatrix A, long int* lrw, long int* liw)
{
  *lrw = (long int)BD(A)->nnz;
  *liw = (long int)(2 * (BD(A)->nblocks + 1));
  return SUN_SUCCESS;
}

// ------------------------------------------------------------ solver API
SUNLinearSolver SUNLinSol_BlockLU_GB300(N_Vector y, SUNMatrix A, int precision, SUNContext ctx)
{
  if (!y || !A || A->ops->getid != SUNMatGetID_BlockDiag_GB300) return nullptr;
  if (precision != SUNBLOCKLU_FP64 && precision != SUNBLOCKLU_MIXED) return nullptr;
  BDContent* a = BD(A);
  if (N_VGetLength_GB300(y) != a->N) return nullptr;
  SUNLinearSolver S = (SUNLinearSolver)calloc(1, sizeof(*S));
  S->ops            = (SUNLinearSolver_Ops)calloc(1, sizeof(*S->ops));
  S->sunctx         = ctx;
  S->ops->gettype   = SUNLinSolGetType_BlockLU_GB300;
  S->ops->getid     = SUNLinSolGetID_BlockLU_GB300;
  S->ops->initialize = SUNLinSolInitialize_BlockLU_GB300;
  S->ops->setup     = SUNLinSolSetup_BlockLU_GB300;
  S->ops->solve     = SUNLinSolSolve_BlockLU_GB300;
  S->ops->lastflag  = SUNLinSolLastFlag_BlockLU_GB300;
  S->ops->free      = SUNLinSolFree_BlockLU_GB300;
  LSContent* c      = (LSContent*)calloc(1, sizeof(LSContent));
  S->content        = c;
  c->precision      = precision;
  c->stream         = (cudaStream_t)N_VGetStream_GB300(y);
  c->N              = a->N;
  c->nnz            = a->nnz;
  c->d_piv          = dalloc<int32_t>(a->N);
  c->d_inv          = precision == SUNBLOCKLU_MIXED ? dalloc<float>(a->nnz) : nullptr;
  c->nblocks        = a->nblocks;
  if (precision == SUNBLOCKLU_MIXED)
  {
    c->d_fb_mark  = dalloc<uint8_t>(a->nblocks);
    c->d_fb_ids   = dalloc<int32_t>(a->nblocks);
    c->d_fb_count = dalloc<unsigned>(1);
    cudaHostAlloc(&c->h_fb_count, sizeof(unsigned), cudaHostAllocDefault);
  }
  c->d_flag         = dalloc<unsigned long long>(1);
  cudaHostAlloc(&c->h_flag, sizeof(unsigned long long), cudaHostAllocDefault);
  return S;
}

SUNLinearSolver_Type SUNLinSolGetType_BlockLU_GB300(SUNLinearSolver) { return SUNLINEARSOLVER_DIRECT; }
SUNLinearSolver_ID SUNLinSolGetID_BlockLU_GB300(SUNLinearSolver) { return SUNLINEARSOLVER_CUSTOM; }
SUNErrCode SUNLinSolInitialize_BlockLU_GB300(SUNLinearSolver S)
{
  LS(S)->last_flag = 0;
  return SUN_SUCCESS;
}

int SUNLinSolSetup_BlockLU_GB300(SUNLinearSolver S, SUNMatrix A)
{
  LSContent* c = LS(S);
  BDContent* a = BD(A);
  cudaStream_t s = c->stream;
  const unsigned long long none = ~0ull;
  cudaMemcpyAsync(c->d_flag, &none, sizeof none, cudaMemcpyHostToDevice, s);
  if (c->precision == SUNBLOCKLU_MIXED)
  {
    cudaMemsetAsync(c->d_fb_mark, 0, a->nblocks, s);
    cudaMemsetAsync(c->d_fb_count, 0, sizeof(unsigned), s);
    k_bd_inv32<<<warp_grid(a->nblocks), kBlock, 0, s>>>(a->d_data, a->d_off, a->d_boff,
                                                         a->nblocks, c->d_inv, c->d_fb_mark);
    k_bd_probe32<<<warp_grid(a->nblocks), kBlock, 0, s>>>(a->d_data, c->d_inv, a->d_off,
                                                           a->d_boff, a->nblocks, c->d_fb_mark,
                                                           c->d_fb_ids, c->d_fb_count);
    count_launch();
    count_launch();
    cudaMemcpyAsync(c->h_fb_count, c->d_fb_count, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (!check_cuda(cudaStreamSynchronize(s), "SUNLinSolSetup_BlockLU_GB300"))
    {
      c->last_flag = SUN_ERR_EXT_FAIL;
      return SUN_ERR_EXT_FAIL;
    }
    c->fb_count = *c->h_fb_count;
    if (c->fb_count > 0)
    {  // FP64 LU of the blocks the FP32 inverse cannot serve
      if (!c->d_lu64) c->d_lu64 = dalloc<double>(a->nnz);
      if (!c->d_lu64)
      {
        c->last_flag = SUN_ERR_MEM_FAIL;
        return SUN_ERR_MEM_FAIL;
      }
      k_bd_copy_blocks<<<warp_grid(c->fb_count), kBlock, 0, s>>>(
        a->d_data, a->d_off, a->d_boff, c->d_fb_ids, c->fb_count, c->d_lu64);
      k_bd_getrf_warp<<<warp_grid(c->fb_count), kBlock, 0, s>>>(
        c->d_lu64, a->d_off, a->d_boff, c->d_fb_ids, c->fb_count, c->d_piv, c->d_flag);
      count_launch();
      count_launch();
    }
  }
  else
  {
    if (a->nsmall)
    {
      k_bd_getrf_small<<<thread_grid(a->nsmall), kBlock, 0, s>>>(
        a->d_data, a->d_off, a->d_boff, a->d_small, a->nsmall, c->d_piv, c->d_flag);
      count_launch();
    }
    if (a->nlarge)
    {
      k_bd_getrf_warp<<<warp_grid(a->nlarge), kBlock, 0, s>>>(
        a->d_data, a->d_off, a->d_boff, a->d_large, a->nlarge, c->d_piv, c->d_flag);
      count_launch();
    }
  }
  cudaMemcpyAsync(c->h_flag, c->d_flag, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
  if (!check_cuda(cudaStreamSynchronize(s), "SUNLinSolSetup_BlockLU_GB300"))
  {
    c->last_flag = SUN_ERR_EXT_FAIL;
    return SUN_ERR_EXT_FAIL;
  }
  if (*c->h_flag != none)
  {
    c->last_flag = (sunindextype)*c->h_flag;
    return SUNLS_LUFACT_FAIL;
  }
  c->last_flag = 0;
  return SUN_SUCCESS;
}

int SUNLinSolSolve_BlockLU_GB300(SUNLinearSolver S, SUNMatrix A, N_Vector x, N_Vector b,
                                 sunrealtype)
{
  LSContent* c = LS(S);
  BDContent* a = BD(A);
  cudaStream_t s = c->stream;
  double* xd     = N_VGetDeviceArrayPointer_GB300(x);
  if (x != b)
    cudaMemcpyAsync(xd, N_VGetDeviceArrayPointer_GB300(b), sizeof(double) * a->N,
                    cudaMemcpyDeviceToDevice, s);
  if (c->precision == SUNBLOCKLU_MIXED)
  {
    k_bd_solve_mixed<<<warp_grid(a->nblocks), kBlock, 0, s>>>(
      a->d_data, c->d_inv, a->d_off, a->d_boff, a->nblocks, c->d_fb_mark, xd);
    count_launch();
    if (c->fb_count > 0)
    {
      k_bd_getrs_warp<<<warp_grid(c->fb_count), kBlock, 0, s>>>(
        c->d_lu64, a->d_off, a->d_boff, c->d_fb_ids, c->fb_count, c->d_piv, xd);
      count_launch();
    }
  }
  else
  {
    if (a->nsmall)
    {
      k_bd_getrs_small<<<thread_grid(a->nsmall), kBlock, 0, s>>>(
        a->d_data, a->d_off, a->d_boff, a->d_small, a->nsmall, c->d_piv, xd);
      count_launch();
    }
    if (a->nlarge)
    {
      k_bd_getrs_warp<<<warp_grid(a->nlarge), kBlock, 0, s>>>(
        a->d_data, a->d_off, a->d_boff, a->d_large, a->nlarge, c->d_piv, xd);
      count_launch();
    }
  }
  c->last_flag = check_cuda(cudaGetLastError(), "SUNLinSolSolve_BlockLU_GB300") ? 0
                                                                                : SUN_ERR_EXT_FAIL;
  return (int)c->last_flag;
}

sunindextype SUNLinSolLastFlag_BlockLU_GB300(SUNLinearSolver S) { return LS(S)->last_flag; }

SUNErrCode SUNLinSolFree_BlockLU_GB300(SUNLinearSolver S)
{
  if (!S) return SUN_SUCCESS;
  LSContent* c = LS(S);
  if (c)
  {
    cudaStreamSynchronize(c->stream);
    cudaFree(c->d_piv);
    cudaFree(c->d_inv);
    cudaFree(c->d_flag);
    cudaFreeHost(c->h_flag);
    cudaFree(c->d_fb_mark);
    cudaFree(c->d_fb_ids);
    cudaFree(c->d_fb_count);
    cudaFreeHost(c->h_fb_count);
    cudaFree(c->d_lu64);
    free(c);
  }
  free(S->ops);
  free(S);
  return SUN_SUCCESS;
}

}  // extern "C"

namespace {
void fill_mat_ops(SUNMatrix_Ops ops)
{
  ops->getid       = SUNMatGetID_BlockDiag_GB300;
  ops->clone       = SUNMatClone_BlockDiag_GB300;
  ops->destroy     = SUNMatDestroy_BlockDiag_GB300;
  ops->zero        = SUNMatZero_BlockDiag_GB300;
  ops->copy        = SUNMatCopy_BlockDiag_GB300;
  ops->scaleadd    = SUNMatScaleAdd_BlockDiag_GB300;
  ops->scaleaddi   = SUNMatScaleAddI_BlockDiag_GB300;
  ops->matvecsetup = SUNMatMatvecSetup_BlockDiag_GB300;
  ops->matvec      = SUNMatMatvec_BlockDiag_GB300;
  ops->space       = SUNMatSpace_BlockDiag_GB300;
}
}  // namespace

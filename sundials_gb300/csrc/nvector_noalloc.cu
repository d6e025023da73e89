// nvector_noalloc.cu -- N_VDotProdMultiNoAlloc_GB300: the fused dot-product
// reduction (d_k = x . Y_k) for callers that must not allocate device memory.
//
// Who needs it: codes that hand the GPU's memory to their own pool at start-up
// and forbid cudaMalloc afterwards (a cudaMalloc/cudaFree synchronises the
// device and can fail once the pool owns the memory), and long-running
// services whose steady state may not call the CUDA allocator.  The regular
// N_Vector reductions allocate a small workspace per stream the first time a
// vector is created; this entry point needs none: the caller passes the
// inputs and the output, and the reduction's scratch (per-block partial sums
// and the last-block counter) is one file-scope static __device__ array that
// every GPU holds from the moment it loads the library until the process
// exits.
//
// Behaviour:
//  * at most SUNGB300_NOALLOC_MAXVEC (8) dot products per call, because the
//    static scratch holds 8 x 1024 partial sums; larger nvec is rejected with
//    SUN_ERR_ARG_OUTOFRANGE and a message, before anything is launched;
//  * the first call on each device (with that device current) looks up the
//    array's device address with cudaGetSymbolAddress; make that first call
//    before any stream capture;
//  * every call shares the array and leaves its contents behind; the counter
//    that must start at zero is cleared by each call (an asynchronous memset
//    on the caller's stream), so calls that overlap on the GPU -- on
//    different streams, or from different host threads -- race;
//  * no cudaMalloc, cudaFree or other allocating routine is called.
// The arithmetic (fused multiply-adds, per-thread order, block tree, block
// order of the partials, launch shape) is the same as N_VDotProdMulti_GB300's,
// so both give the same bits on the same data.
#include <cuda_runtime.h>
#include <stdio.h>

#include <mutex>

#include "../../include/nvector_gb300.h"
#include "gb300_common.cuh"

using namespace gb300;

namespace {

// kMaxRedBlocks partial sums per dot product, then room for the counter.
constexpr int kNoAllocDoubles = SUNGB300_NOALLOC_MAXVEC * kMaxRedBlocks + 32;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {nullptr};

struct PtrArgs
{
  const double* y[SUNGB300_NOALLOC_MAXVEC];
};

template <int NV>
__global__ void __launch_bounds__(kBlock)
  k_dotmulti_static(int64_t n, const double* x, PtrArgs args, int vec, double* partials,
                    unsigned int* counter, double* out)
{
  __shared__ double scratch[kWarps * NV];
  const int64_t tid    = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  double acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) acc[k] = 0.0;
  int64_t head = 0;
  if (vec)
  {
    const int64_t npair = n >> 1;
    for (int64_t p = tid; p < npair; p += stride)
    {
      double2 xv = ((const double2*)x)[p];
#pragma unroll
      for (int k = 0; k < NV; ++k)
      {
        double2 yv = ((const double2*)args.y[k])[p];
        acc[k]     = fma(xv.x, yv.x, acc[k]);
        acc[k]     = fma(xv.y, yv.y, acc[k]);
      }
    }
    head = npair << 1;
  }
  for (int64_t i = head + tid; i < n; i += stride)
  {
    double xv = x[i];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = fma(xv, args.y[k][i], acc[k]);
  }
  block_reduce<SumOp, NV>(acc, scratch);
  if (gridDim.x == 1)
  {
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) out[k] = acc[k];
    return;
  }
  if (grid_finish<SumOp, NV>(acc, partials, counter, gridDim.x, blockIdx.x, scratch))
#pragma unroll
    for (int k = 0; k < NV; ++k) out[k] = acc[k];
}

template <int NV>
void launch(int64_t n, const double* x, const PtrArgs& a, int vec, int grid, double* base,
            double* out, cudaStream_t s)
{
  double* partials      = base;
  unsigned int* counter = (unsigned int*)(base + SUNGB300_NOALLOC_MAXVEC * kMaxRedBlocks);
  k_dotmulti_static<NV><<<grid, kBlock, 0, s>>>(n, x, a, vec, partials, counter, out);
}

// Device address of the static scratch on the current device (looked up once).
double* scratch_address()
{
  int dev = 0;
  if (!check_cuda(cudaGetDevice(&dev), "cudaGetDevice")) return nullptr;
  if (dev < 0 || dev >= kMaxDevices)
  {
    set_error(SUN_ERR_ARG_OUTOFRANGE, "N_VDotProdMultiNoAlloc_GB300: device index too large");
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev])
  {
    double* p = nullptr;
    if (!check_cuda(cudaGetSymbolAddress((void**)&p, g_noalloc_scratch), "cudaGetSymbolAddress"))
      return nullptr;
    g_scratch_addr[dev] = p;
  }
  return g_scratch_addr[dev];
}

inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace

extern "C" SUNErrCode N_VDotProdMultiNoAlloc_GB300(int nvec, const sunrealtype* x,
                                                   const sunrealtype* const* Y, sunindextype n,
                                                   sunrealtype* d_out, void* cuda_stream)
{
  if (nvec < 1 || nvec > SUNGB300_NOALLOC_MAXVEC)
  {
    char msg[160];
    snprintf(msg, sizeof msg,
             "N_VDotProdMultiNoAlloc_GB300: nvec = %d, must be 1..%d (static scratch size)", nvec,
             SUNGB300_NOALLOC_MAXVEC);
    set_error(SUN_ERR_ARG_OUTOFRANGE, msg);
    fprintf(stderr, "[sundials_gb300] %s\n", msg);
    return SUN_ERR_ARG_OUTOFRANGE;
  }
  if (!x || !Y || !d_out || n < 0)
  {
    set_error(SUN_ERR_ARG_CORRUPT, "N_VDotProdMultiNoAlloc_GB300: NULL pointer or n < 0");
    return SUN_ERR_ARG_CORRUPT;
  }
  cudaStream_t s = (cudaStream_t)cuda_stream;
  if (n == 0)
    return check_cuda(cudaMemsetAsync(d_out, 0, sizeof(double) * nvec, s), "cudaMemsetAsync")
             ? SUN_SUCCESS
             : SUN_ERR_EXT_FAIL;
  double* base = scratch_address();
  if (!base) return SUN_ERR_EXT_FAIL;
  PtrArgs a;
  int vec = aligned16(x);
  for (int k = 0; k < nvec; ++k)
  {
    if (!Y[k]) return SUN_ERR_ARG_CORRUPT;
    a.y[k] = Y[k];
    vec    = vec && aligned16(Y[k]);
  }
  // the last-block counter must start at zero
  if (!check_cuda(cudaMemsetAsync(base + SUNGB300_NOALLOC_MAXVEC * kMaxRedBlocks, 0,
                                  sizeof(unsigned int), s),
                  "cudaMemsetAsync(counter)"))
    return SUN_ERR_EXT_FAIL;
  const int64_t items = vec ? (n + 1) / 2 : n;
  const int grid      = reduce_grid(items);
  switch (nvec)
  {
  case 1: launch<1>(n, x, a, vec, grid, base, d_out, s); break;
  case 2: launch<2>(n, x, a, vec, grid, base, d_out, s); break;
  case 3: launch<3>(n, x, a, vec, grid, base, d_out, s); break;
  case 4: launch<4>(n, x, a, vec, grid, base, d_out, s); break;
  case 5: launch<5>(n, x, a, vec, grid, base, d_out, s); break;
  case 6: launch<6>(n, x, a, vec, grid, base, d_out, s); break;
  case 7: launch<7>(n, x, a, vec, grid, base, d_out, s); break;
  default: launch<8>(n, x, a, vec, grid, base, d_out, s); break;
  }
  count_launch();
  return check_cuda(cudaGetLastError(), "k_dotmulti_static launch") ? SUN_SUCCESS
                                                                   : SUN_ERR_EXT_FAIL;
}

// nvector_gb300.cu -- NVECTOR_GB300: every N_Vector operation as an sm_103a
// kernel, plus the ops table that plugs the vector into CVODE/ARKODE.
//
// Operation semantics follow NVECTOR_SERIAL (src/nvector/serial/
// nvector_serial.c:387-1600): the same special cases of LinearSum (a==b ->
// a*(x+y), a==-b -> a*(x-y)) and the same element order of fused sums.  Two
// arithmetic modes: FMA (default; what nvcc makes of NVECTOR_CUDA's kernels)
// and EXACT (every product and sum rounded separately, giving the serial
// vector's bits).  On GB300 the FP64 pipe (~1.2 TFLOP/s) rather than HBM
// bounds most of these operations, so the mode also sets their speed: FMA
// issues 5 instead of 9 FP64 instructions per element of LinearCombination(5).
//
// Kernel design (GB300-first, not a port of NVECTOR_CUDA's kernels):
//  * element pairs move as 16-byte double2 loads/stores when every operand
//    is 16-byte aligned (cudaMalloc gives 256), scalar tail otherwise;
//  * grid-stride loops over <= 8 resident 256-thread blocks per SM;
//  * reductions finish in the same launch (last-block ticket) with a fixed
//    combine order, and deliver the scalar straight into pinned, mapped host
//    memory, so the host pays one stream synchronisation and no copy;
//  * fused and vector-array operations receive coefficients and pointers as
//    kernel parameters (NVECTOR_CUDA stages them through a pinned buffer, an
//    H2D copy and a synchronisation per call, nvector_cuda.cu:2413-2604);
//  * DotProdMulti reads x once for all (up to 8) dot products, on the whole
//    grid (NVECTOR_CUDA launches one block per dot product,
//    nvector_cuda.cu:1527).
#include <cuda_runtime.h>
#include <math.h>

#include <atomic>
#include <chrono>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <mutex>
#include <unordered_map>

#include "../../include/nvector_gb300.h"
#include "gb300_common.cuh"

using namespace gb300;

// ===================================================================== errors

extern "C" {
// Resolved only when the process also links the reference's libsundials_core:
// then errors reach SUNContext_GetLastError like the reference's own modules.
void SUNHandleErrWithMsg(int line, const char* func, const char* file,
                         const char* msg, SUNErrCode code, SUNContext sunctx)
  __attribute__((weak));
}

namespace gb300 {

static thread_local int t_last_err = 0;
static thread_local char t_last_msg[256] = {0};
static std::atomic<long long> g_launches{0};

void set_error(int code, const char* msg)
{
  t_last_err = code;
  snprintf(t_last_msg, sizeof t_last_msg, "%s", msg ? msg : "");
}

bool check_cuda(cudaError_t err, const char* what)
{
  if (err == cudaSuccess) return true;
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(err));
  set_error(SUN_ERR_EXT_FAIL, buf);
  fprintf(stderr, "[sundials_gb300] CUDA error in %s\n", buf);
  return false;
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int num_sms()
{
  static int sms = 0;
  if (sms == 0)
  {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      v = 152;
    sms = v;
  }
  return sms;
}

}  // namespace gb300

extern "C" int SUNGB300_GetLastError(void)
{
  int e      = t_last_err;
  t_last_err = 0;
  return e;
}
extern "C" const char* SUNGB300_GetLastErrorMessage(void) { return t_last_msg; }
extern "C" long long SUNGB300_KernelLaunchCount(void) { return g_launches.load(); }

// ================================================================== content

namespace {

// Reduction workspace shared by a vector and all of its clones (same stream).
struct Workspace
{
  int refs;
  cudaStream_t stream;
  bool own_stream;
  double* d_partials;      // kMaxRedBlocks * kRowsMax doubles
  unsigned int* d_counter; // last-block ticket
  double* h_result;        // pinned, mapped: reduction results land here
  double* d_result;        // device alias of h_result
};
constexpr int kRowsMax   = 32;  // vector-array reductions per launch
constexpr int kResultMax = 64;

struct Content
{
  sunindextype length;
  bool own_host, own_dev;
  double* host;
  double* dev;
  Workspace* ws;
  bool fma;
};

inline Content* C(N_Vector v) { return (Content*)v->content; }
inline double* D(N_Vector v) { return C(v)->dev; }
inline int64_t LEN(N_Vector v) { return (int64_t)C(v)->length; }
inline cudaStream_t S(N_Vector v) { return C(v)->ws->stream; }
inline bool FMA(N_Vector v) { return C(v)->fma; }

// A failed CUDA call: record it, print it, and pass it to the SUNContext.
bool ok_or_report(N_Vector v, cudaError_t err, const char* what)
{
  if (check_cuda(err, what)) return true;
  if (SUNHandleErrWithMsg && v && v->sunctx)
    SUNHandleErrWithMsg(__LINE__, what, __FILE__, SUNGB300_GetLastErrorMessage(),
                        SUN_ERR_EXT_FAIL, v->sunctx);
  return false;
}

Workspace* ws_alloc(cudaStream_t stream)
{
  Workspace* ws = (Workspace*)calloc(1, sizeof(Workspace));
  if (!ws) return nullptr;
  ws->refs       = 1;
  ws->stream     = stream;
  ws->own_stream = false;
  bool ok = check_cuda(cudaMalloc(&ws->d_partials, sizeof(double) * kMaxRedBlocks * kRowsMax),
                       "cudaMalloc(partials)") &&
            check_cuda(cudaMalloc(&ws->d_counter, sizeof(unsigned int)), "cudaMalloc(counter)") &&
            check_cuda(cudaMemset(ws->d_counter, 0, sizeof(unsigned int)), "cudaMemset") &&
            check_cuda(cudaHostAlloc(&ws->h_result, sizeof(double) * kResultMax,
                                     cudaHostAllocMapped),
                       "cudaHostAlloc(result)") &&
            check_cuda(cudaHostGetDevicePointer(&ws->d_result, ws->h_result, 0),
                       "cudaHostGetDevicePointer");
  if (!ok)
  {
    free(ws);
    return nullptr;
  }
  return ws;
}

// All vectors on one CUDA stream share one workspace.  Vectors created without
// an explicit stream use the legacy default stream (NVECTOR_CUDA's default
// policy), so operations on independently created vectors are ordered with
// each other.  All vectors passed to one operation must live on one stream.
std::mutex g_ws_mutex;
std::unordered_map<cudaStream_t, Workspace*> g_ws_by_stream;

Workspace* ws_create(cudaStream_t stream)
{
  std::lock_guard<std::mutex> lock(g_ws_mutex);
  auto it = g_ws_by_stream.find(stream);
  if (it != g_ws_by_stream.end())
  {
    it->second->refs++;
    return it->second;
  }
  Workspace* ws = ws_alloc(stream);
  if (ws) g_ws_by_stream[stream] = ws;
  return ws;
}

void ws_release(Workspace* ws)
{
  if (!ws) return;
  {
    std::lock_guard<std::mutex> lock(g_ws_mutex);
    if (--ws->refs > 0) return;
    g_ws_by_stream.erase(ws->stream);
  }
  cudaStreamSynchronize(ws->stream);
  cudaFree(ws->d_partials);
  cudaFree(ws->d_counter);
  cudaFreeHost(ws->h_result);
  if (ws->own_stream) cudaStreamDestroy(ws->stream);
  free(ws);
}

inline bool sync_stream(N_Vector v)
{
  return ok_or_report(v, cudaStreamSynchronize(S(v)), "cudaStreamSynchronize");
}

inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

// Reduction results reach the host through pinned, mapped memory written by
// the kernel's last block.  Before a launch the host marks the m result slots
// with a signalling-NaN pattern that no arithmetic produces; after it, the
// host polls them until every slot holds a result, which skips the stream
// synchronisation's round trip on the common path.  A reduction still
// running after 2 ms (long vectors) or a failed launch falls back to
// cudaStreamSynchronize, which waits for completion and reports errors.
constexpr uint64_t kResultPending = 0x7ff4dead5eed0001ull;

inline void arm_results(double* h_result, int m)
{
  volatile uint64_t* r = (volatile uint64_t*)h_result;
  for (int j = 0; j < m; ++j) r[j] = kResultPending;
  std::atomic_thread_fence(std::memory_order_seq_cst);
}

inline bool wait_results(N_Vector v, const double* h_result, int m)
{
  const volatile uint64_t* r = (const volatile uint64_t*)h_result;
  const auto t0              = std::chrono::steady_clock::now();
  for (unsigned it = 1;; ++it)
  {
    bool done = true;
    for (int j = 0; j < m && done; ++j) done = r[j] != kResultPending;
    if (done)
    {
      std::atomic_thread_fence(std::memory_order_acquire);
      return true;
    }
    if ((it & 1023u) == 0 &&
        std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(2))
      return sync_stream(v);
  }
}

// ============================================================ device kernels

// Rounding helpers: EXACT (default) rounds every product and sum like
// NVECTOR_SERIAL compiled without contraction; FMA fuses a*x+acc.
template <bool F>
__device__ __forceinline__ double madd(double a, double x, double acc)
{
  if (F) return fma(a, x, acc);
  return __dadd_rn(acc, __dmul_rn(a, x));
}
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }

// ---- elementwise: z = f(x0, x1, x2) ---------------------------------------
template <class F>
__global__ void __launch_bounds__(kBlock)
  k_map(int64_t n, const double* x0, const double* x1,
        const double* x2, double* z, F f, int vec)
{
  const int64_t tid    = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t head         = 0;
  if (vec)
  {
    const int64_t npair = n >> 1;
    const double2* a    = (const double2*)x0;
    const double2* b    = (const double2*)x1;
    const double2* c    = (const double2*)x2;
    double2* zz         = (double2*)z;
    for (int64_t p = tid; p < npair; p += stride)
    {
      double2 va = F::NIN > 0 ? a[p] : make_double2(0, 0);
      double2 vb = F::NIN > 1 ? b[p] : make_double2(0, 0);
      double2 vc = F::NIN > 2 ? c[p] : make_double2(0, 0);
      double2 r;
      r.x   = f(va.x, vb.x, vc.x);
      r.y   = f(va.y, vb.y, vc.y);
      zz[p] = r;
    }
    head = npair << 1;
  }
  for (int64_t i = head + tid; i < n; i += stride)
  {
    double va = F::NIN > 0 ? x0[i] : 0.0;
    double vb = F::NIN > 1 ? x1[i] : 0.0;
    double vc = F::NIN > 2 ? x2[i] : 0.0;
    z[i]      = f(va, vb, vc);
  }
}

template <bool F>
struct FLinSum  // a*x + b*y   (nvector_serial.c:477)
{
  static constexpr int NIN = 2;
  double a, b;
  __device__ double operator()(double x, double y, double) const
  {
    return F ? fma(a, x, mul(b, y)) : add(mul(a, x), mul(b, y));
  }
};
struct FScaleSum  // a*(x+y)   (VScaleSum_Serial)
{
  static constexpr int NIN = 2;
  double a;
  __device__ double operator()(double x, double y, double) const { return mul(a, add(x, y)); }
};
struct FScaleDiff  // a*(x-y)  (VScaleDiff_Serial)
{
  static constexpr int NIN = 2;
  double a;
  __device__ double operator()(double x, double y, double) const { return mul(a, sub(x, y)); }
};
struct FConst
{
  static constexpr int NIN = 0;
  double c;
  __device__ double operator()(double, double, double) const { return c; }
};
struct FProd
{
  static constexpr int NIN = 2;
  __device__ double operator()(double x, double y, double) const { return mul(x, y); }
};
struct FDiv
{
  static constexpr int NIN = 2;
  __device__ double operator()(double x, double y, double) const { return __ddiv_rn(x, y); }
};
struct FScale
{
  static constexpr int NIN = 1;
  double c;
  __device__ double operator()(double x, double, double) const { return mul(c, x); }
};
struct FAbs
{
  static constexpr int NIN = 1;
  __device__ double operator()(double x, double, double) const { return fabs(x); }
};
struct FInv
{
  static constexpr int NIN = 1;
  __device__ double operator()(double x, double, double) const { return __ddiv_rn(1.0, x); }
};
struct FAddConst
{
  static constexpr int NIN = 1;
  double b;
  __device__ double operator()(double x, double, double) const { return add(x, b); }
};
struct FCompare
{
  static constexpr int NIN = 1;
  double c;
  __device__ double operator()(double x, double, double) const { return fabs(x) >= c ? 1.0 : 0.0; }
};

// ---- reductions --------------------------------------------------------------
// E::elem(a, b, c, out, acc) consumes one element; E::NIN inputs are loaded,
// E::WRITES says whether `out` is stored to z.  NV = values per thread.
template <class Op, class E>
__global__ void __launch_bounds__(kBlock)
  k_reduce(int64_t n, const double* x0, const double* x1,
           const double* x2, double* z, E e, int vec,
           double* partials, unsigned int* counter, double* result)
{
  __shared__ double scratch[kWarps];
  const int64_t tid    = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  double acc[1]        = {Op::identity()};
  int64_t head         = 0;
  if (vec)
  {
    const int64_t npair = n >> 1;
    for (int64_t p = tid; p < npair; p += stride)
    {
      double2 va = E::NIN > 0 ? ((const double2*)x0)[p] : make_double2(0, 0);
      double2 vb = E::NIN > 1 ? ((const double2*)x1)[p] : make_double2(0, 0);
      double2 vc = E::NIN > 2 ? ((const double2*)x2)[p] : make_double2(0, 0);
      double2 r;
      e.elem(va.x, vb.x, vc.x, r.x, acc[0]);
      e.elem(va.y, vb.y, vc.y, r.y, acc[0]);
      if (E::WRITES) ((double2*)z)[p] = r;
    }
    head = npair << 1;
  }
  for (int64_t i = head + tid; i < n; i += stride)
  {
    double va = E::NIN > 0 ? x0[i] : 0.0;
    double vb = E::NIN > 1 ? x1[i] : 0.0;
    double vc = E::NIN > 2 ? x2[i] : 0.0;
    double r;
    e.elem(va, vb, vc, r, acc[0]);
    if (E::WRITES) z[i] = r;
  }
  block_reduce<Op, 1>(acc, scratch);
  if (gridDim.x == 1)
  {
    if (threadIdx.x == 0) result[0] = acc[0];
    return;
  }
  if (grid_finish<Op, 1>(acc, partials, counter, gridDim.x, blockIdx.x, scratch))
    result[0] = acc[0];
}

template <bool F>
struct EDot
{
  static constexpr int NIN = 2;
  static constexpr bool WRITES = false;
  __device__ void elem(double x, double y, double, double&, double& s) const { s = madd<F>(x, y, s); }
};
struct EMaxAbs
{
  static constexpr int NIN = 1;
  static constexpr bool WRITES = false;
  __device__ void elem(double x, double, double, double&, double& m) const
  {
    double a = fabs(x);
    if (a > m) m = a;
  }
};
template <bool F>
struct EWSqr
{
  static constexpr int NIN = 2;
  static constexpr bool WRITES = false;
  __device__ void elem(double x, double w, double, double&, double& s) const
  {
    double p = mul(x, w);
    s        = madd<F>(p, p, s);
  }
};
template <bool F>
struct EWSqrMask
{
  static constexpr int NIN = 3;
  static constexpr bool WRITES = false;
  __device__ void elem(double x, double w, double id, double&, double& s) const
  {
    if (id > 0.0)
    {
      double p = mul(x, w);
      s        = madd<F>(p, p, s);
    }
  }
};
struct EMin
{
  static constexpr int NIN = 1;
  static constexpr bool WRITES = false;
  __device__ void elem(double x, double, double, double&, double& m) const
  {
    if (x < m) m = x;
  }
};
struct EL1
{
  static constexpr int NIN = 1;
  static constexpr bool WRITES = false;
  __device__ void elem(double x, double, double, double&, double& s) const { s = add(s, fabs(x)); }
};
// InvTest: z = 1/x where x != 0, z unchanged where x == 0; flag any zero.
struct EInvTest
{
  static constexpr int NIN = 2;  // x, old z
  static constexpr bool WRITES = true;
  __device__ void elem(double x, double zold, double, double& out, double& flag) const
  {
    if (x == 0.0)
    {
      out  = zold;
      flag = 1.0;
    }
    else out = __ddiv_rn(1.0, x);
  }
};
// ConstrMask (nvector_serial.c:800-831): m = 1 where a constraint fails.
struct EConstrMask
{
  static constexpr int NIN = 2;  // c, x
  static constexpr bool WRITES = true;
  __device__ void elem(double c, double x, double, double& m, double& flag) const
  {
    m = 0.0;
    if (c == 0.0) return;
    double xc = mul(x, c);
    bool bad  = (fabs(c) > 1.5 && xc <= 0.0) || (fabs(c) > 0.5 && xc < 0.0);
    if (bad)
    {
      m    = 1.0;
      flag = 1.0;
    }
  }
};
struct EMinQuot
{
  static constexpr int NIN = 2;
  static constexpr bool WRITES = false;
  __device__ void elem(double num, double den, double, double&, double& m) const
  {
    if (den != 0.0)
    {
      double q = __ddiv_rn(num, den);
      if (q < m) m = q;
    }
  }
};

// ---- fused: linear combination z = sum_k c_k X_k ------------------------------
constexpr int kMaxList = 32;
struct LCArgs
{
  const double* x[kMaxList];
  double c[kMaxList];
};

// First term either starts the sum (c0*X0) or continues it (z + c0*X0 ...).
template <bool F, int NV>
__global__ void __launch_bounds__(kBlock)
  k_lincomb(int64_t n, int nv_rt, LCArgs args, double* z, int accumulate, int vec)
{
  const int nv         = NV > 0 ? NV : nv_rt;
  const int64_t tid    = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t head         = 0;
  if (vec)
  {
    const int64_t npair = n >> 1;
    for (int64_t p = tid; p < npair; p += stride)
    {
      // term 0 starts the sum or is added to z; with NV fixed every later
      // term's load is issued up front (the loop unrolls completely)
      const double2 v0 = ((const double2*)args.x[0])[p];
      double2 acc;
      if (accumulate)
      {
        acc   = ((const double2*)z)[p];
        acc.x = madd<F>(args.c[0], v0.x, acc.x);
        acc.y = madd<F>(args.c[0], v0.y, acc.y);
      }
      else acc = make_double2(mul(args.c[0], v0.x), mul(args.c[0], v0.y));
#pragma unroll 8
      for (int k = 1; k < nv; ++k)
      {
        double2 v = ((const double2*)args.x[k])[p];
        acc.x     = madd<F>(args.c[k], v.x, acc.x);
        acc.y     = madd<F>(args.c[k], v.y, acc.y);
      }
      ((double2*)z)[p] = acc;
    }
    head = npair << 1;
  }
  for (int64_t i = head + tid; i < n; i += stride)
  {
    double acc;
    int k0 = 0;
    if (accumulate) acc = z[i];
    else
    {
      acc = mul(args.c[0], args.x[0][i]);
      k0  = 1;
    }
    for (int k = k0; k < nv; ++k) acc = madd<F>(args.c[k], args.x[k][i], acc);
    z[i] = acc;
  }
}

// ---- fused: scale-add-multi Z_k = a_k x + Y_k ----------------------------------
struct SAMArgs
{
  const double* y[kMaxList];
  double* z[kMaxList];
  double a[kMaxList];
};
// NV > 0: a fixed vector count; every Y_k element pair is loaded before any
// Z_k is stored (Z_k may be Y_k: in place), so the loads are all in flight at
// once.  NV == 0: run-time count, one vector at a time.
template <bool F, int NV>
__global__ void __launch_bounds__(kBlock)
  k_scaleaddmulti(int64_t n, int nv, const double* x, SAMArgs args, int vec)
{
  const int64_t tid    = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t head         = 0;
  if (vec)
  {
    const int64_t npair = n >> 1;
    for (int64_t p = tid; p < npair; p += stride)
    {
      double2 xv = ((const double2*)x)[p];
      if (NV > 0)
      {
        double2 yv[NV > 0 ? NV : 1];
#pragma unroll
        for (int k = 0; k < NV; ++k) yv[k] = ((const double2*)args.y[k])[p];
#pragma unroll
        for (int k = 0; k < NV; ++k)
        {
          double2 r;
          r.x                      = madd<F>(args.a[k], xv.x, yv[k].x);
          r.y                      = madd<F>(args.a[k], xv.y, yv[k].y);
          ((double2*)args.z[k])[p] = r;
        }
        continue;
      }
#pragma unroll 6
      for (int k = 0; k < nv; ++k)
      {
        double2 yv = ((const double2*)args.y[k])[p];
        double2 r;
        r.x                    = madd<F>(args.a[k], xv.x, yv.x);
        r.y                    = madd<F>(args.a[k], xv.y, yv.y);
        ((double2*)args.z[k])[p] = r;
      }
    }
    head = npair << 1;
  }
  for (int64_t i = head + tid; i < n; i += stride)
  {
    double xv = x[i];
    for (int k = 0; k < nv; ++k) args.z[k][i] = madd<F>(args.a[k], xv, args.y[k][i]);
  }
}

// ---- fused: dot-product-multi d_k = x . Y_k (x read once) -----------------------
template <bool F, int NV>
__global__ void __launch_bounds__(kBlock)
  k_dotmulti(int64_t n, const double* x, LCArgs args, int vec,
             double* partials, unsigned int* counter, double* result)
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
        double2 yv = ((const double2*)args.x[k])[p];
        acc[k]     = madd<F>(xv.x, yv.x, acc[k]);
        acc[k]     = madd<F>(xv.y, yv.y, acc[k]);
      }
    }
    head = npair << 1;
  }
  for (int64_t i = head + tid; i < n; i += stride)
  {
    double xv = x[i];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = madd<F>(xv, args.x[k][i], acc[k]);
  }
  block_reduce<SumOp, NV>(acc, scratch);
  if (gridDim.x == 1)
  {
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) result[k] = acc[k];
    return;
  }
  if (grid_finish<SumOp, NV>(acc, partials, counter, gridDim.x, blockIdx.x, scratch))
#pragma unroll
    for (int k = 0; k < NV; ++k) result[k] = acc[k];
}

// ---- vector arrays: one row of blocks per vector (blockIdx.y) --------------------
struct VAArgs
{
  const double* x[kMaxList];
  const double* y[kMaxList];
  double* z[kMaxList];
  double c[kMaxList];
};
// mode: 0 z=a x+b y, 1 z=a(x+y), 2 z=a(x-y), 3 z=c_k x, 4 z=c
template <bool F>
__global__ void __launch_bounds__(kBlock)
  k_va_map(int64_t n, int mode, double a, double b, VAArgs args, int vec)
{
  const int k          = blockIdx.y;
  const double* x      = args.x[k];
  const double* y      = args.y[k];
  double* z            = args.z[k];
  const int64_t tid    = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  auto f = [&](double xv, double yv) -> double {
    switch (mode)
    {
    case 0: return F ? fma(a, xv, mul(b, yv)) : add(mul(a, xv), mul(b, yv));
    case 1: return mul(a, add(xv, yv));
    case 2: return mul(a, sub(xv, yv));
    case 3: return mul(args.c[k], xv);
    default: return a;
    }
  };
  const bool needx = mode != 4, needy = mode <= 2;
  int64_t head     = 0;
  if (vec)
  {
    const int64_t npair = n >> 1;
    for (int64_t p = tid; p < npair; p += stride)
    {
      double2 xv = needx ? ((const double2*)x)[p] : make_double2(0, 0);
      double2 yv = needy ? ((const double2*)y)[p] : make_double2(0, 0);
      double2 r;
      r.x              = f(xv.x, yv.x);
      r.y              = f(xv.y, yv.y);
      ((double2*)z)[p] = r;
    }
    head = npair << 1;
  }
  for (int64_t i = head + tid; i < n; i += stride)
    z[i] = f(needx ? x[i] : 0.0, needy ? y[i] : 0.0);
}

// Weighted squared sums of several (X_k, W_k[, id]) pairs; one value per row.
template <bool F, bool MASK>
__global__ void __launch_bounds__(kBlock)
  k_va_wsqr(int64_t n, VAArgs args, const double* id, int vec,
            double* partials, unsigned int* counter, double* result)
{
  __shared__ double scratch[kWarps];
  __shared__ bool is_last;
  const int k          = blockIdx.y;
  const double* x      = args.x[k];
  const double* w      = args.y[k];
  const int64_t tid    = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  double acc[1]        = {0.0};
  int64_t head         = 0;
  if (vec)
  {
    const int64_t npair = n >> 1;
    for (int64_t p = tid; p < npair; p += stride)
    {
      double2 xv = ((const double2*)x)[p], wv = ((const double2*)w)[p];
      double2 iv = MASK ? ((const double2*)id)[p] : make_double2(1, 1);
      if (!MASK || iv.x > 0.0)
      {
        double q = mul(xv.x, wv.x);
        acc[0]   = madd<F>(q, q, acc[0]);
      }
      if (!MASK || iv.y > 0.0)
      {
        double q = mul(xv.y, wv.y);
        acc[0]   = madd<F>(q, q, acc[0]);
      }
    }
    head = npair << 1;
  }
  for (int64_t i = head + tid; i < n; i += stride)
  {
    if (!MASK || id[i] > 0.0)
    {
      double q = mul(x[i], w[i]);
      acc[0]   = madd<F>(q, q, acc[0]);
    }
  }
  block_reduce<SumOp, 1>(acc, scratch);
  const int nb = gridDim.x, rows = gridDim.y;
  if (threadIdx.x == 0)
  {
    partials[k * nb + blockIdx.x] = acc[0];
    __threadfence();
    unsigned int t = atomicAdd(counter, 1u);
    is_last        = (t == (unsigned int)(nb * rows - 1));
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  for (int r = 0; r < rows; ++r)
  {
    double v[1] = {0.0};
    bool first  = true;
    for (int b = threadIdx.x; b < nb; b += kBlock)
    {
      double pv = __ldcg(&partials[r * nb + b]);
      v[0]      = first ? pv : add(v[0], pv);
      first     = false;
    }
    block_reduce<SumOp, 1>(v, scratch);
    if (threadIdx.x == 0) result[r] = v[0];
  }
  if (threadIdx.x == 0) *counter = 0u;
}

// ScaleAddMultiVectorArray: row i computes Z[j][i] = a_j X_i + Y[j][i].
struct SAMVAArgs
{
  const double* x[8];
  const double* y[64];
  double* z[64];
  double a[8];
};
template <bool F>
__global__ void __launch_bounds__(kBlock)
  k_va_scaleaddmulti(int64_t n, int nsum, SAMVAArgs args, int vec)
{
  const int i          = blockIdx.y;
  const double* x      = args.x[i];
  const int64_t tid    = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t head         = 0;
  if (vec)
  {
    const int64_t npair = n >> 1;
    for (int64_t p = tid; p < npair; p += stride)
    {
      double2 xv = ((const double2*)x)[p];
      for (int j = 0; j < nsum; ++j)
      {
        double2 yv = ((const double2*)args.y[i * nsum + j])[p];
        double2 r;
        r.x                                = madd<F>(args.a[j], xv.x, yv.x);
        r.y                                = madd<F>(args.a[j], xv.y, yv.y);
        ((double2*)args.z[i * nsum + j])[p] = r;
      }
    }
    head = npair << 1;
  }
  for (int64_t e = head + tid; e < n; e += stride)
  {
    double xv = x[e];
    for (int j = 0; j < nsum; ++j)
      args.z[i * nsum + j][e] = madd<F>(args.a[j], xv, args.y[i * nsum + j][e]);
  }
}

// LinearCombinationVectorArray: row j computes Z_j = sum_i c_i X[i][j].
struct LCVAArgs
{
  const double* x[64];  // [row * nsum + i]
  double* z[8];
  double c[8];
};
template <bool F>
__global__ void __launch_bounds__(kBlock)
  k_va_lincomb(int64_t n, int nsum, LCVAArgs args, int accumulate, int vec)
{
  const int j          = blockIdx.y;
  double* z            = args.z[j];
  const int64_t tid    = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t head         = 0;
  if (vec)
  {
    const int64_t npair = n >> 1;
    for (int64_t p = tid; p < npair; p += stride)
    {
      double2 acc;
      int i0 = 0;
      if (accumulate) acc = ((const double2*)z)[p];
      else
      {
        double2 v = ((const double2*)args.x[j * nsum])[p];
        acc       = make_double2(mul(args.c[0], v.x), mul(args.c[0], v.y));
        i0        = 1;
      }
      for (int i = i0; i < nsum; ++i)
      {
        double2 v = ((const double2*)args.x[j * nsum + i])[p];
        acc.x     = madd<F>(args.c[i], v.x, acc.x);
        acc.y     = madd<F>(args.c[i], v.y, acc.y);
      }
      ((double2*)z)[p] = acc;
    }
    head = npair << 1;
  }
  for (int64_t e = head + tid; e < n; e += stride)
  {
    double acc;
    int i0 = 0;
    if (accumulate) acc = z[e];
    else
    {
      acc = mul(args.c[0], args.x[j * nsum][e]);
      i0  = 1;
    }
    for (int i = i0; i < nsum; ++i) acc = madd<F>(args.c[i], args.x[j * nsum + i][e], acc);
    z[e] = acc;
  }
}

// ============================================================ host launchers

template <class Fn>
bool launch_map(N_Vector ref, int64_t n, const double* a, const double* b,
                const double* c, double* z, Fn f)
{
  if (n <= 0) return true;
  int vec = aligned16(z) && (Fn::NIN < 1 || aligned16(a)) && (Fn::NIN < 2 || aligned16(b)) &&
            (Fn::NIN < 3 || aligned16(c));
  int64_t items = vec ? (n + 1) / 2 : n;
  k_map<Fn><<<stream_grid(items), kBlock, 0, S(ref)>>>(n, a, b, c, z, f, vec);
  count_launch();
  return ok_or_report(ref, cudaGetLastError(), "k_map launch");
}

// Runs a single-value reduction and returns it on the host (NaN on failure).
template <class Op, class E>
double launch_reduce(N_Vector ref, int64_t n, const double* a, const double* b,
                     const double* c, double* z, E e)
{
  Workspace* ws = C(ref)->ws;
  if (n <= 0) return Op::identity();
  int vec = (E::NIN < 1 || aligned16(a)) && (E::NIN < 2 || aligned16(b)) &&
            (E::NIN < 3 || aligned16(c)) && (!E::WRITES || aligned16(z));
  int64_t items = vec ? (n + 1) / 2 : n;
  int grid      = reduce_grid(items);
  arm_results(ws->h_result, 1);
  k_reduce<Op, E><<<grid, kBlock, 0, ws->stream>>>(n, a, b, c, z, e, vec, ws->d_partials,
                                                   ws->d_counter, ws->d_result);
  count_launch();
  if (!ok_or_report(ref, cudaGetLastError(), "k_reduce launch")) return NAN;
  if (!wait_results(ref, ws->h_result, 1)) return NAN;
  return ws->h_result[0];
}

}  // namespace

// ============================================================ host operations

namespace {

#define DISPATCH_F(v, KERNEL_CALL_T, KERNEL_CALL_F) \
  do {                                              \
    if (FMA(v)) { KERNEL_CALL_T; }                  \
    else { KERNEL_CALL_F; }                         \
  } while (0)

void fill_ops(N_Vector_Ops ops);

N_Vector new_empty(SUNContext sunctx)
{
  N_Vector v = (N_Vector)malloc(sizeof *v);
  if (!v) return nullptr;
  N_Vector_Ops ops = (N_Vector_Ops)calloc(1, sizeof *ops);
  if (!ops)
  {
    free(v);
    return nullptr;
  }
  fill_ops(ops);
  v->ops     = ops;
  v->content = nullptr;
  v->sunctx  = sunctx;
  return v;
}

void free_vector(N_Vector v)
{
  if (!v) return;
  free(v->ops);
  free(v);
}

Content* new_content(sunindextype length, Workspace* ws, bool fma)
{
  Content* c = (Content*)calloc(1, sizeof(Content));
  if (!c) return nullptr;
  c->length = length;
  c->ws     = ws;
  c->fma    = fma;
  return c;
}

bool alloc_device(Content* c)
{
  if (c->length <= 0) return true;
  if (!check_cuda(cudaMalloc(&c->dev, sizeof(double) * (size_t)c->length), "cudaMalloc(vector)"))
    return false;
  c->own_dev = true;
  return true;
}

bool ensure_host(N_Vector v)
{
  Content* c = C(v);
  if (c->host || c->length <= 0) return true;
  if (!check_cuda(cudaMallocHost(&c->host, sizeof(double) * (size_t)c->length),
                  "cudaMallocHost(vector)"))
    return false;
  c->own_host = true;
  return true;
}

N_Vector make_vector(sunindextype length, cudaStream_t stream, SUNContext sunctx,
                     bool alloc)
{
  if (length < 0) return nullptr;
  N_Vector v = new_empty(sunctx);
  if (!v) return nullptr;
  Workspace* ws = ws_create(stream);
  Content* c    = ws ? new_content(length, ws, true) : nullptr;
  if (!c || (alloc && !alloc_device(c)))
  {
    if (c) free(c);
    ws_release(ws);
    free_vector(v);
    return nullptr;
  }
  v->content = c;
  return v;
}

// z = sum_k c_k X_k with the serial vector's accumulation order.
bool lincomb_core(N_Vector ref, int nvec, const double* c, N_Vector* X, N_Vector z,
                  bool accumulate_first)
{
  int64_t n = LEN(z);
  if (n <= 0) return true;
  int k = 0;
  bool accumulate = accumulate_first;
  if (accumulate) k = 1;  // z already holds X[0] with coefficient 1
  while (k < nvec)
  {
    int m = nvec - k < kMaxList ? nvec - k : kMaxList;
    LCArgs args;
    bool vec = aligned16(D(z));
    for (int j = 0; j < m; ++j)
    {
      args.x[j] = D(X[k + j]);
      args.c[j] = c[k + j];
      vec       = vec && aligned16(args.x[j]);
    }
    int64_t items = vec ? (n + 1) / 2 : n;
    int grid      = stream_grid(items);
    const int acc_i = accumulate ? 1 : 0;
    switch (m)
    {  // fixed term counts unroll completely; longer lists use the run-time loop
#define LC_CASE(M)                                                                              \
  case M:                                                                                       \
    DISPATCH_F(ref, (k_lincomb<true, M><<<grid, kBlock, 0, S(ref)>>>(n, m, args, D(z), acc_i, vec)), \
               (k_lincomb<false, M><<<grid, kBlock, 0, S(ref)>>>(n, m, args, D(z), acc_i, vec))); \
    break;
      LC_CASE(1)
      LC_CASE(2)
      LC_CASE(3)
      LC_CASE(4)
      LC_CASE(5)
      LC_CASE(6)
      LC_CASE(7)
      LC_CASE(8)
#undef LC_CASE
    default:
      DISPATCH_F(ref,
                 (k_lincomb<true, 0><<<grid, kBlock, 0, S(ref)>>>(n, m, args, D(z), acc_i, vec)),
                 (k_lincomb<false, 0><<<grid, kBlock, 0, S(ref)>>>(n, m, args, D(z), acc_i, vec)));
    }
    count_launch();
    if (!ok_or_report(ref, cudaGetLastError(), "k_lincomb launch")) return false;
    accumulate = true;
    k += m;
  }
  return true;
}

template <int NV>
void launch_dotmulti(N_Vector x, const LCArgs& args, int vec, int grid)
{
  Workspace* ws = C(x)->ws;
  if (FMA(x))
    k_dotmulti<true, NV><<<grid, kBlock, 0, ws->stream>>>(LEN(x), D(x), args, vec, ws->d_partials,
                                                          ws->d_counter, ws->d_result);
  else
    k_dotmulti<false, NV><<<grid, kBlock, 0, ws->stream>>>(LEN(x), D(x), args, vec, ws->d_partials,
                                                           ws->d_counter, ws->d_result);
}

bool dotmulti_core(int nvec, N_Vector x, N_Vector* Y, double* out)
{
  int64_t n     = LEN(x);
  Workspace* ws = C(x)->ws;
  if (n <= 0)
  {
    for (int k = 0; k < nvec; ++k) out[k] = 0.0;
    return true;
  }
  for (int k0 = 0; k0 < nvec; k0 += kMaxRedVals)
  {
    int m = nvec - k0 < kMaxRedVals ? nvec - k0 : kMaxRedVals;
    LCArgs args;
    int vec = aligned16(D(x));
    for (int j = 0; j < m; ++j)
    {
      args.x[j] = D(Y[k0 + j]);
      vec       = vec && aligned16(args.x[j]);
    }
    int64_t items = vec ? (n + 1) / 2 : n;
    int grid      = reduce_grid(items);
    arm_results(ws->h_result, m);
    switch (m)
    {
    case 1: launch_dotmulti<1>(x, args, vec, grid); break;
    case 2: launch_dotmulti<2>(x, args, vec, grid); break;
    case 3: launch_dotmulti<3>(x, args, vec, grid); break;
    case 4: launch_dotmulti<4>(x, args, vec, grid); break;
    case 5: launch_dotmulti<5>(x, args, vec, grid); break;
    case 6: launch_dotmulti<6>(x, args, vec, grid); break;
    case 7: launch_dotmulti<7>(x, args, vec, grid); break;
    default: launch_dotmulti<8>(x, args, vec, grid); break;
    }
    count_launch();
    if (!ok_or_report(x, cudaGetLastError(), "k_dotmulti launch")) return false;
    if (!wait_results(x, ws->h_result, m)) return false;
    for (int j = 0; j < m; ++j) out[k0 + j] = ws->h_result[j];
  }
  return true;
}

// Vector-array elementwise map over nvec rows (chunks of kMaxList rows).
bool va_map(N_Vector ref, int nvec, int mode, double a, double b, const double* cvals,
            N_Vector* X, N_Vector* Y, N_Vector* Z)
{
  int64_t n = LEN(Z[0]);
  if (n <= 0) return true;
  for (int r0 = 0; r0 < nvec; r0 += kMaxList)
  {
    int m = nvec - r0 < kMaxList ? nvec - r0 : kMaxList;
    VAArgs args;
    int vec = 1;
    for (int j = 0; j < m; ++j)
    {
      args.x[j] = X ? D(X[r0 + j]) : nullptr;
      args.y[j] = Y ? D(Y[r0 + j]) : nullptr;
      args.z[j] = D(Z[r0 + j]);
      args.c[j] = cvals ? cvals[r0 + j] : 0.0;
      vec       = vec && aligned16(args.z[j]) && (!X || aligned16(args.x[j])) &&
            (!Y || aligned16(args.y[j]));
    }
    int64_t items = vec ? (n + 1) / 2 : n;
    int gx        = stream_grid(items);
    gx            = (gx + m - 1) / m;
    if (gx < 1) gx = 1;
    dim3 grid(gx, m);
    DISPATCH_F(ref, (k_va_map<true><<<grid, kBlock, 0, S(ref)>>>(n, mode, a, b, args, vec)),
               (k_va_map<false><<<grid, kBlock, 0, S(ref)>>>(n, mode, a, b, args, vec)));
    count_launch();
    if (!ok_or_report(ref, cudaGetLastError(), "k_va_map launch")) return false;
  }
  return true;
}

int linsum_mode(double a, double b)
{
  bool unit = (a == 1.0) || (b == 1.0) || (a == -1.0) || (b == -1.0);
  if (!unit && a == b) return 1;
  if (!unit && a == -b) return 2;
  return 0;
}

bool va_wsqr(int nvec, N_Vector* X, N_Vector* W, N_Vector id, double* out)
{
  N_Vector ref  = X[0];
  int64_t n     = LEN(ref);
  Workspace* ws = C(ref)->ws;
  if (n <= 0)
  {
    for (int k = 0; k < nvec; ++k) out[k] = 0.0;
    return true;
  }
  for (int r0 = 0; r0 < nvec; r0 += kRowsMax)
  {
    int m = nvec - r0 < kRowsMax ? nvec - r0 : kRowsMax;
    VAArgs args;
    int vec = id ? aligned16(D(id)) : 1;
    for (int j = 0; j < m; ++j)
    {
      args.x[j] = D(X[r0 + j]);
      args.y[j] = D(W[r0 + j]);
      args.z[j] = nullptr;
      vec       = vec && aligned16(args.x[j]) && aligned16(args.y[j]);
    }
    int64_t items = vec ? (n + 1) / 2 : n;
    dim3 grid(reduce_grid(items), m);
    const double* idp = id ? D(id) : nullptr;
    arm_results(ws->h_result, m);
    if (id)
      DISPATCH_F(ref,
                 (k_va_wsqr<true, true><<<grid, kBlock, 0, ws->stream>>>(
                   n, args, idp, vec, ws->d_partials, ws->d_counter, ws->d_result)),
                 (k_va_wsqr<false, true><<<grid, kBlock, 0, ws->stream>>>(
                   n, args, idp, vec, ws->d_partials, ws->d_counter, ws->d_result)));
    else
      DISPATCH_F(ref,
                 (k_va_wsqr<true, false><<<grid, kBlock, 0, ws->stream>>>(
                   n, args, idp, vec, ws->d_partials, ws->d_counter, ws->d_result)),
                 (k_va_wsqr<false, false><<<grid, kBlock, 0, ws->stream>>>(
                   n, args, idp, vec, ws->d_partials, ws->d_counter, ws->d_result)));
    count_launch();
    if (!ok_or_report(ref, cudaGetLastError(), "k_va_wsqr launch")) return false;
    if (!wait_results(ref, ws->h_result, m)) return false;
    for (int j = 0; j < m; ++j) out[r0 + j] = ws->h_result[j];
  }
  return true;
}

}  // namespace

// ------------------------------------------------------------ constructors

extern "C" {

N_Vector N_VNewEmpty_GB300(SUNContext sunctx)
{
  return new_empty(sunctx);
}

N_Vector N_VNew_GB300(sunindextype length, SUNContext sunctx)
{
  return make_vector(length, nullptr, sunctx, true);
}

N_Vector N_VNewWithStream_GB300(sunindextype length, void* cuda_stream, SUNContext sunctx)
{
  return make_vector(length, (cudaStream_t)cuda_stream, sunctx, true);
}

N_Vector N_VMake_GB300(sunindextype length, sunrealtype* h_vdata, sunrealtype* d_vdata,
                       SUNContext sunctx)
{
  N_Vector v = make_vector(length, nullptr, sunctx, d_vdata == nullptr);
  if (!v) return nullptr;
  if (d_vdata) C(v)->dev = d_vdata;
  C(v)->host = h_vdata;
  return v;
}

N_Vector_ID N_VGetVectorID_GB300(N_Vector) { return SUNDIALS_NVEC_CUSTOM; }

N_Vector N_VCloneEmpty_GB300(N_Vector w)
{
  if (!w || !w->content) return nullptr;
  N_Vector v = new_empty(w->sunctx);
  if (!v) return nullptr;
  memcpy(v->ops, w->ops, sizeof *v->ops);  // N_VCopyOps: enabled ops carry over
  Content* c = new_content(C(w)->length, C(w)->ws, C(w)->fma);
  if (!c)
  {
    free_vector(v);
    return nullptr;
  }
  {
    std::lock_guard<std::mutex> lock(g_ws_mutex);
    C(w)->ws->refs++;
  }
  v->content = c;
  return v;
}

N_Vector N_VClone_GB300(N_Vector w)
{
  N_Vector v = N_VCloneEmpty_GB300(w);
  if (!v) return nullptr;
  if (!alloc_device(C(v)))
  {
    N_VDestroy_GB300(v);
    return nullptr;
  }
  return v;
}

void N_VDestroy_GB300(N_Vector v)
{
  if (!v) return;
  Content* c = C(v);
  if (c)
  {
    if (c->own_dev && c->dev) cudaFree(c->dev);
    if (c->own_host && c->host) cudaFreeHost(c->host);
    ws_release(c->ws);
    free(c);
  }
  free_vector(v);
}

void N_VSpace_GB300(N_Vector v, sunindextype* lrw, sunindextype* liw)
{
  *lrw = C(v)->length;
  *liw = 2;
}

sunrealtype* N_VGetArrayPointer_GB300(N_Vector v)
{
  if (!ensure_host(v)) return nullptr;
  return C(v)->host;
}
sunrealtype* N_VGetHostArrayPointer_GB300(N_Vector v) { return N_VGetArrayPointer_GB300(v); }
sunrealtype* N_VGetDeviceArrayPointer_GB300(N_Vector v) { return C(v)->dev; }

void N_VSetArrayPointer_GB300(sunrealtype* v_data, N_Vector v)
{
  Content* c = C(v);
  if (c->own_host && c->host) cudaFreeHost(c->host);
  c->host     = v_data;
  c->own_host = false;
}

void N_VSetDeviceArrayPointer_GB300(sunrealtype* d_vdata, N_Vector v)
{
  Content* c = C(v);
  if (c->own_dev && c->dev) cudaFree(c->dev);
  c->dev     = d_vdata;
  c->own_dev = false;
}

void* N_VGetStream_GB300(N_Vector v) { return (void*)C(v)->ws->stream; }
sunbooleantype N_VIsManagedMemory_GB300(N_Vector) { return SUNFALSE; }
SUNComm N_VGetCommunicator_GB300(N_Vector) { return SUN_COMM_NULL; }
sunindextype N_VGetLength_GB300(N_Vector v) { return C(v)->length; }

void N_VCopyToDevice_GB300(N_Vector v)
{
  Content* c = C(v);
  if (c->length <= 0 || !c->host || !c->dev) return;
  check_cuda(cudaMemcpyAsync(c->dev, c->host, sizeof(double) * (size_t)c->length,
                             cudaMemcpyHostToDevice, c->ws->stream),
             "N_VCopyToDevice");
  sync_stream(v);
}

void N_VCopyFromDevice_GB300(N_Vector v)
{
  Content* c = C(v);
  if (c->length <= 0 || !c->dev || !ensure_host(v)) return;
  check_cuda(cudaMemcpyAsync(c->host, c->dev, sizeof(double) * (size_t)c->length,
                             cudaMemcpyDeviceToHost, c->ws->stream),
             "N_VCopyFromDevice");
  sync_stream(v);
}

// ------------------------------------------------------ standard operations

void N_VLinearSum_GB300(sunrealtype a, N_Vector x, sunrealtype b, N_Vector y, N_Vector z)
{
  int mode = linsum_mode(a, b);
  int64_t n = LEN(z);
  if (mode == 1) launch_map(z, n, D(x), D(y), nullptr, D(z), FScaleSum{a});
  else if (mode == 2) launch_map(z, n, D(x), D(y), nullptr, D(z), FScaleDiff{a});
  else if (FMA(z)) launch_map(z, n, D(x), D(y), nullptr, D(z), FLinSum<true>{a, b});
  else launch_map(z, n, D(x), D(y), nullptr, D(z), FLinSum<false>{a, b});
}

void N_VConst_GB300(sunrealtype c, N_Vector z)
{
  launch_map(z, LEN(z), nullptr, nullptr, nullptr, D(z), FConst{c});
}
void N_VProd_GB300(N_Vector x, N_Vector y, N_Vector z)
{
  launch_map(z, LEN(z), D(x), D(y), nullptr, D(z), FProd{});
}
void N_VDiv_GB300(N_Vector x, N_Vector y, N_Vector z)
{
  launch_map(z, LEN(z), D(x), D(y), nullptr, D(z), FDiv{});
}
void N_VScale_GB300(sunrealtype c, N_Vector x, N_Vector z)
{
  launch_map(z, LEN(z), D(x), nullptr, nullptr, D(z), FScale{c});
}
void N_VAbs_GB300(N_Vector x, N_Vector z)
{
  launch_map(z, LEN(z), D(x), nullptr, nullptr, D(z), FAbs{});
}
void N_VInv_GB300(N_Vector x, N_Vector z)
{
  launch_map(z, LEN(z), D(x), nullptr, nullptr, D(z), FInv{});
}
void N_VAddConst_GB300(N_Vector x, sunrealtype b, N_Vector z)
{
  launch_map(z, LEN(z), D(x), nullptr, nullptr, D(z), FAddConst{b});
}
void N_VCompare_GB300(sunrealtype c, N_Vector x, N_Vector z)
{
  launch_map(z, LEN(z), D(x), nullptr, nullptr, D(z), FCompare{c});
}

sunrealtype N_VDotProd_GB300(N_Vector x, N_Vector y)
{
  if (FMA(x)) return launch_reduce<SumOp>(x, LEN(x), D(x), D(y), nullptr, nullptr, EDot<true>{});
  return launch_reduce<SumOp>(x, LEN(x), D(x), D(y), nullptr, nullptr, EDot<false>{});
}
sunrealtype N_VMaxNorm_GB300(N_Vector x)
{
  return launch_reduce<MaxOp>(x, LEN(x), D(x), nullptr, nullptr, nullptr, EMaxAbs{});
}
sunrealtype N_VWSqrSumLocal_GB300(N_Vector x, N_Vector w)
{
  if (FMA(x)) return launch_reduce<SumOp>(x, LEN(x), D(x), D(w), nullptr, nullptr, EWSqr<true>{});
  return launch_reduce<SumOp>(x, LEN(x), D(x), D(w), nullptr, nullptr, EWSqr<false>{});
}
sunrealtype N_VWSqrSumMaskLocal_GB300(N_Vector x, N_Vector w, N_Vector id)
{
  if (FMA(x))
    return launch_reduce<SumOp>(x, LEN(x), D(x), D(w), D(id), nullptr, EWSqrMask<true>{});
  return launch_reduce<SumOp>(x, LEN(x), D(x), D(w), D(id), nullptr, EWSqrMask<false>{});
}
sunrealtype N_VWrmsNorm_GB300(N_Vector x, N_Vector w)
{
  double s = N_VWSqrSumLocal_GB300(x, w);
  return sqrt(s / (double)C(x)->length);
}
sunrealtype N_VWrmsNormMask_GB300(N_Vector x, N_Vector w, N_Vector id)
{
  double s = N_VWSqrSumMaskLocal_GB300(x, w, id);
  return sqrt(s / (double)C(x)->length);
}
sunrealtype N_VMin_GB300(N_Vector x)
{
  return launch_reduce<MinOp>(x, LEN(x), D(x), nullptr, nullptr, nullptr, EMin{});
}
sunrealtype N_VWL2Norm_GB300(N_Vector x, N_Vector w)
{
  return sqrt(N_VWSqrSumLocal_GB300(x, w));
}
sunrealtype N_VL1Norm_GB300(N_Vector x)
{
  return launch_reduce<SumOp>(x, LEN(x), D(x), nullptr, nullptr, nullptr, EL1{});
}
sunbooleantype N_VInvTest_GB300(N_Vector x, N_Vector z)
{
  double flag = launch_reduce<MaxOp>(x, LEN(x), D(x), D(z), nullptr, D(z), EInvTest{});
  return flag == 0.0 ? SUNTRUE : SUNFALSE;
}
sunbooleantype N_VConstrMask_GB300(N_Vector c, N_Vector x, N_Vector m)
{
  double flag = launch_reduce<MaxOp>(x, LEN(x), D(c), D(x), nullptr, D(m), EConstrMask{});
  return flag == 0.0 ? SUNTRUE : SUNFALSE;
}
sunrealtype N_VMinQuotient_GB300(N_Vector num, N_Vector denom)
{
  return launch_reduce<MinOp>(num, LEN(num), D(num), D(denom), nullptr, nullptr, EMinQuot{});
}

// ------------------------------------------------------------ fused operations

SUNErrCode N_VLinearCombination_GB300(int nvec, sunrealtype* c, N_Vector* X, N_Vector z)
{
  if (nvec < 1) return SUN_ERR_ARG_OUTOFRANGE;
  if (nvec == 1)
  {
    N_VScale_GB300(c[0], X[0], z);
    return SUN_SUCCESS;
  }
  if (nvec == 2)
  {
    N_VLinearSum_GB300(c[0], X[0], c[1], X[1], z);
    return SUN_SUCCESS;
  }
  bool acc = (X[0] == z) && (c[0] == 1.0);
  return lincomb_core(z, nvec, c, X, z, acc) ? SUN_SUCCESS : SUN_ERR_EXT_FAIL;
}

SUNErrCode N_VScaleAddMulti_GB300(int nvec, sunrealtype* a, N_Vector x, N_Vector* Y, N_Vector* Z)
{
  if (nvec < 1) return SUN_ERR_ARG_OUTOFRANGE;
  int64_t n = LEN(x);
  if (n <= 0) return SUN_SUCCESS;
  for (int k0 = 0; k0 < nvec; k0 += kMaxList)
  {
    int m = nvec - k0 < kMaxList ? nvec - k0 : kMaxList;
    SAMArgs args;
    int vec = aligned16(D(x));
    for (int j = 0; j < m; ++j)
    {
      args.y[j] = D(Y[k0 + j]);
      args.z[j] = D(Z[k0 + j]);
      args.a[j] = a[k0 + j];
      vec       = vec && aligned16(args.y[j]) && aligned16(args.z[j]);
    }
    int64_t items = vec ? (n + 1) / 2 : n;
    int grid      = stream_grid(items);
    switch (m)
    {  // fixed vector counts keep every load in flight; longer lists loop
#define SAM_CASE(M)                                                                           \
  case M:                                                                                     \
    DISPATCH_F(x, (k_scaleaddmulti<true, M><<<grid, kBlock, 0, S(x)>>>(n, m, D(x), args, vec)), \
               (k_scaleaddmulti<false, M><<<grid, kBlock, 0, S(x)>>>(n, m, D(x), args, vec))); \
    break;
      SAM_CASE(1)
      SAM_CASE(2)
      SAM_CASE(3)
      SAM_CASE(4)
      SAM_CASE(5)
      SAM_CASE(6)
#undef SAM_CASE
    default:
      DISPATCH_F(x, (k_scaleaddmulti<true, 0><<<grid, kBlock, 0, S(x)>>>(n, m, D(x), args, vec)),
                 (k_scaleaddmulti<false, 0><<<grid, kBlock, 0, S(x)>>>(n, m, D(x), args, vec)));
    }
    count_launch();
    if (!check_cuda(cudaGetLastError(), "k_scaleaddmulti launch")) return SUN_ERR_EXT_FAIL;
  }
  return SUN_SUCCESS;
}

SUNErrCode N_VDotProdMulti_GB300(int nvec, N_Vector x, N_Vector* Y, sunrealtype* dotprods)
{
  if (nvec < 1) return SUN_ERR_ARG_OUTOFRANGE;
  return dotmulti_core(nvec, x, Y, dotprods) ? SUN_SUCCESS : SUN_ERR_EXT_FAIL;
}

SUNErrCode N_VDotProdMultiLocal_GB300(int nvec, N_Vector x, N_Vector* Y, sunrealtype* dotprods)
{
  return N_VDotProdMulti_GB300(nvec, x, Y, dotprods);
}

// One process, one GPU: the local sums are already global.
SUNErrCode N_VDotProdMultiAllReduce_GB300(int, N_Vector, sunrealtype*) { return SUN_SUCCESS; }

// ------------------------------------------------------- vector array operations

SUNErrCode N_VLinearSumVectorArray_GB300(int nvec, sunrealtype a, N_Vector* X, sunrealtype b,
                                         N_Vector* Y, N_Vector* Z)
{
  if (nvec < 1) return SUN_ERR_ARG_OUTOFRANGE;
  if (nvec == 1)
  {
    N_VLinearSum_GB300(a, X[0], b, Y[0], Z[0]);
    return SUN_SUCCESS;
  }
  int mode = linsum_mode(a, b);
  return va_map(Z[0], nvec, mode, a, b, nullptr, X, Y, Z) ? SUN_SUCCESS : SUN_ERR_EXT_FAIL;
}

SUNErrCode N_VScaleVectorArray_GB300(int nvec, sunrealtype* c, N_Vector* X, N_Vector* Z)
{
  if (nvec < 1) return SUN_ERR_ARG_OUTOFRANGE;
  if (nvec == 1)
  {
    N_VScale_GB300(c[0], X[0], Z[0]);
    return SUN_SUCCESS;
  }
  return va_map(Z[0], nvec, 3, 0.0, 0.0, c, X, nullptr, Z) ? SUN_SUCCESS : SUN_ERR_EXT_FAIL;
}

SUNErrCode N_VConstVectorArray_GB300(int nvec, sunrealtype c, N_Vector* Z)
{
  if (nvec < 1) return SUN_ERR_ARG_OUTOFRANGE;
  if (nvec == 1)
  {
    N_VConst_GB300(c, Z[0]);
    return SUN_SUCCESS;
  }
  return va_map(Z[0], nvec, 4, c, 0.0, nullptr, nullptr, nullptr, Z) ? SUN_SUCCESS
                                                                    : SUN_ERR_EXT_FAIL;
}

SUNErrCode N_VWrmsNormVectorArray_GB300(int nvec, N_Vector* X, N_Vector* W, sunrealtype* nrm)
{
  if (nvec < 1) return SUN_ERR_ARG_OUTOFRANGE;
  if (nvec == 1)
  {
    nrm[0] = N_VWrmsNorm_GB300(X[0], W[0]);
    return SUN_SUCCESS;
  }
  if (!va_wsqr(nvec, X, W, nullptr, nrm)) return SUN_ERR_EXT_FAIL;
  double n = (double)C(X[0])->length;
  for (int k = 0; k < nvec; ++k) nrm[k] = sqrt(nrm[k] / n);
  return SUN_SUCCESS;
}

SUNErrCode N_VWrmsNormMaskVectorArray_GB300(int nvec, N_Vector* X, N_Vector* W, N_Vector id,
                                            sunrealtype* nrm)
{
  if (nvec < 1) return SUN_ERR_ARG_OUTOFRANGE;
  if (nvec == 1)
  {
    nrm[0] = N_VWrmsNormMask_GB300(X[0], W[0], id);
    return SUN_SUCCESS;
  }
  if (!va_wsqr(nvec, X, W, id, nrm)) return SUN_ERR_EXT_FAIL;
  double n = (double)C(X[0])->length;
  for (int k = 0; k < nvec; ++k) nrm[k] = sqrt(nrm[k] / n);
  return SUN_SUCCESS;
}

SUNErrCode N_VScaleAddMultiVectorArray_GB300(int nvec, int nsum, sunrealtype* a, N_Vector* X,
                                             N_Vector** Y, N_Vector** Z)
{
  if (nvec < 1 || nsum < 1) return SUN_ERR_ARG_OUTOFRANGE;
  int64_t n = LEN(X[0]);
  if (n <= 0) return SUN_SUCCESS;
  if (nsum > 8)
  {  // wide sums: one fused ScaleAddMulti per row
    N_Vector* YY = (N_Vector*)malloc(sizeof(N_Vector) * nsum);
    N_Vector* ZZ = (N_Vector*)malloc(sizeof(N_Vector) * nsum);
    SUNErrCode err = SUN_SUCCESS;
    for (int i = 0; i < nvec && err == SUN_SUCCESS; ++i)
    {
      for (int j = 0; j < nsum; ++j)
      {
        YY[j] = Y[j][i];
        ZZ[j] = Z[j][i];
      }
      err = N_VScaleAddMulti_GB300(nsum, a, X[i], YY, ZZ);
    }
    free(YY);
    free(ZZ);
    return err;
  }
  int rows_per = 64 / nsum;
  if (rows_per > 8) rows_per = 8;
  for (int r0 = 0; r0 < nvec; r0 += rows_per)
  {
    int m = nvec - r0 < rows_per ? nvec - r0 : rows_per;
    SAMVAArgs args;
    int vec = 1;
    for (int j = 0; j < nsum; ++j) args.a[j] = a[j];
    for (int i = 0; i < m; ++i)
    {
      args.x[i] = D(X[r0 + i]);
      vec       = vec && aligned16(args.x[i]);
      for (int j = 0; j < nsum; ++j)
      {
        args.y[i * nsum + j] = D(Y[j][r0 + i]);
        args.z[i * nsum + j] = D(Z[j][r0 + i]);
        vec = vec && aligned16(args.y[i * nsum + j]) && aligned16(args.z[i * nsum + j]);
      }
    }
    int64_t items = vec ? (n + 1) / 2 : n;
    int gx        = (stream_grid(items) + m - 1) / m;
    dim3 grid(gx < 1 ? 1 : gx, m);
    DISPATCH_F(X[0], (k_va_scaleaddmulti<true><<<grid, kBlock, 0, S(X[0])>>>(n, nsum, args, vec)),
               (k_va_scaleaddmulti<false><<<grid, kBlock, 0, S(X[0])>>>(n, nsum, args, vec)));
    count_launch();
    if (!check_cuda(cudaGetLastError(), "k_va_scaleaddmulti launch")) return SUN_ERR_EXT_FAIL;
  }
  return SUN_SUCCESS;
}

SUNErrCode N_VLinearCombinationVectorArray_GB300(int nvec, int nsum, sunrealtype* c,
                                                 N_Vector** X, N_Vector* Z)
{
  if (nvec < 1 || nsum < 1) return SUN_ERR_ARG_OUTOFRANGE;
  if (nvec == 1)
  {
    if (nsum == 1)
    {
      N_VScale_GB300(c[0], X[0][0], Z[0]);
      return SUN_SUCCESS;
    }
    if (nsum == 2)
    {
      N_VLinearSum_GB300(c[0], X[0][0], c[1], X[1][0], Z[0]);
      return SUN_SUCCESS;
    }
    N_Vector* Yv = (N_Vector*)malloc(sizeof(N_Vector) * nsum);
    for (int i = 0; i < nsum; ++i) Yv[i] = X[i][0];
    SUNErrCode err = N_VLinearCombination_GB300(nsum, c, Yv, Z[0]);
    free(Yv);
    return err;
  }
  if (nsum == 1)
  {
    double* ct = (double*)malloc(sizeof(double) * nvec);
    for (int j = 0; j < nvec; ++j) ct[j] = c[0];
    SUNErrCode err = N_VScaleVectorArray_GB300(nvec, ct, X[0], Z);
    free(ct);
    return err;
  }
  if (nsum == 2) return N_VLinearSumVectorArray_GB300(nvec, c[0], X[0], c[1], X[1], Z);

  int64_t n = LEN(Z[0]);
  if (n <= 0) return SUN_SUCCESS;
  bool accumulate = (X[0] == Z) && (c[0] == 1.0);
  if (nsum > 8)
  {  // wide sums: one fused LinearCombination per row, same term order
    N_Vector* Yv = (N_Vector*)malloc(sizeof(N_Vector) * nsum);
    bool ok      = true;
    for (int j = 0; j < nvec && ok; ++j)
    {
      for (int i = 0; i < nsum; ++i) Yv[i] = X[i][j];
      ok = lincomb_core(Z[j], nsum, c, Yv, Z[j], accumulate);
    }
    free(Yv);
    return ok ? SUN_SUCCESS : SUN_ERR_EXT_FAIL;
  }
  int rows_per = 64 / nsum;
  if (rows_per > 8) rows_per = 8;
  for (int r0 = 0; r0 < nvec; r0 += rows_per)
  {
    int m = nvec - r0 < rows_per ? nvec - r0 : rows_per;
    LCVAArgs args;
    int vec = 1;
    for (int i = 0; i < nsum; ++i) args.c[i] = c[i];
    for (int j = 0; j < m; ++j)
    {
      args.z[j] = D(Z[r0 + j]);
      vec       = vec && aligned16(args.z[j]);
      for (int i = 0; i < nsum; ++i)
      {
        args.x[j * nsum + i] = D(X[i][r0 + j]);
        vec                  = vec && aligned16(args.x[j * nsum + i]);
      }
    }
    int64_t items = vec ? (n + 1) / 2 : n;
    int gx        = (stream_grid(items) + m - 1) / m;
    dim3 grid(gx < 1 ? 1 : gx, m);
    DISPATCH_F(Z[0],
               (k_va_lincomb<true><<<grid, kBlock, 0, S(Z[0])>>>(n, nsum, args, accumulate, vec)),
               (k_va_lincomb<false><<<grid, kBlock, 0, S(Z[0])>>>(n, nsum, args, accumulate, vec)));
    count_launch();
    if (!check_cuda(cudaGetLastError(), "k_va_lincomb launch")) return SUN_ERR_EXT_FAIL;
  }
  return SUN_SUCCESS;
}

// ------------------------------------------------------------ buffers, printing

SUNErrCode N_VBufSize_GB300(N_Vector x, sunindextype* size)
{
  *size = C(x)->length * (sunindextype)sizeof(double);
  return SUN_SUCCESS;
}

SUNErrCode N_VBufPack_GB300(N_Vector x, void* buf)
{
  if (!buf) return SUN_ERR_ARG_CORRUPT;
  if (LEN(x) <= 0) return SUN_SUCCESS;
  if (!check_cuda(cudaMemcpyAsync(buf, D(x), sizeof(double) * (size_t)LEN(x), cudaMemcpyDefault,
                                  S(x)),
                  "N_VBufPack"))
    return SUN_ERR_EXT_FAIL;
  return sync_stream(x) ? SUN_SUCCESS : SUN_ERR_EXT_FAIL;
}

SUNErrCode N_VBufUnpack_GB300(N_Vector x, void* buf)
{
  if (!buf) return SUN_ERR_ARG_CORRUPT;
  if (LEN(x) <= 0) return SUN_SUCCESS;
  if (!check_cuda(cudaMemcpyAsync(D(x), buf, sizeof(double) * (size_t)LEN(x), cudaMemcpyDefault,
                                  S(x)),
                  "N_VBufUnpack"))
    return SUN_ERR_EXT_FAIL;
  return sync_stream(x) ? SUN_SUCCESS : SUN_ERR_EXT_FAIL;
}

void N_VPrintFile_GB300(N_Vector x, FILE* outfile)
{
  N_VCopyFromDevice_GB300(x);
  const double* h = C(x)->host;
  for (int64_t i = 0; i < LEN(x); ++i) fprintf(outfile, "% .15e\n", h[i]);
}

void N_VPrint_GB300(N_Vector x) { N_VPrintFile_GB300(x, stdout); }

// ------------------------------------------------------------ enable / disable

#define ENABLE_FN(NAME, FIELD, FN)                                   \
  SUNErrCode NAME(N_Vector v, sunbooleantype tf)                     \
  {                                                                  \
    if (!v || !v->ops) return SUN_ERR_ARG_CORRUPT;                   \
    v->ops->FIELD = tf ? FN : nullptr;                               \
    return SUN_SUCCESS;                                              \
  }

ENABLE_FN(N_VEnableLinearCombination_GB300, nvlinearcombination, N_VLinearCombination_GB300)
ENABLE_FN(N_VEnableScaleAddMulti_GB300, nvscaleaddmulti, N_VScaleAddMulti_GB300)
ENABLE_FN(N_VEnableDotProdMulti_GB300, nvdotprodmulti, N_VDotProdMulti_GB300)
ENABLE_FN(N_VEnableLinearSumVectorArray_GB300, nvlinearsumvectorarray,
          N_VLinearSumVectorArray_GB300)
ENABLE_FN(N_VEnableScaleVectorArray_GB300, nvscalevectorarray, N_VScaleVectorArray_GB300)
ENABLE_FN(N_VEnableConstVectorArray_GB300, nvconstvectorarray, N_VConstVectorArray_GB300)
ENABLE_FN(N_VEnableWrmsNormVectorArray_GB300, nvwrmsnormvectorarray,
          N_VWrmsNormVectorArray_GB300)
ENABLE_FN(N_VEnableWrmsNormMaskVectorArray_GB300, nvwrmsnormmaskvectorarray,
          N_VWrmsNormMaskVectorArray_GB300)
ENABLE_FN(N_VEnableScaleAddMultiVectorArray_GB300, nvscaleaddmultivectorarray,
          N_VScaleAddMultiVectorArray_GB300)
ENABLE_FN(N_VEnableLinearCombinationVectorArray_GB300, nvlinearcombinationvectorarray,
          N_VLinearCombinationVectorArray_GB300)
ENABLE_FN(N_VEnableDotProdMultiLocal_GB300, nvdotprodmultilocal, N_VDotProdMultiLocal_GB300)

SUNErrCode N_VEnableFusedOps_GB300(N_Vector v, sunbooleantype tf)
{
  if (!v || !v->ops) return SUN_ERR_ARG_CORRUPT;
  N_VEnableLinearCombination_GB300(v, tf);
  N_VEnableScaleAddMulti_GB300(v, tf);
  N_VEnableDotProdMulti_GB300(v, tf);
  N_VEnableLinearSumVectorArray_GB300(v, tf);
  N_VEnableScaleVectorArray_GB300(v, tf);
  N_VEnableConstVectorArray_GB300(v, tf);
  N_VEnableWrmsNormVectorArray_GB300(v, tf);
  N_VEnableWrmsNormMaskVectorArray_GB300(v, tf);
  N_VEnableScaleAddMultiVectorArray_GB300(v, tf);
  N_VEnableLinearCombinationVectorArray_GB300(v, tf);
  N_VEnableDotProdMultiLocal_GB300(v, tf);
  return SUN_SUCCESS;
}

SUNErrCode N_VSetFMA_GB300(N_Vector v, sunbooleantype use_fma)
{
  if (!v || !v->content) return SUN_ERR_ARG_CORRUPT;
  C(v)->fma = use_fma ? true : false;
  return SUN_SUCCESS;
}

sunbooleantype N_VGetFMA_GB300(N_Vector v)
{
  if (!v || !v->content || !v->ops || v->ops->nvlinearsum != N_VLinearSum_GB300) return SUNTRUE;
  return C(v)->fma ? SUNTRUE : SUNFALSE;
}

}  // extern "C"

// ------------------------------------------------------------ the ops table

namespace {
void fill_ops(N_Vector_Ops ops)
{
  ops->nvgetvectorid           = N_VGetVectorID_GB300;
  ops->nvclone                 = N_VClone_GB300;
  ops->nvcloneempty            = N_VCloneEmpty_GB300;
  ops->nvdestroy               = N_VDestroy_GB300;
  ops->nvspace                 = N_VSpace_GB300;
  ops->nvgetarraypointer       = N_VGetArrayPointer_GB300;
  ops->nvgetdevicearraypointer = N_VGetDeviceArrayPointer_GB300;
  ops->nvsetarraypointer       = N_VSetArrayPointer_GB300;
  ops->nvgetcommunicator       = N_VGetCommunicator_GB300;
  ops->nvgetlength             = N_VGetLength_GB300;
  ops->nvgetlocallength        = N_VGetLength_GB300;

  ops->nvlinearsum    = N_VLinearSum_GB300;
  ops->nvconst        = N_VConst_GB300;
  ops->nvprod         = N_VProd_GB300;
  ops->nvdiv          = N_VDiv_GB300;
  ops->nvscale        = N_VScale_GB300;
  ops->nvabs          = N_VAbs_GB300;
  ops->nvinv          = N_VInv_GB300;
  ops->nvaddconst     = N_VAddConst_GB300;
  ops->nvdotprod      = N_VDotProd_GB300;
  ops->nvmaxnorm      = N_VMaxNorm_GB300;
  ops->nvwrmsnorm     = N_VWrmsNorm_GB300;
  ops->nvwrmsnormmask = N_VWrmsNormMask_GB300;
  ops->nvmin          = N_VMin_GB300;
  ops->nvwl2norm      = N_VWL2Norm_GB300;
  ops->nvl1norm       = N_VL1Norm_GB300;
  ops->nvcompare      = N_VCompare_GB300;
  ops->nvinvtest      = N_VInvTest_GB300;
  ops->nvconstrmask   = N_VConstrMask_GB300;
  ops->nvminquotient  = N_VMinQuotient_GB300;

  ops->nvlinearcombination = N_VLinearCombination_GB300;
  ops->nvscaleaddmulti     = N_VScaleAddMulti_GB300;
  ops->nvdotprodmulti      = N_VDotProdMulti_GB300;

  ops->nvlinearsumvectorarray         = N_VLinearSumVectorArray_GB300;
  ops->nvscalevectorarray             = N_VScaleVectorArray_GB300;
  ops->nvconstvectorarray             = N_VConstVectorArray_GB300;
  ops->nvwrmsnormvectorarray          = N_VWrmsNormVectorArray_GB300;
  ops->nvwrmsnormmaskvectorarray      = N_VWrmsNormMaskVectorArray_GB300;
  ops->nvscaleaddmultivectorarray     = N_VScaleAddMultiVectorArray_GB300;
  ops->nvlinearcombinationvectorarray = N_VLinearCombinationVectorArray_GB300;

  ops->nvdotprodlocal     = N_VDotProd_GB300;
  ops->nvmaxnormlocal     = N_VMaxNorm_GB300;
  ops->nvminlocal         = N_VMin_GB300;
  ops->nvl1normlocal      = N_VL1Norm_GB300;
  ops->nvinvtestlocal     = N_VInvTest_GB300;
  ops->nvconstrmasklocal  = N_VConstrMask_GB300;
  ops->nvminquotientlocal = N_VMinQuotient_GB300;
  ops->nvwsqrsumlocal     = N_VWSqrSumLocal_GB300;
  ops->nvwsqrsummasklocal = N_VWSqrSumMaskLocal_GB300;

  ops->nvdotprodmultilocal     = N_VDotProdMultiLocal_GB300;
  ops->nvdotprodmultiallreduce = N_VDotProdMultiAllReduce_GB300;

  ops->nvbufsize   = N_VBufSize_GB300;
  ops->nvbufpack   = N_VBufPack_GB300;
  ops->nvbufunpack = N_VBufUnpack_GB300;

  ops->nvprint     = N_VPrint_GB300;
  ops->nvprintfile = N_VPrintFile_GB300;
}
}  // namespace

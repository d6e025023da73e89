// cvode_fused_gb300.cu -- CVODE's fused integrator kernels
// (include/cvode_fused_gb300.h) over NVECTOR_GB300: each is one grid-stride
// pass that does the work of the reference's N_Vector sequence
// (src/cvode/cvode_fused_stubs.c:30-160).  The EXACT variant rounds every
// product, quotient and sum separately in the stub's order (the serial
// vector's bits); the FMA variant contracts like an nvcc build of
// src/cvode/cvode_fused_gpu.cpp.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/cvode_fused_gb300.h"
#include "../../include/nvector_gb300.h"
#include "gb300_common.cuh"

using namespace gb300;

namespace {

template <bool F>
__device__ __forceinline__ double axpy(double a, double x, double y)  // a*x + y
{
  return F ? fma(a, x, y) : __dadd_rn(__dmul_rn(a, x), y);
}

// Reduction scratch for the atolmin0 test (min of tempv), shared by all calls.
struct MinScratch
{
  double* partials = nullptr;
  unsigned int* counter = nullptr;
  double* h_result = nullptr;
  double* d_result = nullptr;
};
std::mutex g_min_mutex;
MinScratch g_min;

bool min_scratch(MinScratch& m)
{
  std::lock_guard<std::mutex> lock(g_min_mutex);
  if (g_min.partials)
  {
    m = g_min;
    return true;
  }
  if (!check_cuda(cudaMalloc(&g_min.partials, sizeof(double) * kMaxRedBlocks), "fused cudaMalloc") ||
      !check_cuda(cudaMalloc(&g_min.counter, sizeof(unsigned int)), "fused cudaMalloc") ||
      !check_cuda(cudaMemset(g_min.counter, 0, sizeof(unsigned int)), "fused cudaMemset") ||
      !check_cuda(cudaHostAlloc(&g_min.h_result, sizeof(double), cudaHostAllocMapped),
                  "fused cudaHostAlloc") ||
      !check_cuda(cudaHostGetDevicePointer(&g_min.d_result, g_min.h_result, 0), "fused mapped"))
    return false;
  m = g_min;
  return true;
}

// tempv = reltol |y| + abstol (scalar abstol when vabs == nullptr),
// weight = 1 / tempv; with a min-reduction of tempv when partials != nullptr.
template <bool F>
__global__ void __launch_bounds__(kBlock)
  k_ewt(int64_t n, double reltol, double sabs, const double* __restrict__ vabs,
        const double* __restrict__ y, double* __restrict__ tempv, double* __restrict__ weight,
        double* partials, unsigned int* counter, double* result)
{
  __shared__ double scratch[kWarps];
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st  = (int64_t)gridDim.x * blockDim.x;
  double v[1]       = {MinOp::identity()};
  for (int64_t i = tid; i < n; i += st)
  {
    const double a = fabs(y[i]);
    double t;
    if (vabs) t = axpy<F>(reltol, a, vabs[i]);          // VLin1(reltol, |y|, Vabstol)
    else t = F ? fma(reltol, a, sabs) : __dadd_rn(__dmul_rn(a, reltol), sabs);  // VScaleBy, AddConst
    tempv[i]  = t;
    weight[i] = __ddiv_rn(1.0, t);                       // N_VInv
    v[0]      = MinOp::combine(v[0], t);
  }
  if (!partials) return;
  block_reduce<MinOp, 1>(v, scratch);
  if (gridDim.x == 1)
  {
    if (threadIdx.x == 0) *result = v[0];
    return;
  }
  if (grid_finish<MinOp, 1>(v, partials, counter, gridDim.x, blockIdx.x, scratch)) *result = v[0];
}

// tmp = mm * (y - 0.1 * (a c) / ewt), a = (|c| >= 1.5)
template <bool F>
__global__ void __launch_bounds__(kBlock)
  k_constraints(int64_t n, const double* __restrict__ c, const double* __restrict__ ewt,
                const double* __restrict__ y, const double* __restrict__ mm,
                double* __restrict__ tmp)
{
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st  = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = tid; i < n; i += st)
  {
    const double a = fabs(c[i]) >= 1.5 ? 1.0 : 0.0;     // N_VCompare(1.5, c)
    double t       = __dmul_rn(a, c[i]);                // N_VProd
    t              = __ddiv_rn(t, ewt[i]);              // N_VDiv
    t              = axpy<F>(-0.1, t, y[i]);            // LinearSum(1, y, -0.1, t)
    tmp[i]         = __dmul_rn(t, mm[i]);               // N_VProd
  }
}

// res = (rl1 zn1 + ycor) + ngamma ftemp
template <bool F>
__global__ void __launch_bounds__(kBlock)
  k_nls_resid(int64_t n, double rl1, double ngamma, const double* __restrict__ zn1,
              const double* __restrict__ ycor, const double* __restrict__ ftemp,
              double* __restrict__ res)
{
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st  = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = tid; i < n; i += st)
  {
    const double r = axpy<F>(rl1, zn1[i], ycor[i]);
    // N_VLinearSum(ngamma, ftemp, 1, res, res) = Vaxpy (exact for ngamma = +-1)
    double out;
    if (!F && ngamma == 1.0) out = __dadd_rn(r, ftemp[i]);
    else if (!F && ngamma == -1.0) out = __dsub_rn(r, ftemp[i]);
    else out = axpy<F>(ngamma, ftemp[i], r);
    res[i] = out;
  }
}

// ftemp = h fpred - zn1; y = r ftemp + ypred
template <bool F>
__global__ void __launch_bounds__(kBlock)
  k_diag_formy(int64_t n, double h, double r, const double* __restrict__ fpred,
               const double* __restrict__ zn1, const double* __restrict__ ypred,
               double* __restrict__ ftemp, double* __restrict__ y)
{
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st  = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = tid; i < n; i += st)
  {
    const double ft = F ? fma(h, fpred[i], -zn1[i]) : __dsub_rn(__dmul_rn(h, fpred[i]), zn1[i]);
    ftemp[i]        = ft;
    y[i]            = axpy<F>(r, ft, ypred[i]);
  }
}

// M = I - gamma J with J = diag(deltaf/deltay), protected at roundoff level
template <bool F>
__global__ void __launch_bounds__(kBlock)
  k_diag_buildm(int64_t n, double fract, double uround, double h, const double* __restrict__ ftemp,
                const double* __restrict__ fpred, const double* __restrict__ ewt,
                double* __restrict__ bit, double* __restrict__ bitcomp, double* __restrict__ y,
                double* __restrict__ M)
{
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st  = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = tid; i < n; i += st)
  {
    const double ft = ftemp[i];
    double m        = __dsub_rn(M[i], fpred[i]);           // LinearSum(1, M, -1, fpred)
    // LinearSum(fract, ftemp, -h, M): a x + b y, or a (x - y) when a == -b
    if (F) m = fma(-h, m, fract * ft);
    else if (fract == h) m = __dmul_rn(fract, __dsub_rn(ft, m));
    else m = __dadd_rn(__dmul_rn(fract, ft), __dmul_rn(-h, m));
    double yy       = __dmul_rn(ft, ewt[i]);                // N_VProd(ftemp, ewt)
    const double b  = fabs(yy) >= uround ? 1.0 : 0.0;       // N_VCompare(uround, y)
    const double bc = __dadd_rn(b, -1.0);                   // N_VAddConst(bit, -1)
    yy              = __dmul_rn(ft, b);                     // N_VProd(ftemp, bit)
    yy = F ? fma(fract, yy, -bc) : __dsub_rn(__dmul_rn(fract, yy), bc);  // VLin2(fract, y, bitcomp)
    m               = __ddiv_rn(m, yy);                     // N_VDiv(M, y)
    m               = __dmul_rn(m, b);                      // N_VProd(M, bit)
    m               = __dsub_rn(m, bc);                     // LinearSum(1, M, -1, bitcomp)
    bit[i]          = b;
    bitcomp[i]      = bc;
    y[i]            = yy;
    M[i]            = m;
  }
}

// M = r (1/M - 1) + 1
template <bool F>
__global__ void __launch_bounds__(kBlock) k_diag_updatem(int64_t n, double r, double* __restrict__ M)
{
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t st  = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = tid; i < n; i += st)
  {
    const double a = __dadd_rn(__ddiv_rn(1.0, M[i]), -1.0);
    M[i]           = F ? fma(r, a, 1.0) : __dadd_rn(__dmul_rn(a, r), 1.0);
  }
}

inline bool gb(N_Vector v) { return v && v->ops && v->ops->nvlinearsum == N_VLinearSum_GB300; }
inline double* D(N_Vector v) { return N_VGetDeviceArrayPointer_GB300(v); }
inline cudaStream_t S(N_Vector v) { return (cudaStream_t)N_VGetStream_GB300(v); }
inline bool FMA(N_Vector v) { return N_VGetFMA_GB300(v) == SUNTRUE; }

bool same(N_Vector ref, std::initializer_list<N_Vector> vs)
{
  if (!gb(ref)) return false;
  const sunindextype n = N_VGetLength_GB300(ref);
  for (N_Vector v : vs)
    if (!gb(v) || N_VGetLength_GB300(v) != n) return false;
  return true;
}

int finish(const char* what)
{
  count_launch();
  return check_cuda(cudaGetLastError(), what) ? 0 : -1;
}

int ewt(bool atolmin0, double reltol, double sabs, N_Vector vabs, N_Vector ycur, N_Vector tempv,
        N_Vector weight)
{
  const int64_t n = N_VGetLength_GB300(weight);
  if (n <= 0) return 0;
  MinScratch m;
  if (atolmin0 && !min_scratch(m)) return -1;
  const int grid = atolmin0 ? reduce_grid(n) : stream_grid(n);
  const double* va = vabs ? D(vabs) : nullptr;
  if (FMA(weight))
    k_ewt<true><<<grid, kBlock, 0, S(weight)>>>(n, reltol, sabs, va, D(ycur), D(tempv), D(weight),
                                                atolmin0 ? m.partials : nullptr, m.counter,
                                                m.d_result);
  else
    k_ewt<false><<<grid, kBlock, 0, S(weight)>>>(n, reltol, sabs, va, D(ycur), D(tempv), D(weight),
                                                 atolmin0 ? m.partials : nullptr, m.counter,
                                                 m.d_result);
  if (finish("cvEwtSet_fused launch") != 0) return -1;
  if (!atolmin0) return 0;
  if (!check_cuda(cudaStreamSynchronize(S(weight)), "cvEwtSet_fused")) return -1;
  return (*m.h_result <= 0.0) ? -1 : 0;
}

}  // namespace

extern "C" {

int cvEwtSetSS_fused(const sunbooleantype atolmin0, const sunrealtype reltol,
                     const sunrealtype Sabstol, const N_Vector ycur, N_Vector tempv,
                     N_Vector weight)
{
  if (!same(weight, {ycur, tempv})) return -1;
  return ewt(atolmin0, reltol, Sabstol, nullptr, ycur, tempv, weight);
}

int cvEwtSetSV_fused(const sunbooleantype atolmin0, const sunrealtype reltol,
                     const N_Vector Vabstol, const N_Vector ycur, N_Vector tempv, N_Vector weight)
{
  if (!same(weight, {Vabstol, ycur, tempv})) return -1;
  return ewt(atolmin0, reltol, 0.0, Vabstol, ycur, tempv, weight);
}

int cvCheckConstraints_fused(const N_Vector c, const N_Vector ewt_, const N_Vector y,
                             const N_Vector mm, N_Vector tempv)
{
  if (!same(tempv, {c, ewt_, y, mm})) return -1;
  const int64_t n = N_VGetLength_GB300(tempv);
  if (n <= 0) return 0;
  if (FMA(tempv))
    k_constraints<true><<<stream_grid(n), kBlock, 0, S(tempv)>>>(n, D(c), D(ewt_), D(y), D(mm),
                                                                 D(tempv));
  else
    k_constraints<false><<<stream_grid(n), kBlock, 0, S(tempv)>>>(n, D(c), D(ewt_), D(y), D(mm),
                                                                  D(tempv));
  return finish("cvCheckConstraints_fused launch");
}

int cvNlsResid_fused(const sunrealtype rl1, const sunrealtype ngamma, const N_Vector zn1,
                     const N_Vector ycor, const N_Vector ftemp, N_Vector res)
{
  if (!same(res, {zn1, ycor, ftemp})) return -1;
  const int64_t n = N_VGetLength_GB300(res);
  if (n <= 0) return 0;
  if (FMA(res))
    k_nls_resid<true><<<stream_grid(n), kBlock, 0, S(res)>>>(n, rl1, ngamma, D(zn1), D(ycor),
                                                             D(ftemp), D(res));
  else
    k_nls_resid<false><<<stream_grid(n), kBlock, 0, S(res)>>>(n, rl1, ngamma, D(zn1), D(ycor),
                                                              D(ftemp), D(res));
  return finish("cvNlsResid_fused launch");
}

int cvDiagSetup_formY(const sunrealtype h, const sunrealtype r, const N_Vector fpred,
                      const N_Vector zn1, const N_Vector ypred, N_Vector ftemp, N_Vector y)
{
  if (!same(y, {fpred, zn1, ypred, ftemp})) return -1;
  const int64_t n = N_VGetLength_GB300(y);
  if (n <= 0) return 0;
  if (FMA(y))
    k_diag_formy<true><<<stream_grid(n), kBlock, 0, S(y)>>>(n, h, r, D(fpred), D(zn1), D(ypred),
                                                            D(ftemp), D(y));
  else
    k_diag_formy<false><<<stream_grid(n), kBlock, 0, S(y)>>>(n, h, r, D(fpred), D(zn1), D(ypred),
                                                             D(ftemp), D(y));
  return finish("cvDiagSetup_formY launch");
}

int cvDiagSetup_buildM(const sunrealtype fract, const sunrealtype uround, const sunrealtype h,
                       const N_Vector ftemp, const N_Vector fpred, const N_Vector ewt_,
                       N_Vector bit, N_Vector bitcomp, N_Vector y, N_Vector M)
{
  if (!same(M, {ftemp, fpred, ewt_, bit, bitcomp, y})) return -1;
  const int64_t n = N_VGetLength_GB300(M);
  if (n <= 0) return 0;
  if (FMA(M))
    k_diag_buildm<true><<<stream_grid(n), kBlock, 0, S(M)>>>(n, fract, uround, h, D(ftemp),
                                                             D(fpred), D(ewt_), D(bit),
                                                             D(bitcomp), D(y), D(M));
  else
    k_diag_buildm<false><<<stream_grid(n), kBlock, 0, S(M)>>>(n, fract, uround, h, D(ftemp),
                                                              D(fpred), D(ewt_), D(bit),
                                                              D(bitcomp), D(y), D(M));
  return finish("cvDiagSetup_buildM launch");
}

int cvDiagSolve_updateM(const sunrealtype r, N_Vector M)
{
  if (!gb(M)) return -1;
  const int64_t n = N_VGetLength_GB300(M);
  if (n <= 0) return 0;
  if (FMA(M)) k_diag_updatem<true><<<stream_grid(n), kBlock, 0, S(M)>>>(n, r, D(M));
  else k_diag_updatem<false><<<stream_grid(n), kBlock, 0, S(M)>>>(n, r, D(M));
  return finish("cvDiagSolve_updateM launch");
}

}  // extern "C"

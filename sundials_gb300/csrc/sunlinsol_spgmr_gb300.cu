// sunlinsol_spgmr_gb300.cu -- SPGMR (restarted GMRES) over NVECTOR_GB300 with
// fused Gram-Schmidt kernels.
//
// The solver follows SUNLinSolSolve_SPGMR (src/sunlinsol/spgmr/
// sunlinsol_spgmr.c:461-932) step for step: the same initial residual,
// left/right preconditioning and s1/s2 scaling, the same restart loop, Givens
// QR of the Hessenberg matrix on the host (sundials_iterative.c:181-329,
// restated below), the same convergence test and return codes.  What is
// GB300-specific is the Arnoldi step's vector work:
//
//  * classical GS (sundials_iterative.c:116-170): the reference makes
//    N_VDotProdMulti, N_VLinearCombination and N_VDotProd calls (three passes
//    over the new vector, two host synchronisations).  Here pass 1 computes
//    <V_j, w> for every basis vector and <w, w> in ONE read of the basis and
//    w; pass 2 applies w -= sum_j h_j V_j and accumulates the new ||w||^2 in
//    the same loop.  The Hessenberg column is read from pinned host memory
//    after one synchronisation;
//  * modified GS (sundials_iterative.c:45-105): the reference makes a DotProd
//    (host sync) and a LinearSum per basis vector.  Here kernel i applies the
//    projection on V_{i-1} and computes <V_i, w> in one pass; the coefficient
//    h_{i-1} reaches kernel i in device memory (written by the last block of
//    kernel i-1), so the k+1 kernels run back to back with no host round trip;
//  * the reorthogonalisation tests are evaluated on the host after that one
//    synchronisation; when one fires (rare), the second pass runs as in the
//    reference, with its own synchronisations;
//  * the normalisation V_{l+1} *= 1/h_{l+1,l} (sunlinsol_spgmr.c:758) is
//    deferred into the next step's first pass over V_{l+1} (fused with the
//    division by s2, when scaling is on), and copies between the basis and the
//    work vector become exchanges of vector handles.
//
// Every reduction is a fixed-order tree (per-thread sequential, warp
// butterfly, block, last-block ticket), so a solve is bitwise reproducible.
// Host arithmetic (QR, norms, tests) is compiled without floating-point
// contraction, as the reference's is on a baseline x86-64 build.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <utility>

#include "../../include/nvector_gb300.h"
#include "../../include/sunlinsol_spgmr_gb300.h"
#include "gb300_common.cuh"

using namespace gb300;

namespace {

constexpr int kGSMax      = 8;       // vectors per fused launch
constexpr double kFactor  = 1000.0;  // reorthogonalisation factor (sundials_iterative.c:31)

// Up to kGSMax vectors of one launch and, per vector, its slot in the
// Hessenberg-column buffer (coefficient to apply, or result to write).
struct GSList
{
  const double* p[kGSMax];
  int idx[kGSMax];
};

template <bool F>
__device__ __forceinline__ double d_madd(double a, double b, double c)
{
  if (F) return fma(a, b, c);
  return __dadd_rn(__dmul_rn(a, b), c);
}

// w - h v, rounded as the reference's z += (-h) * x.
template <bool F>
__device__ __forceinline__ double d_sub(double w, double h, double v)
{
  if (F) return fma(-h, v, w);
  return __dadd_rn(w, __dmul_rn(-h, v));
}

// One fused Gram-Schmidt pass over the new basis vector w:
//   w -= sum_{k<NU} coef[U.idx[k]] * U.p[k]      (in order k = 0, 1, ...)
//   coef[D.idx[k]] = <D.p[k], w_new>  for k < ND (D.p[k] == w when bit k of
//                                                self_mask is set)
// The ND results go to coef (device, read by later launches) and to out_host
// (pinned, read by the host after the step's synchronisation).
template <bool F, int NU, int ND>
__global__ void __launch_bounds__(kBlock)
  k_gs(int64_t n, double* __restrict__ w, GSList U, GSList D, unsigned self_mask, int vec,
       double* coef, double* partials, unsigned int* counter, double* out_host)
{
  constexpr int NA = ND > 0 ? ND : 1;
  __shared__ double scratch[kWarps * NA];
  double c[NU > 0 ? NU : 1];
#pragma unroll
  for (int k = 0; k < NU; ++k) c[k] = __ldcg(coef + U.idx[k]);
  double acc[NA];
#pragma unroll
  for (int k = 0; k < NA; ++k) acc[k] = 0.0;

  const int64_t tid    = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t head         = 0;
  if (vec)
  {
    const int64_t npair = n >> 1;
    for (int64_t p = tid; p < npair; p += stride)
    {
      double2 wv = ((const double2*)w)[p];
#pragma unroll
      for (int k = 0; k < NU; ++k)
      {
        const double2 u = ((const double2*)U.p[k])[p];
        wv.x            = d_sub<F>(wv.x, c[k], u.x);
        wv.y            = d_sub<F>(wv.y, c[k], u.y);
      }
      if (NU > 0) ((double2*)w)[p] = wv;
#pragma unroll
      for (int k = 0; k < ND; ++k)
      {
        const double2 y = ((self_mask >> k) & 1u) ? wv : ((const double2*)D.p[k])[p];
        acc[k]          = d_madd<F>(wv.x, y.x, acc[k]);
        acc[k]          = d_madd<F>(wv.y, y.y, acc[k]);
      }
    }
    head = npair << 1;
  }
  for (int64_t i = head + tid; i < n; i += stride)
  {
    double wv = w[i];
#pragma unroll
    for (int k = 0; k < NU; ++k) wv = d_sub<F>(wv, c[k], U.p[k][i]);
    if (NU > 0) w[i] = wv;
#pragma unroll
    for (int k = 0; k < ND; ++k)
    {
      const double y = ((self_mask >> k) & 1u) ? wv : D.p[k][i];
      acc[k]         = d_madd<F>(wv, y, acc[k]);
    }
  }
  if (ND == 0) return;
  block_reduce<SumOp, NA>(acc, scratch);
  bool writer = false;
  if (gridDim.x == 1)
    writer = threadIdx.x == 0;
  else
    writer = grid_finish<SumOp, NA>(acc, partials, counter, gridDim.x, blockIdx.x, scratch);
  if (writer)
  {
#pragma unroll
    for (int k = 0; k < ND; ++k)
    {
      coef[D.idx[k]]     = acc[k];
      out_host[D.idx[k]] = acc[k];
    }
  }
}

// v *= c; then, if t: t = s2 ? v / s2 : v.  (N_VScale(c, v, v) followed by
// the next Arnoldi step's N_VDiv(v, s2, vtemp), sunlinsol_spgmr.c:640-647.)
__global__ void __launch_bounds__(kBlock)
  k_gs_normalize(int64_t n, double c, double* __restrict__ v, double* __restrict__ t,
                 const double* __restrict__ s2, int vec)
{
  const int64_t tid    = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t head         = 0;
  if (vec)
  {
    const int64_t npair = n >> 1;
    for (int64_t p = tid; p < npair; p += stride)
    {
      double2 x = ((const double2*)v)[p];
      x.x       = __dmul_rn(x.x, c);
      x.y       = __dmul_rn(x.y, c);
      ((double2*)v)[p] = x;
      if (t)
      {
        if (s2)
        {
          const double2 s = ((const double2*)s2)[p];
          x.x             = __ddiv_rn(x.x, s.x);
          x.y             = __ddiv_rn(x.y, s.y);
        }
        ((double2*)t)[p] = x;
      }
    }
    head = npair << 1;
  }
  for (int64_t i = head + tid; i < n; i += stride)
  {
    double x = __dmul_rn(v[i], c);
    v[i]     = x;
    if (t) t[i] = s2 ? __ddiv_rn(x, s2[i]) : x;
  }
}

using GSKernel = void (*)(int64_t, double*, GSList, GSList, unsigned, int, double*, double*,
                          unsigned int*, double*);

// The (updates, dot products) shapes the solver launches: (0, 1..8) for dot
// passes, (1..8, 0) for update chunks, (1..8, 1) for the last update chunk
// with the new norm or a modified-GS step.
template <bool F>
GSKernel pick_kernel(int nu, int nd)
{
#define GS_CASE8(NU_, ND_EXPR, VAR)                                                        \
  switch (VAR)                                                                             \
  {                                                                                        \
  case 1: return k_gs<F, NU_(1), ND_EXPR(1)>;                                              \
  case 2: return k_gs<F, NU_(2), ND_EXPR(2)>;                                              \
  case 3: return k_gs<F, NU_(3), ND_EXPR(3)>;                                              \
  case 4: return k_gs<F, NU_(4), ND_EXPR(4)>;                                              \
  case 5: return k_gs<F, NU_(5), ND_EXPR(5)>;                                              \
  case 6: return k_gs<F, NU_(6), ND_EXPR(6)>;                                              \
  case 7: return k_gs<F, NU_(7), ND_EXPR(7)>;                                              \
  case 8: return k_gs<F, NU_(8), ND_EXPR(8)>;                                              \
  default: return nullptr;                                                                 \
  }
#define GS_ZERO(x) 0
#define GS_ONE(x)  1
#define GS_SAME(x) x
  if (nu == 0) { GS_CASE8(GS_ZERO, GS_SAME, nd) }
  if (nd == 0) { GS_CASE8(GS_SAME, GS_ZERO, nu) }
  if (nd == 1) { GS_CASE8(GS_SAME, GS_ONE, nu) }
#undef GS_CASE8
#undef GS_ZERO
#undef GS_ONE
#undef GS_SAME
  return nullptr;
}

inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }
inline double* DEV(N_Vector v) { return N_VGetDeviceArrayPointer_GB300(v); }
inline bool is_gb300(N_Vector v)
{
  return v && v->ops && v->ops->nvlinearsum == N_VLinearSum_GB300;
}

// ------------------------------------------------------------------ content
struct Spgmr
{
  int maxl, pretype, gstype, max_restarts;
  sunbooleantype zeroguess;
  int numiters;
  double resnorm;
  int last_flag;
  bool fused;
  long nsyncs;
  SUNATimesFn ATimes;
  void* ATData;
  SUNPSetupFn Psetup;
  SUNPSolveFn Psolve;
  void* PData;
  N_Vector s1, s2;
  N_Vector* V;
  double** Hes;
  double* givens;
  N_Vector xcor;
  double* yg;
  N_Vector vtemp;
  double* cv;
  N_Vector* Xv;
  // device side
  cudaStream_t stream;
  int64_t n;
  double* d_coef;        // Hessenberg-column slots, device copy
  double* h_col;         // the same slots in pinned, mapped host memory
  double* h_col_dev;     // device alias of h_col
  double* d_partials;    // kMaxRedBlocks * kGSMax
  unsigned int* d_counter;
};

inline Spgmr* SP(SUNLinearSolver S) { return (Spgmr*)S->content; }

// Slots of the Hessenberg-column buffer.
inline int slot_h(const Spgmr*, int i) { return i; }
inline int slot_vk(const Spgmr* c) { return c->maxl + 1; }
inline int slot_nn(const Spgmr* c) { return c->maxl + 2; }
inline int slot_p(const Spgmr* c, int i) { return c->maxl + 3 + i; }
inline int slot_nn2(const Spgmr* c) { return 2 * c->maxl + 4; }
inline int num_slots(const Spgmr* c) { return 2 * c->maxl + 8; }

bool launch_gs(Spgmr* c, N_Vector wv, const GSList& U, int nu, const GSList& D, int nd,
               unsigned self_mask)
{
  double* w  = DEV(wv);
  int64_t n  = c->n;
  bool fma_  = N_VGetFMA_GB300(wv) == SUNTRUE;
  GSKernel k = fma_ ? pick_kernel<true>(nu, nd) : pick_kernel<false>(nu, nd);
  if (!k)
  {
    set_error(SUN_ERR_ARG_OUTOFRANGE, "SPGMR_GB300: unsupported Gram-Schmidt launch shape");
    return false;
  }
  int vec = aligned16(w);
  for (int j = 0; j < nu; ++j) vec = vec && aligned16(U.p[j]);
  for (int j = 0; j < nd; ++j) vec = vec && aligned16(D.p[j]);
  int64_t items = vec ? (n + 1) / 2 : n;
  int grid      = nd > 0 ? reduce_grid(items) : stream_grid(items);
  k<<<grid, kBlock, 0, c->stream>>>(n, w, U, D, self_mask, vec, c->d_coef, c->d_partials,
                                    c->d_counter, c->h_col_dev);
  count_launch();
  return check_cuda(cudaGetLastError(), "SPGMR_GB300 k_gs launch");
}

bool launch_normalize(Spgmr* c, double scale, N_Vector v, N_Vector t, N_Vector s2)
{
  double* pv  = DEV(v);
  double* pt  = t ? DEV(t) : nullptr;
  double* ps2 = s2 ? DEV(s2) : nullptr;
  int vec     = aligned16(pv) && (!pt || aligned16(pt)) && (!ps2 || aligned16(ps2));
  int64_t items = vec ? (c->n + 1) / 2 : c->n;
  k_gs_normalize<<<stream_grid(items), kBlock, 0, c->stream>>>(c->n, scale, pv, pt, ps2, vec);
  count_launch();
  return check_cuda(cudaGetLastError(), "SPGMR_GB300 k_gs_normalize launch");
}

bool stream_sync(Spgmr* c)
{
  c->nsyncs++;
  return check_cuda(cudaStreamSynchronize(c->stream), "SPGMR_GB300 stream synchronize");
}

// ---------------------------------------------------- fused Gram-Schmidt
// Orthogonalise V[k] against V[0..k-1]; Hes[0..k-1][k-1] and *new_norm as
// SUNClassicalGS (sundials_iterative.c:116-170) with p = maxl (i0 = 0).
bool gs_classical_fused(Spgmr* c, int k, double* new_norm)
{
  N_Vector* V = c->V;
  N_Vector w  = V[k];
  GSList none = {};
  // pass 1: <V_j, w> for j < k and <w, w>
  const int total = k + 1;
  for (int j0 = 0; j0 < total; j0 += kGSMax)
  {
    int m = total - j0 < kGSMax ? total - j0 : kGSMax;
    GSList D;
    unsigned self = 0;
    for (int t = 0; t < m; ++t)
    {
      int j = j0 + t;
      if (j < k) { D.p[t] = DEV(V[j]); D.idx[t] = slot_h(c, j); }
      else { D.p[t] = DEV(w); D.idx[t] = slot_vk(c); self |= 1u << t; }
    }
    if (!launch_gs(c, w, none, 0, D, m, self)) return false;
  }
  // pass 2: w -= sum_j h_j V_j, with ||w||^2 of the result
  for (int j0 = 0; j0 < k; j0 += kGSMax)
  {
    int m     = k - j0 < kGSMax ? k - j0 : kGSMax;
    bool last = j0 + m == k;
    GSList U, D = {};
    for (int t = 0; t < m; ++t) { U.p[t] = DEV(V[j0 + t]); U.idx[t] = slot_h(c, j0 + t); }
    if (last) { D.p[0] = DEV(w); D.idx[0] = slot_nn(c); }
    if (!launch_gs(c, w, U, m, D, last ? 1 : 0, last ? 1u : 0u)) return false;
  }
  if (!stream_sync(c)) return false;
  const double* h = c->h_col;
  double vk_norm  = sqrt(h[slot_vk(c)]);
  for (int i = 0; i < k; ++i) c->Hes[i][k - 1] = h[slot_h(c, i)];
  *new_norm = sqrt(h[slot_nn(c)]);
  if (!(kFactor * (*new_norm) < vk_norm)) return true;

  // reorthogonalisation: the same two passes with coefficients in slot_p
  for (int j0 = 0; j0 < k; j0 += kGSMax)
  {
    int m = k - j0 < kGSMax ? k - j0 : kGSMax;
    GSList D;
    for (int t = 0; t < m; ++t) { D.p[t] = DEV(V[j0 + t]); D.idx[t] = slot_p(c, j0 + t); }
    if (!launch_gs(c, w, none, 0, D, m, 0u)) return false;
  }
  for (int j0 = 0; j0 < k; j0 += kGSMax)
  {
    int m     = k - j0 < kGSMax ? k - j0 : kGSMax;
    bool last = j0 + m == k;
    GSList U, D = {};
    for (int t = 0; t < m; ++t) { U.p[t] = DEV(V[j0 + t]); U.idx[t] = slot_p(c, j0 + t); }
    if (last) { D.p[0] = DEV(w); D.idx[0] = slot_nn2(c); }
    if (!launch_gs(c, w, U, m, D, last ? 1 : 0, last ? 1u : 0u)) return false;
  }
  if (!stream_sync(c)) return false;
  for (int i = 0; i < k; ++i) c->Hes[i][k - 1] += h[slot_p(c, i)];
  *new_norm = sqrt(h[slot_nn2(c)]);
  return true;
}

// SUNModifiedGS (sundials_iterative.c:45-105) with p = maxl (i0 = 0).
bool gs_modified_fused(Spgmr* c, int k, double* new_norm)
{
  N_Vector* V = c->V;
  N_Vector w  = V[k];
  GSList none = {};
  {
    // ||w||^2 of the input vector and h_0 = <V_0, w>
    GSList D;
    D.p[0] = DEV(w);    D.idx[0] = slot_vk(c);
    D.p[1] = DEV(V[0]); D.idx[1] = slot_h(c, 0);
    if (!launch_gs(c, w, none, 0, D, 2, 1u)) return false;
  }
  for (int i = 1; i <= k; ++i)
  {
    // w -= h_{i-1} V_{i-1}; then h_i = <V_i, w> (or ||w||^2 after the last)
    GSList U, D;
    U.p[0] = DEV(V[i - 1]);
    U.idx[0] = slot_h(c, i - 1);
    unsigned self = 0;
    if (i < k) { D.p[0] = DEV(V[i]); D.idx[0] = slot_h(c, i); }
    else { D.p[0] = DEV(w); D.idx[0] = slot_nn(c); self = 1u; }
    if (!launch_gs(c, w, U, 1, D, 1, self)) return false;
  }
  if (!stream_sync(c)) return false;
  const double* h = c->h_col;
  double vk_norm  = sqrt(h[slot_vk(c)]);
  for (int i = 0; i < k; ++i) c->Hes[i][k - 1] = h[slot_h(c, i)];
  *new_norm   = sqrt(h[slot_nn(c)]);
  double temp = kFactor * vk_norm;
  if ((temp + (*new_norm)) != temp) return true;

  // reorthogonalisation, one basis vector at a time (each test needs the
  // new dot product on the host)
  double new_norm_2 = 0.0;
  for (int i = 0; i < k; ++i)
  {
    GSList D;
    D.p[0]   = DEV(V[i]);
    D.idx[0] = slot_p(c, i);
    if (!launch_gs(c, w, none, 0, D, 1, 0u)) return false;
    if (!stream_sync(c)) return false;
    double prod = h[slot_p(c, i)];
    temp        = kFactor * c->Hes[i][k - 1];
    if ((temp + prod) == temp) continue;
    c->Hes[i][k - 1] += prod;
    GSList U;
    U.p[0]   = DEV(V[i]);
    U.idx[0] = slot_p(c, i);
    if (!launch_gs(c, w, U, 1, none, 0, 0u)) return false;
    new_norm_2 += prod * prod;
  }
  if (new_norm_2 != 0.0)
  {
    double prod = (*new_norm) * (*new_norm) - new_norm_2;
    *new_norm   = prod > 0.0 ? sqrt(prod) : 0.0;
  }
  return true;
}

// ------------------------------------------ reference operation sequences
// The same two algorithms as the reference writes them, through the
// N_Vector operations (used when the fused kernels are switched off).
bool gs_classical_ops(Spgmr* c, int k, double* new_norm)
{
  N_Vector* V   = c->V;
  double* stemp = c->cv;
  N_Vector* vt  = c->Xv;
  if (N_VDotProdMulti_GB300(k + 1, V[k], V, stemp) != SUN_SUCCESS) return false;
  c->nsyncs++;
  double vk_norm = sqrt(stemp[k]);
  for (int i = k - 1; i >= 0; --i)
  {
    c->Hes[i][k - 1] = stemp[i];
    stemp[i + 1]     = -stemp[i];
    vt[i + 1]        = V[i];
  }
  stemp[0] = 1.0;
  vt[0]    = V[k];
  if (N_VLinearCombination_GB300(k + 1, stemp, vt, V[k]) != SUN_SUCCESS) return false;
  *new_norm = sqrt(N_VDotProd_GB300(V[k], V[k]));
  c->nsyncs++;
  if (!(kFactor * (*new_norm) < vk_norm)) return true;
  if (N_VDotProdMulti_GB300(k, V[k], V, stemp + 1) != SUN_SUCCESS) return false;
  c->nsyncs++;
  stemp[0] = 1.0;
  vt[0]    = V[k];
  for (int i = 0; i < k; ++i)
  {
    c->Hes[i][k - 1] += stemp[i + 1];
    stemp[i + 1] = -stemp[i + 1];
    vt[i + 1]    = V[i];
  }
  if (N_VLinearCombination_GB300(k + 1, stemp, vt, V[k]) != SUN_SUCCESS) return false;
  *new_norm = sqrt(N_VDotProd_GB300(V[k], V[k]));
  c->nsyncs++;
  return true;
}

bool gs_modified_ops(Spgmr* c, int k, double* new_norm)
{
  N_Vector* V    = c->V;
  double vk_norm = sqrt(N_VDotProd_GB300(V[k], V[k]));
  c->nsyncs++;
  for (int i = 0; i < k; ++i)
  {
    c->Hes[i][k - 1] = N_VDotProd_GB300(V[i], V[k]);
    c->nsyncs++;
    N_VLinearSum_GB300(1.0, V[k], -c->Hes[i][k - 1], V[i], V[k]);
  }
  *new_norm = sqrt(N_VDotProd_GB300(V[k], V[k]));
  c->nsyncs++;
  double temp = kFactor * vk_norm;
  if ((temp + (*new_norm)) != temp) return true;
  double new_norm_2 = 0.0;
  for (int i = 0; i < k; ++i)
  {
    double prod = N_VDotProd_GB300(V[i], V[k]);
    c->nsyncs++;
    temp = kFactor * c->Hes[i][k - 1];
    if ((temp + prod) == temp) continue;
    c->Hes[i][k - 1] += prod;
    N_VLinearSum_GB300(1.0, V[k], -prod, V[i], V[k]);
    new_norm_2 += prod * prod;
  }
  if (new_norm_2 != 0.0)
  {
    double prod = (*new_norm) * (*new_norm) - new_norm_2;
    *new_norm   = prod > 0.0 ? sqrt(prod) : 0.0;
  }
  return true;
}

// --------------------------------------------------------- Givens QR
// Add column n-1 to the QR factorisation of the (n+1) x n Hessenberg matrix:
// apply the n-1 earlier rotations, then make rotation n-1 (SUNQRfact,
// sundials_iterative.c:181-286; for n = 1 its job-0 branch does the same).
// Returns n if the new diagonal entry is zero.
int qr_add_column(int n, double** h, double* q)
{
  const int col = n - 1;
  for (int k = 0; k < col; ++k)
  {
    double cs = q[2 * k], sn = q[2 * k + 1];
    double t1 = h[k][col], t2 = h[k + 1][col];
    h[k][col]     = cs * t1 - sn * t2;
    h[k + 1][col] = sn * t1 + cs * t2;
  }
  double t1 = h[col][col], t2 = h[col + 1][col], cs, sn;
  if (t2 == 0.0)
  {
    cs = 1.0;
    sn = 0.0;
  }
  else if (fabs(t2) >= fabs(t1))
  {
    double t3 = t1 / t2;
    sn        = -1.0 / sqrt(1.0 + t3 * t3);
    cs        = -sn * t3;
  }
  else
  {
    double t3 = t2 / t1;
    cs        = 1.0 / sqrt(1.0 + t3 * t3);
    sn        = -cs * t3;
  }
  q[2 * col]     = cs;
  q[2 * col + 1] = sn;
  h[col][col]    = cs * t1 - sn * t2;
  return h[col][col] == 0.0 ? n : 0;
}

// Solve R y = Q b in place (SUNQRsol, sundials_iterative.c:297-329);
// returns k+1 for a zero diagonal entry R[k][k].
int qr_solve(int n, double** h, const double* q, double* b)
{
  for (int k = 0; k < n; ++k)
  {
    double cs = q[2 * k], sn = q[2 * k + 1];
    double t1 = b[k], t2 = b[k + 1];
    b[k]      = cs * t1 - sn * t2;
    b[k + 1]  = sn * t1 + cs * t2;
  }
  for (int k = n - 1; k >= 0; --k)
  {
    if (h[k][k] == 0.0) return k + 1;
    b[k] /= h[k][k];
    for (int i = 0; i < k; ++i) b[i] -= b[k] * h[i][k];
  }
  return 0;
}

void free_workspace(Spgmr* c)
{
  if (c->V)
  {
    for (int k = 0; k <= c->maxl; ++k)
      if (c->V[k]) N_VDestroy_GB300(c->V[k]);
    free(c->V);
    c->V = nullptr;
  }
  if (c->Hes)
  {
    for (int k = 0; k <= c->maxl; ++k) free(c->Hes[k]);
    free(c->Hes);
    c->Hes = nullptr;
  }
  free(c->givens);
  free(c->yg);
  free(c->cv);
  free(c->Xv);
  c->givens = c->yg = c->cv = nullptr;
  c->Xv                     = nullptr;
  if (c->d_coef) cudaFree(c->d_coef);
  if (c->h_col) cudaFreeHost(c->h_col);
  if (c->d_partials) cudaFree(c->d_partials);
  if (c->d_counter) cudaFree(c->d_counter);
  c->d_coef = c->h_col = c->h_col_dev = c->d_partials = nullptr;
  c->d_counter = nullptr;
}

}  // namespace

// =================================================================== C API
extern "C" {

SUNLinearSolver SUNLinSol_SPGMR_GB300(N_Vector y, int pretype, int maxl, SUNContext sunctx)
{
  if (!is_gb300(y))
  {
    set_error(SUN_ERR_ARG_INCOMPATIBLE, "SUNLinSol_SPGMR_GB300: y must be an NVECTOR_GB300");
    return nullptr;
  }
  if (pretype != SUN_PREC_NONE && pretype != SUN_PREC_LEFT && pretype != SUN_PREC_RIGHT &&
      pretype != SUN_PREC_BOTH)
    pretype = SUN_PREC_NONE;
  if (maxl <= 0) maxl = SUNSPGMR_GB300_MAXL_DEFAULT;
  SUNLinearSolver S = (SUNLinearSolver)calloc(1, sizeof(*S));
  S->ops            = (SUNLinearSolver_Ops)calloc(1, sizeof(*S->ops));
  S->sunctx         = sunctx;
  S->ops->gettype           = SUNLinSolGetType_SPGMR_GB300;
  S->ops->getid             = SUNLinSolGetID_SPGMR_GB300;
  S->ops->setatimes         = SUNLinSolSetATimes_SPGMR_GB300;
  S->ops->setpreconditioner = SUNLinSolSetPreconditioner_SPGMR_GB300;
  S->ops->setscalingvectors = SUNLinSolSetScalingVectors_SPGMR_GB300;
  S->ops->setzeroguess      = SUNLinSolSetZeroGuess_SPGMR_GB300;
  S->ops->initialize        = SUNLinSolInitialize_SPGMR_GB300;
  S->ops->setup             = SUNLinSolSetup_SPGMR_GB300;
  S->ops->solve             = SUNLinSolSolve_SPGMR_GB300;
  S->ops->numiters          = SUNLinSolNumIters_SPGMR_GB300;
  S->ops->resnorm           = SUNLinSolResNorm_SPGMR_GB300;
  S->ops->resid             = SUNLinSolResid_SPGMR_GB300;
  S->ops->lastflag          = SUNLinSolLastFlag_SPGMR_GB300;
  S->ops->space             = SUNLinSolSpace_SPGMR_GB300;
  S->ops->free              = SUNLinSolFree_SPGMR_GB300;
  Spgmr* c        = (Spgmr*)calloc(1, sizeof(Spgmr));
  S->content      = c;
  c->maxl         = maxl;
  c->pretype      = pretype;
  c->gstype       = SUN_MODIFIED_GS;
  c->max_restarts = SUNSPGMR_GB300_MAXRS_DEFAULT;
  c->zeroguess    = SUNFALSE;
  c->fused        = true;
  c->stream       = (cudaStream_t)N_VGetStream_GB300(y);
  c->n            = (int64_t)N_VGetLength_GB300(y);
  c->xcor         = N_VClone_GB300(y);
  c->vtemp        = N_VClone_GB300(y);
  if (!c->xcor || !c->vtemp)
  {
    SUNLinSolFree_SPGMR_GB300(S);
    return nullptr;
  }
  return S;
}

SUNErrCode SUNLinSol_SPGMR_GB300SetPrecType(SUNLinearSolver S, int pretype)
{
  if (pretype != SUN_PREC_NONE && pretype != SUN_PREC_LEFT && pretype != SUN_PREC_RIGHT &&
      pretype != SUN_PREC_BOTH)
    return SUN_ERR_ARG_OUTOFRANGE;
  SP(S)->pretype = pretype;
  return SUN_SUCCESS;
}

SUNErrCode SUNLinSol_SPGMR_GB300SetGSType(SUNLinearSolver S, int gstype)
{
  if (gstype != SUN_MODIFIED_GS && gstype != SUN_CLASSICAL_GS) return SUN_ERR_ARG_OUTOFRANGE;
  SP(S)->gstype = gstype;
  return SUN_SUCCESS;
}

SUNErrCode SUNLinSol_SPGMR_GB300SetMaxRestarts(SUNLinearSolver S, int maxrs)
{
  if (maxrs < 0) maxrs = SUNSPGMR_GB300_MAXRS_DEFAULT;
  SP(S)->max_restarts = maxrs;
  return SUN_SUCCESS;
}

SUNErrCode SUNLinSol_SPGMR_GB300SetFusedGS(SUNLinearSolver S, sunbooleantype onoff)
{
  SP(S)->fused = onoff ? true : false;
  return SUN_SUCCESS;
}

long int SUNLinSol_SPGMR_GB300NumSyncs(SUNLinearSolver S) { return SP(S)->nsyncs; }

SUNLinearSolver_Type SUNLinSolGetType_SPGMR_GB300(SUNLinearSolver) { return SUNLINEARSOLVER_ITERATIVE; }
SUNLinearSolver_ID SUNLinSolGetID_SPGMR_GB300(SUNLinearSolver) { return SUNLINEARSOLVER_SPGMR; }

SUNErrCode SUNLinSolInitialize_SPGMR_GB300(SUNLinearSolver S)
{
  Spgmr* c = SP(S);
  if (c->max_restarts < 0) c->max_restarts = SUNSPGMR_GB300_MAXRS_DEFAULT;
  if (!c->ATimes)
  {
    set_error(SUN_ERR_ARG_CORRUPT, "SPGMR_GB300: ATimes is not set");
    return SUN_ERR_ARG_CORRUPT;
  }
  if (c->pretype != SUN_PREC_LEFT && c->pretype != SUN_PREC_RIGHT && c->pretype != SUN_PREC_BOTH)
    c->pretype = SUN_PREC_NONE;
  if (c->pretype != SUN_PREC_NONE && !c->Psolve)
  {
    set_error(SUN_ERR_ARG_CORRUPT, "SPGMR_GB300: preconditioning requested without Psolve");
    return SUN_ERR_ARG_CORRUPT;
  }
  const int m = c->maxl;
  if (!c->V)
  {
    c->V = (N_Vector*)calloc(m + 1, sizeof(N_Vector));
    for (int k = 0; k <= m; ++k)
    {
      c->V[k] = N_VClone_GB300(c->vtemp);
      if (!c->V[k]) return SUN_ERR_MEM_FAIL;
    }
  }
  if (!c->Hes)
  {
    c->Hes = (double**)calloc(m + 1, sizeof(double*));
    for (int k = 0; k <= m; ++k) c->Hes[k] = (double*)calloc(m, sizeof(double));
  }
  if (!c->givens) c->givens = (double*)calloc(2 * m, sizeof(double));
  if (!c->yg) c->yg = (double*)calloc(m + 1, sizeof(double));
  if (!c->cv) c->cv = (double*)calloc(m + 1, sizeof(double));
  if (!c->Xv) c->Xv = (N_Vector*)calloc(m + 1, sizeof(N_Vector));
  if (!c->d_coef)
  {
    const size_t bytes = sizeof(double) * num_slots(c);
    if (!check_cuda(cudaMalloc(&c->d_coef, bytes), "SPGMR_GB300 cudaMalloc") ||
        !check_cuda(cudaHostAlloc(&c->h_col, bytes, cudaHostAllocMapped), "SPGMR_GB300 cudaHostAlloc") ||
        !check_cuda(cudaHostGetDevicePointer(&c->h_col_dev, c->h_col, 0), "SPGMR_GB300 mapped pointer") ||
        !check_cuda(cudaMalloc(&c->d_partials, sizeof(double) * kMaxRedBlocks * kGSMax),
                    "SPGMR_GB300 cudaMalloc") ||
        !check_cuda(cudaMalloc(&c->d_counter, sizeof(unsigned int)), "SPGMR_GB300 cudaMalloc") ||
        !check_cuda(cudaMemset(c->d_counter, 0, sizeof(unsigned int)), "SPGMR_GB300 cudaMemset") ||
        !check_cuda(cudaMemset(c->d_coef, 0, bytes), "SPGMR_GB300 cudaMemset"))
      return SUN_ERR_MEM_FAIL;
    memset(c->h_col, 0, bytes);
  }
  c->last_flag = SUN_SUCCESS;
  return SUN_SUCCESS;
}

SUNErrCode SUNLinSolSetATimes_SPGMR_GB300(SUNLinearSolver S, void* ATData, SUNATimesFn ATimes)
{
  SP(S)->ATimes = ATimes;
  SP(S)->ATData = ATData;
  return SUN_SUCCESS;
}

SUNErrCode SUNLinSolSetPreconditioner_SPGMR_GB300(SUNLinearSolver S, void* PData,
                                                  SUNPSetupFn Psetup, SUNPSolveFn Psolve)
{
  SP(S)->Psetup = Psetup;
  SP(S)->Psolve = Psolve;
  SP(S)->PData  = PData;
  return SUN_SUCCESS;
}

SUNErrCode SUNLinSolSetScalingVectors_SPGMR_GB300(SUNLinearSolver S, N_Vector s1, N_Vector s2)
{
  if ((s1 && !is_gb300(s1)) || (s2 && !is_gb300(s2)))
  {
    set_error(SUN_ERR_ARG_INCOMPATIBLE, "SPGMR_GB300: scaling vectors must be NVECTOR_GB300");
    return SUN_ERR_ARG_INCOMPATIBLE;
  }
  SP(S)->s1 = s1;
  SP(S)->s2 = s2;
  return SUN_SUCCESS;
}

SUNErrCode SUNLinSolSetZeroGuess_SPGMR_GB300(SUNLinearSolver S, sunbooleantype onoff)
{
  SP(S)->zeroguess = onoff;
  return SUN_SUCCESS;
}

int SUNLinSolSetup_SPGMR_GB300(SUNLinearSolver S, SUNMatrix)
{
  Spgmr* c = SP(S);
  if (c->Psetup)
  {
    int status = c->Psetup(c->PData);
    if (status != 0)
    {
      c->last_flag = status < 0 ? SUNLS_PSET_FAIL_UNREC : SUNLS_PSET_FAIL_REC;
      return c->last_flag;
    }
  }
  c->last_flag = SUN_SUCCESS;
  return SUN_SUCCESS;
}

int SUNLinSolSolve_SPGMR_GB300(SUNLinearSolver S, SUNMatrix, N_Vector x, N_Vector b,
                               sunrealtype delta)
{
  Spgmr* c               = SP(S);
  c->nsyncs              = 0;
  c->numiters            = 0;
  const int l_max        = c->maxl;
  const int max_restarts = c->max_restarts;
  const bool fused       = c->fused;
  N_Vector* V            = c->V;
  double** Hes           = c->Hes;
  double* givens         = c->givens;
  double* yg             = c->yg;
  N_Vector xcor = c->xcor, s1 = c->s1, s2 = c->s2;
  const bool preOnLeft  = c->pretype == SUN_PREC_LEFT || c->pretype == SUN_PREC_BOTH;
  const bool preOnRight = c->pretype == SUN_PREC_RIGHT || c->pretype == SUN_PREC_BOTH;
  const bool scale1 = s1 != nullptr, scale2 = s2 != nullptr;
  bool converged = false;
  int krydim     = 0;
  double rho, beta, r_norm, rotation_product;

  auto stop = [&](int flag) {
    c->zeroguess = SUNFALSE;
    c->last_flag = flag;
    return flag;
  };
  if (!V || !c->ATimes || ((preOnLeft || preOnRight) && !c->Psolve) || !is_gb300(x) ||
      !is_gb300(b) || N_VGetLength_GB300(x) != c->n || N_VGetLength_GB300(b) != c->n)
  {
    set_error(SUN_ERR_ARG_CORRUPT, "SPGMR_GB300 Solve: solver not initialised or bad vectors");
    return stop(SUN_ERR_ARG_CORRUPT);
  }
  auto atimes = [&](N_Vector in, N_Vector out) -> int {
    int st = c->ATimes(c->ATData, in, out);
    return st == 0 ? 0 : (st < 0 ? SUNLS_ATIMES_FAIL_UNREC : SUNLS_ATIMES_FAIL_REC);
  };
  auto psolve = [&](N_Vector r, N_Vector z, int lr) -> int {
    int st = c->Psolve(c->PData, r, z, delta, lr);
    return st == 0 ? 0 : (st < 0 ? SUNLS_PSOLVE_FAIL_UNREC : SUNLS_PSOLVE_FAIL_REC);
  };
  auto swap_vt = [&](N_Vector& a) { std::swap(a, c->vtemp); };

  // ---- initial residual V[0] = s1 P1^{-1} (b - A x)   (spgmr.c:532-588)
  int st;
  if (fused)
  {
    N_Vector src = b;
    if (!c->zeroguess)
    {
      if ((st = atimes(x, c->vtemp))) return stop(st);
      N_VLinearSum_GB300(1.0, b, -1.0, c->vtemp, c->vtemp);
      src = c->vtemp;
    }
    if (preOnLeft)
    {
      if ((st = psolve(src, V[0], SUN_PREC_LEFT))) return stop(st);
      src = V[0];
    }
    if (scale1) N_VProd_GB300(s1, src, V[0]);
    else if (src == b) N_VScale_GB300(1.0, b, V[0]);
    else if (src == c->vtemp) swap_vt(V[0]);
  }
  else
  {
    if (c->zeroguess) N_VScale_GB300(1.0, b, c->vtemp);
    else
    {
      if ((st = atimes(x, c->vtemp))) return stop(st);
      N_VLinearSum_GB300(1.0, b, -1.0, c->vtemp, c->vtemp);
    }
    N_VScale_GB300(1.0, c->vtemp, V[0]);
    if (preOnLeft)
    {
      if ((st = psolve(V[0], c->vtemp, SUN_PREC_LEFT))) return stop(st);
    }
    else N_VScale_GB300(1.0, V[0], c->vtemp);
    if (scale1) N_VProd_GB300(s1, c->vtemp, V[0]);
    else N_VScale_GB300(1.0, c->vtemp, V[0]);
  }

  r_norm = N_VDotProd_GB300(V[0], V[0]);
  c->nsyncs++;
  c->resnorm = r_norm = beta = sqrt(r_norm);
  if (r_norm <= delta) return stop(SUN_SUCCESS);
  rho = beta;
  N_VConst_GB300(0.0, xcor);

  double pending = 1.0;  // fused: normalisation still owed by V[l] at the start of step l
  for (int ntries = 0; ntries <= max_restarts; ++ntries)
  {
    for (int i = 0; i <= l_max; ++i)
      for (int j = 0; j < l_max; ++j) Hes[i][j] = 0.0;
    rotation_product = 1.0;
    if (fused) pending = 1.0 / r_norm;
    else N_VScale_GB300(1.0 / r_norm, V[0], V[0]);

    for (int l = 0; l < l_max; ++l)
    {
      c->numiters++;
      krydim = l + 1;
      // ---- V[l+1] = s1 P1^{-1} A P2^{-1} s2^{-1} V[l]   (spgmr.c:640-715)
      if (fused)
      {
        N_Vector a = V[l];
        if (scale2)
        {
          if (!launch_normalize(c, pending, V[l], c->vtemp, s2)) return stop(SUN_ERR_EXT_FAIL);
          a = c->vtemp;
        }
        else if (pending != 1.0)
        {
          if (!launch_normalize(c, pending, V[l], nullptr, nullptr)) return stop(SUN_ERR_EXT_FAIL);
        }
        if (preOnRight)
        {
          N_Vector z = (a == V[l]) ? c->vtemp : V[l + 1];
          if ((st = psolve(a, z, SUN_PREC_RIGHT))) return stop(st);
          a = z;
        }
        N_Vector out = (a == V[l + 1]) ? c->vtemp : V[l + 1];
        if ((st = atimes(a, out))) return stop(st);
        if (out == c->vtemp) swap_vt(V[l + 1]);
        if (preOnLeft)
        {
          if ((st = psolve(V[l + 1], c->vtemp, SUN_PREC_LEFT))) return stop(st);
          swap_vt(V[l + 1]);
        }
        if (scale1) N_VProd_GB300(s1, V[l + 1], V[l + 1]);
      }
      else
      {
        if (scale2) N_VDiv_GB300(V[l], s2, c->vtemp);
        else N_VScale_GB300(1.0, V[l], c->vtemp);
        if (preOnRight)
        {
          N_VScale_GB300(1.0, c->vtemp, V[l + 1]);
          if ((st = psolve(V[l + 1], c->vtemp, SUN_PREC_RIGHT))) return stop(st);
        }
        if ((st = atimes(c->vtemp, V[l + 1]))) return stop(st);
        if (preOnLeft)
        {
          if ((st = psolve(V[l + 1], c->vtemp, SUN_PREC_LEFT))) return stop(st);
        }
        else N_VScale_GB300(1.0, V[l + 1], c->vtemp);
        if (scale1) N_VProd_GB300(s1, c->vtemp, V[l + 1]);
        else N_VScale_GB300(1.0, c->vtemp, V[l + 1]);
      }

      // ---- orthogonalise against V[0..l]                (spgmr.c:720-729)
      double* hnew = &Hes[l + 1][l];
      bool ok;
      if (c->gstype == SUN_CLASSICAL_GS)
        ok = fused ? gs_classical_fused(c, l + 1, hnew) : gs_classical_ops(c, l + 1, hnew);
      else
        ok = fused ? gs_modified_fused(c, l + 1, hnew) : gs_modified_ops(c, l + 1, hnew);
      if (!ok) return stop(SUN_ERR_EXT_FAIL);

      // ---- Givens update and convergence test           (spgmr.c:732-756)
      if (qr_add_column(krydim, Hes, givens) != 0) return stop(SUNLS_QRFACT_FAIL);
      rotation_product *= givens[2 * l + 1];
      c->resnorm = rho = fabs(rotation_product * r_norm);
      if (rho <= delta)
      {
        converged = true;
        break;
      }
      if (fused) pending = 1.0 / Hes[l + 1][l];
      else N_VScale_GB300(1.0 / Hes[l + 1][l], V[l + 1], V[l + 1]);
    }

    // ---- xcor += V y, y from the least-squares problem (spgmr.c:771-790)
    yg[0] = r_norm;
    for (int i = 1; i <= krydim; ++i) yg[i] = 0.0;
    if (qr_solve(krydim, Hes, givens, yg) != 0) return stop(SUNLS_QRSOL_FAIL);
    c->cv[0] = 1.0;
    c->Xv[0] = xcor;
    for (int k = 0; k < krydim; ++k)
    {
      c->cv[k + 1] = yg[k];
      c->Xv[k + 1] = V[k];
    }
    if (N_VLinearCombination_GB300(krydim + 1, c->cv, c->Xv, xcor) != SUN_SUCCESS)
      return stop(SUN_ERR_EXT_FAIL);

    if (converged) break;
    if (ntries == max_restarts) break;

    // ---- restart: V[0] from the residual's Krylov representation (spgmr.c:840-862)
    double s_product = 1.0;
    for (int i = krydim; i > 0; --i)
    {
      yg[i] = s_product * givens[2 * i - 2];
      s_product *= givens[2 * i - 1];
    }
    yg[0] = s_product;
    r_norm *= s_product;
    for (int i = 0; i <= krydim; ++i) yg[i] *= r_norm;
    r_norm = fabs(r_norm);
    if (fused && pending != 1.0)
    {
      if (!launch_normalize(c, pending, V[krydim], nullptr, nullptr)) return stop(SUN_ERR_EXT_FAIL);
    }
    for (int k = 0; k <= krydim; ++k)
    {
      c->cv[k] = yg[k];
      c->Xv[k] = V[k];
    }
    if (N_VLinearCombination_GB300(krydim + 1, c->cv, c->Xv, V[0]) != SUN_SUCCESS)
      return stop(SUN_ERR_EXT_FAIL);
  }

  // ---- x update on success or residual reduction       (spgmr.c:795-930)
  if (!converged && !(rho < beta)) return stop(SUNLS_CONV_FAIL);
  if (scale2) N_VDiv_GB300(xcor, s2, xcor);
  if (preOnRight)
  {
    if ((st = psolve(xcor, c->vtemp, SUN_PREC_RIGHT))) return stop(st);
  }
  else N_VScale_GB300(1.0, xcor, c->vtemp);
  if (c->zeroguess) N_VScale_GB300(1.0, c->vtemp, x);
  else N_VLinearSum_GB300(1.0, x, 1.0, c->vtemp, x);
  if (!check_cuda(cudaGetLastError(), "SPGMR_GB300 Solve")) return stop(SUN_ERR_EXT_FAIL);
  return stop(converged ? SUN_SUCCESS : SUNLS_RES_REDUCED);
}

int SUNLinSolNumIters_SPGMR_GB300(SUNLinearSolver S) { return SP(S)->numiters; }
sunrealtype SUNLinSolResNorm_SPGMR_GB300(SUNLinearSolver S) { return SP(S)->resnorm; }
N_Vector SUNLinSolResid_SPGMR_GB300(SUNLinearSolver S) { return SP(S)->vtemp; }
sunindextype SUNLinSolLastFlag_SPGMR_GB300(SUNLinearSolver S) { return SP(S)->last_flag; }

SUNErrCode SUNLinSolSpace_SPGMR_GB300(SUNLinearSolver S, long int* lenrwLS, long int* leniwLS)
{
  Spgmr* c          = SP(S);
  sunindextype lrw1 = 0, liw1 = 0;
  N_VSpace_GB300(c->vtemp, &lrw1, &liw1);
  *lenrwLS = (long int)(lrw1 * (c->maxl + 5) + c->maxl * (c->maxl + 5) + 2);
  *leniwLS = (long int)(liw1 * (c->maxl + 5));
  return SUN_SUCCESS;
}

SUNErrCode SUNLinSolFree_SPGMR_GB300(SUNLinearSolver S)
{
  if (!S) return SUN_SUCCESS;
  if (S->content)
  {
    Spgmr* c = SP(S);
    free_workspace(c);
    if (c->xcor) N_VDestroy_GB300(c->xcor);
    if (c->vtemp) N_VDestroy_GB300(c->vtemp);
    free(c);
    S->content = nullptr;
  }
  free(S->ops);
  free(S);
  return SUN_SUCCESS;
}

}  // extern "C"

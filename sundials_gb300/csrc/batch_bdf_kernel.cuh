// batch_bdf_kernel.cuh -- the per-system BDF integrator, one warp per system.
//
// A restatement, on the device, of one CVode(tout, CV_NORMAL) call with BDF,
// Newton, SUNLINSOL_DENSE and an analytic Jacobian (the same control flow,
// constants and floating-point expressions as src/cvode/cvode.c:1037-3727,
// cvode_nls.c:256-398, cvode_ls.c:1311-1800, sunnonlinsol_newton.c:179-330 and
// sundials_dense.c:85-193).  Function names follow the reference's so the two
// can be read side by side.
//
// Work layout: the 32 lanes of a warp own the elements i = lane, lane + 32 of
// every vector of their system (n <= 64); vectors live in the warp's slice of
// shared memory, so element-wise operations need no synchronisation; the
// right-hand side gathers through shared memory; reductions are a fixed-order
// butterfly (FP64, MIXED) or CVODE's sequential sum (FP64_EXACT); the dense
// factorisation distributes the trailing-submatrix update over all lanes.
// Every scalar of the step control is computed redundantly, and identically,
// by all lanes, so control flow is warp-uniform.
//
// This header is compiled twice: batch_bdf_fast.cu (FP64 with FMA, MIXED) and
// batch_bdf_exact.cu (FP64_EXACT, built with -fmad=false so no product and
// sum is contracted, as in the reference built for x86-64).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "../../include/sunbatchbdf_gb300.h"
#include "ddpow.h"
#include "mlp_device.cuh"

namespace bdf {

constexpr int NMAX  = 64;
constexpr int QMAX  = 5;
constexpr int RMAX  = 2 * NMAX;  // reactions per system
// Global scratch of one warp slot: the saved Jacobian (n x n, leading
// dimension n) followed by the FP64 LU factors (n x ld, ld = n | 1 <= NMAX+1).
constexpr size_t SLOT_J       = (size_t)NMAX * NMAX;
constexpr size_t SLOT_DOUBLES = SLOT_J + (size_t)NMAX * (NMAX + 1);

// CVODE defaults: cvode_impl.h:55-127, cvode.c:118-125, cvode_nls.c:32-34,
// cvode_ls_impl.h:43-45.
constexpr int MXNCF = 10, MXNEF = 7, MXNEF1 = 3, LONG_WAIT = 10, SMALL_NST = 10, SMALL_NEF = 2;
constexpr int MAX_ITERS = 4, NLS_MAXCOR = 3, MSBP = 20, MSBJ = 51;
constexpr double ETA_MAX_FX = 1.5, ETA_MAX_FS = 10000.0, ETA_MAX_ES = 10.0, ETA_MAX_GS = 10.0;
constexpr double ETA_MIN = 0.1, ETA_MAX_EF = 0.2, ETA_MIN_EF = 0.1, ETA_CF = 0.25;
constexpr double ADDON = 0.000001, BIAS1 = 6.0, BIAS2 = 6.0, BIAS3 = 10.0;
constexpr double HLB_FACTOR = 100.0, HUB_FACTOR = 0.1, CORTES = 0.1;
constexpr double CRDOWN = 0.3, RDIV = 2.0, DGMAX_LSETUP = 0.3, DGMAX_JBAD = 0.2;
constexpr double UROUND = 0x1p-52;  // DBL_EPSILON, SUN_UNIT_ROUNDOFF

enum { FIRST_CALL = 6, PREV_CONV_FAIL = 7, PREV_ERR_FAIL = 9 };
enum { NO_FAILURES = 0, FAIL_BAD_J = 1, FAIL_OTHER = 2 };
enum { R_SUCCESS = 0, R_CONTINUE = 901, R_CONV_RECVR = 902 };
enum { DO_ERROR_TEST = 2, PREDICT_AGAIN = 3, TRY_AGAIN = 5 };
enum { CV_SUCCESS = 0, CV_TOO_MUCH_WORK = -1, CV_TOO_MUCH_ACC = -2, CV_ERR_FAILURE = -3,
       CV_CONV_FAILURE = -4 };

// Device-side problem: the host arrays plus the two CSR indexes built at
// creation (species -> signed reactions for f, reactant -> reactions for J).
struct DevProblem
{
  int64_t nsys;
  const int32_t* n;
  const int64_t* y_off;
  const int64_t* r_off;
  const int32_t* rtype;
  const int32_t* ra;
  const int32_t* rb;
  const int32_t* rc;
  const double* rk;
  const int32_t* fptr;   // [y_off[s] + s + i], local offsets into fent
  const int32_t* fent;   // [e_off[s] + e] = r << 1 | (1 if the rate is subtracted)
  const int64_t* e_off;  // [nsys+1]
  const int32_t* jptr;   // [y_off[s] + s + j], local offsets into jent
  const int32_t* jent;   // [je_off[s] + e] = r << 1 | (1 if j is reactant B)
  const int64_t* je_off; // [nsys+1]
  const int32_t* order;  // processing order (largest systems first)
};

// Optional per-section cycle counters (build with -DSUNGB300_BDF_TIMERS):
// each warp accumulates clock64() deltas per section into Params::timers.
enum { T_RHS, T_JAC, T_LU, T_SOLVE, T_NORM, T_SETC, T_PREP, T_OTHER, T_COUNT };
#ifdef SUNGB300_BDF_TIMERS
#define BDF_TIC(v) long long v = clock64()
#define BDF_TOC(v, slot) tacc[slot] += clock64() - (v)
#else
#define BDF_TIC(v)
#define BDF_TOC(v, slot)
#endif

struct Params
{
  DevProblem p;
  double t0, tout, rtol, atol;
  long mxstep;
  int refine;
  const double* y0;
  double* yout;
  SUNBatchBDFStats* stats;
  unsigned int* next;      // work-queue head
  double* scratch;         // per warp slot: SLOT_DOUBLES (saved Jacobian, FP64 LU)
  int* pivots;             // per warp slot: NMAX
  long long* timers;       // [slots][T_COUNT] when built with SUNGB300_BDF_TIMERS
  // learned Newton predictor (fast modes; NULL = off)
  const uint16_t* mlp_w;   // BF16 weights W1 | W2 | W3
  const float* mlp_b;      // FP32 biases b1 | b2 | b3
  unsigned long long* lp_counts;  // [0] predictor calls, [1] learned iterate kept
  // training-data recorder (NULL = off): features and scaled converged correctors
  uint16_t* rec_x;         // [cap][SUNMLP_IN_PAD] BF16
  float* rec_t;            // [cap][64]
  unsigned long long* rec_count;
  long long rec_cap;
  // retry of failed systems: a fast-mode launch appends the ids of systems
  // that end with a failure flag to fail_list (fail_count entries); the retry
  // launch processes order = fail_list with its length read from count_dev
  int32_t* fail_list;
  unsigned int* fail_count;
  const unsigned int* count_dev;
};

// Per-warp shared-memory slice for systems of at most NB species; the warp's
// Newton matrix (its LU factors, or its FP32 inverse) follows it in shared
// memory with an odd leading dimension (no bank conflicts on row access).
template <int NB>
struct WarpMem
{
  double zn[QMAX + 1][NB];
  double ewt[NB], acor[NB], y[NB], tempv[NB], ftemp[NB], delta[NB];
  double rate[2 * NB];
  double red[NB];
  double rdiag[NB];
  float fcol[NB + 4];  // FP32 right-hand side of MIXED solves, zero-padded to the row stride
  int perm[NB];
};

// MIXED keeps its FP32 inverse in shared memory (its solves and the FP32
// elimination are latency-bound); the FP64 modes are bound by the FP64 pipe
// and run faster with more resident warps, so their LU factors stay in the
// warp's global scratch (L1/L2-resident).  min_blocks caps registers at 128
// (16 resident one-warp blocks per SM) wherever shared memory allows that
// many; the 48- and 64-wide MIXED classes are held to 8 by their FP32 inverse.
template <int MODE, int NB>
struct Layout
{
  static constexpr bool mat_in_smem  = (MODE == SUNBATCHBDF_MIXED);
  using MT = typename std::conditional<MODE == SUNBATCHBDF_MIXED, float, double>::type;
  static constexpr size_t mem_bytes  = (sizeof(WarpMem<NB>) + 15) / 16 * 16;
  static constexpr size_t mat_bytes  = mat_in_smem ? sizeof(MT) * NB * (NB + 4) : 0;
  static constexpr size_t warp_bytes = mem_bytes + mat_bytes;
  static constexpr int min_blocks    = (mat_in_smem && NB > 32) ? 8 : 16;
};

// ---------------------------------------------------------------- helpers
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  return v;
}
__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
  {
    double o = __shfl_xor_sync(0xffffffffu, v, off);
    v        = o > v ? o : v;
  }
  return v;
}
__device__ __forceinline__ double dmax(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double dmin(double a, double b) { return a < b ? a : b; }
__device__ __forceinline__ double rsqrt_sun(double x) { return x <= 0.0 ? 0.0 : sqrt(x); }

// 1.0/j for the small integers CVODE divides by (j <= 8): the same bits as
// the run-time division, without spending FP64 instructions on it.
__device__ __forceinline__ double inv_int(int j)
{
  switch (j)
  {
  case 1: return 1.0;
  case 2: return 1.0 / 2.0;
  case 3: return 1.0 / 3.0;
  case 4: return 1.0 / 4.0;
  case 5: return 1.0 / 5.0;
  case 6: return 1.0 / 6.0;
  case 7: return 1.0 / 7.0;
  case 8: return 1.0 / 8.0;
  default: return 1.0 / (double)j;
  }
}

// Order-preserving integer key of |v| (IEEE bits of a non-negative value
// compare like integers), so pivot searches need no FP64 compares.
__device__ __forceinline__ long long abs_key(double v)
{
  return __double_as_longlong(v) & 0x7fffffffffffffffLL;
}
__device__ __forceinline__ long long abs_key(float v)
{
  return (long long)(__float_as_int(v) & 0x7fffffff);
}
__device__ __forceinline__ bool is_zero(double v) { return (__double_as_longlong(v) << 1) == 0; }
__device__ __forceinline__ bool is_zero(float v) { return (__float_as_int(v) << 1) == 0; }

// x^(1/k), k = 1..7, for the fast modes: an FP32 estimate 2^(log2(x)/k)
// refined by one Newton step y <- y - (y^k - x) / (k y^(k-1)) whose residual
// y^k - x is formed in FP64 (the step only needs its divisor to FP32
// accuracy).  From a ~2^-21 estimate the step leaves a relative error below
// 1e-13, at about k + 4 FP64 instructions instead of a full FP64 pow.
__device__ __forceinline__ double fast_root(double x, int k)
{
  if (k == 1) return x;
  if (!(x >= 1e-36 && x <= 1e36)) return x == 0.0 ? 0.0 : pow(x, 1.0 / k);
  const float yf = exp2f(__log2f((float)x) / (float)k);
  const double y = (double)yf;
  double pk1     = y;
  for (int i = 2; i < k; i++) pk1 *= y;  // y^(k-1)
  const double d   = pk1 * y - x;
  const float rdiv = 1.0f / ((float)k * (float)pk1);
  return y - d * (double)rdiv;
}

// SUNRpowerR(x, 1/k) of the step-size controller: the exact mode rounds it
// correctly (double-double), the fast modes use fast_root.
template <bool EXACT>
__device__ __forceinline__ double cv_root(double x, int k)
{
  return EXACT ? dd_pow(x, inv_int(k)) : fast_root(x, k);
}

// LEARN: the learned-predictor inference, its features and the training-data
// recorder are compiled in; the default kernels leave that code out (it is
// cold there, but its size costs instruction-cache misses in the hot loop).
template <int MODE, int NB, bool LEARN = false>
struct Integrator
{
  static constexpr bool EXACT = (MODE == SUNBATCHBDF_FP64_EXACT);
  static constexpr bool MIXED = (MODE == SUNBATCHBDF_MIXED);

  const Params& P;
  WarpMem<NB>& w;
  const int lane;
  // system
  int n, nr;
  bool two;      // n > 32: lanes own a second element (read it through has2())
  // a compile-time false in the 32-wide kernels, so their second-element
  // code is not generated at all
  __device__ __forceinline__ bool has2() const { return NB > 32 && two; }
  double inv_n;  // 1/n (fast modes)
  double* rdiag; // reciprocal pivots of the factorisation (fast modes)
  const int32_t *rt, *ra, *rb, *rc, *fptr, *fent, *jptr, *jent;
  const double* rk;
  double* J;   // saved Jacobian, column-major n x n (global memory)
  double* M;   // Newton matrix / its LU factors (FP64 modes; shared memory)
  float* M32;  // Newton matrix / its inverse (MIXED; shared memory)
  float* J32;  // FP32 copy of J (MIXED; global scratch after J)
  int ld;      // leading dimension of M (FP64 modes, column-major, odd)
  int lr;      // row stride of M32 (MIXED, row-major): a multiple of 4, lr/4 odd
  int* piv;
  // CVODE state (identical in every lane)
  double tn, h, hscale, hprime, next_h, eta, etamax, etaq, etaqm1, etaqp1, hu, h0u;
  int next_q;
  double saved_tq5, rl1, gamma, gammap, gamrat, crate, delp, acnrm;
  double tq[6], l[QMAX + 2], tau[QMAX + 2];
  int q, qprime, qwait, L, indx_acor, nscon, convfail, qu;
  int nls_jcur, cv_jcur;
  long nst, nfe, nsetups, nje, nni, ncfn, netf, nnf, nstlp, nstlj;
  long nlp, nlpu;  // learned predictor: calls, learned iterate kept
  bool learned_start;  // the current Newton solve started from the learned iterate
#ifdef SUNGB300_BDF_TIMERS
  long long tacc[T_COUNT] = {0};
#endif

  __device__ Integrator(const Params& p_, WarpMem<NB>& w_, void* mat, int lane_)
    : P(p_), w(w_), lane(lane_)
  {
    M   = (double*)mat;
    M32 = (float*)mat;
  }

  // ------------------------------------------------------------ norms
  // N_VWrmsNorm_Serial: sqrt(sum((x*w)^2)/n); EXACT sums sequentially.
  __device__ double wrms(const double* x)
  {
    double s;
    if (EXACT)
    {
      for (int i = lane; i < n && (NB > 32 || i < 32); i += 32)
      {
        double p = x[i] * w.ewt[i];
        w.red[i] = p * p;
      }
      __syncwarp();
      s = 0.0;
      for (int i = 0; i < n; i++) s = s + w.red[i];
      __syncwarp();
    }
    else
    {
      double acc = 0.0;
      for (int i = lane; i < n && (NB > 32 || i < 32); i += 32)
      {
        double p = x[i] * w.ewt[i];
        acc      = fma(p, p, acc);
      }
      s = warp_sum(acc);
    }
    s = EXACT ? s / n : s * inv_n;
    return rsqrt_sun(s);
  }

  __device__ void set_ewt(const double* ycur, double* wt)
  {  // cvEwtSetSS (cvode.c:4791)
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32)
    {
      double t   = fabs(ycur[i]);
      t          = P.rtol * t;
      t          = t + P.atol;
      w.tempv[i] = t;
      wt[i]      = 1.0 / t;
    }
  }

  // ------------------------------------------------------------ model
  __device__ void rhs(const double* ysm, double* f)
  {
    BDF_TIC(t0);
    __syncwarp();
    for (int r = lane; r < nr; r += 32)
    {
      double v = rk[r] * ysm[ra[r]];
      if (rt[r]) v = v * ysm[rb[r]];
      w.rate[r] = v;
    }
    __syncwarp();
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32)
    {
      double acc = 0.0;
      for (int e = fptr[i]; e < fptr[i + 1]; e++)
      {
        int ent  = fent[e];
        double v = w.rate[ent >> 1];
        acc      = (ent & 1) ? acc - v : acc + v;
      }
      f[i] = acc;
    }
    __syncwarp();
    nfe++;
    BDF_TOC(t0, T_RHS);
  }

  // J (zeroed first) = df/dy at w.y; lane owns columns j = lane, lane + 32.
  __device__ void jac()
  {
    BDF_TIC(t0);
    for (int e = lane; e < n * n; e += 32) J[e] = 0.0;
    __syncwarp();
    for (int j = lane; j < n && (NB > 32 || j < 32); j += 32)
    {
      double* col = J + j * n;
      for (int e = jptr[j]; e < jptr[j + 1]; e++)
      {
        int ent = jent[e];
        int r   = ent >> 1;
        double d;
        if (rt[r] == 0)
        {
          d         = rk[r];
          col[ra[r]] = col[ra[r]] - d;
          col[rb[r]] = col[rb[r]] + d;
        }
        else
        {
          d          = (ent & 1) ? rk[r] * w.y[ra[r]] : rk[r] * w.y[rb[r]];
          col[ra[r]] = col[ra[r]] - d;
          col[rb[r]] = col[rb[r]] - d;
          col[rc[r]] = col[rc[r]] + d;
        }
      }
    }
    __syncwarp();
    if (MIXED)
    {  // FP32 copy (column-major, like J) the Newton matrices are built from
       // until the next J
      for (int e = lane; e < n * n; e += 32) J32[e] = (float)J[e];
      __syncwarp();
    }
    BDF_TOC(t0, T_JAC);
  }

  // ------------------------------------------------------------ dense LU
  // SUNDlsMat_denseGETRF on a column-major matrix; returns 0 or k+1.
  template <class T>
  __device__ int getrf(T* a)
  {
    for (int k = 0; k < n; k++)
    {
      T* ck        = a + k * ld;
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
      for (int off = 16; off > 0; off >>= 1)
      {
        long long ov = __shfl_xor_sync(0xffffffffu, bk, off);
        int oi       = __shfl_xor_sync(0xffffffffu, bi, off);
        if (ov > bk || (ov == bk && oi < bi))
        {
          bk = ov;
          bi = oi;
        }
      }
      const int l = bi;
      if (lane == 0) piv[k] = l;
      if (bk == 0) return k + 1;
      if (l != k)
        for (int j = lane; j < n && (NB > 32 || j < 32); j += 32)
        {
          T t           = a[j * ld + l];
          a[j * ld + l] = a[j * ld + k];
          a[j * ld + k] = t;
        }
      __syncwarp();
      const T mult = (T)1 / ck[k];
      if (!EXACT && lane == 0) rdiag[k] = (double)mult;
      for (int i = k + 1 + lane; i < n; i += 32) ck[i] *= mult;
      __syncwarp();
      // trailing update, four independent elements per lane at a time
      const int rows = n - k - 1;
      const int tot  = rows * rows;
      const int rdiv = rows > 0 ? rows : 1;
      for (int t0 = lane; t0 < tot; t0 += 128)
      {
        int idx[4];
        T av[4], ak[4], ci[4];
#pragma unroll
        for (int u = 0; u < 4; u++)
        {
          const int t = t0 + 32 * u;
          const int j = t / rdiv, i = t - j * rdiv;
          idx[u]      = t < tot ? (k + 1 + j) * ld + (k + 1 + i) : -1;
          if (idx[u] >= 0)
          {
            ak[u] = a[(k + 1 + j) * ld + k];
            ci[u] = ck[k + 1 + i];
            av[u] = a[idx[u]];
          }
        }
#pragma unroll
        for (int u = 0; u < 4; u++)
          if (idx[u] >= 0)
          {
            if (EXACT)
            {  // the reference skips a zero multiplier (sundials_dense.c:137)
              if (!is_zero(ak[u])) a[idx[u]] = av[u] - ak[u] * ci[u];
            }
            else
              a[idx[u]] = fma(-ak[u], ci[u], av[u]);
          }
      }
      __syncwarp();
    }
    return 0;
  }

  // MIXED: in-place inverse of the FP32 Newton matrix (column-major,
  // a[j*ld + i]) by Gauss-Jordan elimination with partial pivoting: at step k
  // rows k and p swap, row k is scaled by 1/pivot, column k is eliminated
  // from every other row (the pivot column then holds -a_ik/pivot), and the
  // row interchanges are undone on the columns at the end, in reverse order.
  // The pivot choice is the LU factorisation's.  Returns 0 or k+1.
  // In-place Gauss-Jordan inversion with partial pivoting of the FP32 matrix
  // (row-major, row stride lr, padding columns zero); returns 0 or k+1 for a
  // zero pivot in column k.  Lane l owns rows l and l + 32; every row update
  // moves 16-byte chunks (the stride makes 8 consecutive rows' chunks fall in
  // distinct bank quads), so an FMA costs well under one memory instruction.
  __device__ int gauss_jordan(float* a)
  {
    const int nq   = lr >> 2;
    float4* A4     = reinterpret_cast<float4*>(a);
    const int i0   = lane, i1 = lane + 32;
    const bool h0  = i0 < n, h1 = has2() && i1 < n;
    for (int k = 0; k < n; k++)
    {
      long long bk = -1;
      int bi       = n;
      if (h0 && i0 >= k)
      {
        bk = abs_key(a[i0 * lr + k]);
        bi = i0;
      }
      if (h1 && i1 >= k)
      {
        const long long v = abs_key(a[i1 * lr + k]);
        if (v > bk)
        {
          bk = v;
          bi = i1;
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1)
      {
        const long long ov = __shfl_xor_sync(0xffffffffu, bk, off);
        const int oi       = __shfl_xor_sync(0xffffffffu, bi, off);
        if (ov > bk || (ov == bk && oi < bi))
        {
          bk = ov;
          bi = oi;
        }
      }
      if (bk == 0) return k + 1;
      const int l = bi;
      if (lane == 0) w.perm[k] = l;
      if (l != k)
        for (int c = lane; c < nq; c += 32)
        {
          const float4 t  = A4[k * nq + c];
          A4[k * nq + c] = A4[l * nq + c];
          A4[l * nq + c] = t;
        }
      __syncwarp();
      const float rp = 1.f / a[k * lr + k];
      __syncwarp();
      if (lane == 0) a[k * lr + k] = 1.f;  // the pivot position becomes rp
      __syncwarp();
      for (int c = lane; c < nq; c += 32)
      {
        float4 v = A4[k * nq + c];
        v.x *= rp;
        v.y *= rp;
        v.z *= rp;
        v.w *= rp;
        A4[k * nq + c] = v;
      }
      __syncwarp();
      // rows i != k: a[i][:] -= a[i][k] * a[k][:], with a[i][k] first set to 0
      // (so it ends as -a[i][k] * rp)
      const bool e0 = h0 && i0 != k, e1 = h1 && i1 != k;
      const float f0 = e0 ? a[i0 * lr + k] : 0.f;
      const float f1 = e1 ? a[i1 * lr + k] : 0.f;
      if (e0) a[i0 * lr + k] = 0.f;
      if (e1) a[i1 * lr + k] = 0.f;
      if (e0 || e1)
        for (int c0 = 0; c0 < nq; c0 += 4)
        {
          // four chunks' loads issued before any store (row k is never
          // written here, but the compiler cannot prove it)
          float4 y[4], x0[4], x1[4];
#pragma unroll
          for (int u = 0; u < 4; u++)
          {
            const int c = c0 + u < nq ? c0 + u : nq - 1;
            y[u]        = A4[k * nq + c];
            x0[u]       = e0 ? A4[i0 * nq + c] : y[u];
            x1[u]       = e1 ? A4[i1 * nq + c] : y[u];
          }
#pragma unroll
          for (int u = 0; u < 4; u++)
          {
            x0[u].x = fmaf(-f0, y[u].x, x0[u].x);
            x0[u].y = fmaf(-f0, y[u].y, x0[u].y);
            x0[u].z = fmaf(-f0, y[u].z, x0[u].z);
            x0[u].w = fmaf(-f0, y[u].w, x0[u].w);
            x1[u].x = fmaf(-f1, y[u].x, x1[u].x);
            x1[u].y = fmaf(-f1, y[u].y, x1[u].y);
            x1[u].z = fmaf(-f1, y[u].z, x1[u].z);
            x1[u].w = fmaf(-f1, y[u].w, x1[u].w);
          }
#pragma unroll
          for (int u = 0; u < 4; u++)
            if (c0 + u < nq)
            {
              if (e0) A4[i0 * nq + c0 + u] = x0[u];
              if (e1) A4[i1 * nq + c0 + u] = x1[u];
            }
        }
      __syncwarp();
    }
    // undo the row interchanges as column interchanges, last first
    for (int k = n - 1; k >= 0; k--)
    {
      const int p = w.perm[k];
      if (p != k)
      {
        if (h0)
        {
          const float t    = a[i0 * lr + k];
          a[i0 * lr + k] = a[i0 * lr + p];
          a[i0 * lr + p] = t;
        }
        if (h1)
        {
          const float t    = a[i1 * lr + k];
          a[i1 * lr + k] = a[i1 * lr + p];
          a[i1 * lr + p] = t;
        }
      }
    }
    __syncwarp();
    return 0;
  }

  // x = A b for a column-major FP32 matrix (leading dimension ld); b, x in
  // registers; four columns per trip, two accumulators per element.
  // x = A b for the FP32 inverse (row-major, stride lr): b goes through
  // w.fcol (zero-padded to lr), each lane forms the dot products of its rows
  // with 16-byte loads and four partial sums.
  __device__ void matvec32(const float* A, float b0, float b1, float& x0, float& x1)
  {
    if (lane < n) w.fcol[lane] = b0;
    if (lane + 32 < n) w.fcol[lane + 32] = b1;
    for (int i = n + lane; i < lr; i += 32) w.fcol[i] = 0.f;
    __syncwarp();
    const int nq      = lr >> 2;
    const float4* A4  = reinterpret_cast<const float4*>(A);
    const float4* B4  = reinterpret_cast<const float4*>(w.fcol);
    const bool h0 = lane < n, h1 = has2() && lane + 32 < n;
    float4 s0 = make_float4(0.f, 0.f, 0.f, 0.f), s1 = s0;
    for (int c = 0; c < nq; c++)
    {
      const float4 bj = B4[c];
      if (h0)
      {
        const float4 v = A4[lane * nq + c];
        s0.x = fmaf(v.x, bj.x, s0.x);
        s0.y = fmaf(v.y, bj.y, s0.y);
        s0.z = fmaf(v.z, bj.z, s0.z);
        s0.w = fmaf(v.w, bj.w, s0.w);
      }
      if (h1)
      {
        const float4 v = A4[(lane + 32) * nq + c];
        s1.x = fmaf(v.x, bj.x, s1.x);
        s1.y = fmaf(v.y, bj.y, s1.y);
        s1.z = fmaf(v.z, bj.z, s1.z);
        s1.w = fmaf(v.w, bj.w, s1.w);
      }
    }
    __syncwarp();
    x0 = (s0.x + s0.y) + (s0.z + s0.w);
    x1 = (s1.x + s1.y) + (s1.z + s1.w);
  }

  // y = J x with the saved FP64 Jacobian in global memory (column-major,
  // leading dimension n); eight columns' loads in flight per trip.
  __device__ void matvec_j(double x0, double x1, double& y0, double& y1)
  {
    double a0 = 0.0, a1 = 0.0, c0 = 0.0, c1 = 0.0;
    int j = 0;
    for (; j + 8 <= n; j += 8)
    {
      double xj[8], v0[8], v1[8];
#pragma unroll
      for (int u = 0; u < 8; u++)
      {
        xj[u] = __shfl_sync(0xffffffffu, (j + u) < 32 ? x0 : x1, (j + u) & 31);
        v0[u] = lane < n ? J[(j + u) * n + lane] : 0.0;
        v1[u] = (has2() && lane + 32 < n) ? J[(j + u) * n + lane + 32] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 8; u += 2)
      {
        a0 = fma(v0[u], xj[u], a0);
        c0 = fma(v0[u + 1], xj[u + 1], c0);
      }
      if (has2())
#pragma unroll
        for (int u = 0; u < 8; u += 2)
        {
          a1 = fma(v1[u], xj[u], a1);
          c1 = fma(v1[u + 1], xj[u + 1], c1);
        }
    }
    for (; j < n; j++)
    {
      const double xj = __shfl_sync(0xffffffffu, j < 32 ? x0 : x1, j & 31);
      if (lane < n) a0 = fma(J[j * n + lane], xj, a0);
      if (has2() && lane + 32 < n) a1 = fma(J[j * n + lane + 32], xj, a1);
    }
    y0 = a0 + c0;
    y1 = a1 + c1;
  }

  // SUNDlsMat_denseGETRS with b held in registers: b0 = b[lane], b1 = b[lane+32].
  // The fast modes multiply by the reciprocal pivots kept by getrf instead of
  // dividing (one FP64 instruction instead of a division sequence).
  template <class T>
  __device__ void getrs(const T* a, T& b0, T& b1)
  {
    for (int k = 0; k < n; k++)
    {
      const int pk = piv[k];
      if (pk != k)
      {
        T vk = __shfl_sync(0xffffffffu, k < 32 ? b0 : b1, k & 31);
        T vp = __shfl_sync(0xffffffffu, pk < 32 ? b0 : b1, pk & 31);
        if (lane == (k & 31)) { if (k < 32) b0 = vp; else b1 = vp; }
        if (lane == (pk & 31)) { if (pk < 32) b0 = vk; else b1 = vk; }
      }
    }
    for (int k = 0; k < n - 1; k++)
    {
      const T bk  = __shfl_sync(0xffffffffu, k < 32 ? b0 : b1, k & 31);
      const T* ck = a + k * ld;
      if (lane > k && lane < n) b0 -= ck[lane] * bk;
      if (has2() && lane + 32 > k && lane + 32 < n) b1 -= ck[lane + 32] * bk;
    }
    for (int k = n - 1; k > 0; k--)
    {
      const T* ck = a + k * ld;
      if (lane == (k & 31))
      {
        if (EXACT)
        {
          if (k < 32) b0 /= ck[k];
          else b1 /= ck[k];
        }
        else
        {
          const T r = (T)rdiag[k];
          if (k < 32) b0 *= r;
          else b1 *= r;
        }
      }
      const T bk = __shfl_sync(0xffffffffu, k < 32 ? b0 : b1, k & 31);
      if (lane < k) b0 -= ck[lane] * bk;
      if (has2() && lane + 32 < k) b1 -= ck[lane + 32] * bk;
    }
    if (lane == 0)
    {
      if (EXACT) b0 /= a[0];
      else b0 *= (T)rdiag[0];
    }
  }

  // ------------------------------------------------------------ lsetup / lsolve
  // cvNlsLSetup -> cvLsSetup -> cvLsLinSys -> SUNLinSolSetup_Dense
  __device__ int nls_lsetup(int jbad)
  {
    if (jbad) convfail = FAIL_BAD_J;
    double dgamma = fabs((gamma / gammap) - 1.0);
    int ls_jbad   = (nst == 0) || (nst >= nstlj + MSBJ) ||
                  ((convfail == FAIL_BAD_J) && (dgamma < DGMAX_JBAD)) || (convfail == FAIL_OTHER);
    if (ls_jbad)
    {
      cv_jcur = 1;
      jac();
    }
    else cv_jcur = 0;
    BDF_TIC(t0);
    const double c = -gamma;
    int lu;
    if (MIXED)
    {  // M = I - gamma J in FP32 (row-major, zero padding columns), then its
       // inverse; four columns of J32 per trip (coalesced loads), stored as
       // one 16-byte piece of each row (conflict-free: lr = 4 mod 8)
      const float cf = (float)c;
      for (int j0 = 0; j0 < lr; j0 += 4)
      {
        float v0[4], v1[4];
#pragma unroll
        for (int u = 0; u < 4; u++)
        {
          const int j = j0 + u;
          v0[u] = (j < n && lane < n) ? J32[j * n + lane] * cf + (lane == j ? 1.0f : 0.0f) : 0.0f;
          v1[u] = (j < n && lane + 32 < n) ? J32[j * n + lane + 32] * cf + (lane + 32 == j ? 1.0f : 0.0f)
                                           : 0.0f;
        }
        if (lane < n) *reinterpret_cast<float4*>(M32 + lane * lr + j0) = make_float4(v0[0], v0[1], v0[2], v0[3]);
        if (lane + 32 < n)
          *reinterpret_cast<float4*>(M32 + (lane + 32) * lr + j0) = make_float4(v1[0], v1[1], v1[2], v1[3]);
      }
      __syncwarp();
      lu = gauss_jordan(M32);
    }
    else
    {
      for (int e = lane; e < n * n; e += 32)
      {
        const int j = e / n, i = e - j * n;
        M[j * ld + i] = J[e] * c;
      }
      __syncwarp();
      for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) M[i * ld + i] += 1.0;
      __syncwarp();
      lu = getrf<double>(M);
    }
    __syncwarp();
    BDF_TOC(t0, T_LU);
    if (cv_jcur)
    {
      nje++;
      nstlj = nst;
    }
    nsetups++;
    nls_jcur = cv_jcur;
    gamrat   = 1.0;
    gammap   = gamma;
    crate    = 1.0;
    nstlp    = nst;
    return lu > 0 ? R_CONV_RECVR : R_SUCCESS;
  }

  // cvNlsLSolve -> cvLsSolve (direct): b <- A^{-1} b, then the gamrat scaling.
  __device__ void nls_lsolve(double* b)
  {
    BDF_TIC(t0);
    double b0 = lane < n ? b[lane] : 0.0;
    double b1 = lane + 32 < n ? b[lane + 32] : 0.0;
    if (MIXED)
    {
      // x = M32^{-1} b in FP32, then FP64 refinement: r = b - (x - gammap*J x),
      // x += M32^{-1} r; every product is a pipelined matvec (no dependent
      // triangular chains).
      const float* Minv = M32;
      float f0, f1;
      matvec32(Minv, (float)b0, (float)b1, f0, f1);
      double x0 = f0, x1 = f1;
      for (int sweep = 0; sweep < P.refine; sweep++)
      {
        double jx0, jx1;
        matvec_j(x0, x1, jx0, jx1);
        const double r0 = b0 - fma(-gammap, jx0, x0);
        const double r1 = b1 - fma(-gammap, jx1, x1);
        float d0, d1;
        matvec32(Minv, (float)r0, (float)r1, d0, d1);
        x0 += (double)d0;
        x1 += (double)d1;
      }
      b0 = x0;
      b1 = x1;
    }
    else
      getrs<double>(M, b0, b1);
    if (gamrat != 1.0)
    {
      const double c = 2.0 / (1.0 + gamrat);
      b0 *= c;
      b1 *= c;
    }
    if (lane < n) b[lane] = b0;
    if (lane + 32 < n) b[lane + 32] = b1;
    BDF_TOC(t0, T_SOLVE);
  }

  // cvNlsResidual (cvode_nls.c:363)
  __device__ void nls_residual(const double* ycor, double* res)
  {
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.y[i] = w.zn[0][i] + ycor[i];
    rhs(w.y, w.ftemp);
    const double a = -gamma;
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32)
    {
      double r = (rl1 * w.zn[1][i]) + ycor[i];
      res[i]   = r + a * w.ftemp[i];
    }
  }

  // the same residual at ycor = 0 (the BDF predictor itself)
  __device__ void nls_residual0(double* res)
  {
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.y[i] = w.zn[0][i] + 0.0;
    rhs(w.y, w.ftemp);
    const double a = -gamma;
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32)
    {
      double r = (rl1 * w.zn[1][i]) + 0.0;
      res[i]   = r + a * w.ftemp[i];
    }
  }

  // Predictor features (include/sunmlp_gb300.h) of the predicted state zn[0]:
  // xr[c] = feature 32c + lane, rounded to BF16.
  __device__ void mlp_features(float (&xr)[5])
  {
    using namespace gb300mlp;
    double lam[2] = {0.0, 0.0};  // local consumption rates of species lane, lane + 32
#pragma unroll
    for (int h2 = 0; h2 < 2; ++h2)
    {
      const int j = lane + 32 * h2;
      if (j < n)
      {
        double acc = 0.0;
        for (int e = jptr[j]; e < jptr[j + 1]; e++)
        {
          const int ent = jent[e], r = ent >> 1;
          if (rt[r] == 0) acc += rk[r];
          else acc += rk[r] * w.zn[0][(ent & 1) ? ra[r] : rb[r]];
        }
        lam[h2] = acc;
      }
    }
    const float fy0 = lane < n ? feat_y(w.zn[0][lane]) : 0.0f;
    const float fy1 = lane + 32 < n ? feat_y(w.zn[0][lane + 32]) : 0.0f;
    const float fr0 = lane < n ? feat_rate(gamma * lam[0]) : 0.0f;
    const float fr1 = lane + 32 < n ? feat_rate(gamma * lam[1]) : 0.0f;
    const float up0 = __shfl_up_sync(0xffffffffu, fr0, 1);
    const float up1 = __shfl_up_sync(0xffffffffu, fr1, 1);
    const float r31 = __shfl_sync(0xffffffffu, fr0, 31);
    const float r63 = __shfl_sync(0xffffffffu, fr1, 31);
    xr[0] = bf16_round(fy0);
    xr[1] = bf16_round(fy1);
    xr[2] = bf16_round(lane == 0 ? feat_gamma(gamma) : up0);  // 64: gamma; 65+i: species i
    xr[3] = bf16_round(lane == 0 ? r31 : up1);                // species 31 + lane
    xr[4] = bf16_round(lane == 0 ? r63 : 0.0f);               // species 63, then padding
  }

  // cvNlsConvTest (cvode_nls.c:313)
  __device__ int nls_convtest(const double* ycor, double tol, int mcur)
  {
    BDF_TIC(t0);
    int rv;
    double del = wrms(w.delta);
    if (mcur > 0)
    {
      double r = del / delp;
      crate    = (CRDOWN * crate > r) ? CRDOWN * crate : r;
    }
    double dcon = del * (crate < 1.0 ? crate : 1.0) / tol;
    if (dcon <= 1.0)
    {
      // ||ycor|| = ||delta|| after one iteration only when Newton started from 0
      acnrm = (mcur == 0 && !(LEARN && learned_start)) ? del : wrms(ycor);
      rv    = R_SUCCESS;
    }
    else if ((mcur >= 1) && (del > RDIV * delp)) rv = R_CONV_RECVR;
    else
    {
      delp = del;
      rv   = R_CONTINUE;
    }
    BDF_TOC(t0, T_NORM);
    return rv;
  }

  // SUNNonlinSolSolve_Newton (sunnonlinsol_newton.c:179)
  // have_res: w.delta already holds the residual at ycor (first pass only).
  __device__ int newton_solve(double* ycor, double tol, int callLSetup, bool have_res = false)
  {
    int jbad = 0, retval = R_SUCCESS;
    long niters = 0, nconvfails = 0;
    for (;;)
    {
      int curiter = 0;
      if (!have_res) nls_residual(ycor, w.delta);
      have_res = false;
      if (callLSetup)
      {
        retval = nls_lsetup(jbad);
        if (retval != R_SUCCESS) break;
      }
      for (;;)
      {
        niters++;
        for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.delta[i] = -w.delta[i];
        __syncwarp();
        nls_lsolve(w.delta);
        for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) ycor[i] = ycor[i] + w.delta[i];
        retval = nls_convtest(ycor, tol, curiter);
        curiter++;
        if (retval == R_SUCCESS)
        {
          nls_jcur = 0;
          nni += niters;
          nnf += nconvfails;
          return R_SUCCESS;
        }
        if (retval != R_CONTINUE) break;
        if (curiter >= NLS_MAXCOR)
        {
          retval = R_CONV_RECVR;
          break;
        }
        nls_residual(ycor, w.delta);
      }
      if (retval > 0 && !nls_jcur)
      {
        nconvfails++;
        callLSetup    = 1;
        jbad          = 1;
        learned_start = false;
        for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) ycor[i] = 0.0;
        continue;
      }
      break;
    }
    nconvfails++;
    nni += niters;
    nnf += nconvfails;
    return retval;
  }

  // ------------------------------------------------------------ step pieces
  __device__ void rescale()
  {  // cvRescale (cvode.c:2718)
    double c = eta;
    for (int j = 1; j <= q; j++)
    {
      for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.zn[j][i] *= c;
      c = eta * c;
    }
    h      = hscale * eta;
    next_h = h;
    hscale = h;
    nscon  = 0;
  }

  __device__ void increase_bdf()
  {  // cvIncreaseBDF (cvode.c:2632)
    double alpha0, alpha1, prod, xi, xiold, hsum, A1;
    for (int i = 0; i <= QMAX; i++) l[i] = 0.0;
    l[2] = alpha1 = prod = xiold = 1.0;
    alpha0                       = -1.0;
    hsum                         = hscale;
    if (q > 1)
      for (int j = 1; j < q; j++)
      {
        hsum += tau[j + 1];
        xi = hsum / hscale;
        prod *= xi;
        alpha0 -= inv_int(j + 1);
        alpha1 += 1.0 / xi;
        for (int i = j + 2; i >= 2; i--) l[i] = l[i] * xiold + l[i - 1];
        xiold = xi;
      }
    A1 = (-alpha0 - alpha1) / prod;
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.zn[L][i] = A1 * w.zn[indx_acor][i];
    if (q > 1)
      for (int j = 2; j <= q; j++)
        for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.zn[j][i] += l[j] * w.zn[L][i];
  }

  __device__ void decrease_bdf()
  {  // cvDecreaseBDF (cvode.c:2679)
    double hsum, xi;
    for (int i = 0; i <= QMAX; i++) l[i] = 0.0;
    l[2] = 1.0;
    hsum = 0.0;
    for (int j = 1; j <= q - 2; j++)
    {
      hsum += tau[j];
      xi = hsum / hscale;
      for (int i = j + 2; i >= 2; i--) l[i] = l[i] * xi + l[i - 1];
    }
    if (q > 2)
      for (int j = 2; j < q; j++)
      {
        const double c = -l[j];
        for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.zn[j][i] += c * w.zn[q][i];
      }
  }

  __device__ void adjust_order(int deltaq)
  {
    if ((q == 2) && (deltaq != 1)) return;
    if (deltaq == 1) increase_bdf();
    else if (deltaq == -1) decrease_bdf();
  }

  __device__ void adjust_params()
  {
    if (qprime != q)
    {
      adjust_order(qprime - q);
      q     = qprime;
      L     = q + 1;
      qwait = L;
    }
    rescale();
  }

  __device__ void predict()
  {  // cvPredict (cvode.c:2748)
    tn += h;
    for (int k = 1; k <= q; k++)
      for (int j = q; j >= k; j--)
        for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.zn[j - 1][i] = w.zn[j - 1][i] + w.zn[j][i];
  }

  __device__ void restore(double saved_t)
  {  // cvRestore (cvode.c:3315)
    tn = saved_t;
    for (int k = 1; k <= q; k++)
      for (int j = q; j >= k; j--)
        for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.zn[j - 1][i] = w.zn[j - 1][i] - w.zn[j][i];
  }

  __device__ void set_tq_bdf(double hsum, double alpha0, double alpha0_hat, double xi_inv,
                             double xistar_inv)
  {  // cvSetTqBDF (cvode.c:3022)
    double A1 = 1.0 - alpha0_hat + alpha0;
    double A2 = 1.0 + q * A1;
    tq[2]     = fabs(A1 / (alpha0 * A2));
    tq[5]     = fabs(A2 * xistar_inv / (l[q] * xi_inv));
    if (qwait == 1)
    {
      if (q > 1)
      {
        double C     = xistar_inv / l[q];
        double A3    = alpha0 + inv_int(q);
        double A4    = alpha0_hat + xi_inv;
        double Cpinv = (1.0 - A4 + A3) / A3;
        tq[1]        = fabs(C * Cpinv);
      }
      else tq[1] = 1.0;
      hsum += tau[q];
      xi_inv        = h / hsum;
      double A5     = alpha0 - inv_int(q + 1);
      double A6     = alpha0_hat - xi_inv;
      double Cppinv = (1.0 - A6 + A5) / A2;
      tq[3]         = fabs(Cppinv / (xi_inv * (q + 2) * A5));
    }
    tq[4] = CORTES / tq[2];
  }

  __device__ void set_bdf()
  {  // cvSetBDF (cvode.c:2962)
    double alpha0, alpha0_hat, xi_inv, xistar_inv, hsum;
    l[0] = l[1] = xi_inv = xistar_inv = 1.0;
    for (int i = 2; i <= q; i++) l[i] = 0.0;
    alpha0 = alpha0_hat = -1.0;
    hsum                = h;
    if (q > 1)
    {
      for (int j = 2; j < q; j++)
      {
        hsum += tau[j - 1];
        xi_inv = h / hsum;
        alpha0 -= inv_int(j);
        for (int i = j; i >= 1; i--) l[i] += l[i - 1] * xi_inv;
      }
      alpha0 -= inv_int(q);
      xistar_inv = -l[1] - alpha0;
      hsum += tau[q - 1];
      xi_inv     = h / hsum;
      alpha0_hat = -l[1] - xi_inv;
      for (int i = q; i >= 1; i--) l[i] += l[i - 1] * xistar_inv;
    }
    set_tq_bdf(hsum, alpha0, alpha0_hat, xi_inv, xistar_inv);
  }

  // cvSetBDF + cvSetTqBDF with their independent divisions spread over
  // lanes (fast modes): every quotient has the same operands and rounding as
  // in set_bdf / set_tq_bdf, but each round of divisions costs one warp
  // instruction sequence instead of one per quotient.
  __device__ void set_bdf_lanes()
  {
    // hsum_m = h + tau[1] + ... + tau[m-1] (the reference's summation order),
    // xi_inv_m = h / hsum_m for m = 2 .. q+1, on lane m
    double hs = h, my_hsum = h;
    for (int m = 2; m <= q + 1; m++)
    {
      hs += tau[m - 1];
      if (lane == m) my_hsum = hs;
    }
    const double my_xi = h / my_hsum;
    // l[i] on lane i: l[0] = l[1] = 1, then for j = 2..q-1 l[i] += l[i-1] * xi_inv_j
    double li = (lane <= 1) ? 1.0 : 0.0;
    double alpha0 = -1.0, alpha0_hat = -1.0, xi_inv = 1.0, xistar_inv = 1.0, hsum = h;
    if (q > 1)
    {
      for (int j = 2; j < q; j++)
      {
        hsum += tau[j - 1];
        xi_inv = __shfl_sync(0xffffffffu, my_xi, j);
        alpha0 -= inv_int(j);
        const double lm1 = __shfl_up_sync(0xffffffffu, li, 1);
        if (lane >= 1 && lane <= j) li += lm1 * xi_inv;
      }
      alpha0 -= inv_int(q);
      const double l1 = __shfl_sync(0xffffffffu, li, 1);
      xistar_inv      = -l1 - alpha0;
      hsum += tau[q - 1];
      xi_inv     = __shfl_sync(0xffffffffu, my_xi, q);
      alpha0_hat = -l1 - xi_inv;
      const double lm1 = __shfl_up_sync(0xffffffffu, li, 1);
      if (lane >= 1 && lane <= q) li += lm1 * xistar_inv;
    }
#pragma unroll
    for (int i = 0; i <= QMAX; i++) l[i] = __shfl_sync(0xffffffffu, li, i);
    // cvSetTqBDF: first round of quotients
    const double A1  = 1.0 - alpha0_hat + alpha0;
    const double A2  = 1.0 + q * A1;
    const double A3  = alpha0 + inv_int(q);
    const double A4  = alpha0_hat + xi_inv;
    const double xq1 = __shfl_sync(0xffffffffu, my_xi, q + 1);  // h / (hsum + tau[q])
    const double A5  = alpha0 - inv_int(q + 1);
    const double A6  = alpha0_hat - xq1;
    double num = 1.0, den = 1.0;
    switch (lane)
    {
    case 0: num = A1; den = alpha0 * A2; break;                    // tq[2]
    case 1: num = A2 * xistar_inv; den = l[q] * xi_inv; break;     // tq[5]
    case 2: num = xistar_inv; den = l[q]; break;                   // C
    case 3: num = 1.0 - A4 + A3; den = A3; break;                  // Cpinv
    case 4: num = 1.0 - A6 + A5; den = A2; break;                  // Cppinv
    case 5: num = 1.0; den = l[1]; break;                          // rl1
    default: break;
    }
    const double qt    = num / den;
    tq[2]              = fabs(__shfl_sync(0xffffffffu, qt, 0));
    tq[5]              = fabs(__shfl_sync(0xffffffffu, qt, 1));
    const double C     = __shfl_sync(0xffffffffu, qt, 2);
    const double Cpinv = __shfl_sync(0xffffffffu, qt, 3);
    const double Cpp   = __shfl_sync(0xffffffffu, qt, 4);
    rl1                = __shfl_sync(0xffffffffu, qt, 5);
    gamma              = h * rl1;
    if (nst == 0) gammap = gamma;
    // second round: tq[4], tq[3], gamrat
    num = 1.0;
    den = 1.0;
    switch (lane)
    {
    case 0: num = CORTES; den = tq[2]; break;
    case 1: num = Cpp; den = xq1 * (q + 2) * A5; break;
    case 2: num = gamma; den = gammap; break;
    default: break;
    }
    const double qt2 = num / den;
    tq[4]            = __shfl_sync(0xffffffffu, qt2, 0);
    if (qwait == 1)
    {
      tq[1] = (q > 1) ? fabs(C * Cpinv) : 1.0;
      tq[3] = fabs(__shfl_sync(0xffffffffu, qt2, 1));
    }
    gamrat = (nst > 0) ? __shfl_sync(0xffffffffu, qt2, 2) : 1.0;
  }

  __device__ void set_coeffs()
  {  // cvSet (cvode.c:2791)
    BDF_TIC(t0);
    if (!EXACT)
    {
      set_bdf_lanes();
      BDF_TOC(t0, T_SETC);
      return;
    }
    set_bdf();
    rl1   = 1.0 / l[1];
    gamma = h * rl1;
    if (nst == 0) gammap = gamma;
    gamrat = (nst > 0) ? gamma / gammap : 1.0;
    BDF_TOC(t0, T_SETC);
  }

  __device__ int nls(int nflag)
  {  // cvNls (cvode.c:3068)
    convfail      = ((nflag == FIRST_CALL) || (nflag == PREV_ERR_FAIL)) ? NO_FAILURES : FAIL_OTHER;
    int callSetup = (nflag == PREV_CONV_FAIL) || (nflag == PREV_ERR_FAIL) || (nst == 0) ||
                    (nst >= nstlp + MSBP) || (fabs(gamrat - 1.0) > DGMAX_LSETUP);
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.acor[i] = 0.0;
    bool have_res = false;
    learned_start = false;
    float xr[5];
    const bool learn = LEARN && !EXACT && (P.mlp_w != nullptr || P.rec_x != nullptr);
    if (learn) mlp_features(xr);
    if (LEARN && !EXACT && P.mlp_w)
    {
      // learned initial iterate; kept only if its residual is the smaller
      float o0, o1;
      gb300mlp::warp_forward(P.mlp_w, P.mlp_b, xr, lane, o0, o1);
      nlp++;
      __syncwarp();
      if (2 * lane < n) w.acor[2 * lane] = (double)(o0 / (float)w.ewt[2 * lane]);
      if (2 * lane + 1 < n) w.acor[2 * lane + 1] = (double)(o1 / (float)w.ewt[2 * lane + 1]);
      __syncwarp();
      nls_residual(w.acor, w.delta);
      const double rl = wrms(w.delta);
      nls_residual0(w.tempv);
      const double r0 = wrms(w.tempv);
      learned_start = rl < r0;
      if (learned_start) nlpu++;
      else
        for (int i = lane; i < n && (NB > 32 || i < 32); i += 32)
        {
          w.acor[i]  = 0.0;
          w.delta[i] = w.tempv[i];
        }
      __syncwarp();
      have_res = true;
    }
    int flag = newton_solve(w.acor, tq[4], callSetup, have_res);
    if (flag != R_SUCCESS) return flag;
    if (LEARN && !EXACT && P.rec_x)
    {
      // training pair: features and the converged corrector in error-weight units
      unsigned long long idx = 0;
      if (lane == 0) idx = atomicAdd(P.rec_count, 1ull);
      idx = __shfl_sync(0xffffffffu, idx, 0);
      if ((long long)idx < P.rec_cap)
      {
        uint16_t* rx = P.rec_x + idx * gb300mlp::INP;
        float* rtg   = P.rec_t + idx * gb300mlp::OUT;
#pragma unroll
        for (int c = 0; c < 5; ++c)
          if (32 * c + lane < gb300mlp::INP)
            rx[32 * c + lane] = __bfloat16_as_ushort(__float2bfloat16_rn(xr[c]));
        for (int i = lane; i < gb300mlp::OUT; i += 32)
          rtg[i] = i < n ? (float)(w.acor[i] * w.ewt[i]) : 0.0f;
      }
    }
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.y[i] = w.zn[0][i] + w.acor[i];
    cv_jcur = 0;
    return R_SUCCESS;
  }

  __device__ int handle_nflag(int* nflagPtr, double saved_t, int* ncfPtr)
  {  // cvHandleNFlag (cvode.c:3257); hmin = 0
    int nflag = *nflagPtr;
    if (nflag == R_SUCCESS) return DO_ERROR_TEST;
    ncfn++;
    restore(saved_t);
    (*ncfPtr)++;
    etamax = 1.0;
    if (*ncfPtr == MXNCF) return CV_CONV_FAILURE;
    eta       = ETA_CF;
    *nflagPtr = PREV_CONV_FAIL;
    rescale();
    return PREDICT_AGAIN;
  }

  __device__ int do_error_test(int* nflagPtr, double saved_t, int* nefPtr, double* dsmPtr)
  {  // cvDoErrorTest (cvode.c:3359); hmin = 0
    double dsm = acnrm * tq[2];
    *dsmPtr    = dsm;
    if (dsm <= 1.0) return CV_SUCCESS;
    (*nefPtr)++;
    netf++;
    *nflagPtr = PREV_ERR_FAIL;
    restore(saved_t);
    if (*nefPtr == MXNEF) return CV_ERR_FAILURE;
    etamax = 1.0;
    if (*nefPtr <= MXNEF1)
    {
      eta = 1.0 / (cv_root<EXACT>(BIAS2 * dsm, L) + ADDON);
      eta = dmax(ETA_MIN_EF, dmax(eta, 0.0));
      if (*nefPtr >= SMALL_NEF) eta = dmin(eta, ETA_MAX_EF);
      rescale();
      return TRY_AGAIN;
    }
    if (q > 1)
    {
      eta = ETA_MIN_EF;
      adjust_order(-1);
      L = q;
      q--;
      qwait = L;
      rescale();
      return TRY_AGAIN;
    }
    eta = ETA_MIN_EF;
    h *= eta;
    next_h = h;
    hscale = h;
    qwait  = LONG_WAIT;
    nscon  = 0;
    rhs(w.zn[0], w.tempv);
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.zn[1][i] = h * w.tempv[i];
    return TRY_AGAIN;
  }

  __device__ void complete_step()
  {  // cvCompleteStep (cvode.c:3467)
    nst++;
    nscon++;
    hu = h;
    qu = q;
    for (int i = q; i >= 2; i--) tau[i] = tau[i - 1];
    if ((q == 1) && (nst > 1)) tau[2] = tau[1];
    tau[1] = h;
    for (int j = 0; j <= q; j++)
    {
      const double c = l[j];
      for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.zn[j][i] += c * w.acor[i];
    }
    qwait--;
    if ((qwait == 1) && (q != QMAX))
    {
      for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.zn[QMAX][i] = w.acor[i];
      saved_tq5 = tq[5];
      indx_acor = QMAX;
    }
  }

  __device__ void set_eta()
  {  // cvSetEta (cvode.c:3579); eta_min_fx = 0, hmin = 0, hmax_inv = 0
    if ((eta > 0.0) && (eta < ETA_MAX_FX))
    {
      eta    = 1.0;
      hprime = h;
    }
    else
    {
      if (eta >= ETA_MAX_FX)
      {
        eta = dmin(eta, etamax);
        eta /= 1.0;
      }
      else
      {
        eta = dmax(eta, ETA_MIN);
        eta = dmax(eta, 0.0);
      }
      hprime = h * eta;
      if (qprime < q) nscon = 0;
    }
  }

  __device__ double compute_etaqm1()
  {
    etaqm1 = 0.0;
    if (q > 1)
    {
      double ddn = wrms(w.zn[q]) * tq[1];
      etaqm1     = 1.0 / (cv_root<EXACT>(BIAS1 * ddn, q) + ADDON);
    }
    return etaqm1;
  }

  __device__ double compute_etaqp1()
  {
    etaqp1 = 0.0;
    if (q != QMAX)
    {
      if (saved_tq5 == 0.0) return etaqp1;
      double base = h / tau[2], p = 1.0;
      for (int i = 1; i <= L; i++) p *= base;  // SUNRpowerI
      double cquot   = (tq[5] / saved_tq5) * p;
      const double a = -cquot;
      for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.tempv[i] = (a * w.zn[QMAX][i]) + w.acor[i];
      double dup = wrms(w.tempv) * tq[3];
      etaqp1     = 1.0 / (cv_root<EXACT>(BIAS3 * dup, L + 1) + ADDON);
    }
    return etaqp1;
  }

  __device__ void choose_eta()
  {  // cvChooseEta (cvode.c:3670)
    double etam = dmax(etaqm1, dmax(etaq, etaqp1));
    if ((etam > 0.0) && (etam < ETA_MAX_FX))
    {
      eta    = 1.0;
      qprime = q;
    }
    else if (etam == etaq)
    {
      eta    = etaq;
      qprime = q;
    }
    else if (etam == etaqm1)
    {
      eta    = etaqm1;
      qprime = q - 1;
    }
    else
    {
      eta    = etaqp1;
      qprime = q + 1;
      for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.zn[QMAX][i] = w.acor[i];
    }
  }

  __device__ void prepare_next_step(double dsm)
  {  // cvPrepareNextStep (cvode.c:3530)
    if (etamax == 1.0)
    {
      qwait  = qwait > 2 ? qwait : 2;
      qprime = q;
      hprime = h;
      eta    = 1.0;
      return;
    }
    etaq = 1.0 / (cv_root<EXACT>(BIAS2 * dsm, L) + ADDON);
    if (qwait != 0)
    {
      eta    = etaq;
      qprime = q;
      set_eta();
    }
    else
    {
      qwait  = 2;
      etaqm1 = compute_etaqm1();
      etaqp1 = compute_etaqp1();
      choose_eta();
      set_eta();
    }
  }

  __device__ int step()
  {  // cvStep (cvode.c:2367)
    double saved_t, dsm = 0.0;
    int ncf = 0, nef = 0, nflag, kflag, eflag;
    if ((nst > 0) && (hprime != h)) adjust_params();
    saved_t = tn;
    nflag   = FIRST_CALL;
    for (;;)
    {
      predict();
      set_coeffs();
      nflag = nls(nflag);
      kflag = handle_nflag(&nflag, saved_t, &ncf);
      if (kflag == PREDICT_AGAIN) continue;
      if (kflag != DO_ERROR_TEST) return kflag;
      eflag = do_error_test(&nflag, saved_t, &nef, &dsm);
      if (eflag == TRY_AGAIN) continue;
      if (eflag != CV_SUCCESS) return eflag;
      break;
    }
    BDF_TIC(t0);
    complete_step();
    prepare_next_step(dsm);
    BDF_TOC(t0, T_PREP);
    etamax = (nst <= SMALL_NST) ? ETA_MAX_ES : ETA_MAX_GS;
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.acor[i] *= tq[2];
    return CV_SUCCESS;
  }

  // ------------------------------------------------------------ initial step
  __device__ double upper_bound_h0(double tdist)
  {  // cvUpperBoundH0 (cvode.c:2278)
    double* temp1 = w.tempv;
    double* temp2 = w.acor;
    double loc    = 0.0;
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) temp2[i] = fabs(w.zn[0][i]);
    set_ewt(w.zn[0], temp1);
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32)
    {
      double t1 = 1.0 / temp1[i];
      t1        = t1 + HUB_FACTOR * temp2[i];
      double t2 = fabs(w.zn[1][i]);
      t1        = t2 / t1;
      temp1[i]  = t1;
      loc       = fabs(t1) > loc ? fabs(t1) : loc;
    }
    double hub_inv = warp_max(loc);
    double hub     = HUB_FACTOR * tdist;
    if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
    return hub;
  }

  __device__ double ydd_norm(double hg)
  {  // cvYddNorm (cvode.c:2323)
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.y[i] = (hg * w.zn[1][i]) + w.zn[0][i];
    rhs(w.y, w.tempv);
    const double a = 1.0 / hg, b = -1.0 / hg;
    const bool sdiff = (a == -b) && (a != 1.0) && (a != -1.0);
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32)
      w.tempv[i] = sdiff ? a * (w.tempv[i] - w.zn[1][i]) : (a * w.tempv[i]) + (b * w.zn[1][i]);
    return wrms(w.tempv);
  }

  __device__ void hin(double tout)
  {  // cvHin (cvode.c:2161); the right-hand side never fails here
    double tdiff = tout - tn, hnew = 0.0;
    int sign      = (tdiff > 0.0) ? 1 : -1;
    double tdist  = fabs(tdiff);
    double tround = UROUND * dmax(fabs(tn), fabs(tout));
    double hlb    = HLB_FACTOR * tround;
    double hub    = upper_bound_h0(tdist);
    double hg     = rsqrt_sun(hlb * hub);
    if (hub < hlb)
    {
      h = sign == -1 ? -hg : hg;
      return;
    }
    for (int count1 = 1; count1 <= MAX_ITERS; count1++)
    {
      double yddnrm = ydd_norm(hg * sign);
      hnew          = (yddnrm * hub * hub > 2.0) ? rsqrt_sun(2.0 / yddnrm) : rsqrt_sun(hg * hub);
      if (count1 == MAX_ITERS) break;
      double hrat = hnew / hg;
      if ((hrat > 0.5) && (hrat < 2.0)) break;
      if ((count1 > 1) && (hrat > 2.0))
      {
        hnew = hg;
        break;
      }
      hg = hnew;
    }
    double h0 = 0.5 * hnew;
    if (h0 < hlb) h0 = hlb;
    if (h0 > hub) h0 = hub;
    if (sign == -1) h0 = -h0;
    h = h0;
  }

  // CVodeGetDky(t, 0) (cvode.c:1671)
  __device__ void get_dky(double t, double* out)
  {
    double s = (t - tn) / h;
    double c[QMAX + 1];
    int js[QMAX + 1];
    int nvec = 0;
    for (int j = q; j >= 0; j--)
    {
      c[nvec] = 1.0;
      for (int i = 0; i < j; i++) c[nvec] *= s;
      js[nvec] = j;
      nvec++;
    }
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32)
    {
      double v;
      if (nvec == 2) v = (c[0] * w.zn[js[0]][i]) + (c[1] * w.zn[js[1]][i]);
      else
      {
        v = c[0] * w.zn[js[0]][i];
        for (int k = 1; k < nvec; k++) v += c[k] * w.zn[js[k]][i];
      }
      out[i] = v;
    }
  }

  // ------------------------------------------------------------ one system
  __device__ void run(int64_t s, double* scratch, int* pivbuf)
  {
    const DevProblem& p = P.p;
    n    = p.n[s];
    nr   = (int)(p.r_off[s + 1] - p.r_off[s]);
    rt   = p.rtype + p.r_off[s];
    ra   = p.ra + p.r_off[s];
    rb   = p.rb + p.r_off[s];
    rc   = p.rc + p.r_off[s];
    rk   = p.rk + p.r_off[s];
    fptr = p.fptr + p.y_off[s] + s;
    fent = p.fent + p.e_off[s];
    jptr = p.jptr + p.y_off[s] + s;
    jent = p.jent + p.je_off[s];
    J     = scratch;
    J32   = (float*)(scratch + SLOT_J);
    ld    = n | 1;
    lr    = (n + 3) & ~3;
    if (((lr >> 2) & 1) == 0) lr += 4;
    piv   = pivbuf;
    rdiag = w.rdiag;
    two   = n > 32;
    inv_n = 1.0 / n;

    const double* y0 = P.y0 + p.y_off[s];
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.zn[0][i] = y0[i];
    tn = P.t0;
    h = hscale = hprime = next_h = eta = etaq = etaqm1 = etaqp1 = hu = h0u = 0.0;
    next_q = 0;
    saved_tq5 = rl1 = gamma = gammap = gamrat = crate = delp = acnrm = 0.0;
    for (int i = 0; i < 6; i++) tq[i] = 0.0;
    for (int i = 0; i < QMAX + 2; i++) l[i] = tau[i] = 0.0;
    q = 1;
    L = 2;
    qwait = L;
    qprime = 0;
    indx_acor = 0;
    nscon = convfail = qu = 0;
    nls_jcur = cv_jcur = 0;
    etamax = ETA_MAX_FS;
    nst = nfe = nsetups = nje = nni = ncfn = netf = nnf = nstlp = nstlj = 0;
    nlp = nlpu    = 0;
    learned_start = false;
    int istate = CV_SUCCESS;
    const double tout = P.tout;

    set_ewt(w.zn[0], w.ewt);
    rhs(w.zn[0], w.zn[1]);
    hin(tout);
    hscale = h;
    hprime = h;
    h0u    = h;
    for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) w.zn[1][i] *= h;

    long nstloc = 0;
    BDF_TIC(tall);
    for (;;)
    {
      next_h = h;
      next_q = q;
      if (nst > 0) set_ewt(w.zn[0], w.ewt);
      if ((P.mxstep > 0) && (nstloc >= P.mxstep))
      {
        istate = CV_TOO_MUCH_WORK;
        break;
      }
      // ewt was just set from zn[0], so each weighted term is below 1/rtol and
      // UROUND * ||zn[0]|| exceeds 1 only if rtol < UROUND: the fast modes
      // skip the norm when rtol >= 1e-12 (the exact mode always takes it).
      if (EXACT || P.rtol < 1e-12)
      {
        double nrm = wrms(w.zn[0]);
        if (UROUND * nrm > 1.0)
        {
          istate = CV_TOO_MUCH_ACC;
          break;
        }
      }
      int kflag = step();
      if (kflag != CV_SUCCESS)
      {
        istate = kflag;
        break;
      }
      nstloc++;
      if ((tn - tout) * h >= 0.0)
      {
        next_q = qprime;
        next_h = hprime;
        break;
      }
    }
    BDF_TOC(tall, T_OTHER);
    double* yo = P.yout + p.y_off[s];
    if (istate == CV_SUCCESS) get_dky(tout, yo);
    else
      for (int i = lane; i < n && (NB > 32 || i < 32); i += 32) yo[i] = w.zn[0][i];
    if (lane == 0 && P.stats)
    {
      SUNBatchBDFStats st;
      st.nst     = nst;
      st.nfe     = nfe;
      st.nsetups = nsetups;
      st.nje     = nje;
      st.nni     = nni;
      st.ncfn    = ncfn;
      st.netf    = netf;
      st.nnf     = nnf;
      st.flag    = istate;
      st.qu      = qu;
      st.tn      = tn;
      st.hu      = hu;
      st.h0u     = h0u;
      st.next_h  = next_h;
      st.next_q  = next_q;
      P.stats[s] = st;
    }
    if (lane == 0 && P.fail_list && istate != CV_SUCCESS)
      P.fail_list[atomicAdd(P.fail_count, 1u)] = (int32_t)s;
    if (lane == 0 && P.lp_counts && nlp > 0)
    {
      atomicAdd(P.lp_counts, (unsigned long long)nlp);
      atomicAdd(P.lp_counts + 1, (unsigned long long)nlpu);
    }
    __syncwarp();
  }
};

// Persistent kernel, one warp per block: each warp takes the next system of
// its size bucket (n <= NB) from the bucket's queue until the queue is empty
// (no waiting on other warps or blocks).  Dynamic shared memory holds the
// warp's vectors and its Newton matrix.
template <int MODE, int NB, bool LEARN = false>
__global__ void __launch_bounds__(32, Layout<MODE, NB>::min_blocks)
  k_batch_bdf(Params P, const int32_t* order, int64_t count, unsigned int* next)
{
  extern __shared__ __align__(16) unsigned char smem[];
  using L          = Layout<MODE, NB>;
  const int lane   = threadIdx.x & 31;
  const int slot   = blockIdx.x;
  double* scratch  = P.scratch + (size_t)slot * SLOT_DOUBLES;
  int* pivbuf      = P.pivots + (size_t)slot * NMAX;
  WarpMem<NB>* mem = (WarpMem<NB>*)smem;
  void* mat        = L::mat_in_smem ? (void*)(smem + L::mem_bytes) : (void*)(scratch + SLOT_J);
  Integrator<MODE, NB, LEARN> I(P, *mem, mat, lane);
  if (P.count_dev)
  {  // a retry launch: its queue length was produced on the device
    const int64_t c = (int64_t)*P.count_dev;
    count           = c < count ? c : count;
  }
  for (;;)
  {
    unsigned int idx = 0;
    if (lane == 0) idx = atomicAdd(next, 1u);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if ((int64_t)idx >= count) break;
    I.run(order[idx], scratch, pivbuf);
  }
#ifdef SUNGB300_BDF_TIMERS
  if (lane == 0 && P.timers)
    for (int t = 0; t < T_COUNT; t++) P.timers[(size_t)slot * T_COUNT + t] += I.tacc[t];
#endif
}

// Host-side launch and occupancy of the fast modes' kernels (FP64, MIXED);
// each translation unit instantiates one LEARN variant.  The kernel's
// shared-memory limit is set by fast_occupancy at creation.
template <int MODE, int NB, bool LEARN>
cudaError_t fast_launch_one(const Params& P, int grid, cudaStream_t stream, const int32_t* order,
                            int64_t count, unsigned int* next)
{
  const size_t smem = Layout<MODE, NB>::warp_bytes;
  k_batch_bdf<MODE, NB, LEARN><<<grid, 32, smem, stream>>>(P, order, count, next);
  return cudaGetLastError();
}

template <int MODE, int NB, bool LEARN>
cudaError_t fast_occ_one(int* per_sm)
{
  const size_t smem = Layout<MODE, NB>::warp_bytes;
  cudaFuncSetAttribute(k_batch_bdf<MODE, NB, LEARN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k_batch_bdf<MODE, NB, LEARN>, 32,
                                                       smem);
}

template <bool LEARN>
cudaError_t fast_launch(const Params& P, int mode, int nb, int grid, cudaStream_t stream,
                        const int32_t* order, int64_t count, unsigned int* next)
{
  constexpr int M = SUNBATCHBDF_MIXED, F = SUNBATCHBDF_FP64;
  if (mode == M)
    return nb <= 32   ? fast_launch_one<M, 32, LEARN>(P, grid, stream, order, count, next)
           : nb <= 48 ? fast_launch_one<M, 48, LEARN>(P, grid, stream, order, count, next)
                      : fast_launch_one<M, 64, LEARN>(P, grid, stream, order, count, next);
  return nb <= 32   ? fast_launch_one<F, 32, LEARN>(P, grid, stream, order, count, next)
         : nb <= 48 ? fast_launch_one<F, 48, LEARN>(P, grid, stream, order, count, next)
                    : fast_launch_one<F, 64, LEARN>(P, grid, stream, order, count, next);
}

template <bool LEARN>
cudaError_t fast_occupancy(int mode, int nb, int* per_sm)
{
  constexpr int M = SUNBATCHBDF_MIXED, F = SUNBATCHBDF_FP64;
  if (mode == M)
    return nb <= 32   ? fast_occ_one<M, 32, LEARN>(per_sm)
           : nb <= 48 ? fast_occ_one<M, 48, LEARN>(per_sm)
                      : fast_occ_one<M, 64, LEARN>(per_sm);
  return nb <= 32   ? fast_occ_one<F, 32, LEARN>(per_sm)
         : nb <= 48 ? fast_occ_one<F, 48, LEARN>(per_sm)
                    : fast_occ_one<F, 64, LEARN>(per_sm);
}

}  // namespace bdf

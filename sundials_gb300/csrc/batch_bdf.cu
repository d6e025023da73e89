// batch_bdf.cu -- host side of SUNBatchBDF_GB300: problem upload, the
// species/reactant indexes the device right-hand side and Jacobian walk, the
// processing order, per-warp scratch, and the persistent launch.
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "../../include/sunbatchbdf_gb300.h"
#include "batch_bdf_kernel.cuh"
#include "gb300_common.cuh"

namespace bdf {
cudaError_t launch_fast(const Params& P, int mode, int nb, int grid, cudaStream_t stream,
                        const int32_t* order, int64_t count, unsigned int* next);
cudaError_t occupancy_fast(int mode, int nb, int* per_sm);
cudaError_t launch_fast_learn(const Params& P, int mode, int nb, int grid, cudaStream_t stream,
                              const int32_t* order, int64_t count, unsigned int* next);
cudaError_t occupancy_fast_learn(int mode, int nb, int* per_sm);
cudaError_t launch_exact(const Params& P, int nb, int grid, cudaStream_t stream,
                         const int32_t* order, int64_t count, unsigned int* next);
cudaError_t occupancy_exact(int nb, int* per_sm);
}  // namespace bdf

// Systems are sorted into size classes n <= 32, 32 < n <= 48, 48 < n <= 64;
// each class (or, in the FP64 modes, n <= 32 and n > 32) is one persistent
// launch whose shared memory is sized for it (see plan()).

using namespace bdf;

struct SUNBatchBDF_GB300_
{
  cudaStream_t stream;
  int64_t nsys, Y, R;
  DevProblem dp;
  std::vector<void*> allocs;
  double rtol = 1e-6, atol = 1e-12;
  long mxstep  = 1000000;
  int mode     = SUNBATCHBDF_FP64;
  int refine   = 1;
  double* d_y0 = nullptr;
  double* d_yout = nullptr;
  SUNBatchBDFStats* d_stats = nullptr;
  unsigned int* d_next = nullptr;
  double* d_scratch = nullptr;
  int* d_piv = nullptr;
  long long* d_timers = nullptr;
  int slots = 0;
  const int32_t* d_order[3] = {nullptr, nullptr, nullptr};  // n <= 32, <= 48, <= 64
  int64_t count[3]          = {0, 0, 0};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  float last_ms = 0.f;

  // learned predictor and training-data recorder
  const uint16_t* mlp_w = nullptr;
  const float* mlp_b    = nullptr;
  unsigned long long* d_lp = nullptr;  // [2] predictor calls, learned iterate kept
  uint16_t* rec_x = nullptr;
  float* rec_t    = nullptr;
  unsigned long long* rec_count = nullptr;
  long long rec_cap = 0;
  // retry of failed systems (fast modes): mode of the retry launch, or -1
  int retry_mode   = -2;  // the other fast mode
  int per_sm[3][3] = {};   // [mode][width class] resident warps per SM
  int per_sm_learn[3][3] = {};  // the same for the kernels with the learned predictor
  int plan_id[3]   = {0, 0, 1};  // launch plan per mode (index into kPlanWidths)
  std::vector<int32_t> h_order;   // systems by decreasing n (host copy, for sampling)

  int32_t* d_fail  = nullptr;  // [nsys] ids of failed systems
};

namespace {

template <class T>
T* upload(SUNBatchBDF_GB300 b, const T* h, size_t count)
{
  T* d = nullptr;
  if (!gb300::check_cuda(cudaMalloc(&d, sizeof(T) * (count ? count : 1)), "cudaMalloc(batch)"))
    return nullptr;
  b->allocs.push_back(d);
  if (count && !gb300::check_cuda(cudaMemcpy(d, h, sizeof(T) * count, cudaMemcpyHostToDevice),
                                  "cudaMemcpy(batch)"))
    return nullptr;
  return d;
}

bool is_device_ptr(const void* p)
{
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
  {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

constexpr int kBuckets = 3;

// Resident warps per SM of every (mode, width) instantiation, queried once at
// creation (the query also sets each kernel's dynamic shared-memory limit), so
// that SolveAsync makes no such call and can be captured into a CUDA graph.
inline int width_index(int nb) { return nb <= 32 ? 0 : nb <= 48 ? 1 : 2; }

bool query_occupancy(SUNBatchBDF_GB300 b)
{
  const int widths[3] = {32, 48, 64};
  for (int mode : {SUNBATCHBDF_FP64, SUNBATCHBDF_FP64_EXACT, SUNBATCHBDF_MIXED})
    for (int k = 0; k < 3; k++)
    {
      int per_sm    = 0;
      cudaError_t e = (mode == SUNBATCHBDF_FP64_EXACT) ? occupancy_exact(widths[k], &per_sm)
                                                       : occupancy_fast(mode, widths[k], &per_sm);
      if (!gb300::check_cuda(e, "k_batch_bdf occupancy")) return false;
      b->per_sm[mode][k] = per_sm < 1 ? 1 : per_sm;
      if (mode != SUNBATCHBDF_FP64_EXACT)
      {
        int pl = 0;
        if (!gb300::check_cuda(occupancy_fast_learn(mode, widths[k], &pl),
                               "k_batch_bdf occupancy"))
          return false;
        b->per_sm_learn[mode][k] = pl < 1 ? 1 : pl;
      }
    }
  return true;
}

// the predictor or the recorder is attached: the LEARN kernels run
inline bool uses_learn(const Params& P) { return P.mlp_w != nullptr || P.rec_x != nullptr; }

int grid_for(SUNBatchBDF_GB300 b, int mode, int nb, int64_t need)
{
  const bool learn = mode != SUNBATCHBDF_FP64_EXACT && (b->mlp_w || b->rec_x);
  int grid = gb300::num_sms() * (learn ? b->per_sm_learn : b->per_sm)[mode][width_index(nb)];
  if (need < grid) grid = (int)need;
  return grid < 1 ? 1 : grid;
}

// One persistent launch per size class, largest systems first.  A launch plan
// is a set of class widths (the last 64): class k takes the systems with
// n in (W[k-1], W[k]].  MIXED keeps an n x (n+4) FP32 inverse per warp in
// shared memory, so a 48-wide class (12 instead of 8 warps/SM) pays for its
// extra tail; the FP64 modes are register-limited at the same occupancy for
// every width.  Defaults: MIXED {32, 48, 64}, FP64 modes {32, 64};
// SUNBatchBDF_GB300_Autotune times every plan on a sample of the batch.
struct Launch
{
  int nb, grid;
  const int32_t* order;
  int64_t count;
  int queue;
};

constexpr int kPlans = 4;
const int kPlanWidths[kPlans][3] = {{32, 64, 0}, {32, 48, 64}, {48, 64, 0}, {64, 0, 0}};

// number of systems with n > w (the order is by decreasing n)
int64_t count_above(SUNBatchBDF_GB300 b, int w)
{
  if (w >= 64) return 0;
  if (w >= 48) return b->count[2];
  if (w >= 32) return b->count[2] + b->count[1];
  return b->nsys;
}

int plan_with(SUNBatchBDF_GB300 b, int mode, int plan_id, const int32_t* order_base, Launch* L)
{
  const int* W = kPlanWidths[plan_id];
  int nw = 0;
  while (nw < 3 && W[nw]) nw++;
  int nl = 0;
  for (int k = nw - 1; k >= 0; k--)
  {  // largest class first
    const int64_t hi = count_above(b, k ? W[k - 1] : 0);  // end (exclusive) in the order
    const int64_t lo = count_above(b, W[k]);
    if (hi - lo <= 0) continue;
    L[nl++] = {W[k], grid_for(b, mode, W[k], hi - lo), order_base + lo, hi - lo, k};
  }
  return nl;
}

int plan(SUNBatchBDF_GB300 b, int mode, Launch* L)
{
  return plan_with(b, mode, b->plan_id[mode], b->d_order[2], L);
}

bool ensure_scratch(SUNBatchBDF_GB300 b, int slots)
{
  if (slots <= b->slots) return true;
  if (!gb300::check_cuda(cudaMalloc(&b->d_scratch, sizeof(double) * SLOT_DOUBLES * (size_t)slots),
                         "cudaMalloc(scratch)") ||
      !gb300::check_cuda(cudaMalloc(&b->d_piv, sizeof(int) * NMAX * (size_t)slots),
                         "cudaMalloc(pivots)"))
    return false;
#ifdef SUNGB300_BDF_TIMERS
  if (!gb300::check_cuda(cudaMalloc(&b->d_timers, sizeof(long long) * T_COUNT * (size_t)slots),
                         "cudaMalloc(timers)") ||
      !gb300::check_cuda(cudaMemset(b->d_timers, 0, sizeof(long long) * T_COUNT * (size_t)slots),
                         "cudaMemset(timers)"))
    return false;
#endif
  b->slots = slots;
  return true;
}

}  // namespace

extern "C" {

SUNBatchBDF_GB300 SUNBatchBDF_GB300_Create(const SUNBatchBDFProblem* prob, void* cuda_stream)
{
  if (!prob || prob->nsys <= 0) return nullptr;
  const int64_t nsys = prob->nsys;
  for (int64_t s = 0; s < nsys; s++)
    if (prob->n[s] < 1 || prob->n[s] > NMAX ||
        prob->r_off[s + 1] - prob->r_off[s] > RMAX)
    {
      gb300::set_error(SUN_ERR_ARG_OUTOFRANGE, "system size outside 1..64 or > 128 reactions");
      return nullptr;
    }
  SUNBatchBDF_GB300 b = new SUNBatchBDF_GB300_();
  b->stream = (cudaStream_t)cuda_stream;
  b->nsys   = nsys;
  b->Y      = prob->y_off[nsys];
  b->R      = prob->r_off[nsys];

  // Species CSR (f) and reactant CSR (J), both in reaction order.
  std::vector<int32_t> fptr(b->Y + nsys), jptr(b->Y + nsys);
  std::vector<int64_t> e_off(nsys + 1, 0), je_off(nsys + 1, 0);
  std::vector<int32_t> fent, jent;
  fent.reserve(3 * b->R);
  jent.reserve(2 * b->R);
  std::vector<std::vector<int32_t>> fl(NMAX), jl(NMAX);
  for (int64_t s = 0; s < nsys; s++)
  {
    const int n = prob->n[s];
    for (int i = 0; i < n; i++)
    {
      fl[i].clear();
      jl[i].clear();
    }
    for (int64_t r = prob->r_off[s]; r < prob->r_off[s + 1]; r++)
    {
      const int lr = (int)(r - prob->r_off[s]);
      const int a = prob->ra[r], bb = prob->rb[r];
      if (prob->rtype[r] == 0)
      {
        fl[a].push_back(lr << 1 | 1);
        fl[bb].push_back(lr << 1);
        jl[a].push_back(lr << 1);
      }
      else
      {
        const int c = prob->rc[r];
        fl[a].push_back(lr << 1 | 1);
        fl[bb].push_back(lr << 1 | 1);
        fl[c].push_back(lr << 1);
        jl[a].push_back(lr << 1);
        jl[bb].push_back(lr << 1 | 1);
      }
    }
    const int64_t base = prob->y_off[s] + s;
    int32_t fo = 0, jo = 0;
    for (int i = 0; i < n; i++)
    {
      fptr[base + i] = fo;
      jptr[base + i] = jo;
      fent.insert(fent.end(), fl[i].begin(), fl[i].end());
      jent.insert(jent.end(), jl[i].begin(), jl[i].end());
      fo += (int32_t)fl[i].size();
      jo += (int32_t)jl[i].size();
    }
    fptr[base + n] = fo;
    jptr[base + n] = jo;
    e_off[s + 1]   = e_off[s] + fo;
    je_off[s + 1]  = je_off[s] + jo;
  }
  // Within each size bucket, largest systems first (cost grows like n^3).
  std::vector<int32_t> order(nsys);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t x, int32_t y) { return prob->n[x] > prob->n[y]; });
  int64_t n64 = 0, n48 = 0;  // order is by decreasing n
  while (n64 < nsys && prob->n[order[n64]] > 48) n64++;
  n48 = n64;
  while (n48 < nsys && prob->n[order[n48]] > 32) n48++;
  b->count[2] = n64;
  b->count[1] = n48 - n64;
  b->count[0] = nsys - n48;
  b->h_order  = order;

  DevProblem& d = b->dp;
  d.nsys   = nsys;
  d.n      = upload(b, prob->n, nsys);
  d.y_off  = upload(b, prob->y_off, nsys + 1);
  d.r_off  = upload(b, prob->r_off, nsys + 1);
  d.rtype  = upload(b, prob->rtype, b->R);
  d.ra     = upload(b, prob->ra, b->R);
  d.rb     = upload(b, prob->rb, b->R);
  d.rc     = upload(b, prob->rc, b->R);
  d.rk     = upload(b, prob->rk, b->R);
  d.fptr   = upload(b, fptr.data(), fptr.size());
  d.fent   = upload(b, fent.data(), fent.size());
  d.e_off  = upload(b, e_off.data(), e_off.size());
  d.jptr   = upload(b, jptr.data(), jptr.size());
  d.jent   = upload(b, jent.data(), jent.size());
  d.je_off = upload(b, je_off.data(), je_off.size());
  d.order  = upload(b, order.data(), order.size());
  b->d_order[2] = d.order;
  b->d_order[1] = d.order + n64;
  b->d_order[0] = d.order + n48;
  bool ok  = d.n && d.y_off && d.r_off && d.rtype && d.ra && d.rb && d.rc && d.rk && d.fptr &&
            d.fent && d.e_off && d.jptr && d.jent && d.je_off && d.order;
  ok = ok && gb300::check_cuda(cudaMalloc(&b->d_y0, sizeof(double) * b->Y), "cudaMalloc(y0)") &&
       gb300::check_cuda(cudaMalloc(&b->d_yout, sizeof(double) * b->Y), "cudaMalloc(yout)") &&
       gb300::check_cuda(cudaMalloc(&b->d_stats, sizeof(SUNBatchBDFStats) * nsys),
                         "cudaMalloc(stats)") &&
       gb300::check_cuda(cudaMalloc(&b->d_next, 5 * sizeof(unsigned int)), "cudaMalloc(next)") &&
       gb300::check_cuda(cudaMalloc(&b->d_fail, sizeof(int32_t) * (nsys ? nsys : 1)),
                         "cudaMalloc(failed list)") &&
       gb300::check_cuda(cudaEventCreate(&b->ev0), "cudaEventCreate") &&
       gb300::check_cuda(cudaEventCreate(&b->ev1), "cudaEventCreate");
  // Scratch for the largest grid any mode launches, so that SolveAsync
  // allocates nothing.
  ok = ok && query_occupancy(b);
  int maxgrid = 1;
  for (int mode : {SUNBATCHBDF_FP64, SUNBATCHBDF_MIXED, SUNBATCHBDF_FP64_EXACT})
  {
    for (int id = 0; id < kPlans; id++)
    {
      Launch L[kBuckets];
      const int nl = plan_with(b, mode, id, b->d_order[2], L);
      for (int k = 0; k < nl; k++) maxgrid = std::max(maxgrid, L[k].grid);
    }
  }
  ok = ok && ensure_scratch(b, maxgrid);
  if (!ok)
  {
    SUNBatchBDF_GB300_Free(b);
    return nullptr;
  }
  return b;
}

int SUNBatchBDF_GB300_SetTolerances(SUNBatchBDF_GB300 b, double rtol, double atol)
{
  if (!b || rtol < 0 || atol < 0) return SUN_ERR_ARG_OUTOFRANGE;
  b->rtol = rtol;
  b->atol = atol;
  return SUN_SUCCESS;
}

int SUNBatchBDF_GB300_SetMaxNumSteps(SUNBatchBDF_GB300 b, long mxstep)
{
  if (!b) return SUN_ERR_ARG_CORRUPT;
  b->mxstep = mxstep;
  return SUN_SUCCESS;
}

int SUNBatchBDF_GB300_SetMode(SUNBatchBDF_GB300 b, int mode)
{
  if (!b) return SUN_ERR_ARG_CORRUPT;
  if (mode != SUNBATCHBDF_FP64 && mode != SUNBATCHBDF_FP64_EXACT && mode != SUNBATCHBDF_MIXED)
    return SUN_ERR_ARG_OUTOFRANGE;
  b->mode = mode;
  return SUN_SUCCESS;
}

int SUNBatchBDF_GB300_SetRefinementSweeps(SUNBatchBDF_GB300 b, int sweeps)
{
  if (!b) return SUN_ERR_ARG_CORRUPT;
  if (sweeps < 0 || sweeps > 8) return SUN_ERR_ARG_OUTOFRANGE;
  b->refine = sweeps;
  return SUN_SUCCESS;
}

int SUNBatchBDF_GB300_SetPredictor(SUNBatchBDF_GB300 b, const uint16_t* d_weights,
                                   const float* d_biases)
{
  if (!b) return SUN_ERR_ARG_CORRUPT;
  if ((d_weights == nullptr) != (d_biases == nullptr)) return SUN_ERR_ARG_INCOMPATIBLE;
  if (d_weights && !b->d_lp &&
      !gb300::check_cuda(cudaMalloc(&b->d_lp, 2 * sizeof(unsigned long long)),
                         "cudaMalloc(predictor counters)"))
    return SUN_ERR_MEM_FAIL;
  b->mlp_w = d_weights;
  b->mlp_b = d_biases;
  return SUN_SUCCESS;
}

int SUNBatchBDF_GB300_SetRecorder(SUNBatchBDF_GB300 b, uint16_t* d_x, float* d_t,
                                  long long capacity, unsigned long long* d_count)
{
  if (!b) return SUN_ERR_ARG_CORRUPT;
  if (d_x && (!d_t || !d_count || capacity < 0)) return SUN_ERR_ARG_INCOMPATIBLE;
  b->rec_x     = d_x;
  b->rec_t     = d_t;
  b->rec_count = d_count;
  b->rec_cap   = d_x ? capacity : 0;
  return SUN_SUCCESS;
}

int SUNBatchBDF_GB300_GetPredictorCounts(SUNBatchBDF_GB300 b, long long* calls, long long* kept)
{
  if (!b || !calls || !kept) return SUN_ERR_ARG_CORRUPT;
  unsigned long long h[2] = {0, 0};
  if (b->d_lp &&
      !gb300::check_cuda(cudaMemcpyAsync(h, b->d_lp, sizeof h, cudaMemcpyDeviceToHost, b->stream),
                         "cudaMemcpyAsync(predictor counters)"))
    return SUN_ERR_EXT_FAIL;
  if (!gb300::check_cuda(cudaStreamSynchronize(b->stream), "predictor counters"))
    return SUN_ERR_EXT_FAIL;
  *calls = (long long)h[0];
  *kept  = (long long)h[1];
  return SUN_SUCCESS;
}

namespace {
// The launch parameters shared by a solve and by the autotuner's trial runs
// (no predictor, recorder or retry list: the callers add those).
Params base_params(SUNBatchBDF_GB300 b, double t0, const double* d_y0, double tout,
                   double* d_yout, SUNBatchBDFStats* d_stats)
{
  Params P;
  memset(&P, 0, sizeof P);
  P.p       = b->dp;
  P.t0      = t0;
  P.tout    = tout;
  P.rtol    = b->rtol;
  P.atol    = b->atol;
  P.mxstep  = b->mxstep;
  P.refine  = b->refine;
  P.y0      = d_y0;
  P.yout    = d_yout;
  P.stats   = d_stats;
  P.next    = b->d_next;
  P.scratch = b->d_scratch;
  P.pivots  = b->d_piv;
  P.timers  = b->d_timers;
  return P;
}

cudaError_t launch_plan(SUNBatchBDF_GB300 b, const Params& P, const Launch* L, int nl)
{
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < nl && e == cudaSuccess; k++)
  {
    if (L[k].grid > b->slots) return cudaErrorInvalidConfiguration;
    e = (b->mode == SUNBATCHBDF_FP64_EXACT)
          ? launch_exact(P, L[k].nb, L[k].grid, b->stream, L[k].order, L[k].count,
                         b->d_next + L[k].queue)
          : uses_learn(P) ? launch_fast_learn(P, b->mode, L[k].nb, L[k].grid, b->stream,
                                              L[k].order, L[k].count, b->d_next + L[k].queue)
                          : launch_fast(P, b->mode, L[k].nb, L[k].grid, b->stream, L[k].order,
                                        L[k].count, b->d_next + L[k].queue);
    gb300::count_launch();
  }
  return e;
}
}  // namespace

int SUNBatchBDF_GB300_Autotune(SUNBatchBDF_GB300 b, double t0, const double* d_y0, double tout,
                               int stride, double* plan_ms)
{
  if (!b || !d_y0 || stride < 1) return SUN_ERR_ARG_CORRUPT;
  const int64_t nsys = b->nsys;
  if (!is_device_ptr(d_y0))
  {  // a host array: tune on the library's own device copy
    if (!gb300::check_cuda(cudaMemcpyAsync(b->d_y0, d_y0, sizeof(double) * b->Y,
                                           cudaMemcpyHostToDevice, b->stream),
                           "cudaMemcpyAsync(y0)"))
      return SUN_ERR_EXT_FAIL;
    d_y0 = b->d_y0;
  }
  int32_t* d_sample  = nullptr;
  if (!gb300::check_cuda(cudaMalloc(&d_sample, sizeof(int32_t) * (nsys ? nsys : 1)),
                         "cudaMalloc(autotune sample)"))
    return SUN_ERR_MEM_FAIL;
  Params P  = base_params(b, t0, d_y0, tout, b->d_yout, b->d_stats);
  int best  = b->plan_id[b->mode];
  float bms = 0.f;
  int rc    = SUN_SUCCESS;
  for (int id = 0; id < kPlans && rc == SUN_SUCCESS; id++)
  {
    // the plan's classes, each reduced to every stride-th system (in the
    // classes' own largest-first order)
    Launch full[kBuckets], L[kBuckets];
    const int nl = plan_with(b, b->mode, id, b->d_order[2], full);
    std::vector<int32_t> h;
    int nls = 0;
    for (int k = 0; k < nl; k++)
    {
      const int64_t lo = full[k].order - b->d_order[2], start = (int64_t)h.size();
      for (int64_t j = lo; j < lo + full[k].count; j += stride) h.push_back(b->h_order[j]);
      const int64_t cnt = (int64_t)h.size() - start;
      L[nls++] = {full[k].nb, grid_for(b, b->mode, full[k].nb, cnt), d_sample + start, cnt,
                  full[k].queue};
    }
    if (!gb300::check_cuda(cudaMemcpyAsync(d_sample, h.data(), sizeof(int32_t) * h.size(),
                                           cudaMemcpyHostToDevice, b->stream),
                           "cudaMemcpyAsync(autotune sample)"))
    {
      rc = SUN_ERR_EXT_FAIL;
      break;
    }
    float ms = 0.f;
    const int reps = h.size() > 8192 ? 1 : 2;  // small samples: a warm-up run first
    for (int rep = 0; rep < reps; rep++)
    {  // the last run is timed
      cudaMemsetAsync(b->d_next, 0, 5 * sizeof(unsigned int), b->stream);
      cudaEventRecord(b->ev0, b->stream);
      cudaError_t e = launch_plan(b, P, L, nls);
      cudaEventRecord(b->ev1, b->stream);
      if (!gb300::check_cuda(e, "autotune launch") ||
          !gb300::check_cuda(cudaStreamSynchronize(b->stream), "autotune run"))
      {
        rc = SUN_ERR_EXT_FAIL;
        break;
      }
      cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    }
    if (plan_ms) plan_ms[id] = ms;
    if (rc == SUN_SUCCESS && (id == 0 || ms < bms))
    {
      bms  = ms;
      best = id;
    }
  }
  cudaFree(d_sample);
  if (rc == SUN_SUCCESS) b->plan_id[b->mode] = best;
  return rc;
}

int SUNBatchBDF_GB300_GetLaunchPlan(SUNBatchBDF_GB300 b, int mode, int* widths)
{
  if (!b || !widths || mode < 0 || mode > 2) return SUN_ERR_ARG_CORRUPT;
  for (int k = 0; k < 3; k++) widths[k] = kPlanWidths[b->plan_id[mode]][k];
  return SUN_SUCCESS;
}

int SUNBatchBDF_GB300_SolveAsync(SUNBatchBDF_GB300 b, double t0, const double* d_y0, double tout,
                                 double* d_yout, SUNBatchBDFStats* d_stats)
{
  if (!b || !d_y0 || !d_yout) return SUN_ERR_ARG_CORRUPT;
  Params P = base_params(b, t0, d_y0, tout, d_yout, d_stats);
  const bool fast = b->mode != SUNBATCHBDF_FP64_EXACT;  // the exact mode never uses them
  P.mlp_w     = fast ? b->mlp_w : nullptr;
  P.mlp_b     = fast ? b->mlp_b : nullptr;
  P.lp_counts = (fast && b->mlp_w) ? b->d_lp : nullptr;
  P.rec_x     = fast ? b->rec_x : nullptr;
  P.rec_t     = b->rec_t;
  P.rec_count = b->rec_count;
  P.rec_cap   = b->rec_cap;
  // d_next: [0..2] the buckets' queues, [3] the retry queue, [4] failed count
  const int rmode  = b->retry_mode == -2
                      ? (b->mode == SUNBATCHBDF_MIXED ? SUNBATCHBDF_FP64 : SUNBATCHBDF_MIXED)
                      : b->retry_mode;
  const bool retry = fast && rmode >= 0;
  P.fail_list  = retry ? b->d_fail : nullptr;
  P.fail_count = b->d_next + 4;
  P.count_dev  = nullptr;
  if (!gb300::check_cuda(cudaMemsetAsync(b->d_next, 0, 5 * sizeof(unsigned int), b->stream),
                         "cudaMemsetAsync(queue)"))
    return SUN_ERR_EXT_FAIL;
  if (P.lp_counts &&
      !gb300::check_cuda(cudaMemsetAsync(b->d_lp, 0, 2 * sizeof(unsigned long long), b->stream),
                         "cudaMemsetAsync(predictor counters)"))
    return SUN_ERR_EXT_FAIL;
  cudaEventRecord(b->ev0, b->stream);
  Launch L[kBuckets];
  const int nl  = plan(b, b->mode, L);
  cudaError_t e = launch_plan(b, P, L, nl);
  if (retry && e == cudaSuccess)
  {
    // systems that failed in the fast mode are integrated again in the retry
    // mode (by default the other fast mode); the queue length is the
    // device-side failure count, so nothing waits on the host
    Params R      = P;
    R.fail_list   = nullptr;
    R.count_dev   = b->d_next + 4;
    R.mlp_w       = nullptr;
    R.mlp_b       = nullptr;
    R.lp_counts   = nullptr;
    R.rec_x       = nullptr;
    const int grid = std::min(gb300::num_sms(), b->slots);
    e = (rmode == SUNBATCHBDF_FP64_EXACT)
          ? launch_exact(R, 64, grid, b->stream, b->d_fail, b->nsys, b->d_next + 3)
          : launch_fast(R, rmode, 64, grid, b->stream, b->d_fail, b->nsys, b->d_next + 3);
    gb300::count_launch();
  }
  cudaEventRecord(b->ev1, b->stream);
  return gb300::check_cuda(e, "k_batch_bdf launch") ? SUN_SUCCESS : SUN_ERR_EXT_FAIL;
}

int SUNBatchBDF_GB300_SetRetryMode(SUNBatchBDF_GB300 b, int mode)
{
  if (!b) return SUN_ERR_ARG_CORRUPT;
  if (mode != -1 && mode != -2 && mode != SUNBATCHBDF_FP64_EXACT && mode != SUNBATCHBDF_FP64 &&
      mode != SUNBATCHBDF_MIXED)
    return SUN_ERR_ARG_OUTOFRANGE;
  b->retry_mode = mode;
  return SUN_SUCCESS;
}

int SUNBatchBDF_GB300_GetRetryCount(SUNBatchBDF_GB300 b, long long* nretry)
{
  if (!b || !nretry) return SUN_ERR_ARG_CORRUPT;
  unsigned int h = 0;
  if (!gb300::check_cuda(cudaMemcpyAsync(&h, b->d_next + 4, sizeof h, cudaMemcpyDeviceToHost,
                                         b->stream),
                         "cudaMemcpyAsync(retry count)") ||
      !gb300::check_cuda(cudaStreamSynchronize(b->stream), "retry count"))
    return SUN_ERR_EXT_FAIL;
  *nretry = (long long)h;
  return SUN_SUCCESS;
}

int SUNBatchBDF_GB300_Solve(SUNBatchBDF_GB300 b, double t0, const double* y0, double tout,
                            double* yout, SUNBatchBDFStats* stats)
{
  if (!b || !y0 || !yout) return SUN_ERR_ARG_CORRUPT;
  const size_t ybytes = sizeof(double) * b->Y;
  const double* dy0   = y0;
  if (!is_device_ptr(y0))
  {
    if (!gb300::check_cuda(cudaMemcpyAsync(b->d_y0, y0, ybytes, cudaMemcpyHostToDevice, b->stream),
                           "cudaMemcpyAsync(y0)"))
      return SUN_ERR_EXT_FAIL;
    dy0 = b->d_y0;
  }
  const bool dev_out       = is_device_ptr(yout);
  double* dyo              = dev_out ? yout : b->d_yout;
  const bool dev_stats     = stats && is_device_ptr(stats);
  SUNBatchBDFStats* dstats = stats ? (dev_stats ? stats : b->d_stats) : nullptr;
  int rc = SUNBatchBDF_GB300_SolveAsync(b, t0, dy0, tout, dyo, dstats);
  if (rc != SUN_SUCCESS) return rc;
  if (!dev_out &&
      !gb300::check_cuda(cudaMemcpyAsync(yout, dyo, ybytes, cudaMemcpyDeviceToHost, b->stream),
                         "cudaMemcpyAsync(yout)"))
    return SUN_ERR_EXT_FAIL;
  if (stats && !dev_stats &&
      !gb300::check_cuda(cudaMemcpyAsync(stats, dstats, sizeof(SUNBatchBDFStats) * b->nsys,
                                         cudaMemcpyDeviceToHost, b->stream),
                         "cudaMemcpyAsync(stats)"))
    return SUN_ERR_EXT_FAIL;
  if (!gb300::check_cuda(cudaStreamSynchronize(b->stream), "k_batch_bdf"))
    return SUN_ERR_EXT_FAIL;
  cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1);
  return SUN_SUCCESS;
}

double SUNBatchBDF_GB300_LastKernelMs(SUNBatchBDF_GB300 b) { return b ? b->last_ms : 0.0; }

// CVodePrintAllStats (src/cvode/cvode_io.c:1626) for one system of the batch:
// sunfprintf_real / sunfprintf_long (src/sundials/sundials_utils.h:89-117)
// with a 29-character name column and DBL_DIG significant digits.
int SUNBatchBDF_GB300_PrintAllStats(const SUNBatchBDFStats* stats, int64_t nsys, int64_t sys,
                                    FILE* out, int fmt)
{
  if (!stats || !out || sys < 0 || sys >= nsys || (fmt != 0 && fmt != 1))
    return SUN_ERR_ARG_OUTOFRANGE;
  const SUNBatchBDFStats& st = stats[sys];
  bool start = true;
  auto real = [&](const char* name, double v) {
    if (fmt == 0) fprintf(out, "%-29s = %.15g\n", name, v);
    else
    {
      if (!start) fprintf(out, ",");
      fprintf(out, "%s,% .15e", name, v);
    }
    start = false;
  };
  auto lng = [&](const char* name, long v) {
    if (fmt == 0) fprintf(out, "%-29s = %ld\n", name, v);
    else
    {
      if (!start) fprintf(out, ",");
      fprintf(out, "%s,%ld", name, v);
    }
    start = false;
  };
  real("Current time", st.tn);
  lng("Steps", (long)st.nst);
  lng("Error test fails", (long)st.netf);
  lng("NLS step fails", (long)st.ncfn);
  real("Initial step size", st.h0u);
  real("Last step size", st.hu);
  real("Current step size", st.next_h);
  lng("Last method order", (long)st.qu);
  lng("Current method order", (long)st.next_q);
  lng("Stab. lim. order reductions", 0L);
  lng("RHS fn evals", (long)st.nfe);
  lng("NLS iters", (long)st.nni);
  lng("NLS fails", (long)st.nnf);
  if (st.nst > 0) real("NLS iters per step", (double)st.nni / (double)st.nst);
  lng("LS setups", (long)st.nsetups);
  // SUNLINSOL_DENSE with an analytic Jacobian
  lng("Jac fn evals", (long)st.nje);
  lng("LS RHS fn evals", 0L);
  lng("Prec setup evals", 0L);
  lng("Prec solves", 0L);
  lng("LS iters", 0L);
  lng("LS fails", 0L);
  lng("Jac-times setups", 0L);
  lng("Jac-times evals", 0L);
  if (st.nni > 0)
  {
    real("LS iters per NLS iter", 0.0 / (double)st.nni);
    real("Jac evals per NLS iter", (double)st.nje / (double)st.nni);
    real("Prec evals per NLS iter", 0.0 / (double)st.nni);
  }
  lng("Root fn evals", 0L);
  return SUN_SUCCESS;
}

#ifdef SUNGB300_BDF_TIMERS
// Section cycle totals summed over warp slots (instrumented builds only).
SUNGB300_EXPORT int SUNBatchBDF_GB300_SectionCycles(SUNBatchBDF_GB300 b, long long* out)
{
  std::vector<long long> h((size_t)b->slots * T_COUNT);
  cudaMemcpy(h.data(), b->d_timers, sizeof(long long) * h.size(), cudaMemcpyDeviceToHost);
  for (int t = 0; t < T_COUNT; t++) out[t] = 0;
  for (int s = 0; s < b->slots; s++)
    for (int t = 0; t < T_COUNT; t++) out[t] += h[(size_t)s * T_COUNT + t];
  return T_COUNT;
}
#endif

void SUNBatchBDF_GB300_Free(SUNBatchBDF_GB300 b)
{
  if (!b) return;
  cudaStreamSynchronize(b->stream);
  for (void* p : b->allocs) cudaFree(p);
  cudaFree(b->d_y0);
  cudaFree(b->d_yout);
  cudaFree(b->d_stats);
  cudaFree(b->d_next);
  cudaFree(b->d_fail);
  cudaFree(b->d_scratch);
  cudaFree(b->d_piv);
  cudaFree(b->d_timers);
  if (b->d_lp) cudaFree(b->d_lp);
  cudaEventDestroy(b->ev0);
  cudaEventDestroy(b->ev1);
  delete b;
}

}  // extern "C"

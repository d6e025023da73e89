/* ---------------------------------------------------------------------------
 * sunbatchbdf_gb300.h -- SUNBatchBDF_GB300: thousands of independent stiff
 * systems of uneven size integrated by CVODE's BDF method in ONE persistent
 * GPU launch, each system with its own step size, order and counters.
 *
 * The reference has no per-system step control: one CVODE instance owns one
 * h, q and set of counters for its whole N_Vector (src/cvode/cvode_impl.h,
 * cv_h / cv_q), and its batched examples step all systems together
 * (examples/cvode/cuda/cvRoberts_block_cusolversp_batchqr.cu:196-223).  The
 * semantics here are therefore those of one independent CVode(tout,
 * CV_NORMAL) call per system with NVECTOR_SERIAL, SUNLINSOL_DENSE and an
 * analytic Jacobian (src/cvode/cvode.c:1037-3727, cvode_nls.c, cvode_ls.c,
 * sunnonlinsol_newton.c, sundials_dense.c), restated on the device.  The
 * per-system counters have the meaning of CVodeGetNumSteps, GetNumRhsEvals,
 * GetNumLinSolvSetups, GetNumJacEvals, GetNumNonlinSolvIters,
 * GetNumStepSolveFails, GetNumErrTestFails, GetNumNonlinSolvConvFails,
 * GetLastOrder, GetCurrentTime and GetLastStep (src/cvode/cvode_io.c:1053-1626).
 *
 * The right-hand side is a mass-action reaction network given as data
 * (A -> B and A + B -> C reactions with rate constants), evaluated and
 * differentiated on the device.  This entry point has no counterpart in the
 * reference's plugin API (no reference plugin point exists for per-system
 * step control); its problem layout is documented below.
 *
 * Arithmetic modes (SUNBatchBDF_GB300_SetMode):
 *   SUNBATCHBDF_FP64        FP64 throughout, fused multiply-adds (default);
 *   SUNBATCHBDF_FP64_EXACT  FP64 with every product and sum rounded
 *                           separately and sums in CVODE's sequential order,
 *                           i.e. the reference's arithmetic on x86-64 (only
 *                           pow() may differ by an ulp);
 *   SUNBATCHBDF_MIXED       Newton matrix I - gamma*J factored and solved in
 *                           FP32, each solve followed by FP64 iterative
 *                           refinement (residual with the FP64 Jacobian);
 *                           residuals, norms, error test and step control FP64.
 * ------------------------------------------------------------------------- */
#ifndef SUNBATCHBDF_GB300_H
#define SUNBATCHBDF_GB300_H

#include <stdint.h>
#include <stdio.h>

#include "sundials_gb300_abi.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SUNBATCHBDF_FP64       0
#define SUNBATCHBDF_FP64_EXACT 1
#define SUNBATCHBDF_MIXED      2

#define SUNBATCHBDF_NMAX 64 /* largest system size */

/* Mass-action problem.  All arrays are HOST arrays; reaction r of system s
 * is r_off[s] <= r < r_off[s+1], species indices are local (0..n[s]-1):
 *   rtype[r] == 0:  ra -> rb,        rate = rk * y[ra]
 *   rtype[r] == 1:  ra + rb -> rc,   rate = (rk * y[ra]) * y[rb]
 * f sums the signed rates of the reactions in index order (see
 * sundials_gb300/kinetics.py for the definition of every summation order). */
typedef struct
{
  int64_t nsys;
  const int32_t* n;     /* [nsys]   species per system, 1..64 */
  const int64_t* y_off; /* [nsys+1] offsets of each system's state */
  const int64_t* r_off; /* [nsys+1] offsets of each system's reactions */
  const int32_t* rtype; /* [R] */
  const int32_t* ra;    /* [R] */
  const int32_t* rb;    /* [R] */
  const int32_t* rc;    /* [R] (-1 for A -> B) */
  const double* rk;     /* [R] */
} SUNBatchBDFProblem;

/* Per-system result record (same layout as the CPU oracle's KinStats). */
typedef struct
{
  int64_t nst, nfe, nsetups, nje, nni, ncfn, netf, nnf;
  int64_t flag; /* CVode return value: 0 success, <0 failure */
  int64_t qu;   /* last order used */
  double tn;    /* internal time reached */
  double hu;    /* last step size used */
  double h0u;   /* initial step size used (CVodeGetActualInitStep) */
  double next_h;   /* step size to be attempted next (CVodeGetCurrentStep) */
  int64_t next_q;  /* order to be attempted next (CVodeGetCurrentOrder) */
} SUNBatchBDFStats;

typedef struct SUNBatchBDF_GB300_* SUNBatchBDF_GB300;

/* Copies the problem to the device; stream = cudaStream_t (NULL: default). */
SUNGB300_EXPORT SUNBatchBDF_GB300 SUNBatchBDF_GB300_Create(const SUNBatchBDFProblem* prob,
                                                           void* cuda_stream);
SUNGB300_EXPORT int SUNBatchBDF_GB300_SetTolerances(SUNBatchBDF_GB300 b, double rtol,
                                                    double atol);
SUNGB300_EXPORT int SUNBatchBDF_GB300_SetMaxNumSteps(SUNBatchBDF_GB300 b, long mxstep);
SUNGB300_EXPORT int SUNBatchBDF_GB300_SetMode(SUNBatchBDF_GB300 b, int mode);
/* Refinement sweeps after each FP32 solve in SUNBATCHBDF_MIXED (default 1). */
SUNGB300_EXPORT int SUNBatchBDF_GB300_SetRefinementSweeps(SUNBatchBDF_GB300 b, int sweeps);

/* Integrate every system from t0 to tout (one CVode(tout, CV_NORMAL) each).
 * y0 / yout: Sum(n) doubles; host or device pointers (cudaMemcpyDefault
 * semantics).  stats: nsys records (host or device) or NULL.  Returns 0 when
 * the launch succeeded (per-system failures are in stats[s].flag), a
 * SUN_ERR_* code otherwise. */
SUNGB300_EXPORT int SUNBatchBDF_GB300_Solve(SUNBatchBDF_GB300 b, double t0, const double* y0,
                                            double tout, double* yout,
                                            SUNBatchBDFStats* stats);

/* Same as Solve with device pointers only, no synchronisation: enqueued on
 * the object's stream (may be captured into a CUDA graph). */
SUNGB300_EXPORT int SUNBatchBDF_GB300_SolveAsync(SUNBatchBDF_GB300 b, double t0,
                                                 const double* d_y0, double tout,
                                                 double* d_yout, SUNBatchBDFStats* d_stats);

/* Wall time of the last Solve's integration kernel in milliseconds. */
SUNGB300_EXPORT double SUNBatchBDF_GB300_LastKernelMs(SUNBatchBDF_GB300 b);

/* Systems that end a fast-mode solve with a failure flag (CVode < 0) are
 * integrated again, on the device and in the same stream, by a second launch
 * in the retry mode: SUNBATCHBDF_RETRY_OTHER (default: the other fast mode,
 * MIXED <-> FP64, about 1% of a solve when a handful of systems fail),
 * SUNBATCHBDF_FP64_EXACT (the reference's own arithmetic, so those systems'
 * flags and results are the reference CVODE's; one exact integration is
 * ~0.3 s on an otherwise idle GPU), SUNBATCHBDF_FP64 or SUNBATCHBDF_MIXED;
 * SUNBATCHBDF_RETRY_OFF turns it off.  Retried systems report the retry's
 * yout and stats.  A fast-mode failure is a rounding-sensitive edge case of
 * CVODE's error-test heuristics (repeated test failures at one step), and the
 * two fast modes fail on different systems.  No counterpart in the reference
 * (one CVODE instance per system has no other form to fall back to). */
#define SUNBATCHBDF_RETRY_OFF   (-1)
#define SUNBATCHBDF_RETRY_OTHER (-2)
SUNGB300_EXPORT int SUNBatchBDF_GB300_SetRetryMode(SUNBatchBDF_GB300 b, int mode);
/* Number of systems the last solve integrated again. */
SUNGB300_EXPORT int SUNBatchBDF_GB300_GetRetryCount(SUNBatchBDF_GB300 b, long long* nretry);

/* Launch-plan autotuner (no counterpart in the reference).  A plan is the
 * set of kernel widths the systems are split into (one persistent launch per
 * width: systems with n in (previous width, width]): {32,64}, {32,48,64},
 * {48,64} or {64}.  Autotune integrates every stride-th system of each class
 * (t0 -> tout, y0 on the host or the device) under every plan, times it
 * (after a warm-up run when the sample has at most 8,192 systems) and keeps the
 * fastest plan for the current mode; plan_ms (optional, 4 entries) receives
 * the times.  The end of each launch is a tail in which few warps still run,
 * so a sample represents the full batch only if each warp still integrates
 * many systems: use a small stride (2 for 65,536 systems).  Defaults without
 * tuning: MIXED {32,48,64}, FP64 modes {32,64}. */
SUNGB300_EXPORT int SUNBatchBDF_GB300_Autotune(SUNBatchBDF_GB300 b, double t0,
                                               const double* y0, double tout, int stride,
                                               double* plan_ms);
/* The widths of the plan used for `mode` (3 entries, unused ones 0). */
SUNGB300_EXPORT int SUNBatchBDF_GB300_GetLaunchPlan(SUNBatchBDF_GB300 b, int mode, int* widths);

/* Statistics of system `sys` (host array from Solve) in the layout of
 * CVodePrintAllStats (src/cvode/cvode_io.c:1626): the same names, order and
 * number formats, fmt 0 = SUN_OUTPUTFORMAT_TABLE, 1 = SUN_OUTPUTFORMAT_CSV; the
 * linear-solver lines are those of CVODE with SUNLINSOL_DENSE and an analytic
 * Jacobian (no preconditioner, no Krylov iterations, no difference-quotient
 * RHS calls); no root finding, no projection.  Returns 0, or
 * SUN_ERR_ARG_OUTOFRANGE for a bad format or system index. */
SUNGB300_EXPORT int SUNBatchBDF_GB300_PrintAllStats(const SUNBatchBDFStats* stats,
                                                    int64_t nsys, int64_t sys, FILE* outfile,
                                                    int fmt);

/* Learned Newton predictor (include/sunmlp_gb300.h; no counterpart in the
 * reference).  With device weights set, every Newton solve of the fast modes
 * evaluates the network on its system's features and starts Newton from the
 * network's iterate when the WRMS norm of its residual is smaller than the
 * residual of the BDF predictor, else from the predictor (the Newton
 * convergence test is unchanged, so is the accuracy; each solve costs one
 * extra right-hand-side evaluation, counted in nfe).  NULL, NULL turns it
 * off.  The exact mode ignores it. */
SUNGB300_EXPORT int SUNBatchBDF_GB300_SetPredictor(SUNBatchBDF_GB300 b,
                                                   const uint16_t* d_weights,
                                                   const float* d_biases);
/* Over the last solve: predictor evaluations and how often its iterate was kept. */
SUNGB300_EXPORT int SUNBatchBDF_GB300_GetPredictorCounts(SUNBatchBDF_GB300 b, long long* calls,
                                                         long long* kept);
/* Training-data recorder: after every converged Newton solve of the fast
 * modes, append the solve's features (BF16, SUNMLP_IN_PAD per row) to d_x
 * and its converged corrector in error-weight units (64 FP32 per row, zero
 * past n) to d_t, at row atomicAdd(d_count, 1) while it is below capacity.
 * d_x = NULL turns it off. */
SUNGB300_EXPORT int SUNBatchBDF_GB300_SetRecorder(SUNBatchBDF_GB300 b, uint16_t* d_x, float* d_t,
                                                  long long capacity,
                                                  unsigned long long* d_count);

SUNGB300_EXPORT void SUNBatchBDF_GB300_Free(SUNBatchBDF_GB300 b);

#ifdef __cplusplus
}
#endif

#endif /* SUNBATCHBDF_GB300_H */

/* arkstep_port.c -- TEST ORACLE (checker only, never part of the product).
 *
 * ARKODE's ARKStep with an implicit right-hand side (a DIRK method) or an
 * explicit + implicit splitting (an ARK IMEX method), the Newton nonlinear
 * solver with a matrix-free iterative SUNLinearSolver (user or
 * difference-quotient Jacobian-times-vector, a preconditioner solve with or
 * without a preconditioner setup) or a matrix-based direct one (SUNMatrix,
 * user Jacobian), the benchmark's task-local Newton, or the fixed-point
 * solver with Anderson acceleration (oracle/fixedpoint_port.c); and ERKStep
 * (explicit only) -- the ERK, ARK-DIRK and ARK-IMEX configurations of the
 * 3-D advection-reaction benchmark (benchmarks/advection_reaction_3D/raja/
 * arkode_driver.cpp:51-160, 239-370) -- restated over the generic object model: every
 * vector operation is dispatched through the vector's ops table (fused
 * operations when the vector provides them, the reference's fallback
 * compositions otherwise) and the linear solver is driven only through its
 * ops table.  The same code runs the reference's own NVECTOR_SERIAL +
 * SUNLINSOL_SPGMR (pinned bit for bit against the reference's ARKodeEvolve by
 * tests/test_arkstep_port.py) and NVECTOR_GB300 + SUNLinSol_SPGMR_GB300 on
 * a GPU machine where the reference library is not available.
 *
 * The Butcher tables are inputs (A, b, c, d, orders), read from the
 * reference's own table objects where the reference runs, so no coefficient
 * is restated here.
 *
 * Follows, in the same floating-point order (compiled with -ffp-contract=off):
 *   ARKodeEvolve, ARK_NORMAL (no tstop, roots, constraints, relaxation)
 *                                  src/arkode/arkode.c:657-1173
 *   ARKodeGetDky (k = 0)           arkode.c:1175-1240
 *   arkInitialSetup                arkode.c:1978-2250
 *   arkStopTests (tout reached)    arkode.c:2272-2470
 *   arkHin / arkUpperBoundH0 / arkYddNorm   arkode.c:2485-2678
 *   arkCompleteStep                arkode.c:2679-2770
 *   arkCheckConvergence / arkCheckTemporalError   arkode.c:3207-3270, 3335-3395
 *   arkEwtSetSS                    arkode.c:2935-2950
 *   arkAdapt                       src/arkode/arkode_adapt.c:105-205
 *   default controller (I)         src/sunadaptcontroller/soderlind/
 *                                  sunadaptcontroller_soderlind.c:395-420, 566-610, 665-680
 *   ARKodeSetDefaults / ARKStep defaults   src/arkode/arkode_io.c:48-120,
 *                                  arkode_arkstep_io.c:735-795
 *   arkStep_Init (implicit, FIRST_INIT)    src/arkode/arkode_arkstep.c:945-1200
 *   arkStep_FullRHS                arkode_arkstep.c:1297-1660
 *   arkStep_TakeStep_Z             arkode_arkstep.c:1666-2240
 *   arkStep_Predict (trivial)      arkode_arkstep.c:2807-3037
 *   arkStep_StageSetup             arkode_arkstep.c:3038-3160
 *   arkStep_ComputeSolutions       arkode_arkstep.c:3162-3337
 *   arkStep_Nls / NlsResidual_MassIdent / NlsLSolve / NlsConvTest
 *                                  src/arkode/arkode_arkstep_nls.c:364-604, 1152-1200
 *   SUNNonlinSolSolve_Newton       src/sunnonlinsol/newton/sunnonlinsol_newton.c:179-310
 *   ARKodeSetLinearSolver defaults, arkLsInitialize, arkLsATimes,
 *   arkLsDQJtimes, arkLsPSetup, arkLsPSolve, arkLsLinSys, arkLsSetup, arkLsSolve
 *   arkStep_NlsLSetup              arkode_arkstep_nls.c:472-512
 *                                  src/arkode/arkode_ls.c:50-300, 2319-2456, 2842-2880,
 *                                  2981-3160, 3308-3520
 *   Hermite interpolation module    src/arkode/arkode_interp.c:97-170, 307-790
 *   N_VLinearCombination dispatch  src/sundials/sundials_nvector.c:549-580
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../include/sundials_gb300_abi.h"
#include "fixedpoint_port.h"

#define UROUND DBL_EPSILON
#define MAXS 16

/* ARKODE defaults (arkode_impl.h:69-144, arkode_adapt_impl.h:43-66,
 * arkode_arkstep_impl.h:39-52, arkode_ls_impl.h:42-43) */
#define MAXNEF 7
#define MAXNCF 10
#define MAX_DQITERS 3
#define TINY 1.0e-10
#define FUZZ_FACTOR 100.0
#define H0_LBFACTOR 100.0
#define H0_UBFACTOR 0.1
#define H0_BIAS 0.5
#define H0_ITERS 4
#define ONEPSM 1.000001
#define ONEMSM 0.999999
#define SAFETY 0.9
#define GROWTH 20.0
#define HFIXED_LB 1.0
#define HFIXED_UB 1.0
#define ETAMX1 10000.0
#define ETAMXF 0.3
#define ETAMIN 0.1
#define ETACF 0.25
#define SMALL_NEF 2
#define MAXCOR 3
#define CRDOWN 0.3
#define RDIV 2.3
#define NLSCOEF 0.1
#define ARKLS_EPLIN 0.05
#define ARKLS_MSBJ 51
#define DGMAX 0.2
#define MSBP 20
#define INTERP_MAX_DEGREE 5

enum { PREDICT_AGAIN = 3, CONV_FAIL = 4, TRY_AGAIN = 5, FIRST_CALL = 6, PREV_CONV_FAIL = 7,
       PREV_ERR_FAIL = 8, RHSFUNC_RECVR = 9 };
enum { NLS_CONTINUE = 901, NLS_CONV_RECVR = 902 };
enum { NO_FAILURES = 0, FAIL_BAD_J = 1, FAIL_OTHER = 2 };
enum { FULLRHS_START = 0, FULLRHS_END = 1, FULLRHS_OTHER = 2 };
enum { ARK_SUCCESS = 0, ARK_TOO_MUCH_WORK = -1, ARK_TOO_MUCH_ACC = -2, ARK_ERR_FAILURE = -3,
       ARK_CONV_FAILURE = -4, ARK_LSETUP_FAIL = -6, ARK_LSOLVE_FAIL = -7, ARK_RHSFUNC_FAIL = -8,
       ARK_REPTD_RHSFUNC_ERR = -10, ARK_UNREC_RHSFUNC_ERR = -11, ARK_TOO_CLOSE = -27,
       ARK_BAD_T = -25, ARK_ILL_INPUT = -22 };

/* The user callbacks, with ARKODE's signatures (arkode.h, arkode_ls.h). */
typedef int (*ArkRhsFn)(double t, N_Vector y, N_Vector ydot, void* user_data);
typedef int (*ArkJTimesFn)(N_Vector v, N_Vector Jv, double t, N_Vector y, N_Vector fy,
                           void* user_data, N_Vector tmp);
typedef int (*ArkPSolveFn)(double t, N_Vector y, N_Vector fy, N_Vector r, N_Vector z,
                           double gamma, double delta, int lr, void* user_data);
/* ARKLsPrecSetupFn */
typedef int (*ArkPSetupFn)(double t, N_Vector y, N_Vector fy, sunbooleantype jok,
                           sunbooleantype* jcurPtr, double gamma, void* user_data);
/* ARKLsJacFn */
typedef int (*ArkJacFn)(double t, N_Vector y, N_Vector fy, SUNMatrix J, void* user_data,
                        N_Vector tmp1, N_Vector tmp2, N_Vector tmp3);
/* the benchmark's block solve x = (I - gamma dfi/dy)^{-1} b at the state z
 * (rhs3D.hpp SolveReactionLinSys, called with x == b) */
typedef int (*ArkBlockSolveFn)(N_Vector z, N_Vector x, N_Vector b, double gamma,
                               void* user_data);

typedef struct
{
  /* problem, options, method (fe NULL: no explicit partition) */
  ArkRhsFn fe, fi;
  ArkJTimesFn jtimes;
  ArkPSolveFn psolve;
  ArkPSetupFn pset; /* set: SPGMR's preconditioner setup, through arkLsSetup */
  ArkBlockSolveFn block_lsolve; /* set: the task-local Newton, no SUNLinearSolver */
  FPPort* fp;                   /* set: the fixed-point solver, no SUNLinearSolver */
  SUNMatrix Amat, savedJ;       /* set: a matrix-based (direct) linear solver */
  ArkJacFn jac;
  N_Vector Vabstol;             /* ARKodeSVtolerances' copy, or NULL */
  int jcur, nls_jcur, jbad, convfail;
  long nsetups, nje, nstlp, nstlj, npe;
  void* user_data;
  double rtol, atol;
  long mxstep;
  SUNLinearSolver LS;
  int s, q, p, stiffly_accurate, explicit_, sa_e, sa_i;
  double A[MAXS][MAXS], b[MAXS], c[MAXS], d[MAXS];     /* implicit table */
  double Ae[MAXS][MAXS], be[MAXS], ce[MAXS], de[MAXS]; /* explicit table */
  /* vectors (ycur is the caller's output vector, as in ARKodeEvolve) */
  N_Vector yn, fn, ycur, ewt, tempv1, tempv2, tempv3, sdata, zpred, zcor, delta;
  N_Vector Fi[MAXS], Fe[MAXS], ls_x, ls_ytemp, yold, fold, fa, fb;
  /* integrator state */
  double tn, tcur, h, hold, hprime, next_h, eta, h0u, tretlast, tolsf;
  double etamax;
  int initsetup, firststage, fn_is_current;
  long nst, nst_attempts, netf, ncfn, nfi, nfe;
  /* interpolation (Hermite) */
  int interp_degree;
  double hint_told, hint_tnew, hint_h;
  /* stage / nonlinear solver */
  int istage;
  double gamma, gammap, gamrat, crate, delp, eRNrm;
  int curiter;
  long niters, nconvfails, nls_iters, nls_fails, nnlfi, tl_ncnf;
  /* linear solver interface */
  double ls_tcur, nrmfac, eplifac;
  N_Vector ls_ycur, ls_fcur;
  long nli, nps, njtimes, nfeDQ, ncfl;
  /* I controller history (SUNAdaptController_UpdateH_Soderlind) */
  double c_ep, c_hp;
  /* ERKStep instead of ARKStep: the method table is A/b/c/d, the right-hand
   * side fi (counted in nfe); adaptivity safety and growth */
  int erk;
  double safety, growth;
} ArkPort;

/* ------------------------------------------------------ generic vector layer */
static void v_linearsum(double a, N_Vector x, double b, N_Vector y, N_Vector z)
{
  z->ops->nvlinearsum(a, x, b, y, z);
}
static void v_const(double c, N_Vector z) { z->ops->nvconst(c, z); }
static void v_scale(double c, N_Vector x, N_Vector z) { z->ops->nvscale(c, x, z); }
static double v_wrms(N_Vector x, N_Vector w) { return x->ops->nvwrmsnorm(x, w); }

static void v_lincomb(int nvec, double* c, N_Vector* X, N_Vector z)
{
  if (z->ops->nvlinearcombination) z->ops->nvlinearcombination(nvec, c, X, z);
  else
  {
    z->ops->nvscale(c[0], X[0], z);
    for (int i = 1; i < nvec; i++) z->ops->nvlinearsum(c[i], X[i], 1.0, z, z);
  }
}

static double dmax(double a, double b) { return a > b ? a : b; }
static double dmin(double a, double b) { return a < b ? a : b; }

/* arkEwtSetSS (atol > 0, so no N_VMin test) */
static void set_ewt(ArkPort* m, N_Vector ycur, N_Vector w)
{ /* arkEwtSetSS / arkEwtSetSV (all absolute tolerances > 0) */
  N_Vector t = m->tempv1;
  t->ops->nvabs(ycur, t);
  if (m->Vabstol) v_linearsum(m->rtol, t, 1.0, m->Vabstol, t);
  else
  {
    v_scale(m->rtol, t, t);
    t->ops->nvaddconst(t, m->atol, t);
  }
  t->ops->nvinv(t, w);
}

/* the two partitions at (t, y) into Fe[0] / Fi[0] */
static int eval_both(ArkPort* m, double t, N_Vector y)
{
  int r;
  if (m->explicit_)
  {
    r = m->fe(t, y, m->Fe[0], m->user_data);
    m->nfe++;
    if (r != 0) return ARK_RHSFUNC_FAIL;
  }
  r = m->fi(t, y, m->Fi[0], m->user_data);
  m->nfi++;
  if (r != 0) return ARK_RHSFUNC_FAIL;
  return 0;
}

/* f = Fi[0] (+ Fe[0]) */
static void sum_first(ArkPort* m, N_Vector f)
{
  if (m->explicit_) v_linearsum(1.0, m->Fi[0], 1.0, m->Fe[0], f);
  else v_scale(1.0, m->Fi[0], f);
}

/* erkStep_FullRHS (arkode_erkstep.c:591-735) */
static int full_rhs_erk(ArkPort* m, double t, N_Vector y, N_Vector f, int mode)
{
  int r;
  switch (mode)
  {
  case FULLRHS_START:
    if (!m->fn_is_current)
    {
      r = m->fi(t, y, m->Fi[0], m->user_data);
      m->nfe++;
      if (r != 0) return ARK_RHSFUNC_FAIL;
    }
    v_scale(1.0, m->Fi[0], f);
    break;
  case FULLRHS_END:
    if (!m->fn_is_current)
    {
      if (!m->sa_i)
      {
        r = m->fi(t, y, m->Fi[0], m->user_data);
        m->nfe++;
        if (r != 0) return ARK_RHSFUNC_FAIL;
      }
      else v_scale(1.0, m->Fi[m->s - 1], m->Fi[0]);
      v_scale(1.0, m->Fi[0], f);
    }
    break;
  default:
    r = m->fi(t, y, f, m->user_data);
    m->nfe++;
    if (r != 0) return ARK_RHSFUNC_FAIL;
    break;
  }
  return 0;
}

/* arkStep_FullRHS, identity mass matrix */
static int full_rhs(ArkPort* m, double t, N_Vector y, N_Vector f, int mode)
{
  int r;
  if (m->erk) return full_rhs_erk(m, t, y, f, mode);
  switch (mode)
  {
  case FULLRHS_START:
    if (!m->fn_is_current && eval_both(m, t, y)) return ARK_RHSFUNC_FAIL;
    sum_first(m, f);
    break;
  case FULLRHS_END:
    if (!m->fn_is_current)
    {
      const int recompute = (m->explicit_ && !m->sa_e) || !m->sa_i;
      if (recompute)
      {
        if (eval_both(m, t, y)) return ARK_RHSFUNC_FAIL;
      }
      else
      {
        if (m->explicit_) v_scale(1.0, m->Fe[m->s - 1], m->Fe[0]);
        v_scale(1.0, m->Fi[m->s - 1], m->Fi[0]);
      }
    }
    sum_first(m, f);
    break;
  default:
    if (m->explicit_)
    {
      r = m->fe(t, y, m->tempv2, m->user_data);
      m->nfe++;
      if (r != 0) return ARK_RHSFUNC_FAIL;
    }
    r = m->fi(t, y, m->sdata, m->user_data);
    m->nfi++;
    if (r != 0) return ARK_RHSFUNC_FAIL;
    if (m->explicit_) v_linearsum(1.0, m->sdata, 1.0, m->tempv2, f);
    else v_scale(1.0, m->sdata, f);
    break;
  }
  return 0;
}

/* ------------------------------------------------------ ARKLS callbacks */
/* arkLsDQJtimes: Jv = (fi(t, y + sig v) - fy) / sig, sig = 1 / |v|_wrms */
static int dq_jtimes(ArkPort* m, N_Vector v, N_Vector Jv, double t, N_Vector y, N_Vector fy,
                     N_Vector work)
{
  double sig = 1.0 / v_wrms(v, m->ewt);
  int retval = 0;
  for (int iter = 0; iter < MAX_DQITERS; iter++)
  {
    v_linearsum(sig, v, 1.0, y, work);
    retval = m->fi(t, work, Jv, m->user_data);
    m->nfeDQ++;
    if (retval == 0) break;
    if (retval < 0) return -1;
    sig *= 0.25;
  }
  if (retval > 0) return 1;
  const double siginv = 1.0 / sig;
  v_linearsum(siginv, Jv, -siginv, fy, Jv);
  return 0;
}

static int ls_atimes(void* mem, N_Vector v, N_Vector z)
{ /* arkLsATimes (identity mass matrix) */
  ArkPort* m = (ArkPort*)mem;
  int r      = m->jtimes
                 ? m->jtimes(v, z, m->ls_tcur, m->ls_ycur, m->ls_fcur, m->user_data, m->ls_ytemp)
                 : dq_jtimes(m, v, z, m->ls_tcur, m->ls_ycur, m->ls_fcur, m->ls_ytemp);
  m->njtimes++;
  if (r != 0) return r;
  v_linearsum(1.0, v, -m->gamma, z, z);
  return 0;
}

static int ls_psetup(void* mem)
{ /* arkLsPSetup: jok = !jbad, jcurPtr = the step's jcur */
  ArkPort* m = (ArkPort*)mem;
  return m->pset(m->ls_tcur, m->ls_ycur, m->ls_fcur, !(m->jbad), &m->jcur, m->gamma,
                 m->user_data);
}

static int ls_psolve(void* mem, N_Vector r, N_Vector z, double tol, int lr)
{ /* arkLsPSolve */
  ArkPort* m = (ArkPort*)mem;
  int ret = m->psolve(m->ls_tcur, m->ls_ycur, m->ls_fcur, r, z, m->gamma, tol, lr, m->user_data);
  m->nps++;
  return ret;
}

/* arkLsSolve, iterative and matrix-free (rwt = ewt) */
/* arkLsLinSys (arkode_ls.c:2890-2975): A = I - gamma J, J new or saved */
static int ls_linsys(ArkPort* m, double t, N_Vector y, N_Vector fy, int jok)
{
  if (jok)
  {
    m->jcur = SUNFALSE;
    if (m->savedJ->ops->copy(m->savedJ, m->Amat)) return -1;
  }
  else
  {
    m->jcur = SUNTRUE;
    if (m->Amat->ops->zero(m->Amat)) return -1;
    int retval = m->jac(t, y, fy, m->Amat, m->user_data, m->tempv1, m->tempv2, m->tempv3);
    if (retval < 0) return -1;
    if (retval > 0) return 1;
    if (m->Amat->ops->copy(m->Amat, m->savedJ)) return -1;
  }
  if (m->Amat->ops->scaleaddi(-m->gamma, m->Amat)) return -1;
  return 0;
}

/* arkLsSetup with a matrix (arkode_ls.c:3166-3306) */
static int ls_setup(ArkPort* m, int convfail, double tpred, N_Vector ypred, N_Vector fpred)
{
  m->ls_tcur             = tpred;
  m->ls_ycur             = ypred;
  m->ls_fcur             = fpred;
  const int dgamma_fail  = fabs(m->gamrat - 1.0) >= DGMAX;
  m->jbad = m->initsetup || (m->nst >= m->nstlj + ARKLS_MSBJ) ||
            ((convfail == FAIL_BAD_J) && !dgamma_fail) || (convfail == FAIL_OTHER);
  if (!m->Amat)
  { /* matrix-free: the preconditioner setup runs inside the LS setup */
    m->jcur       = m->jbad;
    int last_flag = m->LS->ops->setup(m->LS, NULL);
    if (m->jcur)
    {
      m->npe++;
      m->nstlj = m->nst;
    }
    if (m->jbad) m->jcur = SUNTRUE;
    return last_flag;
  }
  int retval = ls_linsys(m, tpred, ypred, fpred, !m->jbad);
  if (m->jcur)
  {
    m->nje++;
    m->nstlj = m->nst;
  }
  if (retval != 0) return retval;
  return m->LS->ops->setup(m->LS, m->Amat);
}

/* arkLsSolve with a direct solver: no tolerance, x = A^{-1} b, the
 * correction scaled by 2 / (1 + gamrat) when gamma changed since setup */
static int ls_solve_direct(ArkPort* m, N_Vector b, double tnow, N_Vector ynow, N_Vector fnow,
                           int mnewt)
{
  m->ls_tcur = tnow;
  m->ls_ycur = ynow;
  m->ls_fcur = fnow;
  if (m->LS->ops->setscalingvectors) m->LS->ops->setscalingvectors(m->LS, m->ewt, m->ewt);
  v_const(0.0, m->ls_x);
  if (m->LS->ops->setzeroguess) m->LS->ops->setzeroguess(m->LS, SUNTRUE);
  int retval = m->LS->ops->solve(m->LS, m->Amat, m->ls_x, b, 0.0);
  v_scale(1.0, m->ls_x, b);
  if (m->gamrat != 1.0) v_scale(2.0 / (1.0 + m->gamrat), b, b);
  if (retval != 0) m->ncfl++;
  switch (retval)
  {
  case 0: return 0;
  case SUNLS_RES_REDUCED: return mnewt == 0 ? 0 : 1;
  case SUNLS_CONV_FAIL:
  case SUNLS_ATIMES_FAIL_REC:
  case SUNLS_PSOLVE_FAIL_REC:
  case SUNLS_PACKAGE_FAIL_REC:
  case SUNLS_QRFACT_FAIL:
  case SUNLS_LUFACT_FAIL: return 1;
  default: return retval < 0 ? -1 : 0;
  }
}

static int ls_solve(ArkPort* m, N_Vector b, double tnow, N_Vector ynow, N_Vector fnow,
                    double eRNrm, int mnewt)
{
  if (m->Amat) return ls_solve_direct(m, b, tnow, ynow, fnow, mnewt);
  m->ls_tcur        = tnow;
  m->ls_ycur        = ynow;
  m->ls_fcur        = fnow;
  const double deltar = m->eplifac * eRNrm;
  const double bnorm  = v_wrms(b, m->ewt);
  if (bnorm <= deltar)
  {
    if (mnewt > 0) v_const(0.0, b);
    return 0;
  }
  double delta = deltar * m->nrmfac;
  if (m->LS->ops->setscalingvectors) m->LS->ops->setscalingvectors(m->LS, m->ewt, m->ewt);
  else
  {
    v_const(1.0, m->ls_x);
    const double rwt_mean = v_wrms(m->ewt, m->ls_x);
    delta /= rwt_mean;
  }
  v_const(0.0, m->ls_x);
  if (m->LS->ops->setzeroguess) m->LS->ops->setzeroguess(m->LS, SUNTRUE);
  int retval = m->LS->ops->solve(m->LS, NULL, m->ls_x, b, delta);
  v_scale(1.0, m->ls_x, b);
  int nli_inc = m->LS->ops->numiters ? m->LS->ops->numiters(m->LS) : 0;
  m->nli += nli_inc;
  if (retval != 0) m->ncfl++;
  switch (retval)
  {
  case 0: return 0;
  case SUNLS_RES_REDUCED: return mnewt == 0 ? 0 : 1;
  case SUNLS_CONV_FAIL:
  case SUNLS_ATIMES_FAIL_REC:
  case SUNLS_PSOLVE_FAIL_REC:
  case SUNLS_PACKAGE_FAIL_REC:
  case SUNLS_QRFACT_FAIL:
  case SUNLS_LUFACT_FAIL: return 1;
  default: return retval < 0 ? -1 : 0;
  }
}

/* ------------------------------------------------------ Newton + ARKStep NLS */
static int nls_residual(ArkPort* m, N_Vector zcor, N_Vector r)
{ /* arkStep_NlsResidual_MassIdent; with the task-local Newton the
   * benchmark's TaskLocalNlsResidual (arkode_driver.cpp:546-578): the same
   * arithmetic, its evaluations counted apart, failures returned as -1 / +1 */
  double c[3];
  N_Vector X[3];
  v_linearsum(1.0, m->zpred, 1.0, zcor, m->ycur);
  int ret = m->fi(m->tcur, m->ycur, m->Fi[m->istage], m->user_data);
  if (m->block_lsolve)
  {
    m->nnlfi++;
    if (ret != 0) return ret < 0 ? -1 : 1;
  }
  else
  {
    m->nfi++;
    if (ret < 0) return ARK_RHSFUNC_FAIL;
    if (ret > 0) return RHSFUNC_RECVR;
  }
  c[0] = 1.0;
  X[0] = zcor;
  c[1] = -1.0;
  X[1] = m->sdata;
  c[2] = -m->gamma;
  X[2] = m->Fi[m->istage];
  v_lincomb(3, c, X, r);
  return 0;
}

static int nls_lsolve(ArkPort* m, N_Vector b)
{ /* arkStep_NlsLSolve; task-local: TaskLocalLSolve (arkode_driver.cpp:580-596) */
  if (m->block_lsolve) return m->block_lsolve(m->ycur, b, b, m->gamma, m->user_data);
  int retval = ls_solve(m, b, m->tcur, m->ycur, m->Fi[m->istage], m->eRNrm, m->curiter);
  if (retval < 0) return ARK_LSOLVE_FAIL;
  if (retval > 0) return CONV_FAIL;
  return 0;
}

static int nls_convtest(ArkPort* m, N_Vector del, double tol, int mcur)
{ /* arkStep_NlsConvTest */
  const double delnrm = v_wrms(del, m->ewt);
  if (mcur > 0) m->crate = dmax(CRDOWN * m->crate, delnrm / m->delp);
  const double dcon = dmin(m->crate, 1.0) * delnrm / tol;
  if (dcon <= 1.0) return 0;
  if ((mcur >= 1) && (delnrm > RDIV * m->delp)) return NLS_CONV_RECVR;
  m->delp = delnrm;
  return NLS_CONTINUE;
}

/* arkStep_NlsLSetup (arkode_arkstep_nls.c:472-512) */
static int nls_lsetup(ArkPort* m, int jbad)
{
  if (jbad) m->convfail = FAIL_BAD_J;
  m->nsetups++;
  int retval    = ls_setup(m, m->convfail, m->tcur, m->ycur, m->Fi[m->istage]);
  m->nls_jcur   = m->jcur;
  m->firststage = SUNFALSE;
  m->gamrat = m->crate = 1.0;
  m->gammap            = m->gamma;
  m->nstlp             = m->nst;
  if (retval < 0) return ARK_LSETUP_FAIL;
  if (retval > 0) return CONV_FAIL;
  return 0;
}

/* SUNNonlinSolSolve_Newton; a recoverable failure is retried with a fresh
 * setup (jbad) when there is a linear solver setup (a matrix or a
 * preconditioner setup) and the Jacobian was not current */
static int newton_solve(ArkPort* m, N_Vector zcor, double tol, int callLSetup)
{
  N_Vector delta = m->delta;
  int retval, jbad = 0;
  m->niters     = 0;
  m->nconvfails = 0;
  for (;;)
  {
    m->curiter = 0;
    retval     = nls_residual(m, zcor, delta);
    if (retval != 0) break;
    if (callLSetup)
    {
      retval = nls_lsetup(m, jbad);
      if (retval != 0) break;
    }
    for (;;)
    {
      m->niters++;
      v_scale(-1.0, delta, delta);
      retval = nls_lsolve(m, delta);
      if (retval != 0) break;
      v_linearsum(1.0, zcor, 1.0, delta, zcor);
      retval = nls_convtest(m, delta, tol, m->curiter);
      m->curiter++;
      if (retval == 0)
      {
        m->nls_jcur = SUNFALSE;
        return 0;
      }
      if (retval != NLS_CONTINUE) break;
      if (m->curiter >= MAXCOR)
      {
        retval = NLS_CONV_RECVR;
        break;
      }
      retval = nls_residual(m, zcor, delta);
      if (retval != 0) break;
    }
    if ((retval > 0) && !m->nls_jcur && (m->Amat || m->pset))
    {
      m->nconvfails++;
      callLSetup = 1;
      jbad       = 1;
      v_const(0.0, zcor);
      continue;
    }
    break;
  }
  m->nconvfails++;
  return retval;
}

/* arkStep_NlsFPFunction_MassIdent (arkode_arkstep_nls.c:874-900):
 * g = gamma Fi(zpred + zcor) + sdata */
static int fp_sys(void* mem, N_Vector zcor, N_Vector g)
{
  ArkPort* m = (ArkPort*)mem;
  v_linearsum(1.0, m->zpred, 1.0, zcor, m->ycur);
  int ret = m->fi(m->tcur, m->ycur, m->Fi[m->istage], m->user_data);
  m->nfi++;
  if (ret < 0) return ARK_RHSFUNC_FAIL;
  if (ret > 0) return RHSFUNC_RECVR;
  v_linearsum(m->gamma, m->Fi[m->istage], 1.0, m->sdata, g);
  return 0;
}

static int fp_ctest(void* mem, N_Vector zcor, N_Vector del, double tol, int curiter)
{
  (void)zcor;
  return nls_convtest((ArkPort*)mem, del, tol, curiter);
}

static int nls(ArkPort* m, int nflag)
{ /* arkStep_Nls: an lsetup exists with a matrix-based linear solver or a
   * preconditioner setup (arkLsInitialize disables it otherwise) */
  int callLSetup = 0;
  if (m->Amat || m->pset)
  {
    m->convfail = ((nflag == FIRST_CALL) || (nflag == PREV_ERR_FAIL)) ? NO_FAILURES : FAIL_OTHER;
    callLSetup = m->firststage || (fabs(m->gamrat - 1.0) > DGMAX) ||
                 (nflag == PREV_CONV_FAIL) || (nflag == PREV_ERR_FAIL) ||
                 (m->nst >= m->nstlp + MSBP);
  }
  else m->crate = 1.0;
  v_const(0.0, m->zcor);
  m->eRNrm   = 0.1 * NLSCOEF;
  int retval = m->fp ? fp_port_solve(m->fp, m->zcor, NLSCOEF, fp_sys, fp_ctest, m)
                     : newton_solve(m, m->zcor, NLSCOEF, callLSetup);
  if (m->fp)
  {
    m->nls_iters += fp_port_niters(m->fp);
    m->nls_fails += fp_port_nconvfails(m->fp);
  }
  else if (m->block_lsolve)
  { /* TaskLocalNewton_Solve on one task (arkode_driver.cpp:615-640): the
     * status passes through; it reports no iteration count and a running
     * total of CONV_RECVR returns as its convergence-failure count */
    if (retval == NLS_CONV_RECVR) m->tl_ncnf++;
    m->nls_fails += m->tl_ncnf;
  }
  else
  {
    m->nls_iters += m->niters;
    m->nls_fails += m->nconvfails;
  }
  if (retval == 0)
  {
    m->jcur = SUNFALSE;
    v_linearsum(1.0, m->zcor, 1.0, m->zpred, m->ycur);
    return ARK_SUCCESS;
  }
  if (retval == NLS_CONV_RECVR) return CONV_FAIL;
  return retval;
}

/* ------------------------------------------------------ step pieces */
static int stage_setup(ArkPort* m, int implicit)
{ /* arkStep_StageSetup, identity mass */
  double cvals[2 * MAXS + 2];
  N_Vector X[2 * MAXS + 2];
  const int i = m->istage;
  int nvec    = 0;
  if (implicit)
  {
    m->gamma = m->h * m->A[i][i];
    if (m->firststage) m->gammap = m->gamma;
    m->gamrat = m->firststage ? 1.0 : m->gamma / m->gammap;
    v_linearsum(1.0, m->yn, -1.0, m->zpred, m->sdata);
    cvals[0] = 1.0;
    X[0]     = m->sdata;
    nvec     = 1;
  }
  if (m->explicit_)
    for (int j = 0; j < i; j++)
    {
      cvals[nvec] = m->h * m->Ae[i][j];
      X[nvec]     = m->Fe[j];
      nvec++;
    }
  for (int j = 0; j < i; j++)
  {
    cvals[nvec] = m->h * m->A[i][j];
    X[nvec]     = m->Fi[j];
    nvec++;
  }
  v_lincomb(nvec, cvals, X, m->sdata);
  return 0;
}

static int compute_solutions(ArkPort* m, double* dsm)
{ /* arkStep_ComputeSolutions */
  double cvals[2 * MAXS + 2];
  N_Vector X[2 * MAXS + 2];
  N_Vector yerr = m->tempv1;
  int nvec;
  *dsm = 0.0;
  if (!m->stiffly_accurate)
  {
    cvals[0] = 1.0;
    X[0]     = m->yn;
    nvec     = 1;
    for (int j = 0; j < m->s; j++)
    {
      if (m->explicit_)
      {
        cvals[nvec] = m->h * m->be[j];
        X[nvec]     = m->Fe[j];
        nvec++;
      }
      cvals[nvec] = m->h * m->b[j];
      X[nvec]     = m->Fi[j];
      nvec++;
    }
    v_lincomb(nvec, cvals, X, m->ycur);
  }
  nvec = 0;
  for (int j = 0; j < m->s; j++)
  {
    if (m->explicit_)
    {
      cvals[nvec] = m->h * (m->be[j] - m->de[j]);
      X[nvec]     = m->Fe[j];
      nvec++;
    }
    cvals[nvec] = m->h * (m->b[j] - m->d[j]);
    X[nvec]     = m->Fi[j];
    nvec++;
  }
  v_lincomb(nvec, cvals, X, yerr);
  *dsm = v_wrms(yerr, m->ewt);
  return 0;
}

/* erkStep_TakeStep / erkStep_ComputeSolutions (arkode_erkstep.c:736-997,
 * 1413-1516): stage z_i = sum_j h A_ij F_j + yn in one linear combination,
 * y = sum_j h b_j F_j + yn, error = sum_j h (b_j - d_j) F_j */
static int take_step_erk(ArkPort* m, double* dsm, int* nflag)
{
  double cvals[MAXS + 1];
  N_Vector X[MAXS + 1];
  int nvec;
  *nflag = ARK_SUCCESS;
  if (!m->fn_is_current)
  {
    int r = full_rhs(m, m->tn, m->yn, m->fn, m->initsetup ? FULLRHS_START : FULLRHS_END);
    if (r) return ARK_RHSFUNC_FAIL;
    m->fn_is_current = SUNTRUE;
  }
  for (int is = 1; is < m->s; is++)
  {
    m->tcur = m->tn + m->c[is] * m->h;
    nvec    = 0;
    for (int js = 0; js < is; js++)
    {
      cvals[nvec] = m->h * m->A[is][js];
      X[nvec]     = m->Fi[js];
      nvec++;
    }
    cvals[nvec] = 1.0;
    X[nvec]     = m->yn;
    nvec++;
    v_lincomb(nvec, cvals, X, m->ycur);
    int r = m->fi(m->tcur, m->ycur, m->Fi[is], m->user_data);
    m->nfe++;
    if (r < 0) return ARK_RHSFUNC_FAIL;
    if (r > 0) return ARK_UNREC_RHSFUNC_ERR;
  }
  nvec = 0;
  for (int j = 0; j < m->s; j++)
  {
    cvals[nvec] = m->h * m->b[j];
    X[nvec]     = m->Fi[j];
    nvec++;
  }
  cvals[nvec] = 1.0;
  X[nvec]     = m->yn;
  nvec++;
  v_lincomb(nvec, cvals, X, m->ycur);
  nvec = 0;
  for (int j = 0; j < m->s; j++)
  {
    cvals[nvec] = m->h * (m->b[j] - m->d[j]);
    X[nvec]     = m->Fi[j];
    nvec++;
  }
  v_lincomb(nvec, cvals, X, m->tempv1);
  *dsm = v_wrms(m->tempv1, m->ewt);
  return ARK_SUCCESS;
}

static int take_step(ArkPort* m, double* dsm, int* nflag)
{ /* arkStep_TakeStep_Z */
  if (m->erk) return take_step_erk(m, dsm, nflag);
  int implicit_stage = fabs(m->A[0][0]) > TINY;
  const int is_start = implicit_stage ? 0 : 1;
  /* the Hermite module needs fn, so it is always evaluated (or copied) */
  if (!m->fn_is_current)
  {
    int r = full_rhs(m, m->tn, m->yn, m->fn, m->initsetup ? FULLRHS_START : FULLRHS_END);
    if (r) return ARK_RHSFUNC_FAIL;
    m->fn_is_current = SUNTRUE;
  }
  for (int is = is_start; is < m->s; is++)
  {
    m->istage      = is;
    implicit_stage = fabs(m->A[is][is]) > TINY;
    m->tcur        = m->tn + m->c[is] * m->h;
    if (implicit_stage) v_scale(1.0, m->yn, m->zpred); /* trivial predictor */
    stage_setup(m, implicit_stage);
    if (implicit_stage)
    {
      *nflag = nls(m, *nflag);
      if (*nflag != ARK_SUCCESS) return TRY_AGAIN;
    }
    else v_linearsum(1.0, m->yn, 1.0, m->sdata, m->ycur);
    int r = m->fi(m->tcur, m->ycur, m->Fi[is], m->user_data);
    m->nfi++;
    if (r < 0) return ARK_RHSFUNC_FAIL;
    if (r > 0) return ARK_UNREC_RHSFUNC_ERR;
    if (m->explicit_)
    {
      r = m->fe(m->tn + m->ce[is] * m->h, m->ycur, m->Fe[is], m->user_data);
      m->nfe++;
      if (r < 0) return ARK_RHSFUNC_FAIL;
      if (r > 0) return ARK_UNREC_RHSFUNC_ERR;
    }
  }
  *nflag = compute_solutions(m, dsm);
  if (*nflag < 0) return *nflag;
  if (*nflag > 0) return TRY_AGAIN;
  return ARK_SUCCESS;
}

static int check_convergence(ArkPort* m, int* nflag, int* ncf)
{ /* arkCheckConvergence */
  if (*nflag == ARK_SUCCESS) return ARK_SUCCESS;
  m->ncfn++;
  if (*nflag < 0)
  {
    if (*nflag == ARK_LSOLVE_FAIL) return ARK_LSOLVE_FAIL;
    if (*nflag == ARK_RHSFUNC_FAIL) return ARK_RHSFUNC_FAIL;
    return *nflag;
  }
  (*ncf)++;
  m->etamax = 1.0;
  if (*ncf == MAXNCF)
  {
    if (*nflag == CONV_FAIL) return ARK_CONV_FAILURE;
    if (*nflag == RHSFUNC_RECVR) return ARK_REPTD_RHSFUNC_ERR;
  }
  m->eta = ETACF;
  *nflag = PREV_CONV_FAIL;
  return PREDICT_AGAIN;
}

/* arkAdapt with the default I controller: h_acc = h (bias dsm)^(-1/(p+1)) */
static void adapt(ArkPort* m, double hcur, double dsm)
{
  const int ord   = m->p + 1;
  const double e1 = 1.0 * dsm;
  const double k1 = -1.0 / ord;
  double h_acc    = hcur * pow(e1, k1);
  h_acc *= m->safety;
  h_acc = dmin(fabs(h_acc), fabs(m->etamax * hcur));
  h_acc = dmax(h_acc, fabs(ETAMIN * hcur));
  if (dsm <= 1.0)
  {
    if ((h_acc > fabs(hcur * HFIXED_LB * ONEMSM)) && (h_acc < fabs(hcur * HFIXED_UB * ONEPSM)))
      h_acc = hcur;
  }
  h_acc  = copysign(h_acc, hcur);
  m->eta = h_acc / hcur;
  m->eta = dmax(m->eta, 0.0 / fabs(hcur));           /* hmin = 0 */
  m->eta /= dmax(1.0, fabs(hcur) * 0.0 * m->eta);    /* hmax_inv = 0 */
}

static int check_temporal_error(ArkPort* m, int* nflag, int* nef, double dsm)
{ /* arkCheckTemporalError */
  adapt(m, m->h, dsm);
  m->eta = dmin(m->eta, m->etamax);
  m->eta = dmax(m->eta, 0.0 / fabs(m->h));
  m->eta /= dmax(1.0, fabs(m->h) * 0.0 * m->eta);
  if (dsm <= 1.0) return ARK_SUCCESS;
  (*nef)++;
  m->netf++;
  *nflag = PREV_ERR_FAIL;
  if (*nef == MAXNEF) return ARK_ERR_FAILURE;
  m->etamax = 1.0;
  if (*nef >= SMALL_NEF) m->eta = dmin(m->eta, ETAMXF);
  m->eta = dmin(m->eta, m->etamax);
  m->eta = dmax(m->eta, 0.0 / fabs(m->h));
  m->eta /= dmax(1.0, fabs(m->h) * 0.0 * m->eta);
  return TRY_AGAIN;
}

static int complete_step(ArkPort* m, double dsm)
{ /* arkCompleteStep (+ arkInterpUpdate_Hermite, SUNAdaptController_UpdateH) */
  m->tcur = m->tn + m->h;
  if (!m->fn_is_current)
  {
    if (full_rhs(m, m->tn, m->yn, m->fn, FULLRHS_START)) return ARK_RHSFUNC_FAIL;
    m->fn_is_current = SUNTRUE;
  }
  v_scale(1.0, m->yn, m->yold);
  v_scale(1.0, m->fn, m->fold);
  m->hint_told = m->hint_tnew;
  m->hint_tnew = m->tcur;
  m->hint_h    = m->h;
  v_scale(1.0, m->ycur, m->yn);
  m->fn_is_current = SUNFALSE;
  m->c_ep          = 1.0 * dsm;
  m->c_hp          = m->h;
  m->nst++;
  m->hold       = m->h;
  m->tn         = m->tcur;
  m->hprime     = m->h * m->eta;
  m->etamax     = m->growth;
  m->initsetup  = SUNFALSE;
  m->firststage = SUNFALSE;
  return ARK_SUCCESS;
}

/* arkInterpEvaluate_Hermite, d = 0 (arkode_interp.c:441-700): the Hermite
 * interpolant of degree min(order, deg) at tnew + tau (tnew - told); the
 * quartic one bootstraps from the cubic at tau = -1/3 and the full
 * right-hand side there (into fa), the quintic one from quartics at -1/3
 * and -2/3 (fa, fb) */
static int interp_eval(ArkPort* m, double tau, int order, N_Vector dky)
{
  if (!m->fn_is_current)
  {
    if (full_rhs(m, m->tn, m->yn, m->fn, FULLRHS_END)) return ARK_RHSFUNC_FAIL;
    m->fn_is_current = SUNTRUE;
  }
  int qd = order > 0 ? order : 0;
  if (qd > m->interp_degree) qd = m->interp_degree;
  const double tau2 = tau * tau, tau3 = tau * tau2, tau4 = tau * tau3, tau5 = tau * tau4;
  const double h = m->hint_h;
  double a[6];
  N_Vector X[6];
  switch (qd)
  {
  case 0: v_linearsum(0.5, m->yold, 0.5, m->yn, dky); break;
  case 1: v_linearsum(-tau, m->yold, 1.0 + tau, m->yn, dky); break;
  case 2:
    a[0] = tau2;
    a[1] = 1.0 - tau2;
    a[2] = h * (tau2 + tau);
    X[0] = m->yold;
    X[1] = m->yn;
    X[2] = m->fn;
    v_lincomb(3, a, X, dky);
    break;
  case 3:
    a[0] = 3.0 * tau2 + 2.0 * tau3;
    a[1] = 1.0 - 3.0 * tau2 - 2.0 * tau3;
    a[2] = h * (tau2 + tau3);
    a[3] = h * (tau + 2.0 * tau2 + tau3);
    X[0] = m->yold;
    X[1] = m->yn;
    X[2] = m->fold;
    X[3] = m->fn;
    v_lincomb(4, a, X, dky);
    break;
  case 4:
    if (interp_eval(m, -1.0 / 3.0, 3, dky) != 0) return ARK_RHSFUNC_FAIL;
    if (full_rhs(m, m->hint_tnew - h / 3.0, dky, m->fa, FULLRHS_OTHER)) return ARK_RHSFUNC_FAIL;
    a[0] = -6.0 * tau2 - 16.0 * tau3 - 9.0 * tau4;
    a[1] = 1.0 + 6.0 * tau2 + 16.0 * tau3 + 9.0 * tau4;
    a[2] = h * 0.25 * (-5.0 * tau2 - 14.0 * tau3 - 9.0 * tau4);
    a[3] = h * (tau + 2.0 * tau2 + tau3);
    a[4] = h * 27.0 * 0.25 * (-tau4 - 2.0 * tau3 - tau2);
    X[0] = m->yold;
    X[1] = m->yn;
    X[2] = m->fold;
    X[3] = m->fn;
    X[4] = m->fa;
    v_lincomb(5, a, X, dky);
    break;
  case 5: /* from quartics at tau = -1/3 and -2/3 and the right-hand side there */
    if (interp_eval(m, -1.0 / 3.0, 4, dky) != 0) return ARK_RHSFUNC_FAIL;
    if (full_rhs(m, m->hint_tnew - h / 3.0, dky, m->fa, FULLRHS_OTHER)) return ARK_RHSFUNC_FAIL;
    if (interp_eval(m, -2.0 / 3.0, 4, dky) != 0) return ARK_RHSFUNC_FAIL;
    if (full_rhs(m, m->hint_tnew - h * 2.0 / 3.0, dky, m->fb, FULLRHS_OTHER))
      return ARK_RHSFUNC_FAIL;
    a[0] = 54.0 * tau5 + 135.0 * tau4 + 110.0 * tau3 + 30.0 * tau2;
    a[1] = 1.0 - a[0];
    a[2] = h / 4.0 * (27.0 * tau5 + 63.0 * tau4 + 49.0 * tau3 + 13.0 * tau2);
    a[3] = h / 4.0 * (27.0 * tau5 + 72.0 * tau4 + 67.0 * tau3 + 26.0 * tau2 + 4.0 * tau);
    a[4] = h / 4.0 * (81.0 * tau5 + 189.0 * tau4 + 135.0 * tau3 + 27.0 * tau2);
    a[5] = h / 4.0 * (81.0 * tau5 + 216.0 * tau4 + 189.0 * tau3 + 54.0 * tau2);
    X[0] = m->yold;
    X[1] = m->yn;
    X[2] = m->fold;
    X[3] = m->fn;
    X[4] = m->fa;
    X[5] = m->fb;
    v_lincomb(6, a, X, dky);
    break;
  default: return ARK_ILL_INPUT;
  }
  return ARK_SUCCESS;
}

/* ARKodeGetDky(t, 0) */
static int get_dky(ArkPort* m, double t, N_Vector dky)
{
  double tfuzz = FUZZ_FACTOR * UROUND * (fabs(m->tcur) + fabs(m->hold));
  if (m->hold < 0.0) tfuzz = -tfuzz;
  const double tp  = m->tcur - m->hold - tfuzz;
  const double tn1 = m->tcur + tfuzz;
  if ((t - tp) * (t - tn1) > 0.0) return ARK_BAD_T;
  return interp_eval(m, (t - m->tcur) / m->h, INTERP_MAX_DEGREE, dky);
}

/* arkUpperBoundH0 */
static double upper_bound_h0(ArkPort* m, double tdist)
{
  N_Vector temp1 = m->tempv1, temp2 = m->tempv2;
  temp2->ops->nvabs(m->yn, temp2);
  set_ewt(m, m->yn, temp1);
  temp1->ops->nvinv(temp1, temp1);
  v_linearsum(H0_UBFACTOR, temp2, 1.0, temp1, temp1);
  temp2->ops->nvabs(m->fn, temp2);
  temp1->ops->nvdiv(temp2, temp1, temp1);
  const double hub_inv = temp1->ops->nvmaxnorm(temp1);
  double hub           = H0_UBFACTOR * tdist;
  if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
  return hub;
}

/* arkYddNorm */
static int ydd_norm(ArkPort* m, double hg, double* yddnrm)
{
  v_linearsum(hg, m->fn, 1.0, m->yn, m->ycur);
  if (full_rhs(m, m->tcur + hg, m->ycur, m->tempv1, FULLRHS_OTHER)) return ARK_RHSFUNC_FAIL;
  v_linearsum(1.0 / hg, m->tempv1, -1.0 / hg, m->fn, m->tempv1);
  v_scale(1.0, m->yn, m->ycur);
  *yddnrm = v_wrms(m->tempv1, m->ewt);
  return ARK_SUCCESS;
}

static double sun_rsqrt(double x) { return x <= 0.0 ? 0.0 : sqrt(x); } /* SUNRsqrt */

/* arkHin */
static int hin(ArkPort* m, double tout)
{
  const double tdiff = tout - m->tcur;
  if (tdiff == 0.0) return ARK_TOO_CLOSE;
  const int sign      = tdiff > 0.0 ? 1 : -1;
  const double tdist  = fabs(tdiff);
  const double tround = UROUND * dmax(fabs(m->tcur), fabs(tout));
  if (tdist < 2.0 * tround) return ARK_TOO_CLOSE;
  if (!m->fn_is_current)
  {
    if (full_rhs(m, m->tn, m->yn, m->fn, FULLRHS_START)) return ARK_RHSFUNC_FAIL;
    m->fn_is_current = SUNTRUE;
  }
  const double hlb = H0_LBFACTOR * tround;
  const double hub = upper_bound_h0(m, tdist);
  double hg        = sun_rsqrt(hlb * hub);
  if (hub < hlb)
  {
    m->h = sign == -1 ? -hg : hg;
    return ARK_SUCCESS;
  }
  double hs = hg, hnew = hg, yddnrm = 0.0;
  for (int count1 = 1; count1 <= H0_ITERS; count1++)
  {
    int hgOK = 0;
    for (int count2 = 1; count2 <= H0_ITERS; count2++)
    {
      const double hgs = hg * sign;
      int retval       = ydd_norm(m, hgs, &yddnrm);
      if (retval < 0) return ARK_RHSFUNC_FAIL;
      if (retval == ARK_SUCCESS)
      {
        hgOK = 1;
        break;
      }
      hg *= 0.2;
    }
    if (!hgOK)
    {
      if (count1 <= 2) return ARK_REPTD_RHSFUNC_ERR;
      hnew = hs;
      break;
    }
    hs   = hg;
    hnew = (yddnrm * hub * hub > 2.0) ? sun_rsqrt(2.0 / yddnrm) : sun_rsqrt(hg * hub);
    if (count1 == H0_ITERS) break;
    const double hrat = hnew / hg;
    if ((hrat > 0.5) && (hrat < 2.0)) break;
    if ((count1 > 1) && (hrat > 2.0))
    {
      hnew = hg;
      break;
    }
    hg = hnew;
  }
  double h0 = H0_BIAS * hnew;
  if (h0 < hlb) h0 = hlb;
  if (h0 > hub) h0 = hub;
  if (sign == -1) h0 = -h0;
  m->h = h0;
  return ARK_SUCCESS;
}

/* arkInitialSetup (after arkStep_Init, FIRST_INIT) */
static int initial_setup(ArkPort* m, double tout)
{
  set_ewt(m, m->yn, m->ewt);
  if (m->LS && m->LS->ops->initialize && m->LS->ops->initialize(m->LS) != 0)
    return ARK_ILL_INPUT;
  /* Hermite module: degree min(q - 1, 5) for q > 1 (arkStep_Init), then
   * arkInterpInit_Hermite */
  m->interp_degree = INTERP_MAX_DEGREE;
  if (m->q > 1 && m->interp_degree > m->q - 1) m->interp_degree = m->q - 1;
  else if (m->q == 1 && m->interp_degree > 1) m->interp_degree = 1;
  m->hint_told = m->tcur;
  m->hint_tnew = m->tcur;
  m->hint_h    = 0.0;
  /* initial step */
  m->h = fabs(tout - m->tcur);
  if (m->h == 0.0) m->h = 1.0;
  int hflag = hin(m, tout);
  if (hflag != ARK_SUCCESS) return hflag;
  m->etamax = ETAMX1;
  m->h0u    = m->h;
  m->eta    = 1.0;
  m->hprime = m->h;
  return ARK_SUCCESS;
}

/* ------------------------------------------------------ public entry points */
/* fe NULL: implicit only (DIRK); else Ae/be/ce/de is the explicit table of
 * the ARK pair (same number of stages); q, p: the implicit table's orders. */
void* arkstep_port_create(ArkRhsFn fe, ArkRhsFn fi, double t0, N_Vector y0, double rtol,
                          double atol, long mxstep, SUNLinearSolver LS, ArkJTimesFn jtimes,
                          ArkPSolveFn psolve, void* user_data, int stages, int q, int p,
                          const double* A, const double* b, const double* c, const double* d,
                          const double* Ae, const double* be, const double* ce,
                          const double* de)
{
  if (stages < 1 || stages > MAXS) return NULL;
  ArkPort* m = (ArkPort*)calloc(1, sizeof(ArkPort));
  if (!m) return NULL;
  N_Vector (*clone)(N_Vector) = y0->ops->nvclone;
  m->yn     = clone(y0);
  m->fn     = clone(y0);
  m->ewt    = clone(y0);
  m->tempv1 = clone(y0);
  m->tempv2 = clone(y0);
  m->tempv3 = clone(y0);
  m->sdata  = clone(y0);
  m->zpred  = clone(y0);
  m->zcor   = clone(y0);
  m->delta  = clone(y0);
  m->ls_x   = clone(y0);
  m->ls_ytemp = clone(y0);
  m->yold   = clone(y0);
  m->fold   = clone(y0);
  m->fa     = clone(y0);
  m->fb     = clone(y0);
  for (int j = 0; j < stages; j++) m->Fi[j] = clone(y0);
  if (fe)
    for (int j = 0; j < stages; j++) m->Fe[j] = clone(y0);
  v_scale(1.0, y0, m->yn);
  m->fe        = fe;
  m->explicit_ = fe != NULL;
  m->fi        = fi;
  m->jtimes    = jtimes;
  m->psolve    = psolve;
  m->user_data = user_data;
  m->rtol      = rtol;
  m->atol      = atol;
  m->mxstep    = mxstep;
  m->LS        = LS;
  m->s         = stages;
  m->q         = q;
  m->p         = p;
  for (int i = 0; i < stages; i++)
  {
    for (int j = 0; j < stages; j++) m->A[i][j] = A[i * stages + j];
    m->b[i] = b[i];
    m->c[i] = c[i];
    m->d[i] = d[i];
    if (fe)
    {
      for (int j = 0; j < stages; j++) m->Ae[i][j] = Ae[i * stages + j];
      m->be[i] = be[i];
      m->ce[i] = ce[i];
      m->de[i] = de[i];
    }
  }
  /* ARKodeButcherTable_IsStifflyAccurate: b equals the last row of A */
  m->sa_i = m->sa_e = 1;
  for (int j = 0; j < stages; j++)
  {
    if (m->b[j] != m->A[stages - 1][j]) m->sa_i = 0;
    if (fe && m->be[j] != m->Ae[stages - 1][j]) m->sa_e = 0;
  }
  m->stiffly_accurate = m->sa_i && (!fe || m->sa_e);
  m->tn = m->tcur = m->tretlast = t0;
  m->initsetup  = SUNTRUE;
  m->firststage = SUNTRUE;
  m->eplifac    = ARKLS_EPLIN;
  m->nrmfac     = sqrt((double)y0->ops->nvgetlength(y0));
  m->c_ep = m->c_hp = 1.0;
  m->safety = SAFETY;
  m->growth = GROWTH;
  if (LS && LS->ops->setatimes) LS->ops->setatimes(LS, m, ls_atimes);
  if (LS && psolve && LS->ops->setpreconditioner)
    LS->ops->setpreconditioner(LS, m, NULL, ls_psolve);
  return m;
}

/* The benchmark's TaskLocalNewton (arkode_driver.cpp:546-780) on one task:
 * the reference's Newton with the per-cell block solve as its linear solve
 * and no SUNLinearSolver (create with LS and psolve NULL). */
void arkstep_port_set_task_local(void* mem, ArkBlockSolveFn block_lsolve)
{
  ((ArkPort*)mem)->block_lsolve = block_lsolve;
}

/* ARKodeSetLinearSolver(LS, A) with a matrix and a direct LS, and
 * ARKodeSetJacFn(jac): the matrix-based path of ARKLS (create the object
 * with LS and no psolve, then attach A and jac; the saved Jacobian is cloned
 * from A as arkLsInitialize does). */
void arkstep_port_set_matrix(void* mem, SUNMatrix A, ArkJacFn jac)
{
  ArkPort* m = (ArkPort*)mem;
  m->Amat       = A;
  m->jac     = jac;
  if (!m->savedJ) m->savedJ = A->ops->clone(A);
}

/* ARKodeSetPreconditioner(psetup, psolve) with a preconditioner setup: the
 * iterative solver's setup then calls it (arkLsSetup without a matrix). */
void arkstep_port_set_psetup(void* mem, ArkPSetupFn pset)
{
  ArkPort* m = (ArkPort*)mem;
  m->pset    = pset;
  if (m->LS->ops->setpreconditioner) m->LS->ops->setpreconditioner(m->LS, m, ls_psetup, ls_psolve);
}

/* ARKodeSVtolerances(rtol, abstol): a copy of abstol (all entries > 0). */
void arkstep_port_set_vabstol(void* mem, double rtol, N_Vector abstol)
{
  ArkPort* m = (ArkPort*)mem;
  m->rtol    = rtol;
  if (!m->Vabstol) m->Vabstol = abstol->ops->nvclone(abstol);
  v_scale(1.0, abstol, m->Vabstol);
}

/* ERKStepCreate(f, ...) instead of ARKStepCreate: create with fe NULL, fi = f
 * and the explicit table as the method table, then call this (before the
 * first solve); ERKStep's defaults: safety 0.99, growth 25
 * (arkode_erkstep_io.c:308-341). */
void arkstep_port_set_erk(void* mem)
{
  ArkPort* m = (ArkPort*)mem;
  m->erk     = 1;
  m->safety  = 0.99;
  m->growth  = 25.0;
}

/* ARKodeSetNonlinearSolver(SUNNonlinSol_FixedPoint(y, depth)) with no linear
 * solver (create with LS and psolve NULL). */
void arkstep_port_set_fixed_point(void* mem, int depth)
{
  ArkPort* m = (ArkPort*)mem;
  m->fp      = fp_port_create(m->ewt, depth);
}

/* ARKodeEvolve(tout, yout, &tret, ARK_NORMAL) */
int arkstep_port_solve(void* mem, double tout, N_Vector yout, double* tret)
{
  ArkPort* m = (ArkPort*)mem;
  int istate = ARK_SUCCESS;
  m->ycur    = yout;
  if (m->initsetup)
  {
    m->tretlast = *tret = m->tcur;
    int r               = initial_setup(m, tout);
    if (r != ARK_SUCCESS) return r;
  }
  else if ((m->tcur - tout) * m->h >= 0.0)
  { /* arkStopTests: tout already passed */
    int ier = get_dky(m, tout, yout);
    if (ier != ARK_SUCCESS) return ier;
    m->tretlast = *tret = tout;
    return ARK_SUCCESS;
  }
  long nstloc = 0;
  for (;;)
  {
    m->next_h = m->h;
    if (!m->initsetup) set_ewt(m, m->yn, m->ewt);
    if ((m->mxstep > 0) && (nstloc >= m->mxstep))
    {
      istate      = ARK_TOO_MUCH_WORK;
      m->tretlast = *tret = m->tcur;
      v_scale(1.0, m->yn, yout);
      break;
    }
    const double nrm = v_wrms(m->yn, m->ewt);
    m->tolsf         = UROUND * nrm;
    if (m->tolsf > 1.0)
    {
      istate      = ARK_TOO_MUCH_ACC;
      m->tretlast = *tret = m->tcur;
      v_scale(1.0, m->yn, yout);
      m->tolsf *= 2.0;
      break;
    }
    m->tolsf = 1.0;
    if (m->hprime != m->h)
    {
      m->h      = m->h * m->eta;
      m->next_h = m->h;
    }
    double dsm = 0.0;
    int kflag = ARK_SUCCESS, ncf = 0, nef = 0, nflag = FIRST_CALL;
    for (;;)
    {
      m->nst_attempts++;
      kflag = take_step(m, &dsm, &nflag);
      if (kflag < 0) break;
      kflag = check_convergence(m, &nflag, &ncf);
      if (kflag < 0) break;
      if (kflag == ARK_SUCCESS)
      {
        kflag = check_temporal_error(m, &nflag, &nef, dsm);
        if (kflag < 0) break;
      }
      if (kflag == ARK_SUCCESS) break;
      if (fabs(m->h) <= 0.0 * ONEPSM) return ARK_ERR_FAILURE; /* hmin = 0 */
      m->h *= m->eta;
      m->next_h = m->hprime = m->h;
    }
    if (kflag == ARK_SUCCESS) kflag = complete_step(m, dsm);
    if (kflag != ARK_SUCCESS)
    {
      istate      = kflag;
      m->tretlast = *tret = m->tcur;
      v_scale(1.0, m->yn, yout);
      break;
    }
    nstloc++;
    if ((m->tcur - tout) * m->h >= 0.0)
    {
      int r = get_dky(m, tout, yout);
      if (r != ARK_SUCCESS)
      {
        istate = r;
        break;
      }
      m->tretlast = *tret = tout;
      m->next_h           = m->hprime;
      istate              = ARK_SUCCESS;
      break;
    }
  }
  return istate;
}

/* counters: nst, nst_attempts, nfi, netf, ncfn, nni, nnf, nli, nps, njtimes,
 * nfeDQ, ncfl, nfe, nnlfi, nsetups, nje, npe; reals: last step, next step, current time, first step */
void arkstep_port_stats(void* mem, long* cnt, double* r)
{
  ArkPort* m = (ArkPort*)mem;
  cnt[0]     = m->nst;
  cnt[1]     = m->nst_attempts;
  cnt[2]     = m->nfi;
  cnt[3]     = m->netf;
  cnt[4]     = m->ncfn;
  cnt[5]     = m->nls_iters;
  cnt[6]     = m->nls_fails;
  cnt[7]     = m->nli;
  cnt[8]     = m->nps;
  cnt[9]     = m->njtimes;
  cnt[10]    = m->nfeDQ;
  cnt[11]    = m->ncfl;
  cnt[12]    = m->nfe;
  cnt[13]    = m->nnlfi;
  cnt[14]    = m->nsetups;
  cnt[15]    = m->nje;
  cnt[16]    = m->npe;
  r[0]       = m->hold;
  r[1]       = m->next_h;
  r[2]       = m->tcur;
  r[3]       = m->h0u;
}

void arkstep_port_free(void* mem)
{
  ArkPort* m = (ArkPort*)mem;
  if (!m) return;
  N_Vector vs[] = {m->yn,   m->fn,    m->ewt,  m->tempv1, m->tempv2,   m->tempv3, m->sdata,
                   m->zpred, m->zcor, m->delta, m->ls_x,  m->ls_ytemp, m->yold,   m->fold,
                   m->fa,    m->fb};
  for (size_t i = 0; i < sizeof(vs) / sizeof(vs[0]); i++)
    if (vs[i]) vs[i]->ops->nvdestroy(vs[i]);
  for (int j = 0; j < m->s; j++)
  {
    if (m->Fi[j]) m->Fi[j]->ops->nvdestroy(m->Fi[j]);
    if (m->Fe[j]) m->Fe[j]->ops->nvdestroy(m->Fe[j]);
  }
  fp_port_free(m->fp);
  if (m->savedJ) m->savedJ->ops->destroy(m->savedJ);
  if (m->Vabstol) m->Vabstol->ops->nvdestroy(m->Vabstol);
  free(m);
}

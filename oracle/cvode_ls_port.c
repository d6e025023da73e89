/* cvode_ls_port.c -- TEST ORACLE (checker only, never part of the product).
 *
 * CVODE with BDF, the Newton nonlinear solver and either a matrix-free
 * iterative SUNLinearSolver (user or difference-quotient Jacobian-times-
 * vector, optional preconditioner) or a matrix-based direct one (SUNMatrix,
 * user Jacobian) -- or the fixed-point nonlinear solver with Anderson
 * acceleration and no linear solver (oracle/fixedpoint_port.c), with BDF or
 * (CV_ADAMS) Adams-Moulton -- restated
 * over the generic object model: every vector operation is dispatched through
 * the vector's ops table the way the reference's generic layer dispatches it
 * (fused and vector-array operations when the vector provides them, the
 * reference's fallback compositions otherwise), and the linear solver is
 * driven only through its ops table.  The same code therefore runs the
 * reference's own NVECTOR_SERIAL + SUNLINSOL_SPGMR objects (pinned bit for
 * bit against the reference's CVode by tests/test_cvode_ls_port.py) and
 * NVECTOR_GB300 + SUNLinSol_SPGMR_GB300 on a GPU machine where the
 * reference library is not available.
 *
 * Follows, in the same floating-point order (compiled with -ffp-contract=off):
 *   CVode, CV_NORMAL (no tstop, roots, constraints or projection)
 *                                  src/cvode/cvode.c:1037-1640
 *   cvEwtSetSS / cvEwtSetSV        cvode.c:4791-4860
 *   cvHin / cvUpperBoundH0 / cvYddNorm   cvode.c:2161-2340
 *   cvStep and its callees         cvode.c:2367-3727
 *   (Adams: cvAdjustAdams, cvSetAdams, cvAdamsStart, cvAdamsFinish, cvAltSum
 *                                  cvode.c:2545-2600, 2800-2940)
 *   CVodeGetDky (k = 0)            cvode.c:1671-1750
 *   cvNlsResidual / LSetup / LSolve / ConvTest / FPFunction
 *                                  src/cvode/cvode_nls.c:256-425
 *   SUNNonlinSolSolve_Newton       src/sunnonlinsol/newton/sunnonlinsol_newton.c:179-330
 *   CVodeSetLinearSolver defaults, cvLsInitialize (saved J), cvLsLinSys,
 *   cvLsATimes / cvLsDQJtimes / cvLsPSetup / cvLsPSolve, cvLsSetup, cvLsSolve
 *                                  src/cvode/cvode_ls.c:56-285, 895-980, 1536-1900
 *   N_VLinearCombination / N_VScaleAddMulti / N_VScaleVectorArray dispatch
 *                                  src/sundials/sundials_nvector.c:549-670
 * The scalar step logic is the one of oracle/cvode_bdf_port.c. */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "../include/sundials_gb300_abi.h"
#include "fixedpoint_port.h"

#define QMAX 5      /* BDF_Q_MAX */
#define QMAX_ALL 12 /* ADAMS_Q_MAX: array sizes */
#define UROUND DBL_EPSILON

/* CVODE / CVLS / Newton defaults (cvode_impl.h:55-127, cvode.c:118-125,
 * cvode_nls.c:32-34, cvode_ls_impl.h:43-48, sunnonlinsol_newton.c:33) */
#define MXNCF 10
#define MXNEF 7
#define MXNEF1 3
#define LONG_WAIT 10
#define ETA_MAX_FX 1.5
#define ETA_MAX_FS 10000.0
#define ETA_MAX_ES 10.0
#define ETA_MAX_GS 10.0
#define ETA_MIN 0.1
#define ETA_MAX_EF 0.2
#define ETA_MIN_EF 0.1
#define ETA_CF 0.25
#define SMALL_NST 10
#define SMALL_NEF 2
#define ADDON 0.000001
#define BIAS1 6.0
#define BIAS2 6.0
#define BIAS3 10.0
#define HLB_FACTOR 100.0
#define HUB_FACTOR 0.1
#define MAX_ITERS 4
#define FUZZ_FACTOR 100.0
#define CORTES 0.1
#define NLS_MAXCOR 3
#define CRDOWN 0.3
#define RDIV 2.0
#define MSBP 20
#define DGMAX_LSETUP 0.3
#define CVLS_MSBJ 51
#define CVLS_DGMAX 0.2
#define CVLS_EPLIN 0.05

enum { FIRST_CALL = 6, PREV_CONV_FAIL = 7, PREV_ERR_FAIL = 9 };
enum { NO_FAILURES = 0, FAIL_BAD_J = 1, FAIL_OTHER = 2 };
enum { NLS_CONTINUE = 901, NLS_CONV_RECVR = 902, RHSFUNC_RECVR = 9 };
enum { DO_ERROR_TEST = 2, PREDICT_AGAIN = 3, TRY_AGAIN = 5 };
enum { CV_SUCCESS = 0, CV_TOO_MUCH_WORK = -1, CV_TOO_MUCH_ACC = -2, CV_ERR_FAILURE = -3,
       CV_CONV_FAILURE = -4, CV_LSETUP_FAIL = -6, CV_LSOLVE_FAIL = -7, CV_RHSFUNC_FAIL = -8,
       CV_REPTD_RHSFUNC_ERR = -10, CV_BAD_T = -25 };

/* The user callbacks, with CVODE's signatures (cvode.h, cvode_ls.h). */
typedef int (*CvlsRhsFn)(double t, N_Vector y, N_Vector ydot, void* user_data);
typedef int (*CvlsJTimesFn)(N_Vector v, N_Vector Jv, double t, N_Vector y, N_Vector fy,
                            void* user_data, N_Vector tmp);
typedef int (*CvlsPSetupFn)(double t, N_Vector y, N_Vector fy, sunbooleantype jok,
                            sunbooleantype* jcurPtr, double gamma, void* user_data);
typedef int (*CvlsPSolveFn)(double t, N_Vector y, N_Vector fy, N_Vector r, N_Vector z,
                            double gamma, double delta, int lr, void* user_data);
typedef int (*CvlsJacFn)(double t, N_Vector y, N_Vector fy, SUNMatrix J, void* user_data,
                         N_Vector tmp1, N_Vector tmp2, N_Vector tmp3);

typedef struct
{
  /* problem and options */
  CvlsRhsFn f;
  CvlsJTimesFn jtimes;
  CvlsPSetupFn pset;
  CvlsPSolveFn psolve;
  void* user_data;
  double rtol, atol;
  long mxstep;
  SUNLinearSolver LS;
  SUNMatrix A, savedJ; /* matrix-based (direct) solver: A and CVLS's saved J */
  CvlsJacFn jac;
  /* vectors */
  N_Vector zn[QMAX_ALL + 1], ewt, acor, tempv, ftemp, y, delta, ls_x, ls_ytemp;
  N_Vector vtemp1, vtemp2, vtemp3;
  N_Vector ycur, fcur; /* CVLS's pointers to the current state and RHS */
  N_Vector Vabstol;    /* CVodeSVtolerances' copy, or NULL for scalar atol */
  /* CVLS */
  double nrmfac, eplifac;
  sunbooleantype jbad;
  long nstlj, npe, nli, nps, ncfl, njtimes, nfeDQ, nje;
  int initialized;
  /* Newton, or the fixed-point solver when fp is set (no linear solver) */
  FPPort* fp;
  int curiter;
  long niters, nconvfails;
  sunbooleantype nls_jcur;
  /* integrator */
  double tn, h, hscale, hprime, next_h, eta, etamax, etaq, etaqm1, etaqp1, hu, h0u, saved_tq5;
  double rl1, gamma, gammap, gamrat, crate, delp, acnrm;
  double tq[6], l[QMAX_ALL + 2], tau[QMAX_ALL + 2], cvals[QMAX_ALL + 1];
  int qmax, adams; /* CV_ADAMS (qmax 12) or CV_BDF (qmax 5) */
  int q, qprime, qwait, L, indx_acor, nscon, convfail, qu, next_q;
  sunbooleantype cv_jcur;
  long nst, nfe, nsetups, nni, ncfn, netf, nnf, nstlp;
} CvlsPort;

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

static void v_scaleaddmulti(int nvec, double* a, N_Vector x, N_Vector* Y, N_Vector* Z)
{
  if (x->ops->nvscaleaddmulti) x->ops->nvscaleaddmulti(nvec, a, x, Y, Z);
  else
    for (int i = 0; i < nvec; i++) x->ops->nvlinearsum(a[i], x, 1.0, Y[i], Z[i]);
}

static void v_scalevectorarray(int nvec, double* c, N_Vector* X, N_Vector* Z)
{
  if (Z[0]->ops->nvscalevectorarray) Z[0]->ops->nvscalevectorarray(nvec, c, X, Z);
  else
    for (int i = 0; i < nvec; i++) Z[0]->ops->nvscale(c[i], X[i], Z[i]);
}

/* cvEwtSetSS / cvEwtSetSV (absolute tolerances > 0, so no N_VMin test) */
static void set_ewt(CvlsPort* m, N_Vector ycur, N_Vector w)
{
  N_Vector t = m->tempv;
  t->ops->nvabs(ycur, t);
  if (m->Vabstol) v_linearsum(m->rtol, t, 1.0, m->Vabstol, t);
  else
  {
    v_scale(m->rtol, t, t);
    t->ops->nvaddconst(t, m->atol, t);
  }
  t->ops->nvinv(t, w);
}

static int rhs(CvlsPort* m, double t, N_Vector y, N_Vector f)
{
  int r = m->f(t, y, f, m->user_data);
  m->nfe++;
  return r;
}

/* ------------------------------------------------------ CVLS callbacks */
/* cvLsDQJtimes (cvode_ls.c:1266-1305): Jv = (f(t, y + sig v) - fy) / sig,
 * sig = 1 / |v|_wrms, shrunk by 1/4 on a recoverable f failure (3 tries) */
static int dq_jtimes(CvlsPort* m, N_Vector v, N_Vector Jv, double t, N_Vector y, N_Vector fy,
                     N_Vector work)
{
  double sig = 1.0 / v_wrms(v, m->ewt);
  int retval = 0;
  for (int iter = 0; iter < 3; iter++)
  {
    v_linearsum(sig, v, 1.0, y, work);
    retval = m->f(t, work, Jv, m->user_data);
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
{ /* cvLsATimes */
  CvlsPort* m = (CvlsPort*)mem;
  int r       = m->jtimes ? m->jtimes(v, z, m->tn, m->ycur, m->fcur, m->user_data, m->ls_ytemp)
                          : dq_jtimes(m, v, z, m->tn, m->ycur, m->fcur, m->ls_ytemp);
  m->njtimes++;
  if (r != 0) return r;
  v_linearsum(1.0, v, -m->gamma, z, z);
  return 0;
}

static int ls_psetup(void* mem)
{ /* cvLsPSetup */
  CvlsPort* m = (CvlsPort*)mem;
  return m->pset(m->tn, m->ycur, m->fcur, !(m->jbad), &m->cv_jcur, m->gamma, m->user_data);
}

static int ls_psolve(void* mem, N_Vector r, N_Vector z, double tol, int lr)
{ /* cvLsPSolve */
  CvlsPort* m = (CvlsPort*)mem;
  int ret     = m->psolve(m->tn, m->ycur, m->fcur, r, z, m->gamma, tol, lr, m->user_data);
  m->nps++;
  return ret;
}

/* cvLsLinSys (cvode_ls.c:1311-1400): A = I - gamma J with J new or saved */
static int ls_linsys(CvlsPort* m, N_Vector ypred, N_Vector fpred)
{
  if (!m->jbad)
  {
    m->cv_jcur = SUNFALSE;
    if (m->savedJ->ops->copy(m->savedJ, m->A)) return -1;
  }
  else
  {
    m->cv_jcur = SUNTRUE;
    if (m->LS->ops->gettype(m->LS) == SUNLINEARSOLVER_DIRECT && m->A->ops->zero(m->A)) return -1;
    int retval = m->jac(m->tn, ypred, fpred, m->A, m->user_data, m->vtemp1, m->vtemp2, m->vtemp3);
    if (retval < 0) return -1;
    if (retval > 0) return 1;
    if (m->A->ops->copy(m->A, m->savedJ)) return -1;
  }
  if (m->A->ops->scaleaddi(-m->gamma, m->A)) return -1;
  return 0;
}

/* cvLsSetup (cvode_ls.c:1536-1640); jcurPtr is &cv_jcur */
static int ls_setup(CvlsPort* m, int convfail, N_Vector ypred, N_Vector fpred)
{
  m->ycur       = ypred;
  m->fcur       = fpred;
  double dgamma = fabs((m->gamma / m->gammap) - 1.0);
  m->jbad       = (m->nst == 0) || (m->nst >= m->nstlj + CVLS_MSBJ) ||
            ((convfail == FAIL_BAD_J) && (dgamma < CVLS_DGMAX)) || (convfail == FAIL_OTHER);
  if (m->A)
  { /* matrix-based */
    int retval = ls_linsys(m, ypred, fpred);
    if (m->cv_jcur)
    {
      m->nje++;
      m->nstlj = m->nst;
    }
    if (retval != 0) return retval;
    return m->LS->ops->setup(m->LS, m->A);
  }
  m->cv_jcur = m->jbad;
  int flag   = m->LS->ops->setup(m->LS, NULL);
  if (m->cv_jcur)
  {
    m->npe++;
    m->nstlj = m->nst;
  }
  if (m->jbad) m->cv_jcur = SUNTRUE;
  return flag;
}

/* cvLsSolve, iterative, no direct-solver scaling (scalesol is off for a
 * matrix-free solver) */
static int ls_solve(CvlsPort* m, N_Vector b, N_Vector weight, N_Vector ynow, N_Vector fnow)
{
  const int curiter = m->curiter;
  if (m->A)
  { /* direct: no tolerance, x = A^{-1} b, BDF solution scaling (scalesol) */
    m->ycur = ynow;
    m->fcur = fnow;
    if (m->LS->ops->setscalingvectors) m->LS->ops->setscalingvectors(m->LS, weight, weight);
    v_const(0.0, m->ls_x);
    if (m->LS->ops->setzeroguess) m->LS->ops->setzeroguess(m->LS, SUNTRUE);
    int retval = m->LS->ops->solve(m->LS, m->A, m->ls_x, b, 0.0);
    v_scale(1.0, m->ls_x, b);
    if (m->gamrat != 1.0) v_scale(2.0 / (1.0 + m->gamrat), b, b);
    if (retval != 0) m->ncfl++;
    switch (retval)
    {
    case 0: return 0;
    case SUNLS_RES_REDUCED: return curiter == 0 ? 0 : 1;
    case SUNLS_CONV_FAIL:
    case SUNLS_ATIMES_FAIL_REC:
    case SUNLS_PSOLVE_FAIL_REC:
    case SUNLS_PACKAGE_FAIL_REC:
    case SUNLS_QRFACT_FAIL:
    case SUNLS_LUFACT_FAIL: return 1;
    default: return retval < 0 ? -1 : 0;
    }
  }
  double deltar     = m->eplifac * m->tq[4];
  double bnorm      = v_wrms(b, weight);
  if (bnorm <= deltar)
  {
    if (curiter > 0) v_const(0.0, b);
    return 0;
  }
  double delta = deltar * m->nrmfac;
  m->ycur      = ynow;
  m->fcur      = fnow;
  if (m->LS->ops->setscalingvectors) m->LS->ops->setscalingvectors(m->LS, weight, weight);
  else
  {
    v_const(1.0, m->ls_x);
    double w_mean = v_wrms(weight, m->ls_x);
    delta /= w_mean;
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
  case SUNLS_RES_REDUCED: return curiter == 0 ? 0 : 1;
  case SUNLS_CONV_FAIL:
  case SUNLS_ATIMES_FAIL_REC:
  case SUNLS_PSOLVE_FAIL_REC:
  case SUNLS_PACKAGE_FAIL_REC:
  case SUNLS_QRFACT_FAIL:
  case SUNLS_LUFACT_FAIL: return 1;
  default: return retval < 0 ? -1 : 0;
  }
}

/* ------------------------------------------------------ Newton + CVODE NLS */
static int nls_residual(CvlsPort* m, N_Vector ycor, N_Vector res)
{ /* cvNlsResidual */
  v_linearsum(1.0, m->zn[0], 1.0, ycor, m->y);
  int r = rhs(m, m->tn, m->y, m->ftemp);
  if (r < 0) return CV_RHSFUNC_FAIL;
  if (r > 0) return RHSFUNC_RECVR;
  v_linearsum(m->rl1, m->zn[1], 1.0, ycor, res);
  v_linearsum(-m->gamma, m->ftemp, 1.0, res, res);
  return 0;
}

static int nls_lsetup(CvlsPort* m, int jbad)
{ /* cvNlsLSetup */
  if (jbad) m->convfail = FAIL_BAD_J;
  int retval = ls_setup(m, m->convfail, m->y, m->ftemp);
  m->nsetups++;
  m->nls_jcur = m->cv_jcur;
  m->gamrat   = 1.0;
  m->gammap   = m->gamma;
  m->crate    = 1.0;
  m->nstlp    = m->nst;
  if (retval < 0) return CV_LSETUP_FAIL;
  if (retval > 0) return NLS_CONV_RECVR;
  return 0;
}

static int nls_lsolve(CvlsPort* m, N_Vector delta)
{ /* cvNlsLSolve */
  int retval = ls_solve(m, delta, m->ewt, m->y, m->ftemp);
  if (retval < 0) return CV_LSOLVE_FAIL;
  if (retval > 0) return NLS_CONV_RECVR;
  return 0;
}

static int nls_convtest(CvlsPort* m, N_Vector ycor, N_Vector del_v, double tol, int mcur)
{ /* cvNlsConvTest */
  double del = v_wrms(del_v, m->ewt);
  if (mcur > 0)
  {
    double r = del / m->delp;
    m->crate = (CRDOWN * m->crate > r) ? CRDOWN * m->crate : r;
  }
  double dcon = del * (m->crate < 1.0 ? m->crate : 1.0) / tol;
  if (dcon <= 1.0)
  {
    m->acnrm = (mcur == 0) ? del : v_wrms(ycor, m->ewt);
    return 0;
  }
  if ((mcur >= 1) && (del > RDIV * m->delp)) return NLS_CONV_RECVR;
  m->delp = del;
  return NLS_CONTINUE;
}

static int newton_solve(CvlsPort* m, N_Vector ycor, double tol, int callLSetup)
{ /* SUNNonlinSolSolve_Newton */
  N_Vector delta = m->delta;
  int jbad = 0, retval;
  m->niters     = 0;
  m->nconvfails = 0;
  for (;;)
  {
    m->curiter = 0;
    retval     = nls_residual(m, ycor, delta);
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
      v_linearsum(1.0, ycor, 1.0, delta, ycor);
      retval = nls_convtest(m, ycor, delta, tol, m->curiter);
      m->curiter++;
      if (retval == 0)
      {
        m->nls_jcur = SUNFALSE;
        return 0;
      }
      if (retval != NLS_CONTINUE) break;
      if (m->curiter >= NLS_MAXCOR)
      {
        retval = NLS_CONV_RECVR;
        break;
      }
      retval = nls_residual(m, ycor, delta);
      if (retval != 0) break;
    }
    if ((retval > 0) && !m->nls_jcur && (m->pset || m->A))
    {
      m->nconvfails++;
      callLSetup = 1;
      jbad       = 1;
      v_const(0.0, ycor);
      continue;
    }
    break;
  }
  m->nconvfails++;
  return retval;
}

/* ------------------------------------------------------ step pieces */
static void rescale(CvlsPort* m)
{
  m->cvals[0] = m->eta;
  for (int j = 1; j <= m->q; j++) m->cvals[j] = m->eta * m->cvals[j - 1];
  v_scalevectorarray(m->q, m->cvals, m->zn + 1, m->zn + 1);
  m->h      = m->hscale * m->eta;
  m->next_h = m->h;
  m->hscale = m->h;
  m->nscon  = 0;
}

static void increase_bdf(CvlsPort* m)
{
  double alpha0, alpha1, prod, xi, xiold, hsum, A1;
  for (int i = 0; i <= m->qmax; i++) m->l[i] = 0.0;
  m->l[2] = alpha1 = prod = xiold = 1.0;
  alpha0                          = -1.0;
  hsum                            = m->hscale;
  if (m->q > 1)
    for (int j = 1; j < m->q; j++)
    {
      hsum += m->tau[j + 1];
      xi = hsum / m->hscale;
      prod *= xi;
      alpha0 -= 1.0 / (j + 1);
      alpha1 += 1.0 / xi;
      for (int i = j + 2; i >= 2; i--) m->l[i] = m->l[i] * xiold + m->l[i - 1];
      xiold = xi;
    }
  A1 = (-alpha0 - alpha1) / prod;
  v_scale(A1, m->zn[m->indx_acor], m->zn[m->L]);
  if (m->q > 1) v_scaleaddmulti(m->q - 1, m->l + 2, m->zn[m->L], m->zn + 2, m->zn + 2);
}

static void decrease_bdf(CvlsPort* m)
{
  double hsum, xi;
  for (int i = 0; i <= m->qmax; i++) m->l[i] = 0.0;
  m->l[2] = 1.0;
  hsum    = 0.0;
  for (int j = 1; j <= m->q - 2; j++)
  {
    hsum += m->tau[j];
    xi = hsum / m->hscale;
    for (int i = j + 2; i >= 2; i--) m->l[i] = m->l[i] * xi + m->l[i - 1];
  }
  for (int j = 2; j < m->q; j++) m->cvals[j - 2] = -m->l[j];
  if (m->q > 2) v_scaleaddmulti(m->q - 2, m->cvals, m->zn[m->q], m->zn + 2, m->zn + 2);
}

/* cvAdjustAdams (cvode.c:2550-2600): a new zero column on an increase; on
 * a decrease each zn[j] loses a multiple of zn[q] */
static void adjust_adams(CvlsPort* m, int deltaq)
{
  if (deltaq == 1)
  {
    v_const(0.0, m->zn[m->L]);
    return;
  }
  double xi, hsum = 0.0;
  for (int i = 0; i <= m->qmax; i++) m->l[i] = 0.0;
  m->l[1] = 1.0;
  for (int j = 1; j <= m->q - 2; j++)
  {
    hsum += m->tau[j];
    xi = hsum / m->hscale;
    for (int i = j + 1; i >= 1; i--) m->l[i] = m->l[i] * xi + m->l[i - 1];
  }
  for (int j = 1; j <= m->q - 2; j++) m->l[j + 1] = m->q * (m->l[j] / (j + 1));
  for (int j = 2; j < m->q; j++) m->cvals[j - 2] = -m->l[j];
  if (m->q > 2) v_scaleaddmulti(m->q - 2, m->cvals, m->zn[m->q], m->zn + 2, m->zn + 2);
}

static void adjust_order(CvlsPort* m, int deltaq)
{
  if ((m->q == 2) && (deltaq != 1)) return;
  if (m->adams) adjust_adams(m, deltaq);
  else if (deltaq == 1) increase_bdf(m);
  else if (deltaq == -1) decrease_bdf(m);
}

static void adjust_params(CvlsPort* m)
{
  if (m->qprime != m->q)
  {
    adjust_order(m, m->qprime - m->q);
    m->q     = m->qprime;
    m->L     = m->q + 1;
    m->qwait = m->L;
  }
  rescale(m);
}

static void predict(CvlsPort* m)
{
  m->tn += m->h;
  for (int k = 1; k <= m->q; k++)
    for (int j = m->q; j >= k; j--) v_linearsum(1.0, m->zn[j - 1], 1.0, m->zn[j], m->zn[j - 1]);
}

static void restore(CvlsPort* m, double saved_t)
{
  m->tn = saved_t;
  for (int k = 1; k <= m->q; k++)
    for (int j = m->q; j >= k; j--) v_linearsum(1.0, m->zn[j - 1], -1.0, m->zn[j], m->zn[j - 1]);
}

static void set_tq_bdf(CvlsPort* m, double hsum, double alpha0, double alpha0_hat, double xi_inv,
                       double xistar_inv)
{
  double A1, A2, A3, A4, A5, A6, C, Cpinv, Cppinv;
  A1       = 1.0 - alpha0_hat + alpha0;
  A2       = 1.0 + m->q * A1;
  m->tq[2] = fabs(A1 / (alpha0 * A2));
  m->tq[5] = fabs(A2 * xistar_inv / (m->l[m->q] * xi_inv));
  if (m->qwait == 1)
  {
    if (m->q > 1)
    {
      C        = xistar_inv / m->l[m->q];
      A3       = alpha0 + 1.0 / m->q;
      A4       = alpha0_hat + xi_inv;
      Cpinv    = (1.0 - A4 + A3) / A3;
      m->tq[1] = fabs(C * Cpinv);
    }
    else m->tq[1] = 1.0;
    hsum += m->tau[m->q];
    xi_inv   = m->h / hsum;
    A5       = alpha0 - (1.0 / (m->q + 1));
    A6       = alpha0_hat - xi_inv;
    Cppinv   = (1.0 - A6 + A5) / A2;
    m->tq[3] = fabs(Cppinv / (xi_inv * (m->q + 2) * A5));
  }
  m->tq[4] = CORTES / m->tq[2];
}

static void set_bdf(CvlsPort* m)
{
  double alpha0, alpha0_hat, xi_inv, xistar_inv, hsum;
  m->l[0] = m->l[1] = xi_inv = xistar_inv = 1.0;
  for (int i = 2; i <= m->q; i++) m->l[i] = 0.0;
  alpha0 = alpha0_hat = -1.0;
  hsum                = m->h;
  if (m->q > 1)
  {
    for (int j = 2; j < m->q; j++)
    {
      hsum += m->tau[j - 1];
      xi_inv = m->h / hsum;
      alpha0 -= 1.0 / j;
      for (int i = j; i >= 1; i--) m->l[i] += m->l[i - 1] * xi_inv;
    }
    alpha0 -= 1.0 / m->q;
    xistar_inv = -m->l[1] - alpha0;
    hsum += m->tau[m->q - 1];
    xi_inv     = m->h / hsum;
    alpha0_hat = -m->l[1] - xi_inv;
    for (int i = m->q; i >= 1; i--) m->l[i] += m->l[i - 1] * xistar_inv;
  }
  set_tq_bdf(m, hsum, alpha0, alpha0_hat, xi_inv, xistar_inv);
}

/* cvAltSum: sum_{i=0}^{iend} (-1)^i a[i] / (i + k) */
static double alt_sum(int iend, const double* a, int k)
{
  if (iend < 0) return 0.0;
  double sum = 0.0;
  int sign   = 1;
  for (int i = 0; i <= iend; i++)
  {
    sum += sign * (a[i] / (i + k));
    sign = -sign;
  }
  return sum;
}

/* cvSetAdams / cvAdamsStart / cvAdamsFinish (cvode.c:2815-2940) */
static void set_adams(CvlsPort* m)
{
  double mm[QMAX_ALL + 1], M[3], hsum, xi_inv, sum;
  if (m->q == 1)
  {
    m->l[0] = m->l[1] = m->tq[1] = m->tq[5] = 1.0;
    m->tq[2] = 0.5;
    m->tq[3] = 1.0 / 12.0;
    m->tq[4] = CORTES / m->tq[2];
    return;
  }
  hsum  = m->h;
  mm[0] = 1.0;
  for (int i = 1; i <= m->q; i++) mm[i] = 0.0;
  for (int j = 1; j < m->q; j++)
  {
    if ((j == m->q - 1) && (m->qwait == 1))
    {
      sum      = alt_sum(m->q - 2, mm, 2);
      m->tq[1] = m->q * sum / mm[m->q - 2];
    }
    xi_inv = m->h / hsum;
    for (int i = j; i >= 1; i--) mm[i] += mm[i - 1] * xi_inv;
    hsum += m->tau[j];
  }
  M[0] = alt_sum(m->q - 1, mm, 1);
  M[1] = alt_sum(m->q - 1, mm, 2);
  const double M0_inv = 1.0 / M[0];
  m->l[0]             = 1.0;
  for (int i = 1; i <= m->q; i++) m->l[i] = M0_inv * (mm[i - 1] / i);
  const double xi = hsum / m->h;
  xi_inv          = 1.0 / xi;
  m->tq[2]        = M[1] * M0_inv / xi;
  m->tq[5]        = xi / m->l[m->q];
  if (m->qwait == 1)
  {
    for (int i = m->q; i >= 1; i--) mm[i] += mm[i - 1] * xi_inv;
    M[2]     = alt_sum(m->q, mm, 2);
    m->tq[3] = M[2] * M0_inv / m->L;
  }
  m->tq[4] = CORTES / m->tq[2];
}

static void set_coeffs(CvlsPort* m)
{
  if (m->adams) set_adams(m);
  else set_bdf(m);
  m->rl1   = 1.0 / m->l[1];
  m->gamma = m->h * m->rl1;
  if (m->nst == 0) m->gammap = m->gamma;
  m->gamrat = (m->nst > 0) ? m->gamma / m->gammap : 1.0;
}

/* cvNlsFPFunction (cvode_nls.c:401-425): g = rl1 (h f(tn, zn[0] + ycor) - zn[1]) */
static int fp_sys(void* mem, N_Vector ycor, N_Vector res)
{
  CvlsPort* m = (CvlsPort*)mem;
  v_linearsum(1.0, m->zn[0], 1.0, ycor, m->y);
  int r = rhs(m, m->tn, m->y, res);
  if (r < 0) return CV_RHSFUNC_FAIL;
  if (r > 0) return RHSFUNC_RECVR;
  v_linearsum(m->h, res, -1.0, m->zn[1], res);
  v_scale(m->rl1, res, res);
  return 0;
}

static int fp_ctest(void* mem, N_Vector ycor, N_Vector del, double tol, int curiter)
{
  return nls_convtest((CvlsPort*)mem, ycor, del, tol, curiter);
}

static int nls(CvlsPort* m, int nflag)
{ /* cvNls: CVLS has an lsetup only when a preconditioner setup is attached */
  int callSetup = 0;
  if (m->fp)
  { /* SUNNonlinSol_FixedPoint: no linear solver, so no lsetup */
    m->crate = 1.0;
    v_const(0.0, m->acor);
    int flag = fp_port_solve(m->fp, m->acor, m->tq[4], fp_sys, fp_ctest, m);
    m->nni += fp_port_niters(m->fp);
    m->nnf += fp_port_nconvfails(m->fp);
    if (flag != 0) return flag;
    v_linearsum(1.0, m->zn[0], 1.0, m->acor, m->y);
    m->cv_jcur = 0;
    return 0;
  }
  if (m->pset || m->A)
  {
    m->convfail = ((nflag == FIRST_CALL) || (nflag == PREV_ERR_FAIL)) ? NO_FAILURES : FAIL_OTHER;
    callSetup   = (nflag == PREV_CONV_FAIL) || (nflag == PREV_ERR_FAIL) || (m->nst == 0) ||
                (m->nst >= m->nstlp + MSBP) || (fabs(m->gamrat - 1.0) > DGMAX_LSETUP);
  }
  else m->crate = 1.0;
  v_const(0.0, m->acor);
  int flag = newton_solve(m, m->acor, m->tq[4], callSetup);
  m->nni += m->niters;
  m->nnf += m->nconvfails;
  if (flag != 0) return flag;
  v_linearsum(1.0, m->zn[0], 1.0, m->acor, m->y);
  m->cv_jcur = 0;
  return 0;
}

static int handle_nflag(CvlsPort* m, int* nflagPtr, double saved_t, int* ncfPtr)
{ /* cvHandleNFlag, hmin = 0 */
  int nflag = *nflagPtr;
  if (nflag == 0) return DO_ERROR_TEST;
  m->ncfn++;
  restore(m, saved_t);
  if (nflag < 0) return nflag == CV_LSETUP_FAIL   ? CV_LSETUP_FAIL
                        : nflag == CV_LSOLVE_FAIL ? CV_LSOLVE_FAIL
                                                  : CV_RHSFUNC_FAIL;
  (*ncfPtr)++;
  m->etamax = 1.0;
  if (*ncfPtr == MXNCF) return nflag == RHSFUNC_RECVR ? CV_REPTD_RHSFUNC_ERR : CV_CONV_FAILURE;
  m->eta    = ETA_CF > 0.0 ? ETA_CF : 0.0;
  *nflagPtr = PREV_CONV_FAIL;
  rescale(m);
  return PREDICT_AGAIN;
}

static int do_error_test(CvlsPort* m, int* nflagPtr, double saved_t, int* nefPtr, double* dsmPtr)
{ /* cvDoErrorTest, hmin = 0 */
  double dsm = m->acnrm * m->tq[2];
  *dsmPtr    = dsm;
  if (dsm <= 1.0) return CV_SUCCESS;
  (*nefPtr)++;
  m->netf++;
  *nflagPtr = PREV_ERR_FAIL;
  restore(m, saved_t);
  if (*nefPtr == MXNEF) return CV_ERR_FAILURE;
  m->etamax = 1.0;
  if (*nefPtr <= MXNEF1)
  {
    m->eta    = 1.0 / (pow(BIAS2 * dsm, 1.0 / m->L) + ADDON);
    double lo = 0.0;
    m->eta    = ETA_MIN_EF > (m->eta > lo ? m->eta : lo) ? ETA_MIN_EF : (m->eta > lo ? m->eta : lo);
    if (*nefPtr >= SMALL_NEF) m->eta = m->eta < ETA_MAX_EF ? m->eta : ETA_MAX_EF;
    rescale(m);
    return TRY_AGAIN;
  }
  if (m->q > 1)
  {
    m->eta = ETA_MIN_EF;
    adjust_order(m, -1);
    m->L = m->q;
    m->q--;
    m->qwait = m->L;
    rescale(m);
    return TRY_AGAIN;
  }
  m->eta = ETA_MIN_EF;
  m->h *= m->eta;
  m->next_h = m->h;
  m->hscale = m->h;
  m->qwait  = LONG_WAIT;
  m->nscon  = 0;
  int r     = rhs(m, m->tn, m->zn[0], m->tempv);
  if (r < 0) return CV_RHSFUNC_FAIL;
  if (r > 0) return CV_REPTD_RHSFUNC_ERR;
  v_scale(m->h, m->tempv, m->zn[1]);
  return TRY_AGAIN;
}

static void complete_step(CvlsPort* m)
{
  m->nst++;
  m->nscon++;
  m->hu = m->h;
  m->qu = m->q;
  for (int i = m->q; i >= 2; i--) m->tau[i] = m->tau[i - 1];
  if ((m->q == 1) && (m->nst > 1)) m->tau[2] = m->tau[1];
  m->tau[1] = m->h;
  v_scaleaddmulti(m->q + 1, m->l, m->acor, m->zn, m->zn);
  m->qwait--;
  if ((m->qwait == 1) && (m->q != m->qmax))
  {
    v_scale(1.0, m->acor, m->zn[m->qmax]);
    m->saved_tq5 = m->tq[5];
    m->indx_acor = m->qmax;
  }
}

static void set_eta(CvlsPort* m)
{ /* cvSetEta, hmax_inv = 0, hmin = 0 */
  if ((m->eta > 0.0) && (m->eta < ETA_MAX_FX))
  {
    m->eta    = 1.0;
    m->hprime = m->h;
  }
  else
  {
    if (m->eta >= ETA_MAX_FX)
    {
      m->eta = m->eta < m->etamax ? m->eta : m->etamax;
      m->eta /= 1.0;
    }
    else
    {
      m->eta = m->eta > ETA_MIN ? m->eta : ETA_MIN;
      m->eta = m->eta > 0.0 ? m->eta : 0.0;
    }
    m->hprime = m->h * m->eta;
    if (m->qprime < m->q) m->nscon = 0;
  }
}

static double compute_etaqm1(CvlsPort* m)
{
  m->etaqm1 = 0.0;
  if (m->q > 1)
  {
    double ddn = v_wrms(m->zn[m->q], m->ewt) * m->tq[1];
    m->etaqm1  = 1.0 / (pow(BIAS1 * ddn, 1.0 / m->q) + ADDON);
  }
  return m->etaqm1;
}

static double compute_etaqp1(CvlsPort* m)
{
  m->etaqp1 = 0.0;
  if (m->q != m->qmax)
  {
    if (m->saved_tq5 == 0.0) return m->etaqp1;
    double base = m->h / m->tau[2], p = 1.0;
    for (int i = 1; i <= m->L; i++) p *= base; /* SUNRpowerI */
    double cquot = (m->tq[5] / m->saved_tq5) * p;
    v_linearsum(-cquot, m->zn[m->qmax], 1.0, m->acor, m->tempv);
    double dup = v_wrms(m->tempv, m->ewt) * m->tq[3];
    m->etaqp1  = 1.0 / (pow(BIAS3 * dup, 1.0 / (m->L + 1)) + ADDON);
  }
  return m->etaqp1;
}

static void choose_eta(CvlsPort* m)
{
  double etam = m->etaqm1 > (m->etaq > m->etaqp1 ? m->etaq : m->etaqp1)
                  ? m->etaqm1
                  : (m->etaq > m->etaqp1 ? m->etaq : m->etaqp1);
  if ((etam > 0.0) && (etam < ETA_MAX_FX))
  {
    m->eta    = 1.0;
    m->qprime = m->q;
  }
  else if (etam == m->etaq)
  {
    m->eta    = m->etaq;
    m->qprime = m->q;
  }
  else if (etam == m->etaqm1)
  {
    m->eta    = m->etaqm1;
    m->qprime = m->q - 1;
  }
  else
  {
    m->eta    = m->etaqp1;
    m->qprime = m->q + 1;
    if (!m->adams) v_scale(1.0, m->acor, m->zn[m->qmax]);
  }
}

static void prepare_next_step(CvlsPort* m, double dsm)
{
  if (m->etamax == 1.0)
  {
    m->qwait  = m->qwait > 2 ? m->qwait : 2;
    m->qprime = m->q;
    m->hprime = m->h;
    m->eta    = 1.0;
    return;
  }
  m->etaq = 1.0 / (pow(BIAS2 * dsm, 1.0 / m->L) + ADDON);
  if (m->qwait != 0)
  {
    m->eta    = m->etaq;
    m->qprime = m->q;
    set_eta(m);
  }
  else
  {
    m->qwait  = 2;
    m->etaqm1 = compute_etaqm1(m);
    m->etaqp1 = compute_etaqp1(m);
    choose_eta(m);
    set_eta(m);
  }
}

static int step(CvlsPort* m)
{ /* cvStep */
  double saved_t, dsm = 0.0;
  int ncf = 0, nef = 0, nflag, kflag, eflag;
  if ((m->nst > 0) && (m->hprime != m->h)) adjust_params(m);
  saved_t = m->tn;
  nflag   = FIRST_CALL;
  for (;;)
  {
    predict(m);
    set_coeffs(m);
    nflag = nls(m, nflag);
    kflag = handle_nflag(m, &nflag, saved_t, &ncf);
    if (kflag == PREDICT_AGAIN) continue;
    if (kflag != DO_ERROR_TEST) return kflag;
    eflag = do_error_test(m, &nflag, saved_t, &nef, &dsm);
    if (eflag == TRY_AGAIN) continue;
    if (eflag != CV_SUCCESS) return eflag;
    break;
  }
  complete_step(m);
  prepare_next_step(m, dsm);
  m->etamax = (m->nst <= SMALL_NST) ? ETA_MAX_ES : ETA_MAX_GS;
  v_scale(m->tq[2], m->acor, m->acor);
  return CV_SUCCESS;
}

/* ------------------------------------------------------ initial step */
static double upper_bound_h0(CvlsPort* m, double tdist)
{ /* cvUpperBoundH0: temp1 = tempv, temp2 = acor */
  N_Vector temp1 = m->tempv, temp2 = m->acor;
  temp2->ops->nvabs(m->zn[0], temp2);
  set_ewt(m, m->zn[0], temp1);
  temp1->ops->nvinv(temp1, temp1);
  v_linearsum(HUB_FACTOR, temp2, 1.0, temp1, temp1);
  temp2->ops->nvabs(m->zn[1], temp2);
  temp1->ops->nvdiv(temp2, temp1, temp1);
  double hub_inv = temp1->ops->nvmaxnorm(temp1);
  double hub     = HUB_FACTOR * tdist;
  if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
  return hub;
}

static int ydd_norm(CvlsPort* m, double hg, double* yddnrm)
{ /* cvYddNorm */
  v_linearsum(hg, m->zn[1], 1.0, m->zn[0], m->y);
  int r = rhs(m, m->tn + hg, m->y, m->tempv);
  if (r < 0) return CV_RHSFUNC_FAIL;
  if (r > 0) return RHSFUNC_RECVR;
  v_linearsum(1.0 / hg, m->tempv, -1.0 / hg, m->zn[1], m->tempv);
  *yddnrm = v_wrms(m->tempv, m->ewt);
  return 0;
}

static double sun_rsqrt(double x) { return x <= 0.0 ? 0.0 : sqrt(x); } /* SUNRsqrt */

static int hin(CvlsPort* m, double tout)
{ /* cvHin */
  double tdiff = tout - m->tn, tdist, tround, hlb, hub, hg, hs, hnew = 0.0, hrat, h0, yddnrm = 0.0;
  int sign = (tdiff > 0.0) ? 1 : -1;
  tdist    = fabs(tdiff);
  tround   = UROUND * (fabs(m->tn) > fabs(tout) ? fabs(m->tn) : fabs(tout));
  if (tdist < 2.0 * tround) return CV_BAD_T;
  hlb = HLB_FACTOR * tround;
  hub = upper_bound_h0(m, tdist);
  hg  = sun_rsqrt(hlb * hub);
  if (hub < hlb)
  {
    m->h = sign == -1 ? -hg : hg;
    return CV_SUCCESS;
  }
  hs = hg;
  for (int count1 = 1; count1 <= MAX_ITERS; count1++)
  {
    int hgOK = 0;
    for (int count2 = 1; count2 <= MAX_ITERS; count2++)
    {
      int r = ydd_norm(m, hg * sign, &yddnrm);
      if (r < 0) return CV_RHSFUNC_FAIL;
      if (r == 0)
      {
        hgOK = 1;
        break;
      }
      hg *= 0.2;
    }
    if (!hgOK)
    {
      if (count1 <= 2) return CV_REPTD_RHSFUNC_ERR;
      hnew = hs;
      break;
    }
    hs   = hg;
    hnew = (yddnrm * hub * hub > 2.0) ? sun_rsqrt(2.0 / yddnrm) : sun_rsqrt(hg * hub);
    if (count1 == MAX_ITERS) break;
    hrat = hnew / hg;
    if ((hrat > 0.5) && (hrat < 2.0)) break;
    if ((count1 > 1) && (hrat > 2.0))
    {
      hnew = hg;
      break;
    }
    hg = hnew;
  }
  h0 = 0.5 * hnew;
  if (h0 < hlb) h0 = hlb;
  if (h0 > hub) h0 = hub;
  if (sign == -1) h0 = -h0;
  m->h = h0;
  return CV_SUCCESS;
}

static int get_dky(CvlsPort* m, double t, N_Vector dky)
{ /* CVodeGetDky(t, 0) */
  double tfuzz = FUZZ_FACTOR * UROUND * (fabs(m->tn) + fabs(m->hu));
  if (m->hu < 0.0) tfuzz = -tfuzz;
  double tp = m->tn - m->hu - tfuzz, tn1 = m->tn + tfuzz;
  if ((t - tp) * (t - tn1) > 0.0) return CV_BAD_T;
  double s = (t - m->tn) / m->h;
  N_Vector X[QMAX_ALL + 1] = {0};
  int nvec = 0;
  for (int j = m->q; j >= 0; j--)
  {
    m->cvals[nvec] = 1.0;
    for (int i = 0; i < j; i++) m->cvals[nvec] *= s;
    X[nvec] = m->zn[j];
    nvec++;
  }
  v_lincomb(nvec, m->cvals, X, dky);
  return CV_SUCCESS;
}

/* ------------------------------------------------------ public entry points */

/* CVodeCreate(CV_BDF) + CVodeInit(f, t0, y0) + CVodeSStolerances(rtol, atol)
 * + CVodeSetMaxNumSteps(mxstep) + CVodeSetLinearSolver(LS, NULL) +
 * CVodeSetJacTimes(NULL, jtimes) (jtimes NULL: the difference quotient) +
 * CVodeSetPreconditioner(pset, psolve) (pset may be NULL; psolve NULL: no
 * preconditioner is attached). */
void* cvls_port_create(CvlsRhsFn f, double t0, N_Vector y0, double rtol, double atol, long mxstep,
                       SUNLinearSolver LS, CvlsJTimesFn jtimes, CvlsPSetupFn pset,
                       CvlsPSolveFn psolve, void* user_data)
{
  CvlsPort* m = (CvlsPort*)calloc(1, sizeof(CvlsPort));
  if (!m) return NULL;
  N_Vector (*clone)(N_Vector) = y0->ops->nvclone;
  m->ewt   = clone(y0);
  m->acor  = clone(y0);
  m->tempv = clone(y0);
  m->ftemp = clone(y0);
  for (int j = 0; j <= QMAX; j++) m->zn[j] = clone(y0);
  m->y        = clone(y0);
  m->delta    = clone(y0);
  m->ls_ytemp = clone(y0);
  m->ls_x     = clone(y0);
  m->vtemp1   = clone(y0);
  m->vtemp2   = clone(y0);
  m->vtemp3   = clone(y0);
  v_scale(1.0, y0, m->zn[0]);
  m->f         = f;
  m->jtimes    = jtimes;
  m->pset      = pset;
  m->psolve    = psolve;
  m->user_data = user_data;
  m->rtol      = rtol;
  m->atol      = atol;
  m->mxstep    = mxstep;
  m->LS        = LS;
  m->tn        = t0;
  m->q         = 1;
  m->qmax      = QMAX;
  m->L         = 2;
  m->qwait     = m->L;
  m->etamax    = ETA_MAX_FS;
  m->indx_acor = 0;
  m->jbad      = SUNTRUE;
  m->eplifac   = CVLS_EPLIN;
  m->nrmfac    = sqrt((double)y0->ops->nvgetlength(y0));
  if (LS && LS->ops->setatimes) LS->ops->setatimes(LS, m, ls_atimes);
  if (LS && LS->ops->setpreconditioner && psolve)
    LS->ops->setpreconditioner(LS, m, pset ? ls_psetup : NULL, ls_psolve);
  return m;
}

/* CVodeSetLinearSolver(LS, A) with a matrix and a direct solver, and
 * CVodeSetJacFn(jac): the matrix-based path of CVLS (create the object with
 * LS and no J v / preconditioner, then attach A and jac). */
void cvls_port_set_matrix(void* mem, SUNMatrix A, CvlsJacFn jac)
{
  CvlsPort* m = (CvlsPort*)mem;
  m->A        = A;
  m->jac      = jac;
}

/* CVodeSetNonlinearSolver(SUNNonlinSol_FixedPoint(y, m)) with no linear
 * solver (create the object with LS NULL): the fixed-point iteration with
 * Anderson acceleration of depth m replaces Newton. */
void cvls_port_set_fixed_point(void* mem, int depth)
{
  CvlsPort* m = (CvlsPort*)mem;
  m->fp       = fp_port_create(m->ewt, depth);
}

/* CVodeCreate(CV_ADAMS, ...) instead of CV_BDF: Adams-Moulton of orders 1-12
 * (call before the first solve; the history array grows to 13 vectors). */
void cvls_port_set_adams(void* mem)
{
  CvlsPort* m = (CvlsPort*)mem;
  if (m->adams) return;
  m->adams = 1;
  m->qmax  = QMAX_ALL;
  for (int j = QMAX + 1; j <= QMAX_ALL; j++) m->zn[j] = m->zn[0]->ops->nvclone(m->zn[0]);
}

/* CVodeSVtolerances(rtol, abstol): a copy of abstol is kept (all entries > 0). */
void cvls_port_set_vabstol(void* mem, double rtol, N_Vector abstol)
{
  CvlsPort* m = (CvlsPort*)mem;
  m->rtol     = rtol;
  if (!m->Vabstol) m->Vabstol = abstol->ops->nvclone(abstol);
  v_scale(1.0, abstol, m->Vabstol);
}

/* One CVode(tout, yout, &tret, CV_NORMAL) call; returns the CVODE flag. */
int cvls_port_solve(void* mem, double tout, N_Vector yout, double* tret)
{
  CvlsPort* m = (CvlsPort*)mem;
  int istate  = CV_SUCCESS;
  if (m->nst == 0)
  {
    if (!m->initialized)
    { /* cvInitialSetup: ewt, then cvLsInitialize (the saved J of a matrix) */
      set_ewt(m, m->zn[0], m->ewt);
      if (m->A && !m->savedJ) m->savedJ = m->A->ops->clone(m->A);
      if (m->LS) m->LS->ops->initialize(m->LS);
      m->initialized = 1;
    }
    int r = rhs(m, m->tn, m->zn[0], m->zn[1]);
    if (r != 0) return r < 0 ? CV_RHSFUNC_FAIL : -9;
    int hflag = hin(m, tout);
    if (hflag != CV_SUCCESS) return hflag;
    m->hscale = m->h;
    m->h0u    = m->h;
    m->hprime = m->h;
    v_scale(m->h, m->zn[1], m->zn[1]);
  }
  else if ((m->tn - tout) * m->h >= 0.0)
  {
    *tret = tout;
    return get_dky(m, tout, yout) == CV_SUCCESS ? CV_SUCCESS : -22;
  }
  long nstloc = 0;
  for (;;)
  {
    m->next_h = m->h;
    m->next_q = m->q;
    if (m->nst > 0) set_ewt(m, m->zn[0], m->ewt);
    if ((m->mxstep > 0) && (nstloc >= m->mxstep))
    {
      istate = CV_TOO_MUCH_WORK;
      *tret  = m->tn;
      v_scale(1.0, m->zn[0], yout);
      break;
    }
    double nrm = v_wrms(m->zn[0], m->ewt);
    if (UROUND * nrm > 1.0)
    {
      istate = CV_TOO_MUCH_ACC;
      *tret  = m->tn;
      v_scale(1.0, m->zn[0], yout);
      break;
    }
    int kflag = step(m);
    if (kflag != CV_SUCCESS)
    {
      istate = kflag;
      *tret  = m->tn;
      v_scale(1.0, m->zn[0], yout);
      break;
    }
    nstloc++;
    if ((m->tn - tout) * m->h >= 0.0)
    {
      *tret = tout;
      get_dky(m, tout, yout);
      m->next_q = m->qprime;
      m->next_h = m->hprime;
      break;
    }
  }
  return istate;
}

/* Counters in CVodeGet* order: nst, nfe, nni, nnf, ncfn, netf, nsetups, nli,
 * npe, nps, njtimes, ncfl, qu, q (current), nfeDQ (RHS evaluations of the
 * difference-quotient J v), nje; and hu, h (current), tn, h0u. */
void cvls_port_stats(void* mem, long* c, double* r)
{
  CvlsPort* m = (CvlsPort*)mem;
  c[0]  = m->nst;
  c[1]  = m->nfe;
  c[2]  = m->nni;
  c[3]  = m->nnf;
  c[4]  = m->ncfn;
  c[5]  = m->netf;
  c[6]  = m->nsetups;
  c[7]  = m->nli;
  c[8]  = m->npe;
  c[9]  = m->nps;
  c[10] = m->njtimes;
  c[11] = m->ncfl;
  c[12] = m->qu;
  c[13] = m->next_q;
  c[14] = m->nfeDQ;
  c[15] = m->nje;
  r[0]  = m->hu;
  r[1]  = m->next_h;
  r[2]  = m->tn;
  r[3]  = m->h0u;
}

void cvls_port_free(void* mem)
{
  CvlsPort* m = (CvlsPort*)mem;
  if (!m) return;
  N_Vector vs[] = {m->ewt,   m->acor, m->tempv,  m->ftemp,  m->y,     m->delta,
                   m->ls_ytemp, m->ls_x, m->vtemp1, m->vtemp2, m->vtemp3};
  for (int i = 0; i < (int)(sizeof(vs) / sizeof(vs[0])); i++) vs[i]->ops->nvdestroy(vs[i]);
  for (int j = 0; j <= m->qmax; j++) m->zn[j]->ops->nvdestroy(m->zn[j]);
  if (m->Vabstol) m->Vabstol->ops->nvdestroy(m->Vabstol);
  if (m->savedJ) m->savedJ->ops->destroy(m->savedJ);
  fp_port_free(m->fp);
  free(m);
}

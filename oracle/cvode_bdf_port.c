/* cvode_bdf_port.c -- TEST ORACLE (checker and CPU baseline only).
 *
 * A CPU restatement of what the reference's CVODE does for one dense system
 * with BDF, Newton, SUNLINSOL_DENSE and an analytic Jacobian, called once as
 * CVode(tout, CV_NORMAL) with default options (mxstep raised).  It follows,
 * step for step and in the same floating-point order:
 *   CVode main loop            src/cvode/cvode.c:1037-1640
 *   cvHin / UpperBoundH0 / YddNorm  cvode.c:2161-2357
 *   cvStep                     cvode.c:2367-2503
 *   cvAdjustParams/Order/BDF, Increase/DecreaseBDF, cvRescale  cvode.c:2505-2737
 *   cvPredict / cvSet / cvSetBDF / cvSetTqBDF   cvode.c:2748-3060
 *   cvNls                      cvode.c:3068-3163
 *   cvHandleNFlag / cvRestore  cvode.c:3257-3330
 *   cvDoErrorTest              cvode.c:3359-3455
 *   cvCompleteStep / cvPrepareNextStep / cvSetEta / cvComputeEtaqm1/qp1 /
 *   cvChooseEta                cvode.c:3467-3727
 *   cvEwtSetSS                 cvode.c:4791-4830
 *   CVodeGetDky (k = 0)        cvode.c:1671-1750
 *   Newton solve               src/sunnonlinsol/newton/sunnonlinsol_newton.c:179-330
 *   cvNlsLSetup/LSolve/ConvTest/Residual   src/cvode/cvode_nls.c:256-398
 *   cvLsSetup / cvLsLinSys / cvLsSolve     src/cvode/cvode_ls.c:1311-1800
 *   dense LU: SUNDlsMat_denseGETRF/GETRS   src/sundials/sundials_dense.c:85-193
 *   SUNMatScaleAddI_Dense      src/sunmatrix/dense/sunmatrix_dense.c:265-280
 * Vector operations are written with NVECTOR_SERIAL's rounding (its LinearSum
 * special cases included); compiled with -ffp-contract=off.  Pinned against
 * the reference's own CVODE by tests/test_kinetics_oracle.py. */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <omp.h>

#include "kinetics_model.h"
#include "../sundials_gb300/csrc/ddpow.h"

/* Which pow() the step-size controller uses: 0 = the C library's (what the
 * reference calls through SUNRpowerR), 1 = the correctly rounded
 * double-double pow that the GPU integrator's exact mode uses. */
static int g_pow_dd = 0;
void bdf_port_set_pow(int dd) { g_pow_dd = dd; }
static inline double cv_pow(double x, double y) { return g_pow_dd ? dd_pow(x, y) : pow(x, y); }

#define NMAX 64
#define QMAX 5
#define UROUND DBL_EPSILON

/* CVODE defaults (cvode_impl.h:55-127, cvode.c:118-125, cvode_nls.c:32-34,
 * cvode_ls_impl.h:43-45) */
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
#define MSBJ 51
#define DGMAX_JBAD 0.2

enum { FIRST_CALL = 6, PREV_CONV_FAIL = 7, PREV_ERR_FAIL = 9 };
enum { NO_FAILURES = 0, FAIL_BAD_J = 1, FAIL_OTHER = 2 };
enum { R_SUCCESS = 0, R_CONTINUE = 901, R_CONV_RECVR = 902, R_LSETUP_FAIL = -6 };
enum { DO_ERROR_TEST = 2, PREDICT_AGAIN = 3, TRY_AGAIN = 5 };
enum { CV_SUCCESS = 0, CV_TOO_MUCH_WORK = -1, CV_TOO_MUCH_ACC = -2, CV_ERR_FAILURE = -3,
       CV_CONV_FAILURE = -4, CV_LSETUP_FAIL = -6 };

typedef struct
{
  const KinSys* sys;
  int n;
  double rtol, atol;
  double zn[QMAX + 1][NMAX];
  double ewt[NMAX], acor[NMAX], y[NMAX], tempv[NMAX], ftemp[NMAX], delta[NMAX];
  double savedJ[NMAX * NMAX], A[NMAX * NMAX];
  int piv[NMAX];
  double tn, h, hscale, hprime, next_h, eta, etamax, etaq, etaqm1, etaqp1, hu;
  double saved_tq5, rl1, gamma, gammap, gamrat, crate, delp, acnrm;
  double tq[6], l[QMAX + 2], tau[QMAX + 2];
  int q, qprime, qwait, L, indx_acor, nscon, convfail, qu;
  int nls_jcur, cv_jcur;
  long nst, nfe, nsetups, nje, nni, ncfn, netf, nnf, nstlp, nstlj;
} Bdf;

/* ------------------------------------------------------------ vector pieces */
static double wrms(const Bdf* m, const double* x)
{ /* N_VWrmsNorm_Serial: sequential sum, then SUNRsqrt(sum/N) */
  double s = 0.0;
  for (int i = 0; i < m->n; i++)
  {
    double p = x[i] * m->ewt[i];
    s += p * p;
  }
  s = s / m->n;
  return s <= 0.0 ? 0.0 : sqrt(s);
}

static void set_ewt(Bdf* m, const double* ycur, double* w)
{ /* cvEwtSetSS: tempv = |y|; tempv *= rtol; tempv += atol; w = 1/tempv */
  for (int i = 0; i < m->n; i++) m->tempv[i] = fabs(ycur[i]);
  for (int i = 0; i < m->n; i++) m->tempv[i] = m->rtol * m->tempv[i];
  for (int i = 0; i < m->n; i++) m->tempv[i] = m->tempv[i] + m->atol;
  for (int i = 0; i < m->n; i++) w[i] = 1.0 / m->tempv[i];
}

static void rhs(Bdf* m, const double* y, double* f)
{
  kin_rhs(m->sys, y, f);
  m->nfe++;
}

/* ------------------------------------------------------------ dense LU */
static int getrf(double* a, int n, int* p)
{
  for (int k = 0; k < n; k++)
  {
    double* ck = a + (size_t)k * n;
    int l      = k;
    for (int i = k + 1; i < n; i++)
      if (fabs(ck[i]) > fabs(ck[l])) l = i;
    p[k] = l;
    if (ck[l] == 0.0) return k + 1;
    if (l != k)
      for (int i = 0; i < n; i++)
      {
        double t           = a[(size_t)i * n + l];
        a[(size_t)i * n + l] = a[(size_t)i * n + k];
        a[(size_t)i * n + k] = t;
      }
    double mult = 1.0 / ck[k];
    for (int i = k + 1; i < n; i++) ck[i] *= mult;
    for (int j = k + 1; j < n; j++)
    {
      double* cj  = a + (size_t)j * n;
      double a_kj = cj[k];
      if (a_kj != 0.0)
        for (int i = k + 1; i < n; i++) cj[i] -= a_kj * ck[i];
    }
  }
  return 0;
}

static void getrs(const double* a, int n, const int* p, double* b)
{
  for (int k = 0; k < n; k++)
  {
    int pk = p[k];
    if (pk != k)
    {
      double t = b[k];
      b[k]     = b[pk];
      b[pk]    = t;
    }
  }
  for (int k = 0; k < n - 1; k++)
  {
    const double* ck = a + (size_t)k * n;
    for (int i = k + 1; i < n; i++) b[i] -= ck[i] * b[k];
  }
  for (int k = n - 1; k > 0; k--)
  {
    const double* ck = a + (size_t)k * n;
    b[k] /= ck[k];
    for (int i = 0; i < k; i++) b[i] -= ck[i] * b[k];
  }
  b[0] /= a[0];
}

/* ------------------------------------------------------------ lsetup/lsolve */
/* cvNlsLSetup -> cvLsSetup -> cvLsLinSys -> SUNLinSolSetup_Dense */
static int nls_lsetup(Bdf* m, int jbad)
{
  const int n = m->n;
  if (jbad) m->convfail = FAIL_BAD_J;
  double dgamma = fabs((m->gamma / m->gammap) - 1.0);
  int ls_jbad   = (m->nst == 0) || (m->nst >= m->nstlj + MSBJ) ||
                ((m->convfail == FAIL_BAD_J) && (dgamma < DGMAX_JBAD)) ||
                (m->convfail == FAIL_OTHER);
  if (!ls_jbad)
  {
    m->cv_jcur = 0;
    memcpy(m->A, m->savedJ, sizeof(double) * n * n);
  }
  else
  {
    m->cv_jcur = 1;
    memset(m->A, 0, sizeof(double) * n * n);
    kin_jac(m->sys, m->y, m->A);
    memcpy(m->savedJ, m->A, sizeof(double) * n * n);
  }
  const double c = -m->gamma;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++)
    {
      m->A[j * n + i] *= c;
      if (i == j) m->A[j * n + i] += 1.0;
    }
  if (m->cv_jcur)
  {
    m->nje++;
    m->nstlj = m->nst;
  }
  int lu = getrf(m->A, n, m->piv);
  m->nsetups++;
  m->nls_jcur = m->cv_jcur;
  m->gamrat   = 1.0;
  m->gammap   = m->gamma;
  m->crate    = 1.0;
  m->nstlp    = m->nst;
  if (lu > 0) return R_CONV_RECVR; /* SUNLS_LUFACT_FAIL is recoverable */
  return R_SUCCESS;
}

/* cvNlsLSolve -> cvLsSolve (direct): x = A^{-1} b; b = x; scale if gamrat != 1 */
static void nls_lsolve(Bdf* m, double* b)
{
  getrs(m->A, m->n, m->piv, b);
  if (m->gamrat != 1.0)
  {
    double c = 2.0 / (1.0 + m->gamrat);
    for (int i = 0; i < m->n; i++) b[i] *= c;
  }
}

/* cvNlsResidual: y = zn0 + ycor; ftemp = f(y); res = rl1*zn1 + ycor; res += -gamma*ftemp */
static void nls_residual(Bdf* m, const double* ycor, double* res)
{
  const int n = m->n;
  for (int i = 0; i < n; i++) m->y[i] = m->zn[0][i] + ycor[i];
  rhs(m, m->y, m->ftemp);
  for (int i = 0; i < n; i++) res[i] = (m->rl1 * m->zn[1][i]) + ycor[i];
  const double a = -m->gamma;
  for (int i = 0; i < n; i++) res[i] += a * m->ftemp[i];
}

/* cvNlsConvTest */
static int nls_convtest(Bdf* m, const double* ycor, const double* del_v, double tol, int mcur)
{
  double del = wrms(m, del_v);
  if (mcur > 0)
  {
    double r = del / m->delp;
    m->crate = (CRDOWN * m->crate > r) ? CRDOWN * m->crate : r;
  }
  double dcon = del * (m->crate < 1.0 ? m->crate : 1.0) / tol;
  if (dcon <= 1.0)
  {
    m->acnrm = (mcur == 0) ? del : wrms(m, ycor);
    return R_SUCCESS;
  }
  if ((mcur >= 1) && (del > RDIV * m->delp)) return R_CONV_RECVR;
  m->delp = del;
  return R_CONTINUE;
}

/* SUNNonlinSolSolve_Newton; returns 0 or a recoverable / fatal code */
static int newton_solve(Bdf* m, double* ycor, double tol, int callLSetup)
{
  const int n = m->n;
  int jbad = 0, retval;
  long niters = 0, nconvfails = 0;
  for (;;)
  {
    int curiter = 0;
    nls_residual(m, ycor, m->delta);
    if (callLSetup)
    {
      retval = nls_lsetup(m, jbad);
      if (retval != R_SUCCESS) break;
    }
    for (;;)
    {
      niters++;
      for (int i = 0; i < n; i++) m->delta[i] = -m->delta[i];
      nls_lsolve(m, m->delta);
      for (int i = 0; i < n; i++) ycor[i] = ycor[i] + m->delta[i];
      retval = nls_convtest(m, ycor, m->delta, tol, curiter);
      curiter++;
      if (retval == R_SUCCESS)
      {
        m->nls_jcur = 0;
        m->nni += niters;
        m->nnf += nconvfails;
        return R_SUCCESS;
      }
      if (retval != R_CONTINUE) break;
      if (curiter >= NLS_MAXCOR)
      {
        retval = R_CONV_RECVR;
        break;
      }
      nls_residual(m, ycor, m->delta);
    }
    if (retval > 0 && !m->nls_jcur)
    {
      nconvfails++;
      callLSetup = 1;
      jbad       = 1;
      for (int i = 0; i < n; i++) ycor[i] = 0.0;
      continue;
    }
    break;
  }
  nconvfails++;
  m->nni += niters;
  m->nnf += nconvfails;
  return retval;
}

/* ------------------------------------------------------------ step pieces */
static void rescale(Bdf* m)
{
  double c[QMAX + 1];
  c[0] = m->eta;
  for (int j = 1; j <= m->q; j++) c[j] = m->eta * c[j - 1];
  for (int j = 1; j <= m->q; j++)
    for (int i = 0; i < m->n; i++) m->zn[j][i] *= c[j - 1];
  m->h      = m->hscale * m->eta;
  m->next_h = m->h;
  m->hscale = m->h;
  m->nscon  = 0;
}

static void increase_bdf(Bdf* m)
{
  double alpha0, alpha1, prod, xi, xiold, hsum, A1;
  for (int i = 0; i <= QMAX; i++) m->l[i] = 0.0;
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
  for (int i = 0; i < m->n; i++) m->zn[m->L][i] = A1 * m->zn[m->indx_acor][i];
  if (m->q > 1)
    for (int j = 2; j <= m->q; j++)
      for (int i = 0; i < m->n; i++) m->zn[j][i] += m->l[j] * m->zn[m->L][i];
}

static void decrease_bdf(Bdf* m)
{
  double hsum, xi, cvals[QMAX];
  for (int i = 0; i <= QMAX; i++) m->l[i] = 0.0;
  m->l[2] = 1.0;
  hsum    = 0.0;
  for (int j = 1; j <= m->q - 2; j++)
  {
    hsum += m->tau[j];
    xi = hsum / m->hscale;
    for (int i = j + 2; i >= 2; i--) m->l[i] = m->l[i] * xi + m->l[i - 1];
  }
  for (int j = 2; j < m->q; j++) cvals[j - 2] = -m->l[j];
  if (m->q > 2)
    for (int j = 2; j < m->q; j++)
      for (int i = 0; i < m->n; i++) m->zn[j][i] += cvals[j - 2] * m->zn[m->q][i];
}

static void adjust_order(Bdf* m, int deltaq)
{
  if ((m->q == 2) && (deltaq != 1)) return;
  if (deltaq == 1) increase_bdf(m);
  else if (deltaq == -1) decrease_bdf(m);
}

static void adjust_params(Bdf* m)
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

static void predict(Bdf* m)
{
  m->tn += m->h;
  for (int k = 1; k <= m->q; k++)
    for (int j = m->q; j >= k; j--)
      for (int i = 0; i < m->n; i++) m->zn[j - 1][i] = m->zn[j - 1][i] + m->zn[j][i];
}

static void restore(Bdf* m, double saved_t)
{
  m->tn = saved_t;
  for (int k = 1; k <= m->q; k++)
    for (int j = m->q; j >= k; j--)
      for (int i = 0; i < m->n; i++) m->zn[j - 1][i] = m->zn[j - 1][i] - m->zn[j][i];
}

static void set_tq_bdf(Bdf* m, double hsum, double alpha0, double alpha0_hat, double xi_inv,
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

static void set_bdf(Bdf* m)
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

static void set_coeffs(Bdf* m)
{
  set_bdf(m);
  m->rl1   = 1.0 / m->l[1];
  m->gamma = m->h * m->rl1;
  if (m->nst == 0) m->gammap = m->gamma;
  m->gamrat = (m->nst > 0) ? m->gamma / m->gammap : 1.0;
}

static int nls(Bdf* m, int nflag)
{
  m->convfail   = ((nflag == FIRST_CALL) || (nflag == PREV_ERR_FAIL)) ? NO_FAILURES : FAIL_OTHER;
  int callSetup = (nflag == PREV_CONV_FAIL) || (nflag == PREV_ERR_FAIL) || (m->nst == 0) ||
                  (m->nst >= m->nstlp + MSBP) || (fabs(m->gamrat - 1.0) > DGMAX_LSETUP);
  for (int i = 0; i < m->n; i++) m->acor[i] = 0.0;
  int flag = newton_solve(m, m->acor, m->tq[4], callSetup);
  if (flag != R_SUCCESS) return flag;
  for (int i = 0; i < m->n; i++) m->y[i] = m->zn[0][i] + m->acor[i];
  m->cv_jcur = 0;
  return R_SUCCESS;
}

static int handle_nflag(Bdf* m, int* nflagPtr, double saved_t, int* ncfPtr)
{
  int nflag = *nflagPtr;
  if (nflag == R_SUCCESS) return DO_ERROR_TEST;
  m->ncfn++;
  restore(m, saved_t);
  if (nflag < 0) return CV_LSETUP_FAIL;
  (*ncfPtr)++;
  m->etamax = 1.0;
  if (*ncfPtr == MXNCF) return CV_CONV_FAILURE; /* |h| <= hmin*ONEPSM never holds: hmin = 0 */
  m->eta    = ETA_CF > 0.0 ? ETA_CF : 0.0;    /* max(eta_cf, hmin/|h|), hmin = 0 */
  *nflagPtr = PREV_CONV_FAIL;
  rescale(m);
  return PREDICT_AGAIN;
}

static int do_error_test(Bdf* m, int* nflagPtr, double saved_t, int* nefPtr, double* dsmPtr)
{
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
    m->eta = 1.0 / (cv_pow(BIAS2 * dsm, 1.0 / m->L) + ADDON);
    double lo = 0.0; /* hmin/|h| */
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
  rhs(m, m->zn[0], m->tempv);
  for (int i = 0; i < m->n; i++) m->zn[1][i] = m->h * m->tempv[i];
  return TRY_AGAIN;
}

static void complete_step(Bdf* m)
{
  m->nst++;
  m->nscon++;
  m->hu = m->h;
  m->qu = m->q;
  for (int i = m->q; i >= 2; i--) m->tau[i] = m->tau[i - 1];
  if ((m->q == 1) && (m->nst > 1)) m->tau[2] = m->tau[1];
  m->tau[1] = m->h;
  for (int j = 0; j <= m->q; j++)
    for (int i = 0; i < m->n; i++) m->zn[j][i] += m->l[j] * m->acor[i];
  m->qwait--;
  if ((m->qwait == 1) && (m->q != QMAX))
  {
    for (int i = 0; i < m->n; i++) m->zn[QMAX][i] = m->acor[i];
    m->saved_tq5 = m->tq[5];
    m->indx_acor = QMAX;
  }
}

static void set_eta(Bdf* m)
{
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
      m->eta /= 1.0; /* max(1, |h|*hmax_inv*eta) with hmax_inv = 0 */
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

static double compute_etaqm1(Bdf* m)
{
  m->etaqm1 = 0.0;
  if (m->q > 1)
  {
    double ddn = wrms(m, m->zn[m->q]) * m->tq[1];
    m->etaqm1  = 1.0 / (cv_pow(BIAS1 * ddn, 1.0 / m->q) + ADDON);
  }
  return m->etaqm1;
}

static double compute_etaqp1(Bdf* m)
{
  m->etaqp1 = 0.0;
  if (m->q != QMAX)
  {
    if (m->saved_tq5 == 0.0) return m->etaqp1;
    double base = m->h / m->tau[2], p = 1.0;
    for (int i = 1; i <= m->L; i++) p *= base; /* SUNRpowerI */
    double cquot = (m->tq[5] / m->saved_tq5) * p;
    const double a = -cquot;
    for (int i = 0; i < m->n; i++) m->tempv[i] = (a * m->zn[QMAX][i]) + m->acor[i];
    double dup = wrms(m, m->tempv) * m->tq[3];
    m->etaqp1  = 1.0 / (cv_pow(BIAS3 * dup, 1.0 / (m->L + 1)) + ADDON);
  }
  return m->etaqp1;
}

static void choose_eta(Bdf* m)
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
    for (int i = 0; i < m->n; i++) m->zn[QMAX][i] = m->acor[i];
  }
}

static void prepare_next_step(Bdf* m, double dsm)
{
  if (m->etamax == 1.0)
  {
    m->qwait  = m->qwait > 2 ? m->qwait : 2;
    m->qprime = m->q;
    m->hprime = m->h;
    m->eta    = 1.0;
    return;
  }
  m->etaq = 1.0 / (cv_pow(BIAS2 * dsm, 1.0 / m->L) + ADDON);
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

static int step(Bdf* m)
{
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
  for (int i = 0; i < m->n; i++) m->acor[i] *= m->tq[2];
  return CV_SUCCESS;
}

/* ------------------------------------------------------------ initial step */
static double upper_bound_h0(Bdf* m, double tdist)
{
  const int n = m->n;
  double* temp1 = m->tempv;
  double* temp2 = m->acor;
  for (int i = 0; i < n; i++) temp2[i] = fabs(m->zn[0][i]);
  set_ewt(m, m->zn[0], temp1); /* tempv doubles as the weight */
  for (int i = 0; i < n; i++) temp1[i] = 1.0 / temp1[i];
  for (int i = 0; i < n; i++) temp1[i] += HUB_FACTOR * temp2[i];
  for (int i = 0; i < n; i++) temp2[i] = fabs(m->zn[1][i]);
  for (int i = 0; i < n; i++) temp1[i] = temp2[i] / temp1[i];
  double hub_inv = 0.0;
  for (int i = 0; i < n; i++)
    if (fabs(temp1[i]) > hub_inv) hub_inv = fabs(temp1[i]);
  double hub = HUB_FACTOR * tdist;
  if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
  return hub;
}

static double ydd_norm(Bdf* m, double hg)
{
  const int n = m->n;
  for (int i = 0; i < n; i++) m->y[i] = (hg * m->zn[1][i]) + m->zn[0][i];
  rhs(m, m->y, m->tempv);
  const double a = 1.0 / hg, b = -1.0 / hg; /* LinearSum with a == -b: a*(x - y) */
  if (a == -b && a != 1.0 && a != -1.0)
    for (int i = 0; i < n; i++) m->tempv[i] = a * (m->tempv[i] - m->zn[1][i]);
  else
    for (int i = 0; i < n; i++) m->tempv[i] = (a * m->tempv[i]) + (b * m->zn[1][i]);
  return wrms(m, m->tempv);
}

static void hin(Bdf* m, double tout)
{
  double tdiff = tout - m->tn, tdist, tround, hlb, hub, hg, hs, hnew = 0.0, hrat, h0, yddnrm;
  int sign = (tdiff > 0.0) ? 1 : -1;
  tdist    = fabs(tdiff);
  tround   = UROUND * (fabs(m->tn) > fabs(tout) ? fabs(m->tn) : fabs(tout));
  hlb      = HLB_FACTOR * tround;
  hub      = upper_bound_h0(m, tdist);
  hg       = hlb * hub <= 0.0 ? 0.0 : sqrt(hlb * hub);
  if (hub < hlb)
  {
    m->h = sign == -1 ? -hg : hg;
    return;
  }
  hs = hg;
  for (int count1 = 1; count1 <= MAX_ITERS; count1++)
  {
    yddnrm = ydd_norm(m, hg * sign); /* the RHS never fails here */
    hs     = hg;
    if (yddnrm * hub * hub > 2.0)
    {
      double v = 2.0 / yddnrm;
      hnew     = v <= 0.0 ? 0.0 : sqrt(v);
    }
    else
    {
      double v = hg * hub;
      hnew     = v <= 0.0 ? 0.0 : sqrt(v);
    }
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
  (void)hs;
  h0 = 0.5 * hnew;
  if (h0 < hlb) h0 = hlb;
  if (h0 > hub) h0 = hub;
  if (sign == -1) h0 = -h0;
  m->h = h0;
}

/* CVodeGetDky(t, 0): N_VLinearCombination over zn[q..0] with c_j = s^j */
static void get_dky(Bdf* m, double t, double* dky)
{
  const int n = m->n;
  double s = (t - m->tn) / m->h;
  double c[QMAX + 1];
  const double* X[QMAX + 1];
  int nvec = 0;
  for (int j = m->q; j >= 0; j--)
  {
    c[nvec] = 1.0;
    for (int i = 0; i < j; i++) c[nvec] *= s;
    X[nvec] = m->zn[j];
    nvec++;
  }
  if (nvec == 2)
  { /* LinearSum(c0, X0, 1, X1): the b == 1 form rounds as c0*x + y */
    for (int i = 0; i < n; i++) dky[i] = (c[0] * X[0][i]) + (c[1] * X[1][i]);
    return;
  }
  for (int i = 0; i < n; i++) dky[i] = c[0] * X[0][i];
  for (int k = 1; k < nvec; k++)
    for (int i = 0; i < n; i++) dky[i] += c[k] * X[k][i];
}

/* One CVode(tout, CV_NORMAL) call from t0 = 0 with mxstep = mxstep. */
int bdf_port_solve(const KinSys* sys, const double* y0, double rtol, double atol, double tout,
                   long mxstep, double* yout, KinStats* st)
{
  Bdf* m = (Bdf*)calloc(1, sizeof(Bdf));
  m->sys = sys;
  m->n   = sys->n;
  m->rtol = rtol;
  m->atol = atol;
  for (int i = 0; i < m->n; i++) m->zn[0][i] = y0[i];
  m->tn        = 0.0;
  m->q         = 1;
  m->L         = 2;
  m->qwait     = m->L;
  m->etamax    = ETA_MAX_FS;
  m->indx_acor = 0;
  int istate   = CV_SUCCESS;

  /* first call: ewt, f(t0), initial step */
  set_ewt(m, m->zn[0], m->ewt);
  rhs(m, m->zn[0], m->zn[1]);
  hin(m, tout);
  m->hscale = m->h;
  m->hprime = m->h;
  for (int i = 0; i < m->n; i++) m->zn[1][i] *= m->h;

  long nstloc = 0;
  for (;;)
  {
    m->next_h = m->h;
    if (m->nst > 0) set_ewt(m, m->zn[0], m->ewt);
    if ((mxstep > 0) && (nstloc >= mxstep))
    {
      istate = CV_TOO_MUCH_WORK;
      break;
    }
    double nrm = wrms(m, m->zn[0]);
    if (UROUND * nrm > 1.0)
    {
      istate = CV_TOO_MUCH_ACC;
      break;
    }
    int kflag = step(m);
    if (kflag != CV_SUCCESS)
    {
      istate = kflag;
      break;
    }
    nstloc++;
    if ((m->tn - tout) * m->h >= 0.0) break;
  }
  if (istate == CV_SUCCESS) get_dky(m, tout, yout);
  else
    for (int i = 0; i < m->n; i++) yout[i] = m->zn[0][i];
  st->nst     = m->nst;
  st->nfe     = m->nfe;
  st->nsetups = m->nsetups;
  st->nje     = m->nje;
  st->nni     = m->nni;
  st->ncfn    = m->ncfn;
  st->netf    = m->netf;
  st->nnf     = m->nnf;
  st->flag    = istate;
  st->qu      = m->qu;
  st->tn      = m->tn;
  st->hu      = m->hu;
  free(m);
  return istate;
}

/* Batch driver over a problem laid out as in kinetics_model.h; threads > 0
 * sets the OpenMP thread count (systems are independent). */
void bdf_port_batch(int64_t first, int64_t count, const int32_t* n, const int64_t* y_off,
                    const int64_t* r_off, const int32_t* rt, const int32_t* ra, const int32_t* rb,
                    const int32_t* rc, const double* rk, const double* y0, double rtol,
                    double atol, double tout, long mxstep, int threads, double* yout,
                    KinStats* stats)
{
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t s = first; s < first + count; s++)
  {
    KinSys sys = {n[s],          (int)(r_off[s + 1] - r_off[s]), rt + r_off[s], ra + r_off[s],
                  rb + r_off[s], rc + r_off[s],                  rk + r_off[s]};
    bdf_port_solve(&sys, y0 + y_off[s], rtol, atol, tout, mxstep, yout + y_off[s],
                   &stats[s - first]);
  }
}

/* fixedpoint_port.c -- TEST ORACLE (checker only, never part of the product).
 *
 * SUNNonlinSol_FixedPoint with Anderson acceleration of depth m and no
 * damping, restated over the generic vector ops table with the reference's
 * fallbacks for the fused operations it calls, in the same floating-point
 * order (compiled with -ffp-contract=off):
 *   SUNNonlinSolSolve_FixedPoint   src/sunnonlinsol/fixedpoint/sunnonlinsol_fixedpoint.c:174-283
 *   AndersonAccelerate (QR update by modified Gram-Schmidt, Givens
 *   recycling once the subspace is full)   sunnonlinsol_fixedpoint.c:417-609
 *   defaults (maxiters 3, damping off)     sunnonlinsol_fixedpoint.c:50-108
 *   N_VDotProdMulti / N_VLinearCombination dispatch
 *                                  src/sundials/sundials_nvector.c:549-580, 596-616 */
#include "fixedpoint_port.h"

#include <math.h>
#include <stdlib.h>

enum { NLS_CONTINUE = 901, NLS_CONV_RECVR = 902 };

struct FPPort
{
  int m, maxiters, curiter;
  long niters, nconvfails;
  N_Vector yprev, gy, delta, fold, gold, df[16], dg[16], q[16];
  double *R, *gamma, cvals[34];
  int imap[16];
};

static double rsqrt(double x) { return x <= 0.0 ? 0.0 : sqrt(x); } /* SUNRsqrt */
static void v_linearsum(double a, N_Vector x, double b, N_Vector y, N_Vector z)
{
  z->ops->nvlinearsum(a, x, b, y, z);
}
static void v_scale(double c, N_Vector x, N_Vector z) { z->ops->nvscale(c, x, z); }
static double v_dot(N_Vector x, N_Vector y) { return x->ops->nvdotprod(x, y); }

static void v_dotmulti(int nvec, N_Vector x, N_Vector* Y, double* d)
{
  if (x->ops->nvdotprodmulti) x->ops->nvdotprodmulti(nvec, x, Y, d);
  else
    for (int i = 0; i < nvec; i++) d[i] = x->ops->nvdotprod(x, Y[i]);
}

static void v_lincomb(int nvec, double* c, N_Vector* X, N_Vector z)
{
  if (z->ops->nvlinearcombination) z->ops->nvlinearcombination(nvec, c, X, z);
  else
  {
    z->ops->nvscale(c[0], X[0], z);
    for (int i = 1; i < nvec; i++) z->ops->nvlinearsum(c[i], X[i], 1.0, z, z);
  }
}

FPPort* fp_port_create(N_Vector tmpl, int m)
{
  if (m < 0 || m > 16) return NULL;
  FPPort* fp = (FPPort*)calloc(1, sizeof(FPPort));
  if (!fp) return NULL;
  N_Vector (*clone)(N_Vector) = tmpl->ops->nvclone;
  fp->m        = m;
  fp->maxiters = 3;
  fp->yprev    = clone(tmpl);
  fp->gy       = clone(tmpl);
  fp->delta    = clone(tmpl);
  if (m > 0)
  {
    fp->fold  = clone(tmpl);
    fp->gold  = clone(tmpl);
    fp->R     = (double*)calloc((size_t)m * m, sizeof(double));
    fp->gamma = (double*)calloc((size_t)m, sizeof(double));
    for (int i = 0; i < m; i++)
    {
      fp->df[i] = clone(tmpl);
      fp->dg[i] = clone(tmpl);
      fp->q[i]  = clone(tmpl);
    }
  }
  return fp;
}

void fp_port_free(FPPort* fp)
{
  if (!fp) return;
  N_Vector vs[] = {fp->yprev, fp->gy, fp->delta, fp->fold, fp->gold};
  for (int i = 0; i < 5; i++)
    if (vs[i]) vs[i]->ops->nvdestroy(vs[i]);
  for (int i = 0; i < fp->m; i++)
  {
    fp->df[i]->ops->nvdestroy(fp->df[i]);
    fp->dg[i]->ops->nvdestroy(fp->dg[i]);
    fp->q[i]->ops->nvdestroy(fp->q[i]);
  }
  free(fp->R);
  free(fp->gamma);
  free(fp);
}

/* SUNNonlinSolSetMaxIters_FixedPoint (the integrators keep the default 3) */
void fp_port_set_maxiters(FPPort* fp, int maxiters) { fp->maxiters = maxiters; }

long fp_port_niters(const FPPort* fp) { return fp->niters; }
long fp_port_nconvfails(const FPPort* fp) { return fp->nconvfails; }

/* AndersonAccelerate: x = the accelerated iterate from g(x_old) = gval */
static void anderson(FPPort* fp, N_Vector gval, N_Vector x, N_Vector xold, int iter)
{
  const int maa = fp->m;
  double *R = fp->R, *gamma = fp->gamma, *cvals = fp->cvals;
  N_Vector Xvecs[34];
  N_Vector vtemp = x, fv = fp->delta;
  int* ipt_map   = fp->imap;
  for (int i = 0; i < maa; i++) ipt_map[i] = 0;
  const int i_pt = iter - 1 - ((iter - 1) / maa) * maa;
  v_linearsum(1.0, gval, -1.0, xold, fv);
  if (iter > 0)
  {
    v_linearsum(1.0, gval, -1.0, fp->gold, fp->dg[i_pt]);
    v_linearsum(1.0, fv, -1.0, fp->fold, fp->df[i_pt]);
  }
  v_scale(1.0, gval, fp->gold);
  v_scale(1.0, fv, fp->fold);
  if (iter == 0)
  {
    v_scale(1.0, gval, x);
    return;
  }
  if (iter == 1)
  {
    R[0] = v_dot(fp->df[i_pt], fp->df[i_pt]);
    R[0] = rsqrt(R[0]);
    v_scale(1.0 / R[0], fp->df[i_pt], fp->q[i_pt]);
    ipt_map[0] = 0;
  }
  else if (iter <= maa)
  {
    v_scale(1.0, fp->df[i_pt], vtemp);
    for (int j = 0; j < iter - 1; j++)
    {
      ipt_map[j]              = j;
      R[(iter - 1) * maa + j] = v_dot(fp->q[j], vtemp);
      v_linearsum(1.0, vtemp, -R[(iter - 1) * maa + j], fp->q[j], vtemp);
    }
    R[(iter - 1) * maa + iter - 1] = v_dot(vtemp, vtemp);
    R[(iter - 1) * maa + iter - 1] = rsqrt(R[(iter - 1) * maa + iter - 1]);
    if (R[(iter - 1) * maa + iter - 1] == 0.0) v_scale(0.0, vtemp, fp->q[i_pt]);
    else v_scale(1.0 / R[(iter - 1) * maa + iter - 1], vtemp, fp->q[i_pt]);
    ipt_map[iter - 1] = iter - 1;
  }
  else
  { /* subspace full: drop the oldest column by Givens rotations */
    for (int i = 0; i < maa - 1; i++)
    {
      double a = R[(i + 1) * maa + i], b = R[(i + 1) * maa + i + 1];
      double rtemp             = rsqrt(a * a + b * b);
      const double c           = a / rtemp;
      const double s           = b / rtemp;
      R[(i + 1) * maa + i]     = rtemp;
      R[(i + 1) * maa + i + 1] = 0.0;
      for (int j = i + 2; j < maa; j++)
      {
        a                  = R[j * maa + i];
        b                  = R[j * maa + i + 1];
        rtemp              = c * a + s * b;
        R[j * maa + i + 1] = -s * a + c * b;
        R[j * maa + i]     = rtemp;
      }
      v_linearsum(c, fp->q[i], s, fp->q[i + 1], vtemp);
      v_linearsum(-s, fp->q[i], c, fp->q[i + 1], fp->q[i + 1]);
      v_scale(1.0, vtemp, fp->q[i]);
    }
    for (int i = 1; i < maa; i++)
      for (int j = 0; j < maa - 1; j++) R[(i - 1) * maa + j] = R[i * maa + j];
    v_scale(1.0, fp->df[i_pt], vtemp);
    for (int j = 0; j < maa - 1; j++)
    {
      R[(maa - 1) * maa + j] = v_dot(fp->q[j], vtemp);
      v_linearsum(1.0, vtemp, -R[(maa - 1) * maa + j], fp->q[j], vtemp);
    }
    R[(maa - 1) * maa + maa - 1] = v_dot(vtemp, vtemp);
    R[(maa - 1) * maa + maa - 1] = rsqrt(R[(maa - 1) * maa + maa - 1]);
    v_scale(1.0 / R[(maa - 1) * maa + maa - 1], vtemp, fp->q[maa - 1]);
    int j = 0;
    for (int i = i_pt + 1; i < maa; i++) ipt_map[j++] = i;
    for (int i = 0; i < i_pt + 1; i++) ipt_map[j++] = i;
  }
  const int lAA = maa < iter ? maa : iter;
  v_dotmulti(lAA, fv, fp->q, gamma);
  cvals[0] = 1.0;
  Xvecs[0] = gval;
  int nvec = 1;
  for (int i = lAA - 1; i > -1; i--)
  {
    for (int j = i + 1; j < lAA; j++) gamma[i] -= R[j * maa + i] * gamma[j];
    if (gamma[i] == 0.0) gamma[i] = 0.0;
    else gamma[i] /= R[i * maa + i];
    cvals[nvec] = -gamma[i];
    Xvecs[nvec] = fp->dg[ipt_map[i]];
    nvec++;
  }
  v_lincomb(nvec, cvals, Xvecs, x);
}

int fp_port_solve(FPPort* fp, N_Vector ycor, double tol, FPSysFn sys, FPCTestFn ctest,
                  void* mem)
{
  fp->niters     = 0;
  fp->nconvfails = 0;
  for (fp->curiter = 0; fp->curiter < fp->maxiters; fp->curiter++)
  {
    v_scale(1.0, ycor, fp->yprev);
    int retval = sys(mem, ycor, fp->gy);
    if (retval != 0) return retval;
    if (fp->m == 0) v_scale(1.0, fp->gy, ycor);
    else anderson(fp, fp->gy, ycor, fp->yprev, fp->curiter);
    fp->niters++;
    v_linearsum(1.0, ycor, -1.0, fp->yprev, fp->delta);
    retval = ctest(mem, ycor, fp->delta, tol, fp->curiter);
    if (retval == 0) return 0;
    if (retval != NLS_CONTINUE)
    {
      fp->nconvfails++;
      return retval;
    }
  }
  fp->nconvfails++;
  return NLS_CONV_RECVR;
}

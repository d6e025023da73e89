/* nvector_serial_port.c -- TEST ORACLE (checker only; never shipped or timed
 * as the product).  A CPU restatement of the reference's NVECTOR_SERIAL
 * operations on plain arrays, used by tests/ to check the GB300 kernels on
 * the GPU machine, where the reference sources do not exist.
 *
 * Follows src/nvector/serial/nvector_serial.c (v7.5.0):
 *   LinearSum 387-480 (its special cases: a==b -> a*(x+y), a==-b -> a*(x-y)),
 *   Const/Prod/Div/Scale/Abs/Inv/AddConst 482-604, DotProd 605, MaxNorm 622,
 *   WrmsNorm 641/650, WrmsNormMask 671/680, Min 705, WL2Norm 725, L1Norm 746,
 *   Compare 762, InvTest 778, ConstrMask 800, MinQuotient 833,
 *   LinearCombination 871-942, ScaleAddMulti 944-992, DotProdMulti 994-1033.
 * Sums run sequentially in index order; compiled with -ffp-contract=off so
 * every product and sum is rounded separately, like the reference built for
 * x86-64.  Its bits are pinned against the reference itself by
 * tests/test_oracle_pins.py (fixtures in tests/golden/). */
#include <math.h>
#include <stdint.h>
#include <float.h>

typedef int64_t idx;

void port_linearsum(double a, const double* x, double b, const double* y,
                    double* z, idx n)
{
  int unit = (a == 1.0) || (b == 1.0) || (a == -1.0) || (b == -1.0);
  if (!unit && a == b)
  {
    for (idx i = 0; i < n; i++) z[i] = a * (x[i] + y[i]);
    return;
  }
  if (!unit && a == -b)
  {
    for (idx i = 0; i < n; i++) z[i] = a * (x[i] - y[i]);
    return;
  }
  /* every +-1 special case of the reference rounds like a*x + b*y */
  for (idx i = 0; i < n; i++) z[i] = (a * x[i]) + (b * y[i]);
}

void port_const(double c, double* z, idx n)
{
  for (idx i = 0; i < n; i++) z[i] = c;
}
void port_prod(const double* x, const double* y, double* z, idx n)
{
  for (idx i = 0; i < n; i++) z[i] = x[i] * y[i];
}
void port_div(const double* x, const double* y, double* z, idx n)
{
  for (idx i = 0; i < n; i++) z[i] = x[i] / y[i];
}
void port_scale(double c, const double* x, double* z, idx n)
{
  for (idx i = 0; i < n; i++) z[i] = c * x[i];
}
void port_abs(const double* x, double* z, idx n)
{
  for (idx i = 0; i < n; i++) z[i] = fabs(x[i]);
}
void port_inv(const double* x, double* z, idx n)
{
  for (idx i = 0; i < n; i++) z[i] = 1.0 / x[i];
}
void port_addconst(const double* x, double b, double* z, idx n)
{
  for (idx i = 0; i < n; i++) z[i] = x[i] + b;
}
void port_compare(double c, const double* x, double* z, idx n)
{
  for (idx i = 0; i < n; i++) z[i] = (fabs(x[i]) >= c) ? 1.0 : 0.0;
}

double port_dotprod(const double* x, const double* y, idx n)
{
  double s = 0.0;
  for (idx i = 0; i < n; i++) s += x[i] * y[i];
  return s;
}
double port_maxnorm(const double* x, idx n)
{
  double m = 0.0;
  for (idx i = 0; i < n; i++)
    if (fabs(x[i]) > m) m = fabs(x[i]);
  return m;
}
double port_wsqrsum(const double* x, const double* w, idx n)
{
  double s = 0.0;
  for (idx i = 0; i < n; i++)
  {
    double p = x[i] * w[i];
    s += p * p;
  }
  return s;
}
double port_wsqrsummask(const double* x, const double* w, const double* id, idx n)
{
  double s = 0.0;
  for (idx i = 0; i < n; i++)
    if (id[i] > 0.0)
    {
      double p = x[i] * w[i];
      s += p * p;
    }
  return s;
}
double port_wrmsnorm(const double* x, const double* w, idx n)
{
  return sqrt(port_wsqrsum(x, w, n) / (double)n);
}
double port_wrmsnormmask(const double* x, const double* w, const double* id, idx n)
{
  return sqrt(port_wsqrsummask(x, w, id, n) / (double)n);
}
double port_min(const double* x, idx n)
{
  double m = x[0];
  for (idx i = 1; i < n; i++)
    if (x[i] < m) m = x[i];
  return m;
}
double port_wl2norm(const double* x, const double* w, idx n)
{
  return sqrt(port_wsqrsum(x, w, n));
}
double port_l1norm(const double* x, idx n)
{
  double s = 0.0;
  for (idx i = 0; i < n; i++) s += fabs(x[i]);
  return s;
}
int port_invtest(const double* x, double* z, idx n)
{
  int ok = 1;
  for (idx i = 0; i < n; i++)
  {
    if (x[i] == 0.0) ok = 0;
    else z[i] = 1.0 / x[i];
  }
  return ok;
}
int port_constrmask(const double* c, const double* x, double* m, idx n)
{
  int any = 0;
  for (idx i = 0; i < n; i++)
  {
    m[i] = 0.0;
    if (c[i] == 0.0) continue;
    if ((fabs(c[i]) > 1.5 && x[i] * c[i] <= 0.0) || (fabs(c[i]) > 0.5 && x[i] * c[i] < 0.0))
    {
      m[i] = 1.0;
      any  = 1;
    }
  }
  return !any;
}
double port_minquotient(const double* num, const double* den, idx n)
{
  int none = 1;
  double m = DBL_MAX;
  for (idx i = 0; i < n; i++)
  {
    if (den[i] == 0.0) continue;
    double q = num[i] / den[i];
    if (none)
    {
      m    = q;
      none = 0;
    }
    else if (q < m) m = q;
  }
  return m;
}

/* z = sum_k c_k X_k; X[0] may be z (the reference's in-place cases). */
void port_linearcombination(int nvec, const double* c, const double* const* X,
                            double* z, idx n)
{
  if (nvec == 1)
  {
    port_scale(c[0], X[0], z, n);
    return;
  }
  if (nvec == 2)
  {
    port_linearsum(c[0], X[0], c[1], X[1], z, n);
    return;
  }
  if (X[0] == z && c[0] == 1.0)
  {
    for (int k = 1; k < nvec; k++)
      for (idx i = 0; i < n; i++) z[i] += c[k] * X[k][i];
    return;
  }
  if (X[0] == z)
    for (idx i = 0; i < n; i++) z[i] *= c[0];
  else
    for (idx i = 0; i < n; i++) z[i] = c[0] * X[0][i];
  for (int k = 1; k < nvec; k++)
    for (idx i = 0; i < n; i++) z[i] += c[k] * X[k][i];
}

/* Z_k = a_k x + Y_k (Y may be Z). */
void port_scaleaddmulti(int nvec, const double* a, const double* x,
                        const double* const* Y, double* const* Z, idx n)
{
  for (int k = 0; k < nvec; k++)
    for (idx i = 0; i < n; i++) Z[k][i] = a[k] * x[i] + Y[k][i];
}

void port_dotprodmulti(int nvec, const double* x, const double* const* Y,
                       double* d, idx n)
{
  for (int k = 0; k < nvec; k++) d[k] = port_dotprod(x, Y[k], n);
}

/* ---- multi-core timing variants (the CPU baseline on all host cores) ------
 * Same per-element arithmetic as above; the sums split into per-thread
 * partials like the reference's NVECTOR_OPENMP (nvector_openmp.c), so their
 * summation order differs from the serial vector.  Used for timing only. */
#include <omp.h>

void omp_linearsum(double a, const double* x, double b, const double* y, double* z, idx n)
{
#pragma omp parallel for schedule(static)
  for (idx i = 0; i < n; i++) z[i] = (a * x[i]) + (b * y[i]);
}

void omp_linearcombination(int nvec, const double* c, const double* const* X, double* z, idx n)
{
#pragma omp parallel for schedule(static)
  for (idx i = 0; i < n; i++)
  {
    double s = c[0] * X[0][i];
    for (int k = 1; k < nvec; k++) s += c[k] * X[k][i];
    z[i] = s;
  }
}

void omp_dotprodmulti(int nvec, const double* x, const double* const* Y, double* d, idx n)
{
  for (int k = 0; k < nvec; k++) d[k] = 0.0;
#pragma omp parallel
  {
    double loc[64];
    for (int k = 0; k < nvec; k++) loc[k] = 0.0;
#pragma omp for schedule(static)
    for (idx i = 0; i < n; i++)
      for (int k = 0; k < nvec; k++) loc[k] += x[i] * Y[k][i];
#pragma omp critical
    for (int k = 0; k < nvec; k++) d[k] += loc[k];
  }
}

double omp_wrmsnorm(const double* x, const double* w, idx n)
{
  double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
  for (idx i = 0; i < n; i++)
  {
    double p = x[i] * w[i];
    s += p * p;
  }
  return sqrt(s / (double)n);
}

int omp_threads(void) { return omp_get_max_threads(); }

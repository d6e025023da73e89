/* dense_port.c -- TEST ORACLE (checker only): the reference's dense LU with
 * partial pivoting and its solve, restated on plain column-major arrays:
 *   SUNDlsMat_denseGETRF  src/sundials/sundials_dense.c:85-151
 *   SUNDlsMat_denseGETRS  src/sundials/sundials_dense.c:153-193
 * Compiled with -ffp-contract=off; pinned against the reference by
 * tests/test_oracle_pins.py (tests/golden/dense_lu.npz). */
#include <math.h>
#include <stdint.h>

int port_dense_getrf(double* a, int64_t n, int64_t* p)
{
  for (int64_t k = 0; k < n; k++)
  {
    double* ck = a + k * n;
    int64_t l  = k;
    for (int64_t i = k + 1; i < n; i++)
      if (fabs(ck[i]) > fabs(ck[l])) l = i;
    p[k] = l;
    if (ck[l] == 0.0) return (int)(k + 1);
    if (l != k)
      for (int64_t i = 0; i < n; i++)
      {
        double t     = a[i * n + l];
        a[i * n + l] = a[i * n + k];
        a[i * n + k] = t;
      }
    double mult = 1.0 / ck[k];
    for (int64_t i = k + 1; i < n; i++) ck[i] *= mult;
    for (int64_t j = k + 1; j < n; j++)
    {
      double* cj  = a + j * n;
      double a_kj = cj[k];
      if (a_kj != 0.0)
        for (int64_t i = k + 1; i < n; i++) cj[i] -= a_kj * ck[i];
    }
  }
  return 0;
}

void port_dense_getrs(const double* a, int64_t n, const int64_t* p, double* b)
{
  for (int64_t k = 0; k < n; k++)
  {
    int64_t pk = p[k];
    if (pk != k)
    {
      double t = b[k];
      b[k]     = b[pk];
      b[pk]    = t;
    }
  }
  for (int64_t k = 0; k < n - 1; k++)
    for (int64_t i = k + 1; i < n; i++) b[i] -= a[k * n + i] * b[k];
  for (int64_t k = n - 1; k > 0; k--)
  {
    b[k] /= a[k * n + k];
    for (int64_t i = 0; i < k; i++) b[i] -= a[k * n + i] * b[k];
  }
  b[0] /= a[0];
}

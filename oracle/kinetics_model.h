/* kinetics_model.h -- TEST ORACLE: the mass-action right-hand side and
 * Jacobian of the uneven kinetics batch, shared by the reference-CVODE driver
 * (kinetics_cvode_ref.c) and the CVODE restatement (cvode_bdf_port.c).
 *
 * The batch and its summation order are defined in sundials_gb300/kinetics.py:
 *   A -> B      : rate = k*y_A;        f_A -= rate; f_B += rate
 *   A + B -> C  : rate = (k*y_A)*y_B;  f_A -= rate; f_B -= rate; f_C += rate
 * accumulated over the reactions in index order (f starts at zero), and the
 * Jacobian entries likewise, column-major J[j*n + i] = d f_i / d y_j. */
#ifndef ORACLE_KINETICS_MODEL_H
#define ORACLE_KINETICS_MODEL_H

#include <stdint.h>

typedef struct
{
  int n;              /* species */
  int nr;             /* reactions (2n) */
  const int32_t* rt;  /* 0: A->B, 1: A+B->C */
  const int32_t* ra;
  const int32_t* rb;
  const int32_t* rc;
  const double* rk;
} KinSys;

static inline void kin_rhs(const KinSys* s, const double* y, double* f)
{
  for (int i = 0; i < s->n; i++) f[i] = 0.0;
  for (int r = 0; r < s->nr; r++)
  {
    const int a = s->ra[r], b = s->rb[r];
    if (s->rt[r] == 0)
    {
      const double rate = s->rk[r] * y[a];
      f[a] = f[a] - rate;
      f[b] = f[b] + rate;
    }
    else
    {
      const int c       = s->rc[r];
      const double rate = (s->rk[r] * y[a]) * y[b];
      f[a] = f[a] - rate;
      f[b] = f[b] - rate;
      f[c] = f[c] + rate;
    }
  }
}

/* J must be zero on entry (CVODE zeroes A before calling the Jacobian). */
static inline void kin_jac(const KinSys* s, const double* y, double* J)
{
  const int n = s->n;
  for (int r = 0; r < s->nr; r++)
  {
    const int a = s->ra[r], b = s->rb[r];
    const double k = s->rk[r];
    if (s->rt[r] == 0)
    {
      J[a * n + a] = J[a * n + a] - k;
      J[a * n + b] = J[a * n + b] + k;
    }
    else
    {
      const int c     = s->rc[r];
      const double dA = k * y[b]; /* d rate / d y_A */
      const double dB = k * y[a]; /* d rate / d y_B */
      J[a * n + a] = J[a * n + a] - dA;
      J[a * n + b] = J[a * n + b] - dA;
      J[a * n + c] = J[a * n + c] + dA;
      J[b * n + a] = J[b * n + a] - dB;
      J[b * n + b] = J[b * n + b] - dB;
      J[b * n + c] = J[b * n + c] + dB;
    }
  }
}

/* Binary problem file (little endian):
 *   int64 nsys, Y, R
 *   int32 n[nsys]; int64 y_off[nsys+1]; int64 r_off[nsys+1]
 *   int32 rt[R], ra[R], rb[R], rc[R]; double rk[R]; double y0[Y]        */

/* Per-system result record written by the drivers. */
typedef struct
{
  int64_t nst, nfe, nsetups, nje, nni, ncfn, netf, nnf;
  int64_t flag, qu;
  double tn, hu;
} KinStats;

#endif

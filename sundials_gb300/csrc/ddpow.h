/* ddpow.h -- pow(x, y) for x >= 0 evaluated in double-double arithmetic and
 * rounded once to double, for host and device code.
 *
 * Purpose: CVODE's step-size controller calls pow() at every step
 * (cvode.c:3443, 3553, 3624, 3651).  The reference's results come from the C
 * library's pow, whose error is a small fraction of an ulp; CUDA's device pow
 * may be off by up to 2 ulp.  Evaluating log and exp with ~100-bit
 * intermediates and rounding once gives the correctly rounded result except
 * when the exact value lies within about 2^-40 ulp of a rounding boundary,
 * so it agrees with an accurate C library pow in essentially every call.
 *
 * Methods (published, textbook):
 *   - error-free transformations two_sum (Knuth), fast_two_sum (Dekker) and
 *     two_prod via fused multiply-add;
 *   - double-double add / mul / div (Dekker 1971; Hida, Li, Bailey 2001);
 *   - log(x) = e*ln2 + 2*atanh((f-1)/(f+1)), f in [1/sqrt2, sqrt2), with the
 *     atanh series summed in double-double (21 terms: |s| <= 0.1716);
 *   - exp(z) = 2^k * (exp(r/256))^256, r = z - k*ln2, Taylor series for
 *     exp(r/256) (11 terms), eight double-double squarings.
 * ln 2 is split into two doubles (hi + lo) from its decimal expansion
 * 0.69314718055994530941723212145817656807...
 * Every operation uses explicit fma() where a fused product is meant, so the
 * bits are the same on the host and on the device, with or without
 * -fmad=false. */
#ifndef SUNGB300_DDPOW_H
#define SUNGB300_DDPOW_H

#include <math.h>

#if defined(__CUDACC__)
#define DDQ __host__ __device__ __forceinline__
#else
#define DDQ static inline
#endif

typedef struct
{
  double hi, lo;
} dd_t;

DDQ dd_t dd_from(double a)
{
  dd_t r = {a, 0.0};
  return r;
}

DDQ dd_t dd_two_sum(double a, double b)
{
  double s  = a + b;
  double bb = s - a;
  double e  = (a - (s - bb)) + (b - bb);
  dd_t r    = {s, e};
  return r;
}
DDQ dd_t dd_fast_two_sum(double a, double b)
{
  double s = a + b;
  double e = b - (s - a);
  dd_t r   = {s, e};
  return r;
}
DDQ dd_t dd_two_prod(double a, double b)
{
  double p = a * b;
  double e = fma(a, b, -p);
  dd_t r   = {p, e};
  return r;
}
DDQ dd_t dd_add(dd_t x, dd_t y)
{
  dd_t s = dd_two_sum(x.hi, y.hi);
  dd_t t = dd_two_sum(x.lo, y.lo);
  s.lo   = s.lo + t.hi;
  s      = dd_fast_two_sum(s.hi, s.lo);
  s.lo   = s.lo + t.lo;
  return dd_fast_two_sum(s.hi, s.lo);
}
DDQ dd_t dd_mul(dd_t x, dd_t y)
{
  dd_t p = dd_two_prod(x.hi, y.hi);
  p.lo   = p.lo + (x.hi * y.lo + x.lo * y.hi);
  return dd_fast_two_sum(p.hi, p.lo);
}
DDQ dd_t dd_mul_d(dd_t x, double y)
{
  dd_t p = dd_two_prod(x.hi, y);
  p.lo   = p.lo + x.lo * y;
  return dd_fast_two_sum(p.hi, p.lo);
}
DDQ dd_t dd_div(dd_t x, dd_t y)
{ /* long division: q1 + q2 + q3 */
  double q1 = x.hi / y.hi;
  dd_t r    = dd_add(x, dd_mul_d(y, -q1));
  double q2 = r.hi / y.hi;
  r         = dd_add(r, dd_mul_d(y, -q2));
  double q3 = r.hi / y.hi;
  dd_t q    = dd_fast_two_sum(q1, q2);
  return dd_add(q, dd_from(q3));
}

DDQ dd_t dd_ln2(void)
{
  dd_t r = {0.6931471805599453094172321214581766, 2.319046813846299558417771e-17};
  return r;
}

/* natural log of x > 0 (finite, normal) in double-double */
DDQ dd_t dd_log(double x)
{
  int e;
  double f = frexp(x, &e); /* x = f * 2^e, f in [0.5, 1) */
  if (f < 0.70710678118654752440)
  {
    f = f * 2.0;
    e = e - 1;
  }
  dd_t num = {f - 1.0, 0.0}; /* exact (Sterbenz) */
  dd_t den = dd_two_sum(f, 1.0);
  dd_t s   = dd_div(num, den);
  dd_t s2  = dd_mul(s, s);
  const int K = 21;
  dd_t one = {1.0, 0.0};
  dd_t p   = dd_div(one, dd_from(2.0 * K + 1.0));
  for (int k = K - 1; k >= 0; k--)
  {
    dd_t c = dd_div(one, dd_from(2.0 * k + 1.0));
    p      = dd_add(dd_mul(p, s2), c);
  }
  dd_t lf = dd_mul(dd_mul_d(s, 2.0), p);
  return dd_add(dd_mul_d(dd_ln2(), (double)e), lf);
}

/* exp of a double-double argument of moderate size (|z| < 700) */
DDQ dd_t dd_exp(dd_t z)
{
  const dd_t ln2 = dd_ln2();
  double k       = nearbyint(z.hi / ln2.hi);
  dd_t r         = dd_add(z, dd_mul_d(ln2, -k));
  r.hi           = r.hi * (1.0 / 256.0); /* exact scaling */
  r.lo           = r.lo * (1.0 / 256.0);
  /* Taylor: sum_{j=0}^{11} r^j / j!, Horner from the top */
  dd_t one = {1.0, 0.0};
  dd_t p   = one;
  for (int j = 11; j >= 1; j--)
  {
    p = dd_add(one, dd_div(dd_mul(p, r), dd_from((double)j)));
  }
  for (int i = 0; i < 8; i++) p = dd_mul(p, p);
  p.hi = ldexp(p.hi, (int)k);
  p.lo = ldexp(p.lo, (int)k);
  return p;
}

/* pow(x, y) for x >= 0 and moderate results, rounded once. */
DDQ double dd_pow(double x, double y)
{
  if (x == 0.0) return y > 0.0 ? 0.0 : (y == 0.0 ? 1.0 : INFINITY);
  if (!(x < INFINITY) || x != x || y != y) return pow(x, y);
  if (y == 1.0) return x;
  dd_t l = dd_log(x);
  dd_t z = dd_mul_d(l, y);
  if (fabs(z.hi) > 700.0) return pow(x, y);
  dd_t r = dd_exp(z);
  return r.hi + r.lo;
}

#endif

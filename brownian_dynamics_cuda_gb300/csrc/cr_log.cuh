// Natural logarithm of a positive double, correctly rounded to nearest in
// all but (by construction) astronomically rare cases, for the device-side
// polar noise transform.
//
// Method: argument reduction x = 2^k m with m in [1/sqrt2, sqrt2), then
//   log x = k ln2 + 2 atanh(z),  z = (m - 1) / (m + 1),  |z| <= 0.1716,
//   2 atanh(z) = 2 z (1 + w/3 + w^2/5 + w^3/7 + ...),  w = z^2 <= 0.0295
// (the classical atanh series for the logarithm), evaluated in
// double-double arithmetic: Knuth's TwoSum and the FMA form of Dekker's
// TwoProduct for every operation on the first nine series terms, plain
// doubles for the tail (relative weight < w^9 ~ 1.7e-14 of the sum, so its
// own rounding enters below 2^-95), ln 2 as a double-double constant
// (hi + lo to ~2^-107).  The double-double result carries a relative error
// far below 2^-90; rounding hi + lo to double then gives the correctly
// rounded logarithm unless the exact value lies within that error of a
// rounding midpoint.
//
// Compiles for the device (CUDA) and the host (C++, with fma from <cmath>),
// so the host test checks the very same code against high-precision values.
#pragma once
#include <math.h>

#if defined(__CUDACC__)
#define CRLOG_HD __host__ __device__ inline
#else
#define CRLOG_HD inline
#endif

namespace crlog {

struct dd {
  double hi, lo;
};

// s + e = a + b exactly (Knuth)
CRLOG_HD dd two_sum(double a, double b) {
  const double s = a + b;
  const double bb = s - a;
  const double e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
// s + e = a + b exactly, |a| >= |b| (Dekker)
CRLOG_HD dd fast_two_sum(double a, double b) {
  const double s = a + b;
  return {s, b - (s - a)};
}
// p + e = a b exactly (FMA)
CRLOG_HD dd two_prod(double a, double b) {
  const double p = a * b;
  return {p, fma(a, b, -p)};
}
CRLOG_HD dd dd_add(dd a, dd b) {
  dd s = two_sum(a.hi, b.hi);
  const dd t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = fast_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return fast_two_sum(s.hi, s.lo);
}
CRLOG_HD dd dd_mul(dd a, dd b) {
  dd p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return fast_two_sum(p.hi, p.lo);
}
// 1 / n as a double-double (n a small odd integer): hi = RN(1/n), and the
// residual 1 - n hi is exact through the FMA
CRLOG_HD dd dd_recip(double n) {
  const double h = 1.0 / n;
  return {h, fma(-n, h, 1.0) / n};
}

CRLOG_HD double log_cr(double x) {
  if (!(x > 0.0)) return x == 0.0 ? -INFINITY : NAN;
  if (isinf(x)) return x;
  // x = 2^k f, f in [1, 2); then m = f or f / 2 in [1/sqrt2, sqrt2)
  int k;
  double f = frexp(x, &k);  // f in [0.5, 1)
  f *= 2.0;
  k -= 1;
  if (f > 1.4142135623730951) {
    f *= 0.5;
    k += 1;
  }
  if (f == 1.0 && k == 0) return 0.0;
  // z = (f - 1) / (f + 1): f - 1 is exact (Sterbenz); f + 1 as a double-double
  const double num = f - 1.0;
  const dd den = two_sum(f, 1.0);
  const double zh = num / den.hi;
  // residual num - zh (den.hi + den.lo), the first product exact by the FMA
  const double r = fma(-zh, den.hi, num) - zh * den.lo;
  const dd z = fast_two_sum(zh, r / den.hi);
  const dd w = dd_mul(z, z);
  // tail (terms j >= 9) in doubles: 1/19 + w/21 + w^2/23 + ...
  double t = 0.0;
  for (int j = 24; j >= 9; j--) t = t * w.hi + 1.0 / (2 * j + 1);
  dd P = {t, 0.0};
  for (int j = 8; j >= 0; j--) P = dd_add(dd_mul(P, w), dd_recip(2 * j + 1));
  dd y = dd_mul(z, P);
  y.hi *= 2.0;
  y.lo *= 2.0;
  // k ln2 with ln2 = L_HI + L_LO
  const double L_HI = 0.6931471805599453094172321;     // 0x1.62e42fefa39efp-1
  const double L_LO = 2.3190468138462996154e-17;       // 0x1.abc9e3b39803fp-56
  const dd kl = dd_add(two_prod((double)k, L_HI), dd{(double)k * L_LO, 0.0});
  const dd s = dd_add(kl, y);
  return s.hi + s.lo;
}

}  // namespace crlog

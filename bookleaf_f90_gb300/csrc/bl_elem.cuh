// bl_elem.cuh -- exp, log and pow for the equations of state, written for
// this project so that the device and the CPU restatement (oracle/oracle.c,
// orc_exp/orc_log/orc_pow) evaluate them with the same IEEE operations in
// the same order: with FMA contraction off (the exact build) the two agree
// bit for bit, which the hardware's and the C library's own functions,
// different implementations, cannot promise.  Measured against the C
// library on the host they stay within 1-2 units in the last place (the
// CPU test of the restatement's copies).
//
// Methods (textbook, constants computed for this file):
//   exp(x): x = k ln2 + r with k = nearest(x / ln2), ln2 split into a
//     40-bit head (k * head exact for |k| < 2^13) and the rounded rest
//     (Cody and Waite 1980); exp(r), |r| <= ln2/2, from its Taylor series
//     to r^13 (remainder below 1e-17 relative) as 1 + (r + r^2 P(r)), then
//     scaled by 2^k with exact power-of-two products.
//   log(a): a = m 2^e with m in [sqrt(1/2), sqrt(2)); log m = 2 atanh(s),
//     s = (m - 1)/(m + 1), |s| < 0.1716, from the odd series to s^23
//     (remainder below 1e-18); log a = e ln2 + log m with ln2 split as above.
//   pow(a, b) = exp(b log a) for a > 0, log a and its product with b
//     carried as double-doubles (Dekker 1971, Knuth's two-sum; no FMA
//     needed) into exp's reduced argument, with the IEEE special cases the
//     equations of state can meet (a = 1, b = 0, a = 0, NaN, infinity).
#pragma once
#include <cmath>
#include <cstdint>

namespace bl {

namespace elem {
constexpr double kInvLn2 = 1.4426950408889634;
constexpr double kLn2Hi = 0.6931471805592082;     // 40 significant bits of ln 2
constexpr double kLn2Lo = 7.371002565167799e-13;  // ln 2 - kLn2Hi, rounded
constexpr double kSqrt2 = 1.4142135623730951;

__device__ __forceinline__ double pow2i(int k) {  // 2^k, -1022 <= k <= 1023
  return __longlong_as_double((long long)(k + 1023) << 52);
}
}  // namespace elem

// exp(x + xl) for a small correction xl (0 for plain exp), added to the
// reduced argument
__device__ __forceinline__ double bl_exp2p(double x, double xl) {
  using namespace elem;
  if (x != x) return x;
  if (x > 709.782712893384) return HUGE_VAL;
  if (x < -745.1332191019412) return 0.0;
  const double kd = rint(x * kInvLn2);
  const double r = ((x - kd * kLn2Hi) - kd * kLn2Lo) + xl;
  double p = 1.6059043836821613e-10;  // 1/13!
  p = p * r + 2.08767569878681e-09;   // 1/12!
  p = p * r + 2.505210838544172e-08;
  p = p * r + 2.755731922398589e-07;
  p = p * r + 2.7557319223985893e-06;
  p = p * r + 2.48015873015873e-05;
  p = p * r + 0.0001984126984126984;
  p = p * r + 0.001388888888888889;
  p = p * r + 0.008333333333333333;
  p = p * r + 0.041666666666666664;
  p = p * r + 0.16666666666666666;
  p = p * r + 0.5;                    // 1/2!
  const double q = r + (r * r) * p;
  double e = 1.0 + q;
  int k = (int)kd;
  if (k > 1023) {
    e = e * pow2i(1023);
    k -= 1023;
  } else if (k < -1022) {
    e = e * pow2i(-1022);
    k += 1022;
    if (k < -1022) return 0.0;
  }
  return e * pow2i(k);
}

__device__ __forceinline__ double bl_exp(double x) { return bl_exp2p(x, 0.0); }

// Dekker's exact product without FMA: a*b = p + e (Veltkamp splitting into
// 26-bit halves; |a|, |b| well below 2^996)
__device__ __forceinline__ void two_prod(double a, double b, double& p, double& e) {
  p = a * b;
  double c = 134217729.0 * a;
  const double ah = c - (c - a), al = a - ah;
  c = 134217729.0 * b;
  const double bh = c - (c - b), bl = b - bh;
  e = ((ah * bh - p) + ah * bl + al * bh) + al * bl;
}

// log(a) as a double-double hi + lo (a > 0 finite): the reduction's
// quotient s = f/(2+f) is corrected by its remainder and the sum with
// e ln2 is taken exactly (Knuth's two-sum)
__device__ __forceinline__ void bl_log_dd(double a, double& hi, double& lo) {
  using namespace elem;
  long long b = __double_as_longlong(a);
  int e = 0;
  if ((b >> 52) == 0) {
    a = a * 18014398509481984.0;
    b = __double_as_longlong(a);
    e = -54;
  }
  e += (int)((b >> 52) & 0x7ff) - 1023;
  double m = __longlong_as_double((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
  if (m > kSqrt2) {
    m = m * 0.5;
    e += 1;
  }
  const double f = m - 1.0;
  const double uh = 2.0 + f, ul = f - (uh - 2.0);  // 2 + f exactly
  const double s = f / uh;
  double P, Pe;
  two_prod(s, uh, P, Pe);
  const double serr = (((f - P) - Pe) - s * ul) / uh;  // f/(2+f) - s
  const double s2 = s * s;
  double R = 0.043478260869565216;
  R = R * s2 + 0.047619047619047616;
  R = R * s2 + 0.05263157894736842;
  R = R * s2 + 0.058823529411764705;
  R = R * s2 + 0.06666666666666667;
  R = R * s2 + 0.07692307692307693;
  R = R * s2 + 0.09090909090909091;
  R = R * s2 + 0.1111111111111111;
  R = R * s2 + 0.14285714285714285;
  R = R * s2 + 0.2;
  R = R * s2 + 0.3333333333333333;
  R = R * s2;
  const double t = s + s;
  const double ed = (double)e;
  const double A = ed * kLn2Hi;               // exact
  const double H = A + t;
  const double bv = H - A;
  const double L1 = (A - (H - bv)) + (t - bv);  // two-sum error
  hi = H;
  lo = L1 + ((t * R + (serr + serr)) + ed * kLn2Lo);
}

__device__ __forceinline__ double bl_log(double a) {
  using namespace elem;
  if (a != a) return a;
  if (a <= 0.0) return a == 0.0 ? -HUGE_VAL : __longlong_as_double(0x7ff8000000000000LL);
  if (a == HUGE_VAL) return a;
  long long b = __double_as_longlong(a);
  int e = 0;
  if ((b >> 52) == 0) {  // subnormal: scale into the normal range
    a = a * 18014398509481984.0;  // 2^54
    b = __double_as_longlong(a);
    e = -54;
  }
  e += (int)((b >> 52) & 0x7ff) - 1023;
  double m = __longlong_as_double((b & 0x000fffffffffffffLL) | 0x3ff0000000000000LL);
  if (m > kSqrt2) {
    m = m * 0.5;
    e += 1;
  }
  const double f = m - 1.0;
  const double s = f / (2.0 + f);
  const double s2 = s * s;
  double R = 0.043478260869565216;  // 1/23
  R = R * s2 + 0.047619047619047616;
  R = R * s2 + 0.05263157894736842;
  R = R * s2 + 0.058823529411764705;
  R = R * s2 + 0.06666666666666667;
  R = R * s2 + 0.07692307692307693;
  R = R * s2 + 0.09090909090909091;
  R = R * s2 + 0.1111111111111111;
  R = R * s2 + 0.14285714285714285;
  R = R * s2 + 0.2;
  R = R * s2 + 0.3333333333333333;  // 1/3
  R = R * s2;
  const double t = s + s;
  const double ed = (double)e;
  return ed * kLn2Hi + (t + (t * R + ed * kLn2Lo));
}

__device__ __forceinline__ double bl_pow(double a, double b) {
  if (b == 0.0 || a == 1.0) return 1.0;
  if (a != a || b != b) return a + b;
  if (a < 0.0) return __longlong_as_double(0x7ff8000000000000LL);
  if (a == 0.0) return b > 0.0 ? 0.0 : HUGE_VAL;
  if (a == HUGE_VAL) return b > 0.0 ? HUGE_VAL : 0.0;
  double lh, ll;
  bl_log_dd(a, lh, ll);
  if (fabs(b) > 1e300 || fabs(lh * b) > 1e300) return bl_exp(b * lh);
  double yh, yl;
  two_prod(b, lh, yh, yl);  // b (lh + ll) = yh + yl + b ll
  return bl_exp2p(yh, yl + b * ll);
}

}  // namespace bl

// bl_fp64.cuh -- correctly rounded FP64 division and square root, and FP64
// comparisons, on the integer pipe.
//
// GB300 issues FP64 at 1/64 of the FP32 rate (2 lanes per SM per clock),
// and DSETP/DMNMX comparisons, the MUFU.*64H seeds and the DFMA refinements
// of the hardware divide and square root all queue on that one pipe, which
// the hot path saturates.  The integer and FP32 pipes sit idle beside it.
// The routines here return exactly what the IEEE-754 operations return
// (round to nearest even) using integer arithmetic and one FP32 MUFU seed:
//
// ddiv_rn(a, b)
//   1. D = divisor significand << 11 (bit 63 set); N = dividend significand
//      shifted so that N < D <= 2N; Q = floor(N * 2^64 / D) has bit 63 set.
//   2. y = 2^64 + v ~ 2^128 / D from below: an FP32 rcp.approx of the top
//      24 bits of D, lowered by a margin of 2^-19, then two Newton-Raphson
//      steps y <- y + y (2^128 - D y) / 2^128, the first on the 24-bit seed
//      (64 x 24-bit products), the second in full 64-bit fixed point, every
//      truncation downwards (Newton-Raphson division, Flynn 1970, in the
//      fixed-point form of Moller and Granlund, "Improved division by
//      invariant integers", IEEE TC 2011).  After the second step
//      0 <= 2^128/D - y <= 4 units.
//   3. q = N + umulhi(N, v) satisfies q <= Q <= q + 5.
//   4. Rounding from q alone when its low 11 bits are more than 5 away from
//      the half-way point 0x400 and from the carry into bit 11; otherwise
//      (about 0.5% of operands) the exact remainder N*2^64 - q*D fixes q
//      and supplies the sticky bit.
//
// dsqrt_rn(x)
//   x = M * 2^(k-52), k even, M in [2^52, 2^54); N = M * 2^74 in
//   [2^126, 2^128), whose top word is Nhi = M << 10; S = floor(sqrt(N)).
//   R ~ 2^127 / sqrt(N) from below: FP32 rsqrt.approx seed of the top 24
//   bits less a 2^-19 margin, Newton-Raphson y <- y (3 - n y^2) / 2 once on
//   the 24-bit seed and once in 64-bit fixed point (this iteration
//   approaches 1/sqrt(n) from below from either side).  S0 = N R / 2^127,
//   then one residual step S1 = S0 + (N - S0^2) R / 2^128 leaves
//   S1 <= S <= S1 + 2.  Rounding as for the divide (no ties exist for a
//   square root), with the exact remainder N - S^2 near the boundary.
//
// Zero and subnormal operands are handled inline (a signed zero, or the
// significand normalised with an extended exponent); infinite and NaN
// operands, zero divisors, and quotients whose exponent could leave the
// normal range take the hardware path, which returns the identical result.
// bl_selftest_fp64 checks these routines (and dmul_rn below) against the
// hardware bit for bit on the device.
//
// Comparisons: an FP64 comparison is decided on the integer pipe through an
// order key (the bit pattern for sign-clear values, its reflection for
// negative ones, so that -0 and +0 share the key 0), with explicit NaN
// tests where an operand may be NaN, reproducing the IEEE predicate.
#pragma once
#include <climits>
#include <cstdint>

namespace bl {

// Bit patterns through inline PTX moves: the compiler cannot see through
// them, so it cannot turn the integer tests of the patterns below back into
// FP64 comparisons, class tests or abs (which would issue on the FP64 pipe).
__device__ __forceinline__ long long bits64(double x) {
  long long r;
  asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
  return r;
}
__device__ __forceinline__ double from_bits64(long long b) {
  double r;
  asm("mov.b64 %0, %1;" : "=d"(r) : "l"(b));
  return r;
}

__device__ __forceinline__ float rcp_approx_f32(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ float rsqrt_approx_f32(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// (a * b) >> 64 for b < 2^32
__device__ __forceinline__ uint64_t umulhi_64x32(uint64_t a, uint32_t b) {
  const uint64_t lo = (uint64_t)(uint32_t)a * b;
  const uint64_t hi = (a >> 32) * (uint64_t)b;
  return (hi + (lo >> 32)) >> 32;
}

// v with 2^64 + v ~ 2^128 / D, never above it; D in [2^63, 2^64).
__device__ __forceinline__ uint64_t recip_fixed(uint64_t D) {
  // seed: r = rcp(top 24 bits of D) in (2^-24, 2^-23]; Y0 = r * 2^47 is the
  // 24-bit seed, y0 = Y0 * 2^41
  const uint32_t d24 = (uint32_t)(D >> 40);
  const uint32_t rb = __float_as_uint(rcp_approx_f32((float)d24));
  // an approximation that lands outside (2^-24, 2^-23] is replaced by the
  // nearer end of that range (2^128/D lies in (2^64, 2^65])
  const uint32_t er = rb >> 23;
  uint32_t Y0 = er == 103u ? (0x800000u | (rb & 0x7FFFFFu)) : (er > 103u ? (1u << 24) : (1u << 23));
  Y0 = Y0 - 16u;                       // margin 2^-19
  if (Y0 < (1u << 23)) Y0 = 1u << 23;  // y0 >= 2^64 <= 2^128/D always
  // step 1: P = D * Y0 (< 2^87); E32 = floor((2^128 - P 2^41) / 2^87)
  //         = 2^41 - ceil(P / 2^46); y1 = y0 + Y0 * E32
  const uint64_t Plo = D * (uint64_t)Y0;
  const uint64_t Phi = umulhi_64x32(D, Y0);
  const uint64_t P46 = (Phi << 18) | (Plo >> 46);
  const uint64_t cP = P46 + (((Plo & ((1ull << 46) - 1)) != 0) ? 1ull : 0ull);
  const uint32_t E32 = (uint32_t)((1ull << 41) - cP);
  uint64_t v = ((uint64_t)Y0 << 41) + (uint64_t)Y0 * E32;   // mod 2^64: y1 - 2^64
  // step 2: e = 2^128 - D y1 (its high word, < 2^28); y2 = y1 + y1 e / 2^128
  const uint64_t plo = D * v;
  const uint64_t shi = D + __umul64hi(D, v);
  const uint64_t ehi = ~shi + (plo == 0 ? 1ull : 0ull);
  v = v + ehi + umulhi_64x32(v, (uint32_t)ehi);
  return v;
}

// The hardware operations for the rare operands, out of line so that none
// of their FP64 instructions is issued on the common path.
static __device__ __noinline__ double div_hw(double a, double b) { return a / b; }
static __device__ __noinline__ double sqrt_hw(double x) { return sqrt(x); }

// Slow-path rounding of a quotient: q <= Q <= q + 8, remainder fixed exactly.
static __device__ __noinline__ uint64_t ddiv_fix(uint64_t N, uint64_t D, uint64_t q) {
  const uint64_t plo = q * D;
  const uint64_t phi = __umul64hi(q, D);
  uint64_t rlo = 0ull - plo;
  uint64_t rhi = N - phi - (plo != 0 ? 1ull : 0ull);
#pragma unroll 1
  for (int k = 0; k < 8 && (rhi != 0 || rlo >= D); k++) {
    rhi -= (rlo < D) ? 1ull : 0ull;
    rlo -= D;
    q += 1;
  }
  // q = Q now; significand and round-up flag packed as (q >> 11) + up
  const uint64_t s = q >> 11;
  const bool g = ((q >> 10) & 1ull) != 0;
  const bool sticky = ((q & 0x3FFull) != 0) || (rlo != 0);
  return s + ((g && (sticky || (s & 1ull))) ? 1ull : 0ull);
}

__device__ __forceinline__ double ddiv_rn(double a, double b) {
  const uint64_t ua = (uint64_t)bits64(a);
  const uint64_t ub = (uint64_t)bits64(b);
  const uint64_t M52 = (1ull << 52) - 1;
  int ea = (int)((ua >> 52) & 0x7FF);
  int eb = (int)((ub >> 52) & 0x7FF);
  uint64_t ma = (ua & M52) | (1ull << 52);
  uint64_t mb = (ub & M52) | (1ull << 52);
  int ed = ea - eb;
  if ((unsigned)(ea - 1) >= 2046u || (unsigned)(eb - 1) >= 2046u || (unsigned)(ed + 1021) > 2043u) {
    const bool az = (ua << 1) == 0, bz = (ub << 1) == 0;
    // infinities, NaNs and zero divisors: the hardware
    if (ea == 2047 || eb == 2047 || bz) return div_hw(a, b);
    // a zero dividend (common: fluid at rest) gives the zero with the
    // product of the signs
    if (az) return from_bits64((long long)((ua ^ ub) & 0x8000000000000000ull));
    // subnormal operands (tiny velocity differences ahead of a shock) are
    // normalised, their exponent extended below 1
    if (ea == 0) {
      const int s = __clzll((long long)(ua & M52)) - 11;
      ma = (ua & M52) << s;
      ea = 1 - s;
    }
    if (eb == 0) {
      const int s = __clzll((long long)(ub & M52)) - 11;
      mb = (ub & M52) << s;
      eb = 1 - s;
    }
    ed = ea - eb;
    // a quotient that may be subnormal or overflow: the hardware
    if ((unsigned)(ed + 1021) > 2043u) return div_hw(a, b);
  }
  const bool ge = ma >= mb;
  const uint64_t N = ma << (ge ? 10 : 11);
  const uint64_t D = mb << 11;
  const int E = ed + (ge ? 1023 : 1022);   // in [1, 2045]
  const uint64_t v = recip_fixed(D);
  const uint64_t q = N + __umul64hi(N, v);
  const uint32_t L = (uint32_t)q & 0x7FFu;
  uint64_t sig;  // significand with the implicit bit, rounded
  if ((L + 5u >= 0x400u && L <= 0x400u) || L + 5u > 0x7FFu) sig = ddiv_fix(N, D, q);
  else sig = (q >> 11) + (L > 0x400u ? 1ull : 0ull);
  // the implicit bit of sig carries into the exponent field: (E-1) << 52
  const uint64_t r = (((uint64_t)(E - 1) << 52) + sig) | ((ua ^ ub) & 0x8000000000000000ull);
  return from_bits64((long long)r);
}

// Slow-path rounding of a square root: S1 <= S <= S1 + 4.
static __device__ __noinline__ uint64_t dsqrt_fix(uint64_t Nhi, uint64_t S) {
  uint64_t slo = S * S;
  uint64_t rlo = 0ull - slo;
  uint64_t rhi = Nhi - __umul64hi(S, S) - (slo != 0 ? 1ull : 0ull);
#pragma unroll 1
  for (int k = 0; k < 4; k++) {
    // N - S^2 >= 2S + 1 means S + 1 fits
    const uint64_t t = 2 * S + 1, thi = S >> 63;
    if (!(rhi > thi || (rhi == thi && rlo >= t))) break;
    rhi = rhi - thi - (rlo < t ? 1ull : 0ull);
    rlo -= t;
    S += 1;
  }
  const uint64_t s = S >> 11;
  const bool g = ((S >> 10) & 1ull) != 0;
  const bool sticky = ((S & 0x3FFull) != 0) || (rlo != 0) || (rhi != 0);
  return s + ((g && (sticky || (s & 1ull))) ? 1ull : 0ull);
}

__device__ __forceinline__ double dsqrt_rn(double x) {
  const uint64_t ux = (uint64_t)bits64(x);
  const uint64_t M52 = (1ull << 52) - 1;
  const int ex = (int)(ux >> 52);  // with the sign bit: negative x fails the test
  uint64_t M = (ux & M52) | (1ull << 52);
  int u = ex - 1023;
  if ((unsigned)(ex - 1) >= 2046u) {
    if ((ux << 1) == 0) return x;  // sqrt(+-0) = +-0
    if (ex != 0) return sqrt_hw(x);  // negative, infinite, NaN
    // positive subnormal: normalise (its square root is a normal number)
    const int s = __clzll((long long)ux) - 11;
    M = ux << s;
    u = -1022 - s;
  }
  const int odd = u & 1;
  const uint64_t Nhi = M << (10 + odd);
  const int E = ((u - odd) >> 1) + 1023;
  // seed: r = rsqrt(top 24 bits of Nhi) in (2^-12, 2^-11]; Y0 = r * 2^35,
  // R0 = Y0 * 2^40 ~ 2^127 / sqrt(N)
  const uint32_t rb = __float_as_uint(rsqrt_approx_f32((float)(uint32_t)(Nhi >> 40)));
  const uint32_t er = rb >> 23;
  uint32_t Y0 = er == 115u ? (0x800000u | (rb & 0x7FFFFFu)) : (er > 115u ? (1u << 24) : (1u << 23));
  Y0 = Y0 - 16u;
  if (Y0 < (1u << 23)) Y0 = 1u << 23;
  // step 1: t = n y0^2 2^62 = Nhi Y0^2 / 2^48 (rounded up), h = 3 2^62 - t,
  //         R1 = R0 h / 2^63 = Y0 h / 2^23
  const uint64_t Y2 = (uint64_t)Y0 * Y0;                      // < 2^48
  uint64_t t = __umul64hi(Nhi, Y2 << 16) + 1;
  uint64_t h = 3ull * (1ull << 62) - t;
  uint64_t R = (umulhi_64x32(h, Y0) << 41) | ((h * Y0) >> 23);
  // step 2 in 64-bit: t >= Nhi R^2 / 2^128 (two dropped words: +2)
  t = __umul64hi(Nhi, __umul64hi(R, R)) + 2;
  h = 3ull * (1ull << 62) - t;
  {
    const uint64_t plo = R * h, phi = __umul64hi(R, h);
    R = (phi << 1) | (plo >> 63);
  }
  // S0 = floor(Nhi R / 2^63) <= sqrt(N)
  uint64_t S;
  {
    const uint64_t plo = Nhi * R, phi = __umul64hi(Nhi, R);
    S = (phi << 1) | (plo >> 63);
  }
  // residual step: rem = N - S0^2 (< 2^70); S1 = S0 + floor(rem R / 2^128)
  {
    const uint64_t slo = S * S;
    const uint64_t rlo = 0ull - slo;
    const uint64_t rhi = Nhi - __umul64hi(S, S) - (slo != 0 ? 1ull : 0ull);
    const uint64_t alo = R * rhi;
    const uint64_t ahi = umulhi_64x32(R, (uint32_t)rhi);
    const uint64_t sum = alo + __umul64hi(rlo, R);
    S += ahi + (sum < alo ? 1ull : 0ull);
  }
  const uint32_t L = (uint32_t)S & 0x7FFu;
  uint64_t sig;
  if ((L + 3u >= 0x400u && L <= 0x400u) || L + 3u > 0x7FFu) sig = dsqrt_fix(Nhi, S);
  else sig = (S >> 11) + (L > 0x400u ? 1ull : 0ull);
  return from_bits64((long long)(((uint64_t)(E - 1) << 52) + sig));
}

// ------------------------------------------------------------ multiply

// dmul_rn(a, b): the FP64 product on the integer pipe, rounded to nearest
// even, bit for bit the FP64 multiply's result.  The significands with
// their implicit bit, shifted to bit 63 (A = ma << 11, B = mb << 11), are
// multiplied in 32-bit limbs; the product's top word hi lies in
// [2^62, 2^64) and s is its top bit.  X = hi >> s, with the bit shifted out
// and the low word's non-zero test folded into bit 0 (the sticky bit), lies
// in [2^62, 2^63), and (X + 0x1FF + bit 10 of X) >> 10 is the significand
// rounded to nearest even (guard bit 9), at most 2^53: added to the biased
// exponent field it carries into the exponent by itself.  A zero operand
// with a finite other operand gives the signed zero inline; subnormal,
// infinite and NaN operands, and products whose exponent could leave the
// normal range, take the FP64 multiply.  Measured on GB300 it issues no
// faster than the FP64 pipe multiplies (bl_fp64_rates: 522 against 513 G
// products/s), and moving k_getdt's 84 products that do not fold into an
// FMA here made the kernel slower (160 against 144 us on Sedov 512x512,
// with more spills at the same registers), so the kernels keep the FP64
// multiply; the routine and its self-test record that measurement.
static __device__ __noinline__ double mul_hw(double a, double b) { return a * b; }
__device__ __forceinline__ double dmul_rn(double a, double b) {
  const uint64_t ia = (uint64_t)bits64(a), ib = (uint64_t)bits64(b);
  const int ea = (int)(ia >> 52) & 0x7FF, eb = (int)(ib >> 52) & 0x7FF;
  const uint64_t sgn = (ia ^ ib) & 0x8000000000000000ull;
  const int e = ea + eb - 1023;  // the product's exponent field when s = 0
  if ((unsigned)(ea - 1) < 2046u && (unsigned)(eb - 1) < 2046u && (unsigned)(e - 1) < 2044u) {
    const uint32_t al = (uint32_t)ia << 11, ah = (uint32_t)(ia >> 21) | 0x80000000u;
    const uint32_t bl = (uint32_t)ib << 11, bh = (uint32_t)(ib >> 21) | 0x80000000u;
    const uint64_t p0 = (uint64_t)al * bl;
    const uint64_t p1 = (uint64_t)ah * bl + (p0 >> 32);
    const uint64_t p2 = (uint64_t)al * bh + (uint32_t)p1;
    const uint64_t hi = (uint64_t)ah * bh + (p1 >> 32) + (p2 >> 32);
    const uint64_t sticky = (((uint32_t)p0 | (uint32_t)p2) != 0u) ? 1ull : 0ull;
    const unsigned s = (unsigned)(hi >> 63);
    const uint64_t X = (hi >> s) | (hi & (uint64_t)s) | sticky;
    const uint64_t m = (X + 0x1FFull + ((X >> 10) & 1ull)) >> 10;
    return from_bits64((long long)(sgn | (((uint64_t)(e + (int)s - 1) << 52) + m)));
  }
  if (((ia << 1) == 0 && eb != 0x7FF) || ((ib << 1) == 0 && ea != 0x7FF))
    return from_bits64((long long)sgn);
  return mul_hw(a, b);
}

// ------------------------------------------------------------ powers of two

// x * 2^K exactly as the FP64 multiply rounds it, by adding K to the
// exponent field when x and the product are normal numbers; zeros return
// themselves, and subnormal, infinite or NaN operands and products that
// leave the normal range take the FP64 multiply.  The scalings by 0.5,
// 0.25, 2 and 4 that the reference's formulas are full of then cost no
// FP64 issue slot.
static __device__ __noinline__ double ldexp_slow(double x, double s) { return x * s; }
template <int K>
__device__ __forceinline__ double ldexpF(double x) {
  const long long b = bits64(x);
  const int e = (int)((b >> 52) & 0x7FF);
  if ((unsigned)(e - 1) < 2046u && (unsigned)(e + K - 1) < 2046u)
    return from_bits64(b + (long long)((unsigned long long)(long long)K << 52));
  if (((unsigned long long)b << 1) == 0) return x;
  return ldexp_slow(x, K >= 0 ? (double)(1 << (K >= 0 ? K : 0)) : 1.0 / (double)(1 << (K < 0 ? -K : 0)));
}
__device__ __forceinline__ double half(double x) { return ldexpF<-1>(x); }
__device__ __forceinline__ double quarter(double x) { return ldexpF<-2>(x); }
__device__ __forceinline__ double twice(double x) { return ldexpF<1>(x); }
__device__ __forceinline__ double times4(double x) { return ldexpF<2>(x); }

// ------------------------------------------------------------ sign bits

// |x| and Fortran SIGN(|a|, b) as operations on the sign bit of the high
// word (integer pipe); an FP64 abs or negate that the compiler cannot fold
// into a neighbouring instruction would otherwise occupy an FP64 issue slot.
__device__ __forceinline__ double negF(double x) {
  return from_bits64(bits64(x) ^ (long long)0x8000000000000000ull);
}
__device__ __forceinline__ double absF(double x) {
  return from_bits64(bits64(x) & 0x7FFFFFFFFFFFFFFFll);
}
__device__ __forceinline__ double signF(double a, double b) {
  return from_bits64((bits64(a) & 0x7FFFFFFFFFFFFFFFll) | (bits64(b) & (long long)0x8000000000000000ull));
}

// ------------------------------------------------------------ comparisons

// Order key: monotone in the value over non-NaN doubles, with -0 and +0 both
// mapped to 0 (for negative x the key is minus the magnitude bits).
__device__ __forceinline__ long long okey(double x) {
  const long long i = bits64(x);
  return i < 0 ? (LLONG_MIN - i) : i;
}
__device__ __forceinline__ bool nanF(double x) {
  return ((unsigned long long)bits64(x) & 0x7FFFFFFFFFFFFFFFull) >
         0x7FF0000000000000ull;
}
// IEEE a > b, a >= b (false when either is NaN)
__device__ __forceinline__ bool gtF(double a, double b) {
  return okey(a) > okey(b) && !nanF(a) && !nanF(b);
}
__device__ __forceinline__ bool geF(double a, double b) {
  return okey(a) >= okey(b) && !nanF(a) && !nanF(b);
}
// IEEE a > b when b's sign bit is clear (b in +0..+inf or a positive NaN),
// for any a: a sign-bit-set a is then never above b, and the plain integer
// order of sign-clear patterns is the value order with NaNs at the top.
__device__ __forceinline__ bool gt_nn(double a, double b) {
  const long long ia = bits64(a), ib = bits64(b);
  return ia > ib && ia <= 0x7FF0000000000000ll;
}
// IEEE a <= b when a's sign bit is clear, for any b
__device__ __forceinline__ bool le_nn(double a, double b) {
  const long long ia = bits64(a);
  return ia <= okey(b) && ia <= 0x7FF0000000000000ll && !nanF(b);
}

}  // namespace bl

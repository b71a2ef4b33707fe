// bl_lreal.cuh -- the type of the limiter and edge-viscosity arithmetic,
// and FP32 versions of the helpers it uses.
//
// The fast and exact builds evaluate everything in FP64 (lr = double; the
// helpers resolve to bl_fp64.cuh's).  The mixed build (BL_MIXED, the
// demoted batched form) evaluates the edge viscosity's limiter ratios,
// edge coefficients and edge forces, the CFL lengths and the divergence
// in FP32 (lr = float) on the FP32 pipe, 64 times the FP64 issue rate on
// GB300; positions, the geometry and its volume cancellation, the
// pressure forces, the energy update and the dt reduction stay FP64.  The
// FP32 helpers below keep the FP64 helpers' names, so that one source
// serves both types by overload.
#pragma once
#include <cfloat>
#include <cmath>

#include "bl_fp64.cuh"

#ifndef BL_MIXED
#define BL_MIXED 0
#endif

namespace bl {

#if BL_MIXED
using lr = float;
#else
using lr = double;
#endif

// FP32: IEEE divide and square root (the FP32 pipe), and the scalings,
// sign-bit operations and comparisons of bl_fp64.cuh with the same
// semantics (MAX/MIN keep the first argument on ties and NaN).
static __device__ __forceinline__ float ddiv_call(float a, float b) { return a / b; }
static __device__ __forceinline__ float dsqrt_call(float x) { return sqrtf(x); }
static __device__ __forceinline__ float ddiv_rn(float a, float b) { return a / b; }
static __device__ __forceinline__ float dsqrt_rn(float x) { return sqrtf(x); }
__device__ __forceinline__ float half(float x) { return 0.5f * x; }
__device__ __forceinline__ float quarter(float x) { return 0.25f * x; }
__device__ __forceinline__ float twice(float x) { return 2.0f * x; }
__device__ __forceinline__ float times4(float x) { return 4.0f * x; }
__device__ __forceinline__ float negF(float x) { return __int_as_float(__float_as_int(x) ^ 0x80000000); }
__device__ __forceinline__ float absF(float x) { return fabsf(x); }
__device__ __forceinline__ float signF(float a, float b) { return copysignf(a, b); }
__device__ __forceinline__ bool gtF(float a, float b) { return a > b; }
__device__ __forceinline__ bool geF(float a, float b) { return a >= b; }
__device__ __forceinline__ bool gt_nn(float a, float b) { return a > b; }
__device__ __forceinline__ bool le_nn(float a, float b) { return a <= b; }
__device__ __forceinline__ float maxF(float a, float b) { return b > a ? b : a; }
__device__ __forceinline__ float minF(float a, float b) { return a > b ? b : a; }
__device__ __forceinline__ float maxF_nn(float a, float b) { return b > a ? b : a; }
__device__ __forceinline__ float minF_nn(float a, float b) { return a > b ? b : a; }

// a with its sign flipped where s is negative (sign bit of s), and -a
// likewise
__device__ __forceinline__ double xorsign(double a, double s) {
  return from_bits64(bits64(a) ^ (bits64(s) & (long long)0x8000000000000000ull));
}
__device__ __forceinline__ double negxorsign(double a, double s) {
  return from_bits64(bits64(a) ^ (long long)0x8000000000000000ull ^
                     (bits64(s) & (long long)0x8000000000000000ull));
}
__device__ __forceinline__ float xorsign(float a, float s) {
  return __int_as_float(__float_as_int(a) ^ (__float_as_int(s) & 0x80000000));
}
__device__ __forceinline__ float negxorsign(float a, float s) {
  return __int_as_float(__float_as_int(a) ^ 0x80000000 ^ (__float_as_int(s) & 0x80000000));
}

// FP64 <-> FP32 on the integer pipe, with a power-of-two scaling folded
// into the exponent: f32_of(x, k) is x * 2^k truncated to FP32 (its
// leading 24 significant bits), zero where that falls below FP32's normal
// range and infinite above it; f64_of(f, k) is f * 2^k exactly for a
// normal f (zero for zero or subnormal f).  The FP64 unit, 1/64 of the
// FP32 rate on GB300, is not used.
__device__ __forceinline__ float f32_of(double x, int k) {
  const long long b = bits64(x);
  const unsigned sign = (unsigned)((unsigned long long)b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7ff);
  const int fe = e - 1023 + 127 + k;
  const unsigned m = (unsigned)((unsigned long long)b >> 29) & 0x7fffffu;
  if (e == 0 || fe <= 0) return __int_as_float((int)sign);
  if (fe >= 255) return __int_as_float((int)(sign | 0x7f800000u));
  return __int_as_float((int)(sign | ((unsigned)fe << 23) | m));
}
__device__ __forceinline__ double f64_of(float f, int k) {
  const unsigned b = (unsigned)__float_as_int(f);
  const long long sign = (long long)(b & 0x80000000u) << 32;
  const int fe = (int)((b >> 23) & 0xff);
  if (fe == 0) return from_bits64(sign);
  int e = fe == 255 ? 0x7ff : fe - 127 + 1023 + k;
  if (fe != 255 && e <= 0) return from_bits64(sign);
  if (fe != 255 && e >= 0x7ff) return from_bits64(sign | 0x7ff0000000000000ll);
  return from_bits64(sign | ((long long)e << 52) | ((long long)(b & 0x7fffffu) << 29));
}
// an FP64 value as an lr (FP32: f32_of), and back
__device__ __forceinline__ lr to_lr(double x) {
#if BL_MIXED
  return f32_of(x, 0);
#else
  return x;
#endif
}
__device__ __forceinline__ double from_lr(lr x) {
#if BL_MIXED
  return f64_of(x, 0);
#else
  return x;
#endif
}

// the cut-off zerocut as an lr: FP32 has no 1e-40, so the smallest
// normal FP32 stands in for cut-offs below it
__device__ __forceinline__ lr lr_cut(double zc) {
#if BL_MIXED
  return zc < (double)FLT_MIN ? FLT_MIN : (float)zc;
#else
  return zc;
#endif
}

}  // namespace bl

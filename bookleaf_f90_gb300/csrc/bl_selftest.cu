// bl_selftest.cu -- on-device check of the integer-pipe FP64 arithmetic
// (bl_fp64.cuh) against the hardware operations, bit for bit.
//
// bl_selftest_fp64(op, n, seed, &mismatches, &first_a, &first_b) draws n
// operand pairs from a counter-based generator (splitmix64 of seed and the
// index), mixes in hand-picked hard cases (all-ones and all-zeros
// significands, ratios next to 1, exponent-range edges, zeros, infinities,
// NaNs, subnormals of every width) and counts results that differ from the hardware in any
// bit (two NaNs compare equal).  op 0 is the divide, op 1 the square root
// (its operand is the first of the pair; for op 1 the second reports 0),
// op 2 the multiply (one pair in four with significands of 28 and 27 bits,
// whose 54- and 55-bit products round from exact ties).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "../../include/bookleaf_gb300.h"
#include "bl_fp64.cuh"

namespace {

__device__ __forceinline__ uint64_t splitmix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__device__ double pick(uint64_t r, uint64_t r2) {
  const uint64_t M52 = (1ull << 52) - 1;
  const int kind = (int)(r2 & 15);
  uint64_t sign = (r2 >> 8) & 1ull;
  uint64_t mant = r & M52;
  int e;
  switch (kind) {
    case 0: mant = M52; break;                          // all ones
    case 1: mant = 0; break;                            // power of two
    case 2: mant = M52 - (r2 >> 20 & 0xFF); break;      // just below 2
    case 3: mant = (r2 >> 20) & 0xFF; break;            // just above 1
    default: break;
  }
  const int ek = (int)((r2 >> 4) & 15);
  if (ek < 10) e = 1023 + (int)((r >> 52) & 127) - 64;        // moderate range
  else if (ek < 13) e = (int)((r >> 52) & 0x7FF);             // anything, incl. 0/2047
  else if (ek < 14) e = 1 + (int)((r2 >> 30) & 3);            // bottom of the range
  else if (ek < 15) e = 2046 - (int)((r2 >> 30) & 3);         // top of the range
  else e = 1023;
  if (e < 0) e = 0;
  if (e > 2047) e = 2047;
  if (kind == 4) {  // subnormal, with a significand of 1..52 bits
    e = 0;
    mant = (r & M52) >> ((r2 >> 40) % 52);
    if (mant == 0) mant = 1;
  }
  return __longlong_as_double((long long)((sign << 63) | ((uint64_t)e << 52) | mant));
}

__global__ void k_selftest(int op, long long n, unsigned long long seed,
                           unsigned long long* bad, unsigned long long* first) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t r1 = splitmix(seed ^ (2 * (uint64_t)i));
    const uint64_t r2 = splitmix(r1 + 0x1234567ull);
    const uint64_t r3 = splitmix(r2);
    const uint64_t r4 = splitmix(r3);
    double a = pick(r1, r2), b = pick(r3, r4);
    double h, s;
    if (op == 0) {
      if ((r4 >> 60) == 0) a = b * __longlong_as_double((long long)(0x3FF0000000000000ull | (r1 & 0xF)));
      h = a / b;
      s = bl::ddiv_rn(a, b);
    } else if (op == 2) {
      if (((r4 >> 58) & 3) == 0) {
        a = __longlong_as_double(__double_as_longlong(a) & ~((1ll << 25) - 1));
        b = __longlong_as_double(__double_as_longlong(b) & ~((1ll << 26) - 1));
      }
      h = a * b;
      s = bl::dmul_rn(a, b);
    } else {
      // squares of doubles and their neighbours, and integers next to squares
      const int kind = (int)((r4 >> 56) & 7);
      if (kind == 0) a = fabs(b) * fabs(b);
      if (kind == 1) a = __longlong_as_double(__double_as_longlong(fabs(b) * fabs(b)) + (long long)((r4 >> 8) % 5) - 2);
      if (kind == 2) {
        const double t = (double)(r3 & ((1ull << 26) - 1));
        a = t * t + (((r4 >> 3) & 1) ? 0.5 : -0.5);
      }
      b = 0.0;
      h = sqrt(a);
      s = bl::dsqrt_rn(a);
    }
    const uint64_t hb = (uint64_t)__double_as_longlong(h), sb = (uint64_t)__double_as_longlong(s);
    const bool same = (hb == sb) || (h != h && s != s);
    if (!same) {
      if (atomicAdd(bad, 1ull) == 0) {
        first[0] = (unsigned long long)__double_as_longlong(a);
        first[1] = (unsigned long long)__double_as_longlong(b);
      }
    }
  }
}

}  // namespace

extern "C" int bl_selftest_fp64(int op, long long n, unsigned long long seed,
                                long long* mismatches, double* first_a, double* first_b) {
  if (op < 0 || op > 2 || n < 0 || !mismatches) return BL_FAILURE;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 3 * sizeof(unsigned long long)) != cudaSuccess) return BL_FAILURE;
  cudaMemset(d, 0, 3 * sizeof(unsigned long long));
  k_selftest<<<152 * 8, 256>>>(op, n, seed, d, d + 1);
  unsigned long long h[3] = {0, 0, 0};
  cudaError_t r = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (r != cudaSuccess) return BL_FAILURE;
  *mismatches = (long long)h[0];
  if (first_a) {
    long long t = (long long)h[1];
    std::memcpy(first_a, &t, 8);
  }
  if (first_b) {
    long long t = (long long)h[2];
    std::memcpy(first_b, &t, 8);
  }
  return BL_SUCCESS;
}

// ------------------------------------------------------------------ rates
// Issue-rate probe of the FP64 operations the hot path is made of: each
// thread runs independent dependency chains (enough to cover the pipe
// latency) and writes one double, so the time is the pipe's throughput.
namespace {

constexpr int kRateBlocks = 152 * 8, kRateThreads = 256;

__global__ void k_rate_dfma(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4,
         x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <int OP>
__global__ void k_rate_op(double* out, int iters, double a) {
  double x0 = 1.5 + threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  for (int i = 0; i < iters; i++) {
    if (OP == 0) { x0 = a / x0 + 1.0; x1 = a / x1 + 1.0; x2 = a / x2 + 1.0; x3 = a / x3 + 1.0; }
    if (OP == 1) {
      x0 = bl::ddiv_rn(a, x0) + 1.0; x1 = bl::ddiv_rn(a, x1) + 1.0;
      x2 = bl::ddiv_rn(a, x2) + 1.0; x3 = bl::ddiv_rn(a, x3) + 1.0;
    }
    if (OP == 2) { x0 = sqrt(x0) + 1.0; x1 = sqrt(x1) + 1.0; x2 = sqrt(x2) + 1.0; x3 = sqrt(x3) + 1.0; }
    if (OP == 3) {
      x0 = bl::dsqrt_rn(x0) + 1.0; x1 = bl::dsqrt_rn(x1) + 1.0;
      x2 = bl::dsqrt_rn(x2) + 1.0; x3 = bl::dsqrt_rn(x3) + 1.0;
    }
    if (OP == 4) { x0 = x0 * a; x1 = x1 * a; x2 = x2 * a; x3 = x3 * a; }
    if (OP == 5) {
      x0 = bl::dmul_rn(x0, a); x1 = bl::dmul_rn(x1, a);
      x2 = bl::dmul_rn(x2, a); x3 = bl::dmul_rn(x3, a);
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}

}  // namespace

extern "C" int bl_fp64_rates(double* rates, int n) {
  if (!rates || n < 5) return BL_FAILURE;
  const int total = kRateBlocks * kRateThreads;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * total) != cudaSuccess) return BL_FAILURE;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float ms = 0.f;
  int rc = BL_SUCCESS;
  const int nrates = n >= 7 ? 7 : 5;
  for (int which = 0; which < nrates && rc == BL_SUCCESS; which++) {
    const int iters = which == 0 ? 1024 : 128;
    const double ops = (which == 0 ? 8.0 : 4.0) * iters * (double)total;
    for (int rep = 0; rep < 2; rep++) {  // first pass warms up
      cudaEventRecord(e0);
      switch (which) {
        case 0: k_rate_dfma<<<kRateBlocks, kRateThreads>>>(d, iters, 0.999999, 1e-7); break;
        case 1: k_rate_op<0><<<kRateBlocks, kRateThreads>>>(d, iters, 3.0); break;
        case 2: k_rate_op<1><<<kRateBlocks, kRateThreads>>>(d, iters, 3.0); break;
        case 3: k_rate_op<2><<<kRateBlocks, kRateThreads>>>(d, iters, 0.0); break;
        case 4: k_rate_op<3><<<kRateBlocks, kRateThreads>>>(d, iters, 0.0); break;
        case 5: k_rate_op<4><<<kRateBlocks, kRateThreads>>>(d, iters, 0.9999999); break;
        default: k_rate_op<5><<<kRateBlocks, kRateThreads>>>(d, iters, 0.9999999); break;
      }
      cudaEventRecord(e1);
      if (cudaEventSynchronize(e1) != cudaSuccess) { rc = BL_FAILURE; break; }
      cudaEventElapsedTime(&ms, e0, e1);
    }
    rates[which] = ops / (ms * 1e-3) / 1e9;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (cudaGetLastError() != cudaSuccess) rc = BL_FAILURE;
  return rc;
}

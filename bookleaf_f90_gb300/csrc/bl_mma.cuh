// bl_mma.cuh -- the closure network's building blocks on the tensor cores,
// shared by its training kernels (bl_mlp.cu) and the solver's closure
// kernel (hydro_kernels.cuh): the parameter layout, 16x8x16 BF16 tile
// products (mma.sync m16n8k16, FP32 accumulation) with their fragment
// layouts, and the forward pass of 16 samples per warp.
//
// Fragments of a 16x16 A tile and a 16x8 B tile are read through accessors
// a(row, col) and b(k, n); the accumulator element c[i] of a lane is at row
// g + 8*(i/2), column 2t + (i%2) (g = lane/4, t = lane%4), as the PTX ISA
// defines the m16n8k16 layouts.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "../../include/bookleaf_gb300.h"

namespace bl {
namespace mlp {

constexpr int NI = BL_MLP_IN, NH = BL_MLP_HIDDEN, NO = BL_MLP_OUT;
// parameter layout: W1[NH][NI], b1[NH], W2[NH][NH], b2[NH], W3[NO][NH], b3[NO]
constexpr int OW1 = 0, OB1 = OW1 + NH * NI, OW2 = OB1 + NH, OB2 = OW2 + NH * NH,
              OW3 = OB2 + NH, OB3 = OW3 + NO * NH, NP = OB3 + NO;
static_assert(NP == BL_MLP_NPARAM, "parameter count");
constexpr int WARPS = 4, TPB = 32 * WARPS, SPB = 16 * WARPS;  // samples per block

__device__ __forceinline__ uint32_t pack(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  uint32_t u;
  memcpy(&u, &v, 4);
  return u;
}

// D = A(16x16, row) * B(16x8, col) + D, BF16 operands, FP32 accumulators
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Fragments of a 16x16 A tile and a 16x8 B tile read through accessors
// a(row, col) and b(k, n); the accumulator element c[i] of a lane is at row
// g + 8*(i/2), column 2t + (i%2) (g = lane/4, t = lane%4).
template <class FA>
__device__ __forceinline__ void frag_a(uint32_t (&r)[4], FA a) {
  const int l = threadIdx.x & 31, g = l >> 2, t = l & 3;
  r[0] = pack(a(g, 2 * t), a(g, 2 * t + 1));
  r[1] = pack(a(g + 8, 2 * t), a(g + 8, 2 * t + 1));
  r[2] = pack(a(g, 2 * t + 8), a(g, 2 * t + 9));
  r[3] = pack(a(g + 8, 2 * t + 8), a(g + 8, 2 * t + 9));
}
template <class FB>
__device__ __forceinline__ void frag_b(uint32_t (&r)[2], FB b) {
  const int l = threadIdx.x & 31, g = l >> 2, t = l & 3;
  r[0] = pack(b(2 * t, g), b(2 * t + 1, g));
  r[1] = pack(b(2 * t + 8, g), b(2 * t + 9, g));
}
template <class FS>
__device__ __forceinline__ void store_c(const float (&c)[4], FS s) {
  const int l = threadIdx.x & 31, g = l >> 2, t = l & 3;
  s(g, 2 * t, c[0]);
  s(g, 2 * t + 1, c[1]);
  s(g + 8, 2 * t, c[2]);
  s(g + 8, 2 * t + 1, c[3]);
}

// the logistic function with the fast single-precision divide: its error of
// a few ulp is far below the BF16 rounding every activation goes through,
// and for z below about -87 it gives the limit 0
__device__ __forceinline__ float sigm(float z) { return __fdividef(1.0f, 1.0f + __expf(-z)); }

// The parameters in shared memory, zero-padded to whole tiles: W1 as 64x16,
// W3 as 16x64.
struct SmemW {
  float w1[NH][16], b1[NH], w2[NH][NH], b2[NH], w3[16][NH], b3[16];
};
// The image of SmemW in global memory: the offset of parameter i in it
// (the padding stays zero).  Kernels copy the image with 16-byte loads, all
// issued before the first store, instead of gathering and padding the
// parameters one by one.
constexpr int kImgB1 = NH * 16, kImgW2 = kImgB1 + NH, kImgB2 = kImgW2 + NH * NH,
              kImgW3 = kImgB2 + NH, kImgB3 = kImgW3 + 16 * NH, kImgN = kImgB3 + 16;
static_assert(kImgN * sizeof(float) == sizeof(SmemW) && sizeof(SmemW) % 16 == 0, "image");
__host__ __device__ constexpr int image_offset(int i) {
  return i < OB1   ? (i / NI) * 16 + i % NI
         : i < OW2 ? kImgB1 + (i - OB1)
         : i < OB2 ? kImgW2 + (i - OW2)
         : i < OW3 ? kImgB2 + (i - OB2)
         : i < OB3 ? kImgW3 + (i - OW3)
                   : kImgB3 + (i - OB3);
}
template <int NT>
__device__ __forceinline__ void copy_weights(SmemW& w, const float* img) {
  constexpr int N4 = kImgN / 4, K = (N4 + NT - 1) / NT;
  const float4* src = reinterpret_cast<const float4*>(img);
  float4* dst = reinterpret_cast<float4*>(&w);
  float4 r[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    const int i = threadIdx.x + k * NT;
    if (i < N4) r[k] = __ldg(src + i);
  }
#pragma unroll
  for (int k = 0; k < K; k++) {
    const int i = threadIdx.x + k * NT;
    if (i < N4) dst[i] = r[k];
  }
}

// One warp's 16 samples: x (16x16, padded), pre-activations and activations
struct SmemS {
  float x[16][16], z1[16][NH], h1[16][NH], z2[16][NH], h2[16][NH], y[16][16];
};

// Forward pass of a warp's samples (rows of s.x) into s.z1 ... s.y
static __device__ void forward_warp(const SmemW& w, SmemS& s) {
  // layer 1: z1 = x W1^T + b1 (K = 16 padded inputs, N = 64)
  uint32_t a[4];
  frag_a(a, [&](int r, int c) { return s.x[r][c]; });
#pragma unroll
  for (int nt = 0; nt < NH / 8; nt++) {
    float d[4] = {0, 0, 0, 0};
    uint32_t b[2];
    frag_b(b, [&](int k, int n) { return w.w1[nt * 8 + n][k]; });
    mma16816(d, a, b);
    // the activation straight from the accumulators (z kept for the backward pass)
    store_c(d, [&](int r, int c, float v) {
      const float z = v + w.b1[nt * 8 + c];
      s.z1[r][nt * 8 + c] = z;
      s.h1[r][nt * 8 + c] = z * sigm(z);
    });
  }
  __syncwarp();
  // layer 2: z2 = h1 W2^T + b2 (K = 64, N = 64)
#pragma unroll
  for (int nt = 0; nt < NH / 8; nt++) {
    float d[4] = {0, 0, 0, 0};
#pragma unroll
    for (int kt = 0; kt < NH / 16; kt++) {
      frag_a(a, [&](int r, int c) { return s.h1[r][kt * 16 + c]; });
      uint32_t b[2];
      frag_b(b, [&](int k, int n) { return w.w2[nt * 8 + n][kt * 16 + k]; });
      mma16816(d, a, b);
    }
    store_c(d, [&](int r, int c, float v) {
      const float z = v + w.b2[nt * 8 + c];
      s.z2[r][nt * 8 + c] = z;
      s.h2[r][nt * 8 + c] = z * sigm(z);
    });
  }
  __syncwarp();
  // layer 3: y = h2 W3^T + b3 (K = 64, N = 8 of which NO used)
  float d[4] = {0, 0, 0, 0};
#pragma unroll
  for (int kt = 0; kt < NH / 16; kt++) {
    frag_a(a, [&](int r, int c) { return s.h2[r][kt * 16 + c]; });
    uint32_t b[2];
    frag_b(b, [&](int k, int n) { return w.w3[n][kt * 16 + k]; });
    mma16816(d, a, b);
  }
  store_c(d, [&](int r, int c, float v) { s.y[r][c] = v + w.b3[c]; });
  __syncwarp();
}

}  // namespace mlp
}  // namespace bl

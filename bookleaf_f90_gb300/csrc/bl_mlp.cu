// bl_mlp.cu -- the learned mixed-cell closure's network: 10 inputs, two
// hidden layers of 64 with SiLU, 2 outputs, trained and evaluated on the
// tensor cores (BF16 operands, FP32 accumulation) by the kernels below.
//
//   z1 = W1 x + b1, h1 = silu(z1), z2 = W2 h1 + b2, h2 = silu(z2),
//   y = W3 h2 + b3,  loss = sum over samples and outputs of (y - t)^2 / (2 n)
//
// Every product of the forward and backward passes is a 16x8x16 tile
// product (mma.sync m16n8k16, BF16 x BF16 -> FP32) of 16 samples per warp:
// the activations and weights are rounded to BF16 where they enter a
// product, everything else (biases, SiLU, sums, Adam) stays FP32.  The
// weight gradients of a block of 64 samples are summed on the tensor cores
// too (the sample dimension is the product's k), then over blocks in a
// fixed order, so training is deterministic.  Parameters are FP32 master
// copies in one array (layout below); no CPU path exists.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/bookleaf_gb300.h"
#include "bl_mma.cuh"

namespace {

using namespace bl::mlp;

__device__ void load_x(SmemS& s, const float* X, int base, int n) {
  for (int i = threadIdx.x & 31; i < 16 * 16; i += 32) {
    const int r = i / 16, c = i % 16, row = base + r;
    s.x[r][c] = (c < NI && row < n) ? X[(size_t)row * NI + c] : 0.0f;
  }
  __syncwarp();
}

__global__ void __launch_bounds__(TPB) k_mlp_forward(const float* img, const float* X, float* Y,
                                                     int n) {
  extern __shared__ unsigned char smem[];
  SmemW& w = *reinterpret_cast<SmemW*>(smem);
  SmemS* S = reinterpret_cast<SmemS*>(smem + sizeof(SmemW));
  copy_weights<TPB>(w, img);
  __syncthreads();
  const int warp = threadIdx.x >> 5;
  SmemS& s = S[warp];
  const int base = blockIdx.x * SPB + warp * 16;
  load_x(s, X, base, n);
  forward_warp(w, s);
  for (int i = threadIdx.x & 31; i < 16 * NO; i += 32) {
    const int r = i / NO, c = i % NO;
    if (base + r < n) Y[(size_t)(base + r) * NO + c] = s.y[r][c];
  }
}

// Forward and backward of one block's 64 samples; the block's gradient sum
// and loss sum go to G[blockIdx][NP] and L[blockIdx].
__global__ void __launch_bounds__(TPB) k_mlp_grad(const float* img, const float* X, const float* T,
                                                  const int* idx, int n, float inv_n, float* G,
                                                  float* L) {
  extern __shared__ unsigned char smem[];
  SmemW& w = *reinterpret_cast<SmemW*>(smem);
  SmemS* S = reinterpret_cast<SmemS*>(smem + sizeof(SmemW));
  // per block: dz1, dz2 (64 samples x 64), dy (64 x 16), gathered x (64 x 16)
  float(*dz1)[NH] = reinterpret_cast<float(*)[NH]>(smem + sizeof(SmemW) + WARPS * sizeof(SmemS));
  float(*dz2)[NH] = dz1 + SPB;
  float(*dy)[16] = reinterpret_cast<float(*)[16]>(dz2 + SPB);
  float* lsum = reinterpret_cast<float*>(dy + SPB);
  copy_weights<TPB>(w, img);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x < WARPS) lsum[threadIdx.x] = 0.0f;
  __syncthreads();
  SmemS& s = S[warp];
  const int base = blockIdx.x * SPB + warp * 16;
  // the samples of this warp (through the permutation idx, if given)
  for (int i = lane; i < 16 * 16; i += 32) {
    const int r = i / 16, c = i % 16, row = base + r;
    const int src = row < n ? (idx ? idx[row] : row) : -1;
    s.x[r][c] = (c < NI && src >= 0) ? X[(size_t)src * NI + c] : 0.0f;
  }
  __syncwarp();
  forward_warp(w, s);
  // dy = (y - t) / n for valid samples; loss terms
  float lp = 0.0f;
  for (int i = lane; i < 16 * 16; i += 32) {
    const int r = i / 16, c = i % 16, row = base + r;
    float g = 0.0f;
    if (c < NO && row < n) {
      const int src = idx ? idx[row] : row;
      const float e = s.y[r][c] - T[(size_t)src * NO + c];
      lp += e * e;
      g = e * inv_n;
    }
    dy[warp * 16 + r][c] = g;
  }
  for (int o = 16; o > 0; o >>= 1) lp += __shfl_xor_sync(0xffffffffu, lp, o);
  if (lane == 0) lsum[warp] = lp;
  __syncwarp();
  const int row0 = warp * 16;
  // dh2 = dy W3 (K = 16 padded outputs, N = 64); dz2 = dh2 silu'(z2)
  uint32_t a[4];
  frag_a(a, [&](int r, int c) { return dy[row0 + r][c]; });
#pragma unroll
  for (int nt = 0; nt < NH / 8; nt++) {
    float d[4] = {0, 0, 0, 0};
    uint32_t b[2];
    frag_b(b, [&](int k, int nn) { return w.w3[k][nt * 8 + nn]; });
    mma16816(d, a, b);
    store_c(d, [&](int r, int c, float v) {
      const float z = s.z2[r][nt * 8 + c], sg = sigm(z);
      dz2[row0 + r][nt * 8 + c] = v * sg * (1.0f + z * (1.0f - sg));
    });
  }
  __syncwarp();
  // dh1 = dz2 W2 (K = 64, N = 64); dz1 = dh1 silu'(z1)
#pragma unroll
  for (int nt = 0; nt < NH / 8; nt++) {
    float d[4] = {0, 0, 0, 0};
#pragma unroll
    for (int kt = 0; kt < NH / 16; kt++) {
      frag_a(a, [&](int r, int c) { return dz2[row0 + r][kt * 16 + c]; });
      uint32_t b[2];
      frag_b(b, [&](int k, int nn) { return w.w2[kt * 16 + k][nt * 8 + nn]; });
      mma16816(d, a, b);
    }
    store_c(d, [&](int r, int c, float v) {
      const float z = s.z1[r][nt * 8 + c], sg = sigm(z);
      dz1[row0 + r][nt * 8 + c] = v * sg * (1.0f + z * (1.0f - sg));
    });
  }
  __syncthreads();
  // Weight gradients summed over the block's 64 samples (the k of the
  // products): dW = dZ^T A with A the layer's input activations.  Warp w
  // takes the output rows [16w, 16w + 16) of dW1 and dW2 and, for dW3, the
  // columns [16w, 16w + 16).
  float* Gb = G + (size_t)blockIdx.x * NP;
  // dW2[o][i] = sum_s dz2[s][o] h1[s][i]; dW1[o][i] = sum_s dz1[s][o] x[s][i]
  for (int layer = 0; layer < 2; layer++) {
    const int ncols = layer == 0 ? NH : 16;
    for (int nt = 0; nt < ncols / 8; nt++) {
      float d[4] = {0, 0, 0, 0};
      for (int kt = 0; kt < SPB / 16; kt++) {   // 16 samples of warp kt
        SmemS& sk = S[kt];
        frag_a(a, [&](int r, int c) {
          return layer == 0 ? dz2[kt * 16 + c][warp * 16 + r] : dz1[kt * 16 + c][warp * 16 + r];
        });
        uint32_t b[2];
        frag_b(b, [&](int k, int nn) {
          return layer == 0 ? sk.h1[k][nt * 8 + nn] : sk.x[k][nt * 8 + nn];
        });
        mma16816(d, a, b);
      }
      store_c(d, [&](int r, int c, float v) {
        const int o = warp * 16 + r, i = nt * 8 + c;
        if (layer == 0) Gb[OW2 + o * NH + i] = v;
        else if (i < NI) Gb[OW1 + o * NI + i] = v;
      });
    }
  }
  // dW3[o][i] = sum_s dy[s][o] h2[s][i] (o < NO of 16 padded rows)
  for (int nt = 0; nt < 2; nt++) {
    float d[4] = {0, 0, 0, 0};
    for (int kt = 0; kt < SPB / 16; kt++) {
      SmemS& sk = S[kt];
      frag_a(a, [&](int r, int c) { return dy[kt * 16 + c][r]; });
      uint32_t b[2];
      frag_b(b, [&](int k, int nn) { return sk.h2[k][warp * 16 + nt * 8 + nn]; });
      mma16816(d, a, b);
    }
    store_c(d, [&](int r, int c, float v) {
      if (r < NO) Gb[OW3 + r * NH + warp * 16 + nt * 8 + c] = v;
    });
  }
  // bias gradients: column sums over the block's samples (FP32)
  for (int i = threadIdx.x; i < NH; i += blockDim.x) {
    float g1 = 0.0f, g2 = 0.0f;
    for (int r = 0; r < SPB; r++) {
      g1 += dz1[r][i];
      g2 += dz2[r][i];
    }
    Gb[OB1 + i] = g1;
    Gb[OB2 + i] = g2;
  }
  if (threadIdx.x < NO) {
    float g3 = 0.0f;
    for (int r = 0; r < SPB; r++) g3 += dy[r][threadIdx.x];
    Gb[OB3 + threadIdx.x] = g3;
  }
  __syncthreads();
  if (threadIdx.x == 0) L[blockIdx.x] = 0.5f * inv_n * (lsum[0] + lsum[1] + lsum[2] + lsum[3]);
}

// Sums the per-block gradients and losses in block order; the loss times
// wgt is also added to *acc (an epoch's running sum), in launch order.
__global__ void k_mlp_reduce(const float* G, const float* L, int nblk, float* grad, float* loss,
                             double* acc, double wgt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NP) {
    float s = 0.0f;
    for (int b = 0; b < nblk; b++) s += G[(size_t)b * NP + i];
    grad[i] = s;
  }
  if (i == 0) {
    float s = 0.0f;
    for (int b = 0; b < nblk; b++) s += L[b];
    *loss = s;
    if (acc) *acc += (double)s * wgt;
  }
}

// The parameters' shared-memory image (its padding is zeroed once).
__global__ void k_mlp_image(const float* P, float* img) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NP) img[image_offset(i)] = P[i];
}

// Adam on the FP32 master parameters (Kingma and Ba, 2015).
// The image is kept current with the parameters.
// Adam; the bias corrections of this update are entry *ebase + k of the
// tables c1t, c2t (the mini-batch k of an epoch whose first update is
// *ebase), so that one captured epoch replays with the next epoch's values
__global__ void k_mlp_adam(float* P, float* M, float* V, float* img, const float* grad, float lr,
                           float b1, float b2, float eps, const float* c1t, const float* c2t,
                           const int* ebase, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NP) return;
  const float c1 = c1t[*ebase + k], c2 = c2t[*ebase + k];
  const float g = grad[i];
  const float m = b1 * M[i] + (1.0f - b1) * g, v = b2 * V[i] + (1.0f - b2) * g * g;
  M[i] = m;
  V[i] = v;
  const float p = P[i] - lr * (m * c1) / (sqrtf(v * c2) + eps);
  P[i] = p;
  img[image_offset(i)] = p;
}

constexpr size_t kSmemFwd = sizeof(SmemW) + WARPS * sizeof(SmemS);
constexpr size_t kSmemGrad = kSmemFwd + (2 * SPB * NH + SPB * 16 + WARPS) * sizeof(float);

}  // namespace

struct bl_mlp {
  float *P = nullptr, *M = nullptr, *V = nullptr, *grad = nullptr, *loss = nullptr;
  float* img = nullptr;  // SmemW image of P
  double* acc = nullptr;  // an epoch's loss sum
  int step = 0;
};

extern "C" {

int bl_mlp_create(bl_mlp** out, const float* params) {
  if (!out || !params) return BL_FAILURE;
  *out = nullptr;
  bl_mlp* m = new bl_mlp();
  bool ok = cudaMalloc(&m->P, NP * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->M, NP * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->V, NP * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->grad, NP * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->loss, sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->img, kImgN * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&m->acc, sizeof(double)) == cudaSuccess;
  ok = ok && cudaMemcpy(m->P, params, NP * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemset(m->M, 0, NP * sizeof(float)) == cudaSuccess &&
       cudaMemset(m->V, 0, NP * sizeof(float)) == cudaSuccess &&
       cudaMemset(m->img, 0, kImgN * sizeof(float)) == cudaSuccess;
  if (ok) {
    k_mlp_image<<<(NP + 255) / 256, 256>>>(m->P, m->img);
    ok = cudaDeviceSynchronize() == cudaSuccess;
  }
  ok = ok && cudaFuncSetAttribute(k_mlp_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kSmemFwd) == cudaSuccess &&
       cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                            (int)kSmemGrad) == cudaSuccess;
  if (!ok) {
    bl_mlp_destroy(m);
    return BL_FAILURE;
  }
  *out = m;
  return BL_SUCCESS;
}

int bl_mlp_destroy(bl_mlp* m) {
  if (!m) return BL_SUCCESS;
  cudaFree(m->P);
  cudaFree(m->M);
  cudaFree(m->V);
  cudaFree(m->grad);
  cudaFree(m->loss);
  cudaFree(m->img);
  cudaFree(m->acc);
  delete m;
  return BL_SUCCESS;
}

int bl_mlp_params(bl_mlp* m, float* params) {
  if (!m || !params) return BL_FAILURE;
  return cudaMemcpy(params, m->P, NP * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess
             ? BL_SUCCESS : BL_FAILURE;
}

// The device image of the current parameters (the layout the closure
// kernel copies into shared memory); bl_set_closure takes a copy.
const float* bl_mlp_device_image(bl_mlp* m) { return m ? m->img : nullptr; }

int bl_mlp_predict(bl_mlp* m, const float* x, int n, float* y) {
  if (!m || !x || !y || n < 0) return BL_FAILURE;
  if (n == 0) return BL_SUCCESS;
  float *dx = nullptr, *dy = nullptr;
  bool ok = cudaMalloc(&dx, (size_t)n * NI * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&dy, (size_t)n * NO * sizeof(float)) == cudaSuccess;
  ok = ok && cudaMemcpy(dx, x, (size_t)n * NI * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
  if (ok) {
    k_mlp_forward<<<(n + SPB - 1) / SPB, TPB, kSmemFwd>>>(m->img, dx, dy, n);
    ok = cudaMemcpy(y, dy, (size_t)n * NO * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  cudaFree(dx);
  cudaFree(dy);
  return ok ? BL_SUCCESS : BL_FAILURE;
}

int bl_mlp_gradient(bl_mlp* m, const float* x, const float* t, int n, float* grad, float* loss) {
  if (!m || !x || !t || !grad || n < 1) return BL_FAILURE;
  const int nblk = (n + SPB - 1) / SPB;
  float *dx = nullptr, *dt = nullptr, *G = nullptr, *L = nullptr;
  bool ok = cudaMalloc(&dx, (size_t)n * NI * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&dt, (size_t)n * NO * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&G, (size_t)nblk * NP * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&L, (size_t)nblk * sizeof(float)) == cudaSuccess;
  ok = ok && cudaMemcpy(dx, x, (size_t)n * NI * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(dt, t, (size_t)n * NO * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
  if (ok) {
    k_mlp_grad<<<nblk, TPB, kSmemGrad>>>(m->img, dx, dt, nullptr, n, 1.0f / (float)n, G, L);
    k_mlp_reduce<<<(NP + 255) / 256, 256>>>(G, L, nblk, m->grad, m->loss, nullptr, 0.0);
    ok = cudaMemcpy(grad, m->grad, NP * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess;
    if (ok && loss) ok = cudaMemcpy(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  cudaFree(dx);
  cudaFree(dt);
  cudaFree(G);
  cudaFree(L);
  return ok ? BL_SUCCESS : BL_FAILURE;
}

int bl_mlp_train(bl_mlp* m, const float* x, const float* t, int n, int epochs, int batch,
                 float lr, unsigned long long seed, float* losses) {
  if (!m || !x || !t || n < 1 || epochs < 1 || batch < SPB) return BL_FAILURE;
  const int nb_per = (batch + SPB - 1) / SPB;
  const int nbat = (n + batch - 1) / batch;  // mini-batches per epoch
  const long nupd = (long)epochs * nbat;
  float *dx = nullptr, *dt = nullptr, *G = nullptr, *L = nullptr, *c1t = nullptr, *c2t = nullptr;
  int *didx = nullptr, *ebase = nullptr;
  bool ok = cudaMalloc(&dx, (size_t)n * NI * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&dt, (size_t)n * NO * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&didx, (size_t)n * sizeof(int)) == cudaSuccess &&
            cudaMalloc(&G, (size_t)nb_per * NP * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&L, (size_t)nb_per * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&c1t, (size_t)nupd * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&c2t, (size_t)nupd * sizeof(float)) == cudaSuccess &&
            cudaMalloc(&ebase, sizeof(int)) == cudaSuccess;
  ok = ok && cudaMemcpy(dx, x, (size_t)n * NI * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(dt, t, (size_t)n * NO * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  // Adam's bias corrections for every update of the run (update u has step
  // count m->step + 1 + u)
  if (ok) {
    std::vector<float> c1(nupd), c2(nupd);
    for (long u = 0; u < nupd; u++) {
      const float st = (float)(m->step + 1 + u);
      c1[u] = 1.0f / (1.0f - powf(b1, st));
      c2[u] = 1.0f / (1.0f - powf(b2, st));
    }
    ok = cudaMemcpy(c1t, c1.data(), nupd * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(c2t, c2.data(), nupd * sizeof(float), cudaMemcpyHostToDevice) == cudaSuccess;
  }
  // one epoch's mini-batches (gradient, block sum, Adam for each) captured
  // once as a graph and replayed every epoch: the launches of a 256-sample
  // mini-batch take longer to issue than to run
  cudaStream_t cs = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ok = ok && cudaStreamCreate(&cs) == cudaSuccess &&
       cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  if (ok) {
    for (int k = 0; k < nbat; k++) {
      const int b0 = k * batch, nb = std::min(batch, n - b0);
      const int nblk = (nb + SPB - 1) / SPB;
      k_mlp_grad<<<nblk, TPB, kSmemGrad, cs>>>(m->img, dx, dt, didx + b0, nb, 1.0f / (float)nb, G, L);
      k_mlp_reduce<<<(NP + 255) / 256, 256, 0, cs>>>(G, L, nblk, m->grad, m->loss, m->acc, (double)nb);
      k_mlp_adam<<<(NP + 255) / 256, 256, 0, cs>>>(m->P, m->M, m->V, m->img, m->grad, lr, b1, b2,
                                                   eps, c1t, c2t, ebase, k);
    }
    ok = cudaStreamEndCapture(cs, &graph) == cudaSuccess &&
         cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
  }
  std::vector<int> perm(n);
  for (int i = 0; i < n; i++) perm[i] = i;
  uint64_t r = seed * 0x9E3779B97F4A7C15ull + 1;
  for (int ep = 0; ep < epochs && ok; ep++) {
    // Fisher-Yates shuffle with a splitmix-style generator
    for (int i = n - 1; i > 0; i--) {
      r += 0x9E3779B97F4A7C15ull;
      uint64_t z = r;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      z ^= z >> 31;
      const int j = (int)(z % (uint64_t)(i + 1));
      std::swap(perm[i], perm[j]);
    }
    const int eb = ep * nbat;
    double eloss = 0.0;
    ok = cudaMemcpyAsync(didx, perm.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice, cs) == cudaSuccess &&
         cudaMemcpyAsync(ebase, &eb, sizeof(int), cudaMemcpyHostToDevice, cs) == cudaSuccess &&
         cudaMemsetAsync(m->acc, 0, sizeof(double), cs) == cudaSuccess &&
         cudaGraphLaunch(exec, cs) == cudaSuccess &&
         cudaMemcpyAsync(&eloss, m->acc, sizeof(double), cudaMemcpyDeviceToHost, cs) == cudaSuccess &&
         cudaStreamSynchronize(cs) == cudaSuccess;
    if (losses) losses[ep] = (float)(eloss / n);
  }
  if (ok) m->step += (int)nupd;
  ok = ok && cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess;
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  if (cs) cudaStreamDestroy(cs);
  cudaFree(dx);
  cudaFree(dt);
  cudaFree(didx);
  cudaFree(G);
  cudaFree(L);
  cudaFree(c1t);
  cudaFree(c2t);
  cudaFree(ebase);
  return ok ? BL_SUCCESS : BL_FAILURE;
}

}  // extern "C"

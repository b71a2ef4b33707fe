// bl_setup.cuh -- the device half of bl_init: the connectivity's range
// checks and its conversion to 0-based indices, and the node -> corner
// tables of the nodal gathers.
//
// The host uploads the connectivity as the caller holds it (1-based,
// four entries per element); k_check_pack checks every range and converts
// in place, raising error bits that the host reads before anything indexes
// with the tables.  The node -> corner tables are a counting sort by node
// of a corner sequence: counts (atomics), an exclusive scan of the counts
// (the node offsets), a fill through per-node cursors (atomics, so the
// order within a node is arbitrary), then per node a sort of its corners
// by their position in the sequence, which makes the tables those of a
// stable sort: every node's corners in sequence order, the summation order
// of the reference's gathers.  Integer work only: the result does not
// depend on the order in which the atomics land.
#pragma once
#include <cuda_runtime.h>

namespace bl {
namespace setup {

// error bits, reported by bl_init in this order of precedence
enum : int { kBadConn = 1, kBadRegSort = 2, kBadPerm = 4, kBadMat = 8 };

constexpr int kThreads = 256;                     // every set-up kernel
constexpr int kScanV = 16;                        // scan values per thread
constexpr int kScanTile = kThreads * kScanV;      // scan values per block

inline int blocks_for(long n, int per) { return (int)((n + per - 1) / per); }

__device__ __forceinline__ bool in1(int v, int hi) { return (unsigned)(v - 1) < (unsigned)hi; }

// Element i: nodes nd and neighbours ee (1-based on entry, in place),
// neighbour faces fc4 (1-based, packed one byte per side into fc), region
// rg (in place), sort position srt (in place; seen[] counts each position
// to check that ielsort1 is a permutation), material mt (checked only:
// <= 0 marks a mixed cell).
__global__ void __launch_bounds__(kThreads)
    k_check_pack(int4* __restrict__ nd, int4* __restrict__ ee, const int4* __restrict__ fc4,
                 int* __restrict__ fc, int* __restrict__ rg, int* __restrict__ srt,
                 const int* __restrict__ mt, int* __restrict__ seen, int nel, int nnd,
                 int nreg, int nmat, int* __restrict__ bad) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  int b = 0;
  if (i < nel) {
    const int4 n = nd[i], e = ee[i], f = fc4[i];
    if (!(in1(n.x, nnd) && in1(n.y, nnd) && in1(n.z, nnd) && in1(n.w, nnd) && in1(e.x, nel) &&
          in1(e.y, nel) && in1(e.z, nel) && in1(e.w, nel) && in1(f.x, 4) && in1(f.y, 4) &&
          in1(f.z, 4) && in1(f.w, 4)))
      b |= kBadConn;
    const int r = rg[i], s = srt[i];
    if (!in1(r, nreg)) b |= kBadRegSort;
    if (!in1(s, nel)) {
      b |= kBadRegSort;
    } else if (atomicAdd(seen + (s - 1), 1) != 0) {
      b |= kBadPerm;
    }
    if (mt[i] > nmat) b |= kBadMat;
    nd[i] = make_int4(n.x - 1, n.y - 1, n.z - 1, n.w - 1);
    ee[i] = make_int4(e.x - 1, e.y - 1, e.z - 1, e.w - 1);
    fc[i] = (f.x - 1) | ((f.y - 1) << 8) | ((f.z - 1) << 16) | ((f.w - 1) << 24);
    rg[i] = r - 1;
    srt[i] = s - 1;
  }
  b = __reduce_or_sync(0xffffffffu, b);
  if (b && (threadIdx.x & 31) == 0) atomicOr(bad, b);
}

// corners per node (the same for every corner sequence of one mesh)
__global__ void __launch_bounds__(kThreads)
    k_count(const int4* __restrict__ nd, int nel, int nnd, int* __restrict__ cnt) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= nel) return;
  const int4 n = nd[i];
  const int c[4] = {n.x, n.y, n.z, n.w};
  for (int j = 0; j < 4; j++)
    if ((unsigned)c[j] < (unsigned)nnd) atomicAdd(cnt + c[j], 1);
}

// exclusive prefix of one value per thread over the block; *total = the
// block's sum
__device__ __forceinline__ int block_exclusive(int v, int* total) {
  __shared__ int ws[kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    int s = lane < kThreads / 32 ? ws[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kThreads / 32) ws[lane] = s;
  }
  __syncthreads();
  const int before = (w ? ws[w - 1] : 0) + x - v;
  *total = ws[kThreads / 32 - 1];
  __syncthreads();
  return before;
}

// scan, pass 1: each block's sum of its tile of kScanTile values
__global__ void __launch_bounds__(kThreads)
    k_scan_tiles(const int* __restrict__ in, int n, int* __restrict__ bsum) {
  const long base = (long)blockIdx.x * kScanTile + (long)threadIdx.x * kScanV;
  int s = 0;
  for (int k = 0; k < kScanV; k++)
    if (base + k < n) s += in[base + k];
  int total;
  block_exclusive(s, &total);
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// scan, pass 2 (one block): the tiles' sums to their exclusive prefixes
__global__ void __launch_bounds__(kThreads) k_scan_sums(int* __restrict__ bsum, int nb) {
  int carry = 0;
  for (int c0 = 0; c0 < nb; c0 += kThreads) {
    const int i = c0 + threadIdx.x;
    const int v = i < nb ? bsum[i] : 0;
    int total;
    const int before = block_exclusive(v, &total);
    if (i < nb) bsum[i] = carry + before;
    carry += total;
  }
}

// scan, pass 3: off[i] = sum of cnt[0..i), off[n] = the total; cnt[i]
// becomes off[i] (the fill's cursor)
__global__ void __launch_bounds__(kThreads)
    k_scan_apply(int* __restrict__ cnt, int n, const int* __restrict__ bsum,
                 int* __restrict__ off) {
  const long base = (long)blockIdx.x * kScanTile + (long)threadIdx.x * kScanV;
  int v[kScanV];
  int s = 0;
  for (int k = 0; k < kScanV; k++) {
    v[k] = base + k < n ? cnt[base + k] : 0;
    s += v[k];
  }
  int total;
  int p = bsum[blockIdx.x] + block_exclusive(s, &total);
  for (int k = 0; k < kScanV; k++) {
    if (base + k < n) {
      off[base + k] = p;
      cnt[base + k] = p;
    }
    p += v[k];
  }
  if (base <= n - 1 && n - 1 < base + kScanV) off[n] = p;
}

// the cursor reset for a second corner sequence over the same offsets
__global__ void __launch_bounds__(kThreads)
    k_copy(const int* __restrict__ off, int n, int* __restrict__ cur) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i < n) cur[i] = off[i];
}

// Fill, corner-major sequence: corner j of the elements in ielsort1 order
// (position k of the sort holds element srt[k]), sequence number
// j*nel + k.  Element-major sequence (srt null): corner j of element i in
// natural order, sequence number 4*i + j.
__global__ void __launch_bounds__(kThreads)
    k_fill(const int4* __restrict__ nd, const int* __restrict__ srt, int nel, int nnd,
           int* __restrict__ cur, int* __restrict__ key) {
  const int k = blockIdx.x * kThreads + threadIdx.x;
  if (k >= nel) return;
  const int i = srt ? srt[k] : k;
  if ((unsigned)i >= (unsigned)nel) return;
  const int4 n = nd[i];
  const int c[4] = {n.x, n.y, n.z, n.w};
  for (int j = 0; j < 4; j++) {
    if ((unsigned)c[j] >= (unsigned)nnd) continue;
    const int pos = atomicAdd(cur + c[j], 1);
    key[pos] = srt ? j * nel + k : 4 * k + j;
  }
}

// Per node: its corners sorted by sequence number (insertion sort: a
// node has a handful of corners), then each sequence number replaced by
// its corner's entry 4*element + corner.
__global__ void __launch_bounds__(kThreads)
    k_sort(const int* __restrict__ off, const int* __restrict__ srt, int nel, int nnd,
           int* __restrict__ key) {
  const int n = blockIdx.x * kThreads + threadIdx.x;
  if (n >= nnd) return;
  const int b = off[n], e = off[n + 1];
  for (int a = b + 1; a < e; a++) {
    const int v = key[a];
    int c = a - 1;
    while (c >= b && key[c] > v) {
      key[c + 1] = key[c];
      c--;
    }
    key[c + 1] = v;
  }
  if (srt)
    for (int a = b; a < e; a++) {
      const int q = key[a];
      key[a] = 4 * srt[q % nel] + q / nel;
    }
}

}  // namespace setup
}  // namespace bl

// Binned SAH build on the device, reproducing buildNodeSAH
// (renderer.go:526-633) node for node: the same bounds, axis, bins, split
// costs and leaf rule in fp64 with the reference's operation order, the same
// in-place partition of Scene.Order, and the reference's pre-order node
// numbering (left subtree first).
//
// The tree is built a level at a time. Each level's tasks (node ranges of the
// Order array) are cut into chunks of kChunk elements; per-chunk partial
// results (bounds, the 32 bins) are reduced per task. Bounds use an
// order-preserving 64-bit key of each double so min/max run as integer
// atomics; the key orders -0 before +0, which is what Go's math.Min/Max do
// with signed zeros, and a min/max reduction is order-independent, so the
// boxes equal the sequential ones bit for bit.
//
// The partition loop of the reference (i from the left, j from the right;
// a right-side element at i is swapped with the element at j, j moves down)
// has a closed form, computed here with per-task prefix counts. With L the
// number of left-side elements of the range [s, e):
//   * a left element in [s, s+L) stays;
//   * the m-th right element in [s, s+L) (m = 1, 2, ...) goes to l_{m-1} - 1,
//     where l_k is the position of the k-th left element of [s+L, e) counted
//     from the end (l_0 = e), and that k-th left element goes to the position
//     of the k-th right element of [s, s+L);
//   * a right element at p in (s+L, e) goes to p - 1, and the one at s+L (if it
//     is a right element) to l_M - 1 (e - 1 if M = 0), M being the number of
//     right elements in [s, s+L).
// The median fallback of the reference is unreachable (the chosen split has
// both sides non-empty); if it were reached, the build reports an error.
#include <cstring>
#include <vector>

#include "../../include/bc_host_scene.h"
#include "context.h"

namespace bcgx {
namespace {

constexpr int kChunk = 1024;
constexpr int kBins = 32;
constexpr int kThreads = 256;

__device__ __forceinline__ unsigned long long dkey(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double kdbl(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}
constexpr unsigned long long kKeyPosInf = 0xfff0000000000000ull;  // dkey(+inf): identity of min
constexpr unsigned long long kKeyNegInf = 0x000fffffffffffffull;  // dkey(-inf): identity of max

// AABB.SurfaceArea (renderer.go:133-139), unfused.
__device__ __forceinline__ double box_area(const double* mn, const double* mx) {
  const double ex = __dsub_rn(mx[0], mn[0]), ey = __dsub_rn(mx[1], mn[1]), ez = __dsub_rn(mx[2], mn[2]);
  if (ex < 0 || ey < 0 || ez < 0) return 0;
  return __dmul_rn(2.0, __dadd_rn(__dadd_rn(__dmul_rn(ex, ey), __dmul_rn(ey, ez)), __dmul_rn(ez, ex)));
}

// Task state
constexpr int kLeaf = 0, kSplit = 1;

struct BuildArgs {
  // inputs
  const double* pbox;  // 6 per primitive (padded box)
  const double* cent;  // 3 per primitive
  int n, nb, leaf;
  // Order and scratch
  int32_t *order, *order2, *lbefore, *rpos, *lpos;
  uint8_t* bin;
  // tasks of the current level and of the next
  const int32_t *ts, *te, *tnode;
  const int* T;  // task count of the level
  int32_t *nts, *nte, *ntnode;
  int* nT;
  // per task
  int32_t* chunk_off;  // T + 1
  int8_t *tstate, *taxis;
  double *tminc, *tinv;
  int32_t *tbest, *tL, *tM;
  // per chunk partials, and their per-task reductions
  unsigned long long* part_b;     // 12 per chunk
  unsigned long long* part_bins;  // 32 * 7 per chunk (count, box keys)
  int32_t* part_left;             // left count per chunk; then the chunk's base
  unsigned long long* task_b;     // 12 per task
  unsigned long long* task_bins;  // 32 * 7 per task
  // BFS node arrays
  double* nbox;                   // 6 per node
  int32_t *nleft, *nright, *nstart, *ncount;
  int* n_nodes;
  unsigned* error;
};

__device__ __forceinline__ int task_of_chunk(const BuildArgs& a, int c, int T) {
  int lo = 0, hi = T - 1;  // last task with chunk_off <= c
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (a.chunk_off[mid] <= c) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// chunk offsets of the level (single block: a chunked scan)
__global__ void k_chunk_offsets(BuildArgs a) {
  __shared__ int carry;
  __shared__ int tmp[1024];
  const int T = *a.T;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < T; base += 1024) {
    const int k = base + threadIdx.x;
    const int v = k < T ? (a.te[k] - a.ts[k] + kChunk - 1) / kChunk : 0;
    tmp[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const int add = threadIdx.x >= (unsigned)o ? tmp[threadIdx.x - o] : 0;
      __syncthreads();
      tmp[threadIdx.x] += add;
      __syncthreads();
    }
    if (k < T) a.chunk_off[k] = carry + tmp[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += tmp[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) a.chunk_off[T] = carry;
}

// bounds and centroid bounds per chunk
__global__ void __launch_bounds__(kThreads) k_bounds(BuildArgs a) {
  __shared__ unsigned long long sk[12];
  const int T = *a.T;
  const int total = a.chunk_off[T];
  for (int c = blockIdx.x; c < total; c += gridDim.x) {
    if (threadIdx.x < 12) sk[threadIdx.x] = (threadIdx.x % 6) < 3 ? kKeyPosInf : kKeyNegInf;
    __syncthreads();
    const int k = task_of_chunk(a, c, T);
    const int p0 = a.ts[k] + (c - a.chunk_off[k]) * kChunk, p1 = min(a.te[k], p0 + kChunk);
    unsigned long long m[12];
#pragma unroll
    for (int j = 0; j < 12; j++) m[j] = (j % 6) < 3 ? kKeyPosInf : kKeyNegInf;
    for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
      const int q = a.order[p];
#pragma unroll
      for (int j = 0; j < 3; j++) {
        m[j] = min(m[j], dkey(a.pbox[6 * (size_t)q + j]));
        m[3 + j] = max(m[3 + j], dkey(a.pbox[6 * (size_t)q + 3 + j]));
        const unsigned long long ck = dkey(a.cent[3 * (size_t)q + j]);
        m[6 + j] = min(m[6 + j], ck);
        m[9 + j] = max(m[9 + j], ck);
      }
    }
#pragma unroll
    for (int j = 0; j < 12; j++) {
      if ((j % 6) < 3) atomicMin(&sk[j], m[j]);
      else atomicMax(&sk[j], m[j]);
    }
    __syncthreads();
    if (threadIdx.x < 12) a.part_b[12 * (size_t)c + threadIdx.x] = sk[threadIdx.x];
    __syncthreads();
  }
}

// Per-task reduction of chunk partials, one thread per (task, field): F = 12
// bound keys (fields 0-2, 6-8 min, the rest max), or F = 32 * 7 bin fields
// (count sums; box fields 1-3 min, 4-6 max). Tasks that are not split are
// skipped for the bins.
template <bool BINS>
__global__ void k_reduce(BuildArgs a) {
  const int T = *a.T;
  const int F = BINS ? kBins * 7 : 12;
  const long long total = (long long)T * F;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i / F), f = (int)(i - (long long)k * F);
    if (BINS && a.tstate[k] != kSplit) continue;
    const unsigned long long* src = BINS ? a.part_bins : a.part_b;
    const int g = BINS ? f % 7 : f % 6;
    const bool is_sum = BINS && g == 0;
    const bool is_min = BINS ? (g >= 1 && g <= 3) : g < 3;
    unsigned long long v = is_sum ? 0ull : (is_min ? kKeyPosInf : kKeyNegInf);
    for (int c = a.chunk_off[k]; c < a.chunk_off[k + 1]; c++) {
      const unsigned long long x = src[(size_t)c * F + f];
      v = is_sum ? v + x : (is_min ? min(v, x) : max(v, x));
    }
    (BINS ? a.task_bins : a.task_b)[(size_t)k * F + f] = v;
  }
}

// per task: node box, leaf tests before binning, axis and bin parameters
__global__ void k_task_bounds(BuildArgs a) {
  const int T = *a.T;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < T; k += gridDim.x * blockDim.x) {
    unsigned long long m[12];
#pragma unroll
    for (int j = 0; j < 12; j++) m[j] = a.task_b[12 * (size_t)k + j];
    const int node = a.tnode[k];
    for (int j = 0; j < 6; j++) a.nbox[6 * (size_t)node + j] = kdbl(m[j]);
    const int s = a.ts[k], cnt = a.te[k] - s;
    a.nstart[node] = s;
    a.ncount[node] = cnt;
    a.nleft[node] = -1;
    a.nright[node] = -1;
    a.tstate[k] = kLeaf;
    if (cnt <= a.leaf) continue;
    double cmn[3], cmx[3], ext[3];
    for (int j = 0; j < 3; j++) {
      cmn[j] = kdbl(m[6 + j]);
      cmx[j] = kdbl(m[9 + j]);
      ext[j] = __dsub_rn(cmx[j], cmn[j]);
    }
    int axis = 0;  // largestAxis (renderer.go:485-493)
    if (ext[1] > ext[0] && ext[1] >= ext[2]) axis = 1;
    else if (ext[2] > ext[0] && ext[2] > ext[1]) axis = 2;
    const double axis_extent = __dsub_rn(cmx[axis], cmn[axis]);
    if (axis_extent < 1e-12) continue;
    a.tstate[k] = kSplit;
    a.taxis[k] = (int8_t)axis;
    a.tminc[k] = cmn[axis];
    a.tinv[k] = __ddiv_rn(1.0, axis_extent);
  }
}

__device__ __forceinline__ int bin_of(const BuildArgs& a, int k, int q) {
  const double c = a.cent[3 * (size_t)q + a.taxis[k]];
  const double x = __dmul_rn(__dmul_rn(__dsub_rn(c, a.tminc[k]), a.tinv[k]), (double)a.nb);
  int b = (int)x;  // truncation toward zero, as Go's int()
  return b < 0 ? 0 : (b >= a.nb ? a.nb - 1 : b);
}

// bins per chunk: count and box
__global__ void __launch_bounds__(kThreads) k_bins(BuildArgs a) {
  __shared__ unsigned long long sb[kBins * 7];
  const int T = *a.T;
  const int total = a.chunk_off[T];
  for (int c = blockIdx.x; c < total; c += gridDim.x) {
    const int k = task_of_chunk(a, c, T);
    if (a.tstate[k] != kSplit) continue;  // uniform over the block
    for (int j = threadIdx.x; j < kBins * 7; j += blockDim.x) {
      const int f = j % 7;
      sb[j] = f == 0 ? 0ull : (f <= 3 ? kKeyPosInf : kKeyNegInf);
    }
    __syncthreads();
    const int p0 = a.ts[k] + (c - a.chunk_off[k]) * kChunk, p1 = min(a.te[k], p0 + kChunk);
    for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
      const int q = a.order[p];
      const int b = bin_of(a, k, q);
      a.bin[p] = (uint8_t)b;
      atomicAdd(&sb[7 * b], 1ull);
#pragma unroll
      for (int j = 0; j < 3; j++) {
        atomicMin(&sb[7 * b + 1 + j], dkey(a.pbox[6 * (size_t)q + j]));
        atomicMax(&sb[7 * b + 4 + j], dkey(a.pbox[6 * (size_t)q + 3 + j]));
      }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < kBins * 7; j += blockDim.x) a.part_bins[(size_t)c * kBins * 7 + j] = sb[j];
    __syncthreads();
  }
}

// per task: the split of least SAH cost, or a leaf (renderer.go:566-604)
__global__ void k_split(BuildArgs a) {
  const int T = *a.T;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < T; k += gridDim.x * blockDim.x) {
    if (a.tstate[k] != kSplit) continue;
    const int nb = a.nb;
    long long cntb[kBins];
    double bmn[kBins][3], bmx[kBins][3];
    for (int b = 0; b < nb; b++) {
      const unsigned long long* tb = a.task_bins + (size_t)k * kBins * 7 + 7 * b;
      cntb[b] = (long long)tb[0];
      for (int j = 0; j < 3; j++) {
        bmn[b][j] = kdbl(tb[1 + j]);
        bmx[b][j] = kdbl(tb[4 + j]);
      }
    }
    double lArea[kBins - 1], rArea[kBins - 1];
    long long lCnt[kBins - 1], rCnt[kBins - 1];
    double amn[3] = {INFINITY, INFINITY, INFINITY}, amx[3] = {-INFINITY, -INFINITY, -INFINITY};
    long long acc = 0;
    for (int i = 0; i < nb - 1; i++) {
      if (cntb[i] > 0)
        for (int j = 0; j < 3; j++) {
          amn[j] = kdbl(min(dkey(amn[j]), dkey(bmn[i][j])));
          amx[j] = kdbl(max(dkey(amx[j]), dkey(bmx[i][j])));
        }
      acc += cntb[i];
      lCnt[i] = acc;
      lArea[i] = box_area(amn, amx);
    }
    for (int j = 0; j < 3; j++) {
      amn[j] = INFINITY;
      amx[j] = -INFINITY;
    }
    acc = 0;
    for (int i = nb - 1; i > 0; i--) {
      if (cntb[i] > 0)
        for (int j = 0; j < 3; j++) {
          amn[j] = kdbl(min(dkey(amn[j]), dkey(bmn[i][j])));
          amx[j] = kdbl(max(dkey(amx[j]), dkey(bmx[i][j])));
        }
      acc += cntb[i];
      rCnt[i - 1] = acc;
      rArea[i - 1] = box_area(amn, amx);
    }
    int best = -1;
    double best_cost = INFINITY;
    for (int i = 0; i < nb - 1; i++) {
      if (lCnt[i] == 0 || rCnt[i] == 0) continue;
      const double cost = __dadd_rn(__dmul_rn(lArea[i], (double)lCnt[i]), __dmul_rn(rArea[i], (double)rCnt[i]));
      if (cost < best_cost) {
        best_cost = cost;
        best = i;
      }
    }
    const int node = a.tnode[k];
    const int cnt = a.te[k] - a.ts[k];
    const double leaf_cost = __dmul_rn(box_area(a.nbox + 6 * (size_t)node, a.nbox + 6 * (size_t)node + 3), (double)cnt);
    if (best < 0 || (cnt <= a.leaf * 2 && best_cost >= __dmul_rn(leaf_cost, 0.98))) {
      a.tstate[k] = kLeaf;
      continue;
    }
    a.tbest[k] = best;
  }
}

// left-side count per chunk
__global__ void __launch_bounds__(kThreads) k_left_count(BuildArgs a) {
  __shared__ int s;
  const int T = *a.T;
  const int total = a.chunk_off[T];
  for (int c = blockIdx.x; c < total; c += gridDim.x) {
    const int k = task_of_chunk(a, c, T);
    if (a.tstate[k] != kSplit) continue;
    if (threadIdx.x == 0) s = 0;
    __syncthreads();
    const int p0 = a.ts[k] + (c - a.chunk_off[k]) * kChunk, p1 = min(a.te[k], p0 + kChunk);
    const int best = a.tbest[k];
    int cntl = 0;
    for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) cntl += a.bin[p] <= best;
    atomicAdd(&s, cntl);
    __syncthreads();
    if (threadIdx.x == 0) a.part_left[c] = s;
    __syncthreads();
  }
}

// per task: chunk bases of the left counts, L
__global__ void k_task_scan(BuildArgs a) {
  const int T = *a.T;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < T; k += gridDim.x * blockDim.x) {
    if (a.tstate[k] != kSplit) continue;
    int acc = 0;
    for (int c = a.chunk_off[k]; c < a.chunk_off[k + 1]; c++) {
      const int v = a.part_left[c];
      a.part_left[c] = acc;
      acc += v;
    }
    a.tL[k] = acc;
    a.tM[k] = 0;
    const int cnt = a.te[k] - a.ts[k];
    if (acc <= 0 || acc >= cnt) {  // the median fallback: never taken for a split with both sides non-empty
      atomicOr(a.error, 1u);
      a.tstate[k] = kLeaf;
    }
  }
}

// block-wide exclusive scan of one int per thread
__device__ __forceinline__ int block_excl_scan(int v, int* tmp) {
  tmp[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {
    const int add = (int)threadIdx.x >= o ? tmp[threadIdx.x - o] : 0;
    __syncthreads();
    tmp[threadIdx.x] += add;
    __syncthreads();
  }
  const int r = tmp[threadIdx.x] - v;
  __syncthreads();
  return r;
}

// ranks: lefts before each element; the tables of misplaced elements; M
__global__ void __launch_bounds__(kThreads) k_rank(BuildArgs a) {
  __shared__ int tmp[kThreads];
  const int T = *a.T;
  const int total = a.chunk_off[T];
  for (int c = blockIdx.x; c < total; c += gridDim.x) {
    const int k = task_of_chunk(a, c, T);
    if (a.tstate[k] != kSplit) continue;
    const int s = a.ts[k];
    const int p0 = s + (c - a.chunk_off[k]) * kChunk, p1 = min(a.te[k], p0 + kChunk);
    const int best = a.tbest[k], L = a.tL[k];
    int base = a.part_left[c];
    for (int p = p0; p < p1; p += blockDim.x) {  // kChunk / blockDim.x rounds, in order
      const int pp = p + threadIdx.x;
      const bool in = pp < p1;
      const bool left = in && a.bin[pp] <= best;
      const int lb = base + block_excl_scan(left ? 1 : 0, tmp);
      if (in) {
        a.lbefore[pp] = lb;
        if (pp == s + L) a.tM[k] = L - lb;
        if (pp < s + L && !left) a.rpos[s + ((pp - s) - lb)] = pp;  // misplaced right, rank (pp - s) - lb
        if (pp >= s + L && left) a.lpos[s + (L - lb) - 1] = pp;     // left beyond L, rank L - lb from the end
      }
      // next round's base: the last thread's exclusive prefix plus its own flag
      if (threadIdx.x == blockDim.x - 1) tmp[0] = lb + (left ? 1 : 0);
      __syncthreads();
      base = tmp[0];
      __syncthreads();
    }
  }
}

// the reference's partition as a permutation
__global__ void __launch_bounds__(kThreads) k_permute(BuildArgs a) {
  const int T = *a.T;
  const int total = a.chunk_off[T];
  for (int c = blockIdx.x; c < total; c += gridDim.x) {
    const int k = task_of_chunk(a, c, T);
    if (a.tstate[k] != kSplit) continue;
    const int s = a.ts[k], e = a.te[k];
    const int p0 = s + (c - a.chunk_off[k]) * kChunk, p1 = min(e, p0 + kChunk);
    const int best = a.tbest[k], L = a.tL[k], M = a.tM[k];
    for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
      const bool left = a.bin[p] <= best;
      const int lb = a.lbefore[p];
      int dest;
      if (left) {
        dest = p < s + L ? p : a.rpos[s + (L - lb) - 1];
      } else if (p < s + L) {
        const int m0 = (p - s) - lb;  // right elements of [s, p)
        dest = (m0 == 0 ? e : a.lpos[s + m0 - 1]) - 1;
      } else if (p == s + L) {
        dest = (M > 0 ? a.lpos[s + M - 1] : e) - 1;
      } else {
        dest = p - 1;
      }
      if (dest < s || dest >= e) {  // cannot happen for consistent ranks; never write outside the task
        atomicOr(a.error, 2u);
        continue;
      }
      a.order2[dest] = a.order[p];
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_copy_back(BuildArgs a) {
  const int T = *a.T;
  const int total = a.chunk_off[T];
  for (int c = blockIdx.x; c < total; c += gridDim.x) {
    const int k = task_of_chunk(a, c, T);
    if (a.tstate[k] != kSplit) continue;
    const int p0 = a.ts[k] + (c - a.chunk_off[k]) * kChunk, p1 = min(a.te[k], p0 + kChunk);
    for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) a.order[p] = a.order2[p];
  }
}

// children of split tasks: two nodes each, two tasks of the next level
__global__ void k_children(BuildArgs a) {
  const int T = *a.T;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < T; k += gridDim.x * blockDim.x) {
    if (a.tstate[k] != kSplit) continue;
    const int node = a.tnode[k];
    const int id = atomicAdd(a.n_nodes, 2);
    const int t = atomicAdd(a.nT, 2);
    const int s = a.ts[k], e = a.te[k], mid = s + a.tL[k];
    a.nleft[node] = id;
    a.nright[node] = id + 1;
    a.ncount[node] = 0;
    a.nstart[node] = 0;
    a.nts[t] = s;
    a.nte[t] = mid;
    a.ntnode[t] = id;
    a.nts[t + 1] = mid;
    a.nte[t + 1] = e;
    a.ntnode[t + 1] = id + 1;
  }
}

// subtree sizes of nodes [lo, hi) (children already sized)
__global__ void k_sizes(int lo, int hi, const int32_t* nl, const int32_t* nr, int32_t* size) {
  const int i = lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hi) return;
  size[i] = nl[i] < 0 ? 1 : 1 + size[nl[i]] + size[nr[i]];
}

// pre-order indices of the children of nodes [lo, hi)
__global__ void k_preorder(int lo, int hi, const int32_t* nl, const int32_t* nr, const int32_t* size, int32_t* pre) {
  const int i = lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= hi || nl[i] < 0) return;
  pre[nl[i]] = pre[i] + 1;
  pre[nr[i]] = pre[i] + 1 + size[nl[i]];
}

__global__ void k_emit(int n_nodes, const int32_t* pre, const double* nbox, const int32_t* nl, const int32_t* nr,
                       const int32_t* ns, const int32_t* nc, double* obox, int32_t* ol, int32_t* orr, int32_t* os,
                       int32_t* oc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  const int d = pre[i];
  for (int j = 0; j < 6; j++) obox[6 * (size_t)d + j] = nbox[6 * (size_t)i + j];
  ol[d] = nl[i] < 0 ? -1 : pre[nl[i]];
  orr[d] = nr[i] < 0 ? -1 : pre[nr[i]];
  os[d] = nl[i] < 0 ? ns[i] : 0;
  oc[d] = nl[i] < 0 ? nc[i] : 0;
}

}  // namespace

// Carves 256-byte aligned sub-buffers out of one device allocation.
struct Carver {
  char* p;
  template <class T>
  T* take(size_t n) {
    T* r = reinterpret_cast<T*>(p);
    p += ((n * sizeof(T) + 255) / 256) * 256;
    return r;
  }
};

// Device build: fills the caller's host arrays (node arrays sized 2n - 1).
bc_status build_sah_device(bc_context* ctx, int32_t n, const double* prim_box, const double* centroid, int32_t bins,
                           int32_t leaf, int32_t* n_nodes_out, double* node_box, int32_t* node_left,
                           int32_t* node_right, int32_t* node_start, int32_t* node_count, int32_t* order_out) {
  cudaStream_t st = ctx->stream;
  const size_t N = (size_t)n, NN = 2 * N;
  // fixed arrays (per primitive, per task, per node)
  const size_t fixed = 256 * 48 + N * (6 * 8 + 3 * 8 + 5 * 4 + 1) + N * (6 * 4 + 4 + 2 + 2 * 8 + 3 * 4 + 12 * 8) +
                       NN * (6 * 8 + 6 * 4) + 64;
  cudaError_t e = ctx->d_build.ensure(fixed);
  if (e) return cuda_status(ctx, e, "BVH build buffers");
  Carver cv{(char*)ctx->d_build.p};
  BuildArgs a;
  double* pbox = cv.take<double>(N * 6);
  double* cent = cv.take<double>(N * 3);
  a.pbox = pbox;
  a.cent = cent;
  a.n = n;
  a.nb = bins;
  a.leaf = leaf;
  a.order = cv.take<int32_t>(N);
  a.order2 = cv.take<int32_t>(N);
  a.lbefore = cv.take<int32_t>(N);
  a.rpos = cv.take<int32_t>(N);
  a.lpos = cv.take<int32_t>(N);
  a.bin = cv.take<uint8_t>(N);
  int32_t* ts[2] = {cv.take<int32_t>(N), cv.take<int32_t>(N)};
  int32_t* te[2] = {cv.take<int32_t>(N), cv.take<int32_t>(N)};
  int32_t* tn[2] = {cv.take<int32_t>(N), cv.take<int32_t>(N)};
  a.chunk_off = cv.take<int32_t>(N + 1);
  a.tstate = cv.take<int8_t>(N);
  a.taxis = cv.take<int8_t>(N);
  a.tminc = cv.take<double>(N);
  a.tinv = cv.take<double>(N);
  a.tbest = cv.take<int32_t>(N);
  a.tL = cv.take<int32_t>(N);
  a.tM = cv.take<int32_t>(N);
  a.task_b = cv.take<unsigned long long>(N * 12);
  a.nbox = cv.take<double>(NN * 6);
  a.nleft = cv.take<int32_t>(NN);
  a.nright = cv.take<int32_t>(NN);
  a.nstart = cv.take<int32_t>(NN);
  a.ncount = cv.take<int32_t>(NN);
  int32_t* size = cv.take<int32_t>(NN);
  int32_t* pre = cv.take<int32_t>(NN);
  int* counters = cv.take<int>(16);  // [0], [1] task counts; [2] nodes; [3] error
  a.n_nodes = counters + 2;
  a.error = reinterpret_cast<unsigned*>(counters + 3);

  std::vector<int32_t> iota(n);
  for (int32_t i = 0; i < n; i++) iota[i] = i;
  const int32_t root_task[3] = {0, n, 0};
  const int init[4] = {1, 0, 1, 0};
  e = cudaMemcpyAsync(pbox, prim_box, N * 6 * 8, cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(cent, centroid, N * 3 * 8, cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(a.order, iota.data(), N * 4, cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(ts[0], &root_task[0], 4, cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(te[0], &root_task[1], 4, cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(tn[0], &root_task[2], 4, cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(counters, init, sizeof(init), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaStreamSynchronize(st);  // the host vectors above die at return
  if (e) return cuda_status(ctx, e, "BVH build upload");

  int sms = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int cgrid = std::max(1, sms * 8), tgrid = std::max(1, sms * 8);
  std::vector<int> level_lo{0};  // node ids of level d: [level_lo[d], level_lo[d + 1])
  int cur = 0;
  for (int level = 0;; level++) {
    if (level >= 4096) return set_error(ctx, BC_ERR_CAPACITY, "BVH deeper than 4096 levels: build on the host");
    int hdr[3] = {0, 0, 0};  // task counts, nodes
    e = cudaMemcpyAsync(hdr, counters, 3 * sizeof(int), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (e) return cuda_status(ctx, e, "BVH build");
    const int T = hdr[cur];
    if (T == 0) break;
    if (level > 0) level_lo.push_back(hdr[2] - T);
    a.ts = ts[cur];
    a.te = te[cur];
    a.tnode = tn[cur];
    a.T = counters + cur;
    a.nts = ts[cur ^ 1];
    a.nte = te[cur ^ 1];
    a.ntnode = tn[cur ^ 1];
    a.nT = counters + (cur ^ 1);
    e = cudaMemsetAsync(a.nT, 0, sizeof(int), st);
    if (e) return cuda_status(ctx, e, "BVH build");
    k_chunk_offsets<<<1, 1024, 0, st>>>(a);
    int chunks = 0;
    e = cudaMemcpyAsync(&chunks, a.chunk_off + T, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (e) return cuda_status(ctx, e, "BVH build");
    // per-level partials: 12 + 224 keys and one count per chunk, 224 keys per task
    e = ctx->d_build_out.ensure((size_t)chunks * (12 + kBins * 7) * 8 + (size_t)chunks * 4 +
                                (size_t)T * kBins * 7 * 8 + 4 * 256);
    if (e) return cuda_status(ctx, e, "BVH build partials");
    Carver pc{(char*)ctx->d_build_out.p};
    a.part_b = pc.take<unsigned long long>((size_t)chunks * 12);
    a.part_bins = pc.take<unsigned long long>((size_t)chunks * kBins * 7);
    a.part_left = pc.take<int32_t>((size_t)chunks);
    a.task_bins = pc.take<unsigned long long>((size_t)T * kBins * 7);
    const int rgrid = std::max(1, std::min(sms * 16, (int)(((long long)T * kBins * 7 + 255) / 256)));
    k_bounds<<<cgrid, kThreads, 0, st>>>(a);
    k_reduce<false><<<rgrid, 256, 0, st>>>(a);
    k_task_bounds<<<tgrid, 128, 0, st>>>(a);
    k_bins<<<cgrid, kThreads, 0, st>>>(a);
    k_reduce<true><<<rgrid, 256, 0, st>>>(a);
    k_split<<<tgrid, 128, 0, st>>>(a);
    k_left_count<<<cgrid, kThreads, 0, st>>>(a);
    k_task_scan<<<tgrid, 128, 0, st>>>(a);
    k_rank<<<cgrid, kThreads, 0, st>>>(a);
    k_permute<<<cgrid, kThreads, 0, st>>>(a);
    k_copy_back<<<cgrid, kThreads, 0, st>>>(a);
    k_children<<<tgrid, 128, 0, st>>>(a);
    if ((e = cudaGetLastError())) return cuda_status(ctx, e, "BVH build launch");
    cur ^= 1;
  }
  int n_nodes = 0;
  unsigned err = 0;
  e = cudaMemcpyAsync(&n_nodes, a.n_nodes, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaMemcpyAsync(&err, a.error, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  if (e) return cuda_status(ctx, e, "BVH build");
  if (err & 1u) return set_error(ctx, BC_ERR_BAD_SCENE, "BVH build reached the median fallback");
  if (err) return set_error(ctx, BC_ERR_DEVICE, "BVH build: inconsistent partition ranks");
  if (n_nodes > (int)NN) return set_error(ctx, BC_ERR_CAPACITY, "BVH build node count");
  level_lo.push_back(n_nodes);
  // subtree sizes bottom-up, pre-order indices top-down
  for (int d = (int)level_lo.size() - 2; d >= 0; d--) {
    const int lo = level_lo[d], hi = level_lo[d + 1];
    if (hi > lo) k_sizes<<<(hi - lo + 255) / 256, 256, 0, st>>>(lo, hi, a.nleft, a.nright, size);
  }
  e = cudaMemsetAsync(pre, 0, sizeof(int32_t), st);
  if (e) return cuda_status(ctx, e, "BVH build");
  for (int d = 0; d + 1 < (int)level_lo.size(); d++) {
    const int lo = level_lo[d], hi = level_lo[d + 1];
    if (hi > lo) k_preorder<<<(hi - lo + 255) / 256, 256, 0, st>>>(lo, hi, a.nleft, a.nright, size, pre);
  }
  // the tree in the reference's numbering, staged in the (no longer needed) partials buffer
  e = ctx->d_build_out.ensure((size_t)n_nodes * (6 * 8 + 4 * 4) + 8 * 256);
  if (e) return cuda_status(ctx, e, "BVH build output");
  Carver oc{(char*)ctx->d_build_out.p};
  double* ob = oc.take<double>((size_t)n_nodes * 6);
  int32_t* oL = oc.take<int32_t>((size_t)n_nodes);
  int32_t* oR = oc.take<int32_t>((size_t)n_nodes);
  int32_t* oS = oc.take<int32_t>((size_t)n_nodes);
  int32_t* oC = oc.take<int32_t>((size_t)n_nodes);
  k_emit<<<(n_nodes + 255) / 256, 256, 0, st>>>(n_nodes, pre, a.nbox, a.nleft, a.nright, a.nstart, a.ncount, ob, oL,
                                                  oR, oS, oC);
  e = cudaGetLastError();
  if (!e) e = cudaMemcpyAsync(node_box, ob, (size_t)n_nodes * 48, cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaMemcpyAsync(node_left, oL, (size_t)n_nodes * 4, cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaMemcpyAsync(node_right, oR, (size_t)n_nodes * 4, cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaMemcpyAsync(node_start, oS, (size_t)n_nodes * 4, cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaMemcpyAsync(node_count, oC, (size_t)n_nodes * 4, cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaMemcpyAsync(order_out, a.order, N * 4, cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  if (e) return cuda_status(ctx, e, "BVH build readback");
  *n_nodes_out = n_nodes;
  return BC_OK;
}

using TreeBuildFn = bc_status (*)(void* user, int32_t n, const double* pbox, const double* cent, int32_t bins,
                                  int32_t leaf, int32_t* n_nodes, double* box, int32_t* left, int32_t* right,
                                  int32_t* start, int32_t* count, int32_t* order);
bc_status hscene_build_external(bc_hscene* s, TreeBuildFn fn, void* user);  // host_scene.cpp

}  // namespace bcgx

using namespace bcgx;

extern "C" bc_status bc_build_sah(bc_context* ctx, int32_t n_prims, const double* prim_box, const double* centroid,
                                  int32_t bins, int32_t leaf_size, int32_t* n_nodes_out, double* node_box,
                                  int32_t* node_left, int32_t* node_right, int32_t* node_start, int32_t* node_count,
                                  int32_t* order_out) {
  if (!ctx || n_prims < 1 || !prim_box || !centroid || !n_nodes_out || !node_box || !node_left || !node_right ||
      !node_start || !node_count || !order_out)
    return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument or no primitives");
  if (n_prims >= (1 << 27)) return set_error(ctx, BC_ERR_INVALID_ARG, "at most 2^27 primitives");
  if (bins < 4) bins = 16;  // Scene.Build's clamps (renderer.go:413-427)
  if (bins > 32) bins = 32;
  if (leaf_size < 1) leaf_size = 4;
  if (leaf_size > 16) leaf_size = 16;
  cudaSetDevice(ctx->device);
  return build_sah_device(ctx, n_prims, prim_box, centroid, bins, leaf_size, n_nodes_out, node_box, node_left,
                          node_right, node_start, node_count, order_out);
}

static bc_status device_tree(void* user, int32_t n, const double* pbox, const double* cent, int32_t bins,
                             int32_t leaf, int32_t* n_nodes, double* box, int32_t* left, int32_t* right,
                             int32_t* start, int32_t* count, int32_t* order) {
  return bc_build_sah(static_cast<bc_context*>(user), n, pbox, cent, bins, leaf, n_nodes, box, left, right, start,
                      count, order);
}

extern "C" bc_status bc_hscene_build_device(bc_hscene* s, bc_context* ctx) {
  if (!s || !ctx) return BC_ERR_INVALID_ARG;
  return hscene_build_external(s, device_tree, ctx);
}

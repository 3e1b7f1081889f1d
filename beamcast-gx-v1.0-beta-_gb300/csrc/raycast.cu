// Ray-cast kernels: exact closest hit and any hit over the BVH8, one thread
// per ray. Rays are 32-byte records (ox, oy, oz, tmin, dx, dy, dz, tmax) read
// with two 128-bit loads; results are written as coalesced 4-byte streams.
#include <algorithm>

#include "kernels.h"
#include "trace_core.cuh"

namespace bcgx {

int stack_variant(int need) {
  if (need <= 64) return 64;
  if (need <= 128) return 128;
  if (need <= 256) return 256;
  return 0;
}

namespace {

template <int STACK, bool SPHERES, int MINB>
__global__ void __launch_bounds__(128, MINB) k_closest_exact(SceneView sv, const float4* __restrict__ rays, int64_t n,
                                                       float* __restrict__ t_out, int32_t* __restrict__ prim_out,
                                                       unsigned* status) {
  // No early return: every lane reaches the warp-converged fp64 settlement.
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n;
  float4 a = make_float4(0, 0, 0, 0), b = a;
  if (active) {
    a = __ldg(rays + 2 * i);
    b = __ldg(rays + 2 * i + 1);
  }
  const Ray32 r = make_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w);
  const HitResult h = closest_hit_exact<STACK, SPHERES>(sv, r, b.w, status, active);
  if (!active) return;
  if (h.slot >= 0) {
    t_out[i] = __double2float_rn(h.t64);
    prim_out[i] = h.tie ? kTieMark : __ldg(sv.slot_prim + h.slot);
  } else {
    t_out[i] = -1.0f;
    prim_out[i] = -1;
  }
}

template <int STACK, bool SPHERES, int MINB>
__global__ void __launch_bounds__(128, MINB) k_any_exact(SceneView sv, const float4* __restrict__ rays, int64_t n,
                                                   uint8_t* __restrict__ out, unsigned* status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = __ldg(rays + 2 * i);
  const float4 b = __ldg(rays + 2 * i + 1);
  const Ray32 r = make_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w);
  out[i] = any_hit_exact<STACK, SPHERES>(sv, r, b.w, status) ? 1 : 0;
}

// Fast variant: the same walk with plain fp32 tests (no exactness contract:
// near ties and edge grazes may differ from the fp64 path).
template <int STACK, bool SPHERES>
__global__ void __launch_bounds__(128) k_closest_fast(SceneView sv, const float4* __restrict__ rays, int64_t n,
                                                      float* __restrict__ t_out, int32_t* __restrict__ prim_out,
                                                      unsigned* status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = __ldg(rays + 2 * i);
  const float4 b = __ldg(rays + 2 * i + 1);
  const Ray32 r = make_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w);
  const HitResult h = closest_hit_fast<STACK, SPHERES>(sv, r, b.w, status);
  t_out[i] = h.slot >= 0 ? h.t32 : -1.0f;
  prim_out[i] = h.slot >= 0 ? __ldg(sv.slot_prim + h.slot) : -1;
}

// ---- persistent kernels with per-lane refill -------------------------------
// Lanes whose rays are done fetch the next ray indices once kRefillLanes of the
// warp's lanes are idle (one atomic per warp for all of them), so the warp does
// not idle until its slowest ray ends. The exact kernel parks each finished ray's contenders in a
// per-warp queue in shared memory; when 32 are parked, the warp settles them
// in fp64 with every lane active. Triangle-only scenes (spheres settle at
// once and use the kernels above).
constexpr int kParkTie = 0x100;  // npend flag: the walk already compared two equal fp64 distances

struct ParkQueue {
  long long idx[32];
  int bslot[32];
  float bhi[32];
  int npend[32];
  int pslot[kPending][32];
  float plo[kPending][32];
};

__device__ __forceinline__ void settle_parked(const SceneView& sv, const float4* __restrict__ rays,
                                              const ParkQueue& q, int k, float* __restrict__ t_out,
                                              int32_t* __restrict__ prim_out, unsigned* status) {
  const long long i = q.idx[k];
  const float4 a = __ldg(rays + 2 * i), b = __ldg(rays + 2 * i + 1);
  const D3 o{(double)a.x, (double)a.y, (double)a.z}, d{(double)b.x, (double)b.y, (double)b.z};
  const double tmin = (double)a.w, tmax = (double)b.w;
  const int bslot = q.bslot[k];
  const float bhi = q.bhi[k];
  int win = -1;
  double wt = 0.0;
  if (bslot >= 0) {
    double t;
    if (tri_hit64(sv.slot64 + 9 * (size_t)bslot, o, d, tmin, tmax, &t)) {
      win = bslot;
      wt = t;
    } else {
      atomicOr(status, kStatusBound);  // a certain hit must pass its fp64 test
    }
  }
  const int np = q.npend[k] & 0xff;
  bool tie = (q.npend[k] & kParkTie) != 0;
#pragma unroll
  for (int j = 0; j < kPending; j++) {
    if (j < np && !(bslot >= 0 && q.plo[j][k] > bhi)) {
      const int sj = q.pslot[j][k];
      double t;
      if (tri_hit64(sv.slot64 + 9 * (size_t)sj, o, d, tmin, tmax, &t)) {
        tie = tie || (win >= 0 && t == wt);
        if (win < 0 || t < wt || (t == wt && sj > win)) {
          win = sj;
          wt = t;
        }
      }
    }
  }
  if (win >= 0) {
    t_out[i] = __double2float_rn(wt);
    prim_out[i] = tie ? kTieMark : __ldg(sv.slot_prim + win);
  } else {
    t_out[i] = -1.0f;
    prim_out[i] = -1;
  }
}

template <int STACK, int MINB>
__global__ void __launch_bounds__(128, MINB) k_closest_exact_persistent(SceneView sv, const float4* __restrict__ rays,
                                                                        int64_t n, float* __restrict__ t_out,
                                                                        int32_t* __restrict__ prim_out,
                                                                        unsigned* status, unsigned long long* work,
                                                                        const int32_t* __restrict__ perm) {
  __shared__ ParkQueue park[4];
  ParkQueue& q = park[threadIdx.x >> 5];
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  long long idx = -1;
  bool exhausted = false;
  Ray32 r = make_ray(0, 0, 0, 0, 0, 0, 0);
  ExactClosestLeaf<false> leaf(sv, r, 0.0f, status);
  Walker<STACK, kExactLeafVote> w;
  w.reset(r);
  int parked = 0;  // warp-uniform
  for (;;) {
    const bool need = idx < 0 && !exhausted;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m && (__popc(m) >= kRefillLanes || !__any_sync(0xffffffffu, idx >= 0))) {
      const int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if ((int)lane == leader) base = atomicAdd(work, (unsigned long long)__popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const unsigned long long my = base + (unsigned long long)__popc(m & below);
        if (my < (unsigned long long)n) {
          idx = perm ? (long long)perm[my] : (long long)my;
          const float4 a = __ldg(rays + 2 * idx), b = __ldg(rays + 2 * idx + 1);
          r = make_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w);
          leaf.reset(b.w);
          w.reset(r);
        } else {
          exhausted = true;
        }
      }
    }
    const bool active = idx >= 0;
    if (!__any_sync(0xffffffffu, active)) break;
    bool finished = false;
    if (active) finished = w.step(sv, r, leaf, status);
    const unsigned pm = __ballot_sync(0xffffffffu, finished);
    if (pm) {
      if (parked + __popc(pm) > 32) {
        __syncwarp();
        if ((int)lane < parked) settle_parked(sv, rays, q, (int)lane, t_out, prim_out, status);
        __syncwarp();
        parked = 0;
      }
      if (finished) {
        const int k = parked + __popc(pm & below);
        q.idx[k] = idx;
        q.bslot[k] = leaf.best.slot;
        q.bhi[k] = leaf.best.hi;
        q.npend[k] = leaf.npend | (leaf.tie ? kParkTie : 0);
#pragma unroll
        for (int j = 0; j < kPending; j++) {
          q.pslot[j][k] = leaf.pend[j].slot;
          q.plo[j][k] = leaf.pend[j].lo;
        }
        idx = -1;
      }
      parked += __popc(pm);
    }
  }
  __syncwarp();
  if ((int)lane < parked) settle_parked(sv, rays, q, (int)lane, t_out, prim_out, status);
}

// ---- exact closest hit in passes: walk, then settle ----------------------------
// The one-kernel form above keeps the fp64 settlement (and the in-walk fp64
// re-test of a full contender list) in the walking kernel, whose register
// allocation then covers the fp64 code: 80 registers with spills at six
// 128-thread blocks per SM. Split, the walk holds no fp64 code and fits 40
// registers without spills (twelve blocks per SM; 9.74 ms -> 7.71 ms on the
// 1M-triangle / 4M-ray cast, settlement and ray order included):
//   pass 1, k_exact_walk: the persistent walk with the fp32 classifier; a
//     finished ray leaves a record (best certain hit: slot and upper bound of
//     its distance; the pending contenders: slot and lower bound). A ray with
//     more contenders than the list holds stops walking and is marked.
//   pass 2, k_exact_settle: one thread per ray settles its record in fp64 with
//     triHit's operation order (the same decisions as settle_parked) and writes
//     the result; marked rays go to a list.
//   pass 3, k_closest_exact_list: the marked rays, traced again by the
//     one-kernel exact walk, whose full list falls back to fp64 in the walk.
// Triangle-only scenes (as the persistent one-kernel form). The rays and the
// records pass through L2 once each way, so the walk and the settlement read
// and write them evict-first (ld/st.global.cs): L2 stays with the scene.
struct ExactRecords {
  int32_t* bslot;   // [n]: best certain hit, -1 none
  float* bhi;       // [n]: upper bound of its distance
  int32_t* npend;   // [n]: pending contenders; kPending + 1: list overflowed
  int32_t* pslot;   // [kPending * n]
  float* plo;       // [kPending * n]
  long long* redo;  // [n]: rays of pass 3
  unsigned long long* n_redo;
};


size_t up256(size_t b) { return (b + 255) / 256 * 256; }

// Layout of the records in the caller's scratch (exact_record_bytes(n) bytes).
ExactRecords exact_records(void* p, int64_t n) {
  auto up = up256;
  char* q = (char*)p;
  ExactRecords r;
  r.n_redo = (unsigned long long*)q;
  q += 256;
  r.bslot = (int32_t*)q;
  q += up((size_t)n * 4);
  r.bhi = (float*)q;
  q += up((size_t)n * 4);
  r.npend = (int32_t*)q;
  q += up((size_t)n * 4);
  r.pslot = (int32_t*)q;
  q += up((size_t)n * 4 * kPending);
  r.plo = (float*)q;
  q += up((size_t)n * 4 * kPending);
  r.redo = (long long*)q;
  return r;
}

// ExactClosestLeaf's decisions without its fp64 fallback: where that leaf
// resolves a contender in fp64 because its list is full, this one marks the
// ray (npend = kPending + 1) and ends the walk (done).
struct FilterLeaf {
  const SceneView& sv;
  const Ray32& r;
  float tmax_ray;
  float tlim;
  bool done;
  int32_t bslot;
  float blo, bhi;
  int npend;
  PendEntry pend[kPending];

  __device__ FilterLeaf(const SceneView& s, const Ray32& ray) : sv(s), r(ray) { reset(0.0f); }
  __device__ __forceinline__ void reset(float tmax) {
    tmax_ray = tmax;
    tlim = widen(tmax);
    done = false;
    npend = 0;
    bslot = -1;
    blo = tmax;
    bhi = tmax;
  }
  __device__ __forceinline__ void overflow() {
    npend = kPending + 1;
    done = true;
  }
  __device__ __forceinline__ void take_certain(int slot, float lo, float hi) {
    if (bslot < 0 || hi < blo) {
      bslot = slot;
      blo = lo;
      bhi = hi;
    } else if (lo > bhi) {
      return;
    } else if (npend < kPending) {
      if (hi < bhi) {
        pend[npend++] = PendEntry{bslot, blo};
        bslot = slot;
        blo = lo;
        bhi = hi;
      } else {
        pend[npend++] = PendEntry{slot, lo};
      }
    } else {
      overflow();
      return;
    }
    tlim = widen(bhi);
  }
  __device__ __forceinline__ void operator()(uint32_t ref) {
    const int cnt = (int)((ref >> 27) & 15u) + 1;
    const int s0 = (int)(ref & kSlotMask);
    for (int k = 0; k < cnt && !done; k++) {
      const int s = s0 + k;
      const float4 A = __ldg(sv.tri + 3 * s);
      const float4 E1 = __ldg(sv.tri + 3 * s + 1);
      const float4 E2 = __ldg(sv.tri + 3 * s + 2);
      const TriClass tc = tri_classify(A, E1, E2, r, tmax_ray, tlim);
      if (tc.state == kMiss) continue;
      const float lo = __fsub_rd(tc.t, tc.et), hi = __fadd_ru(tc.t, tc.et);
      if (bslot >= 0 && lo > bhi) continue;
      if (tc.state == kHit) take_certain(s, lo, hi);
      else if (npend < kPending) pend[npend++] = PendEntry{s, lo};
      else overflow();
    }
  }
};

template <int STACK>
__global__ void __launch_bounds__(128, 12) k_exact_walk(SceneView sv, const float4* __restrict__ rays, int64_t n,
                                                       ExactRecords rec, unsigned* status, unsigned long long* work,
                                                       const int32_t* __restrict__ perm) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  long long idx = -1;
  bool exhausted = false;
  Ray32 r = make_ray(0, 0, 0, 0, 0, 0, 0);
  FilterLeaf leaf(sv, r);
  Walker<STACK, kExactLeafVote> w;
  w.reset(r);
  for (;;) {
    const bool need = idx < 0 && !exhausted;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m && (__popc(m) >= kRefillLanes || !__any_sync(0xffffffffu, idx >= 0))) {
      const int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if ((int)lane == leader) base = atomicAdd(work, (unsigned long long)__popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const unsigned long long my = base + (unsigned long long)__popc(m & below);
        if (my < (unsigned long long)n) {
          idx = perm ? (long long)perm[my] : (long long)my;
          const float4 a = __ldcs(rays + 2 * idx), b = __ldcs(rays + 2 * idx + 1);
          r = make_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w);
          leaf.reset(b.w);
          w.reset(r);
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, idx >= 0)) break;
    if (idx >= 0 && w.step(sv, r, leaf, status)) {
      __stcs(rec.bslot + idx, leaf.bslot);
      __stcs(rec.bhi + idx, leaf.bhi);
      __stcs(rec.npend + idx, leaf.npend);
      const int np = min(leaf.npend, kPending);
      for (int j = 0; j < np; j++) {
        __stcs(rec.pslot + (size_t)j * n + idx, leaf.pend[j].slot);
        __stcs(rec.plo + (size_t)j * n + idx, leaf.pend[j].lo);
      }
      idx = -1;
    }
  }
}

__global__ void __launch_bounds__(128) k_exact_settle(SceneView sv, const float4* __restrict__ rays, int64_t n,
                                                      ExactRecords rec, float* __restrict__ t_out,
                                                      int32_t* __restrict__ prim_out, unsigned* status) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int np = __ldcs(rec.npend + i);
    if (np > kPending) {
      rec.redo[atomicAdd(rec.n_redo, 1ull)] = i;
      continue;
    }
    const float4 a = __ldcs(rays + 2 * i), b = __ldcs(rays + 2 * i + 1);
    const D3 o{(double)a.x, (double)a.y, (double)a.z}, d{(double)b.x, (double)b.y, (double)b.z};
    const double tmin = (double)a.w, tmax = (double)b.w;
    const int bslot = __ldcs(rec.bslot + i);
    const float bhi = __ldcs(rec.bhi + i);
    int win = -1;
    double wt = 0.0;
    bool tie = false;
    if (bslot >= 0) {
      double t;
      if (tri_hit64(sv.slot64 + 9 * (size_t)bslot, o, d, tmin, tmax, &t)) {
        win = bslot;
        wt = t;
      } else {
        atomicOr(status, kStatusBound);  // a certain hit must pass its fp64 test
      }
    }
    for (int j = 0; j < np; j++) {
      const float lo = __ldcs(rec.plo + (size_t)j * n + i);
      if (bslot >= 0 && lo > bhi) continue;
      const int sj = __ldcs(rec.pslot + (size_t)j * n + i);
      double t;
      if (tri_hit64(sv.slot64 + 9 * (size_t)sj, o, d, tmin, tmax, &t)) {
        tie = tie || (win >= 0 && t == wt);
        if (win < 0 || t < wt || (t == wt && sj > win)) {
          win = sj;
          wt = t;
        }
      }
    }
    t_out[i] = win >= 0 ? __double2float_rn(wt) : -1.0f;
    prim_out[i] = win >= 0 ? (tie ? kTieMark : __ldg(sv.slot_prim + win)) : -1;
  }
}

// Pass 3: the listed rays with the one-kernel exact walk. Every lane of a warp
// runs the same number of iterations (the warp-converged settlement inside
// closest_hit_exact needs all 32 lanes).
template <int STACK>
__global__ void __launch_bounds__(128) k_closest_exact_list(SceneView sv, const float4* __restrict__ rays,
                                                            ExactRecords rec, float* __restrict__ t_out,
                                                            int32_t* __restrict__ prim_out, unsigned* status) {
  const long long cnt = (long long)*((volatile unsigned long long*)rec.n_redo);
  for (long long base = (long long)blockIdx.x * blockDim.x; base < cnt; base += (long long)gridDim.x * blockDim.x) {
    const long long k = base + threadIdx.x;
    const bool active = k < cnt;
    const long long i = active ? rec.redo[k] : 0;
    float4 a = make_float4(0, 0, 0, 0), b = a;
    if (active) {
      a = __ldg(rays + 2 * i);
      b = __ldg(rays + 2 * i + 1);
    }
    const Ray32 r = make_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w);
    const HitResult h = closest_hit_exact<STACK, false>(sv, r, b.w, status, active);
    if (active) {
      t_out[i] = h.slot >= 0 ? __double2float_rn(h.t64) : -1.0f;
      prim_out[i] = h.slot >= 0 ? (h.tie ? kTieMark : __ldg(sv.slot_prim + h.slot)) : -1;
    }
  }
}

// ---- exact any hit in passes -----------------------------------------------------
// The same split for Scene.Occluded: the walk (no fp64 code) decides a ray when
// a triangle certainly blocks it or when no triangle might; a ray with
// undecided ("maybe") triangles is appended to a list with up to kPending of
// them, which the second pass tests in fp64 (triAnyHit's operation order); a
// ray with more is re-traced there by the one-kernel exact any-hit walk.
struct AnyRecords {
  long long* idx;   // [n] listed rays
  int32_t* npend;   // [n] maybe-triangles listed; kPending + 1: list overflowed
  int32_t* pslot;   // [kPending * n]
  unsigned long long* count;
};

AnyRecords any_records(void* p, int64_t n) {
  char* q = (char*)p;
  AnyRecords r;
  r.count = (unsigned long long*)q;
  q += 256;
  r.idx = (long long*)q;
  q += up256((size_t)n * 8);
  r.npend = (int32_t*)q;
  q += up256((size_t)n * 4);
  r.pslot = (int32_t*)q;
  return r;
}

// ExactAnyLeaf's decisions without its fp64 test: a maybe-triangle is listed.
struct FilterAnyLeaf {
  const SceneView& sv;
  const Ray32& r;
  float tmax_ray;
  float tlim;
  bool done, hit;
  int npend;
  int32_t pend[kPending];

  __device__ FilterAnyLeaf(const SceneView& s, const Ray32& ray) : sv(s), r(ray) { reset(0.0f); }
  __device__ __forceinline__ void reset(float tmax) {
    tmax_ray = tmax;
    tlim = widen(tmax);
    done = false;
    hit = false;
    npend = 0;
  }
  __device__ __forceinline__ void operator()(uint32_t ref) {
    const int cnt = (int)((ref >> 27) & 15u) + 1;
    const int s0 = (int)(ref & kSlotMask);
    for (int k = 0; k < cnt && !done; k++) {
      const int s = s0 + k;
      const float4 A = __ldg(sv.tri + 3 * s);
      const float4 E1 = __ldg(sv.tri + 3 * s + 1);
      const float4 E2 = __ldg(sv.tri + 3 * s + 2);
      const TriClass tc = tri_classify(A, E1, E2, r, tmax_ray, tlim);
      if (tc.state == kHit) {
        hit = true;
        done = true;
      } else if (tc.state == kMaybe) {
        if (npend < kPending) {
          pend[npend++] = s;
        } else {
          npend = kPending + 1;
          done = true;
        }
      }
    }
  }
};

template <int STACK>
__global__ void __launch_bounds__(128, 12) k_any_walk(SceneView sv, const float4* __restrict__ rays, int64_t n,
                                                      uint8_t* __restrict__ out, AnyRecords rec, unsigned* status,
                                                      unsigned long long* work,
                                                      const int32_t* __restrict__ perm) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  long long idx = -1;
  bool exhausted = false;
  Ray32 r = make_ray(0, 0, 0, 0, 0, 0, 0);
  FilterAnyLeaf leaf(sv, r);
  Walker<STACK, kAnyLeafVote> w;
  w.reset(r);
  for (;;) {
    const bool need = idx < 0 && !exhausted;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m && (__popc(m) >= kRefillLanes || !__any_sync(0xffffffffu, idx >= 0))) {
      const int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if ((int)lane == leader) base = atomicAdd(work, (unsigned long long)__popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const unsigned long long my = base + (unsigned long long)__popc(m & below);
        if (my < (unsigned long long)n) {
          idx = perm ? (long long)perm[my] : (long long)my;
          const float4 a = __ldcs(rays + 2 * idx), b = __ldcs(rays + 2 * idx + 1);
          r = make_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w);
          leaf.reset(b.w);
          w.reset(r);
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, idx >= 0)) break;
    if (idx >= 0 && w.step(sv, r, leaf, status)) {
      if (leaf.hit || leaf.npend == 0) {
        out[idx] = leaf.hit ? 1 : 0;
      } else {
        const unsigned long long k = atomicAdd(rec.count, 1ull);
        rec.idx[k] = idx;
        rec.npend[k] = leaf.npend;
        const int np = min(leaf.npend, kPending);
        for (int j = 0; j < np; j++) rec.pslot[(size_t)j * n + k] = leaf.pend[j];
      }
      idx = -1;
    }
  }
}

template <int STACK>
__global__ void __launch_bounds__(128) k_any_settle(SceneView sv, const float4* __restrict__ rays, int64_t n,
                                                    uint8_t* __restrict__ out, AnyRecords rec, unsigned* status) {
  const long long cnt = (long long)*((volatile unsigned long long*)rec.count);
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += (long long)gridDim.x * blockDim.x) {
    const long long i = rec.idx[k];
    const float4 a = __ldcs(rays + 2 * i), b = __ldcs(rays + 2 * i + 1);
    const int np = rec.npend[k];
    if (np > kPending) {
      const Ray32 r = make_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w);
      out[i] = any_hit_exact<STACK, false>(sv, r, b.w, status) ? 1 : 0;
      continue;
    }
    const D3 o{(double)a.x, (double)a.y, (double)a.z}, d{(double)b.x, (double)b.y, (double)b.z};
    bool hit = false;
    for (int j = 0; j < np && !hit; j++) {
      double t;
      hit = tri_hit64(sv.slot64 + 9 * (size_t)rec.pslot[(size_t)j * n + k], o, d, (double)a.w, (double)b.w, &t);
    }
    out[i] = hit ? 1 : 0;
  }
}

template <int STACK>
__global__ void __launch_bounds__(128) k_closest_fast_persistent(SceneView sv, const float4* __restrict__ rays,
                                                                 int64_t n, float* __restrict__ t_out,
                                                                 int32_t* __restrict__ prim_out, unsigned* status,
                                                                 unsigned long long* work,
                                                                 const int32_t* __restrict__ perm) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  long long idx = -1;
  bool exhausted = false;
  Ray32 r = make_ray(0, 0, 0, 0, 0, 0, 0);
  FastClosestLeaf<false> leaf(sv, r, 0.0f);
  FastWalker<STACK, kLeafVote> w;
  w.reset(r);
  for (;;) {
    const bool need = idx < 0 && !exhausted;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m && (__popc(m) >= kRefillLanes || !__any_sync(0xffffffffu, idx >= 0))) {
      const int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if ((int)lane == leader) base = atomicAdd(work, (unsigned long long)__popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const unsigned long long my = base + (unsigned long long)__popc(m & below);
        if (my < (unsigned long long)n) {
          idx = perm ? (long long)perm[my] : (long long)my;
          const float4 a = __ldg(rays + 2 * idx), b = __ldg(rays + 2 * idx + 1);
          r = make_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w);
          leaf.reset(b.w);
          w.reset(r);
        } else {
          exhausted = true;
        }
      }
    }
    const bool active = idx >= 0;
    if (!__any_sync(0xffffffffu, active)) break;
    if (active && w.step(sv, r, leaf, status)) {
      t_out[idx] = leaf.best_slot >= 0 ? leaf.best_t : -1.0f;
      prim_out[idx] = leaf.best_slot >= 0 ? __ldg(sv.slot_prim + leaf.best_slot) : -1;
      idx = -1;
    }
  }
}

// ---- ray order -------------------------------------------------------------------
// Rays are traced in the order of a 21-bit key: the Morton code of the origin
// on a 64^3 grid over the scene bounds, then the direction octant, so a warp's
// rays start near each other and head the same way (fewer divergent node
// visits, better L1 reuse). A counting sort over the 2^21 keys gives the
// permutation; rays and results stay in the caller's order.
constexpr int kKeyBits = 21, kKeyBins = 1 << kKeyBits, kScanBlock = 1024;

__device__ __forceinline__ uint32_t spread3(uint32_t v) {  // 6 bits -> every third bit
  v &= 63u;
  v = (v | (v << 8)) & 0x0000f00fu;
  v = (v | (v << 4)) & 0x000c30c3u;
  v = (v | (v << 2)) & 0x00249249u;
  return v;
}

__global__ void k_ray_keys(const float4* __restrict__ rays, int64_t n, float3 lo, float3 scale,
                           uint32_t* __restrict__ keys, int32_t* __restrict__ bins) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = __ldg(rays + 2 * i), b = __ldg(rays + 2 * i + 1);
  const uint32_t qx = (uint32_t)min(max((a.x - lo.x) * scale.x, 0.0f), 63.0f);
  const uint32_t qy = (uint32_t)min(max((a.y - lo.y) * scale.y, 0.0f), 63.0f);
  const uint32_t qz = (uint32_t)min(max((a.z - lo.z) * scale.z, 0.0f), 63.0f);
  const uint32_t oct = (b.x < 0.0f ? 1u : 0u) | (b.y < 0.0f ? 2u : 0u) | (b.z < 0.0f ? 4u : 0u);
  const uint32_t key = ((spread3(qx) | (spread3(qy) << 1) | (spread3(qz) << 2)) << 3) | oct;  // NaN origins -> 0
  keys[i] = key;
  atomicAdd(&bins[key], 1);
}

// exclusive scan of each 1024-bin block in place; block totals out
__global__ void __launch_bounds__(kScanBlock) k_scan_bins(int32_t* __restrict__ bins, int32_t* __restrict__ totals) {
  __shared__ int32_t sh[kScanBlock];
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  const int v = bins[i];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    const int add = (int)threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += add;
    __syncthreads();
  }
  bins[i] = sh[threadIdx.x] - v;
  if (threadIdx.x == kScanBlock - 1) totals[blockIdx.x] = sh[threadIdx.x];
}

// exclusive scan of the block totals (kKeyBins / kScanBlock = 2048 of them), one block
__global__ void __launch_bounds__(kScanBlock) k_scan_totals(int32_t* __restrict__ totals) {
  __shared__ int32_t sh[kScanBlock];
  const int a = totals[2 * threadIdx.x], b = totals[2 * threadIdx.x + 1];
  sh[threadIdx.x] = a + b;
  __syncthreads();
  for (int o = 1; o < kScanBlock; o <<= 1) {
    const int add = (int)threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += add;
    __syncthreads();
  }
  const int ex = sh[threadIdx.x] - (a + b);
  totals[2 * threadIdx.x] = ex;
  totals[2 * threadIdx.x + 1] = ex + a;
}

__global__ void k_ray_scatter(int64_t n, const uint32_t* __restrict__ keys, int32_t* __restrict__ bins,
                              const int32_t* __restrict__ totals, int32_t* __restrict__ perm) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = keys[i];
  perm[totals[k / kScanBlock] + atomicAdd(&bins[k], 1)] = (int32_t)i;
}

// ---- exact ties: the reference's own walk ------------------------------------
// A ray marked kTieMark has its closest fp64 distance shared by two or more
// primitives. Which of them the reference returns depends on its traversal
// order: triHit accepts t == closest (renderer.go:702), so the last one tested
// at that distance wins. Such a ray is walked again here exactly as Scene.Hit
// walks the caller's binary BVH (renderer.go:777-849): a 16-entry stack of
// (node, entry distance); a popped entry at or beyond the closest hit is
// skipped (796); a leaf tests its primitives in Order (800-808); both children
// are box-tested against the closest hit and pushed far first, the left one
// nearer on equal entry distances (828-839); with the stack full, the
// recursive descent of hitRecursive (815-826, 914-939) takes the left subtree,
// then the right one, each node box-tested when it is reached. Arithmetic is
// fp64 in the reference's operation order: prepareRay and HitAccel
// (renderer.go:59-81, 147-210), triHit and sphereHitAccel.
constexpr int kReplayDepth = 256;  // pending subtrees of the recursive descent

struct Accel64 {
  D3 o, inv;
  bool zx, zy, zz;
};

// One slab of HitAccel: an axis with |d| < 1e-15 only checks the origin.
__device__ __forceinline__ bool slab64(bool zero, double o, double inv, double mn, double mx, double* near,
                                       double* far) {
  if (zero) return !(o < mn || o > mx);
  double t0 = __dmul_rn(__dsub_rn(mn, o), inv);
  double t1 = __dmul_rn(__dsub_rn(mx, o), inv);
  if (inv < 0) {
    const double x = t0;
    t0 = t1;
    t1 = x;
  }
  if (t0 > *near) *near = t0;
  if (t1 < *far) *far = t1;
  return !(*far <= *near);
}

__device__ __forceinline__ bool box64(const BinNode* __restrict__ b, const Accel64& a, double tmin, double tmax,
                                      double* near_out) {
  double near = tmin, far = tmax;
  if (!slab64(a.zx, a.o.x, a.inv.x, __ldg(&b->lo[0]), __ldg(&b->hi[0]), &near, &far)) return false;
  if (!slab64(a.zy, a.o.y, a.inv.y, __ldg(&b->lo[1]), __ldg(&b->hi[1]), &near, &far)) return false;
  if (!slab64(a.zz, a.o.z, a.inv.z, __ldg(&b->lo[2]), __ldg(&b->hi[2]), &near, &far)) return false;
  *near_out = near;
  return true;
}

// A leaf's primitives in Order; each accepted hit becomes the closest.
__device__ __forceinline__ void leaf64(const SceneView& sv, const BinNode* __restrict__ b, D3 o, D3 d, double tmin,
                                       double* closest, int* best) {
  const int s0 = __ldg(&b->start), cnt = __ldg(&b->count);
  for (int k = 0; k < cnt; k++) {
    const int s = s0 + k;
    const bool sphere = __ldg(reinterpret_cast<const float*>(sv.tri + 3 * (size_t)s + 2) + 3) < 0.0f;
    double t;
    const bool hit = sphere ? sphere_hit64(sv.slot64 + 9 * (size_t)s, o, d, tmin, *closest, &t)
                            : tri_hit64(sv.slot64 + 9 * (size_t)s, o, d, tmin, *closest, &t);
    if (hit) {
      *closest = t;
      *best = s;
    }
  }
}

// Returns the winning slot (-1: miss) and its distance.
__device__ int replay_closest(const SceneView& sv, const BinNode* __restrict__ bin, D3 o, D3 d, double tmin,
                              double tmax, double* t_out, unsigned* status) {
  Accel64 a;
  a.o = o;
  a.zx = fabs(d.x) < 1e-15;
  a.zy = fabs(d.y) < 1e-15;
  a.zz = fabs(d.z) < 1e-15;
  a.inv.x = a.zx ? 0.0 : __ddiv_rn(1.0, d.x);
  a.inv.y = a.zy ? 0.0 : __ddiv_rn(1.0, d.y);
  a.inv.z = a.zz ? 0.0 : __ddiv_rn(1.0, d.z);
  double closest = tmax;
  int best = -1;
  double root_near;
  if (!box64(bin, a, tmin, tmax, &root_near)) return -1;
  int sn[16];
  double sd[16];
  int dfs[kReplayDepth];
  int sp = 1;
  sn[0] = 0;
  sd[0] = root_near;
  while (sp > 0) {
    sp--;
    if (sd[sp] >= closest) continue;
    const BinNode* n = bin + sn[sp];
    if (__ldg(&n->count) > 0) {
      leaf64(sv, n, o, d, tmin, &closest, &best);
      continue;
    }
    const int l = __ldg(&n->left), r = __ldg(&n->right);
    double ln = 0.0, rn = 0.0;
    const bool lok = box64(bin + l, a, tmin, closest, &ln);
    const bool rok = box64(bin + r, a, tmin, closest, &rn);
    if (!lok && !rok) continue;
    if (sp + 2 > 16) {  // hitRecursive on the left child, then on the right one
      int dp = 0;
      if (rok) dfs[dp++] = r;
      if (lok) dfs[dp++] = l;
      while (dp > 0) {
        const BinNode* m = bin + dfs[--dp];
        double mn;
        if (!box64(m, a, tmin, closest, &mn)) continue;
        if (__ldg(&m->count) > 0) {
          leaf64(sv, m, o, d, tmin, &closest, &best);
          continue;
        }
        if (dp + 2 > kReplayDepth) {  // a tree deeper than the replay holds: report, never guess
          atomicOr(status, kStatusStackOverflow);
          return -1;
        }
        dfs[dp++] = __ldg(&m->right);
        dfs[dp++] = __ldg(&m->left);
      }
      continue;
    }
    if (lok && rok) {
      if (ln <= rn) {
        sn[sp] = r; sd[sp++] = rn;
        sn[sp] = l; sd[sp++] = ln;
      } else {
        sn[sp] = l; sd[sp++] = ln;
        sn[sp] = r; sd[sp++] = rn;
      }
    } else if (lok) {
      sn[sp] = l; sd[sp++] = ln;
    } else {
      sn[sp] = r; sd[sp++] = rn;
    }
  }
  *t_out = closest;
  return best;
}

__global__ void __launch_bounds__(128) k_tie_replay(SceneView sv, const BinNode* __restrict__ bin,
                                                    const float4* __restrict__ rays, int64_t n,
                                                    float* __restrict__ t_out, int32_t* __restrict__ prim_out,
                                                    unsigned* status) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (prim_out[i] != kTieMark) continue;
    const float4 a = __ldg(rays + 2 * i), b = __ldg(rays + 2 * i + 1);
    const D3 o{(double)a.x, (double)a.y, (double)a.z}, d{(double)b.x, (double)b.y, (double)b.z};
    double t = 0.0;
    const int s = replay_closest(sv, bin, o, d, (double)a.w, (double)b.w, &t, status);
    t_out[i] = s >= 0 ? __double2float_rn(t) : -1.0f;
    prim_out[i] = s >= 0 ? __ldg(sv.slot_prim + s) : -1;
  }
}

template <class K>
int persistent_blocks(K kernel) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 128, 0);
  return sms * (per > 0 ? per : 1);
}

SceneView view_of(const DeviceScene& s) {
  SceneView v;
  v.nodes = s.nodes;
  v.tri = s.tri;
  v.slot64 = s.slot64;
  v.snorm = s.snorm;
  v.slot_prim = s.slot_prim;
  return v;
}

// Occupancy variants: MINB = minimum resident 128-thread blocks per SM the
// register allocation must allow (1: unconstrained, 6: <= 80 registers,
// 8: <= 64 registers). Selected per context (bc_set_option "raycast_minblocks").
template <int STACK, int MINB>
cudaError_t closest_stack(const DeviceScene& s, const float4* rays, int64_t n, float* t, int32_t* p, unsigned* status,
                          unsigned long long* work, const int32_t* perm, cudaStream_t st) {
  const int64_t grid = (n + 127) / 128;
  if (s.has_spheres) {
    k_closest_exact<STACK, true, MINB><<<(unsigned)grid, 128, 0, st>>>(view_of(s), rays, n, t, p, status);
  } else {
    static int blocks = 0;
    if (!blocks) blocks = persistent_blocks(k_closest_exact_persistent<STACK, MINB>);
    cudaError_t e = cudaMemsetAsync(work, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    const int g = (int)std::min<int64_t>(blocks, (n + 127) / 128);
    k_closest_exact_persistent<STACK, MINB><<<g, 128, 0, st>>>(view_of(s), rays, n, t, p, status, work, perm);
  }
  return cudaGetLastError();
}

template <int STACK>
cudaError_t closest_split(const DeviceScene& s, const float4* rays, int64_t n, float* t, int32_t* p, unsigned* status,
                          unsigned long long* work, const int32_t* perm, void* rec_scratch, cudaStream_t st) {
  static int blocks = 0;
  if (!blocks) blocks = persistent_blocks(k_exact_walk<STACK>);
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms < 1) sms = 1;
  }
  const ExactRecords rec = exact_records(rec_scratch, n);
  cudaError_t e = cudaMemsetAsync(work, 0, sizeof(unsigned long long), st);
  if (!e) e = cudaMemsetAsync(rec.n_redo, 0, sizeof(unsigned long long), st);
  if (e) return e;
  const int64_t grid = (n + 127) / 128;
  k_exact_walk<STACK><<<(int)std::min<int64_t>(blocks, grid), 128, 0, st>>>(view_of(s), rays, n, rec, status, work,
                                                                           perm);
  k_exact_settle<<<(int)std::min<int64_t>((int64_t)sms * 16, grid), 128, 0, st>>>(view_of(s), rays, n, rec, t, p,
                                                                                 status);
  k_closest_exact_list<STACK><<<sms * 4, 128, 0, st>>>(view_of(s), rays, rec, t, p, status);
  return cudaGetLastError();
}

template <int STACK>
cudaError_t any_split(const DeviceScene& s, const float4* rays, int64_t n, uint8_t* out, unsigned* status,
                      unsigned long long* work, void* rec_scratch, const int32_t* perm, cudaStream_t st) {
  static int blocks = 0;
  if (!blocks) blocks = persistent_blocks(k_any_walk<STACK>);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const AnyRecords rec = any_records(rec_scratch, n);
  cudaError_t e = cudaMemsetAsync(work, 0, sizeof(unsigned long long), st);
  if (!e) e = cudaMemsetAsync(rec.count, 0, sizeof(unsigned long long), st);
  if (e) return e;
  const int64_t grid = (n + 127) / 128;
  k_any_walk<STACK><<<(int)std::min<int64_t>(blocks, grid), 128, 0, st>>>(view_of(s), rays, n, out, rec, status, work, perm);
  k_any_settle<STACK><<<std::max(sms, 1) * 4, 128, 0, st>>>(view_of(s), rays, n, out, rec, status);
  return cudaGetLastError();
}

template <int STACK, int MINB>
cudaError_t any_stack(const DeviceScene& s, const float4* rays, int64_t n, uint8_t* out, unsigned* status,
                      cudaStream_t st) {
  const int64_t grid = (n + 127) / 128;
  if (s.has_spheres)
    k_any_exact<STACK, true, MINB><<<(unsigned)grid, 128, 0, st>>>(view_of(s), rays, n, out, status);
  else
    k_any_exact<STACK, false, MINB><<<(unsigned)grid, 128, 0, st>>>(view_of(s), rays, n, out, status);
  return cudaGetLastError();
}

template <int STACK>
cudaError_t closest_var(const DeviceScene& s, const float4* rays, int64_t n, float* t, int32_t* p, unsigned* status,
                        unsigned long long* work, int variant, const int32_t* perm, void* rec_scratch,
                        cudaStream_t st) {
  if (variant != 0 && rec_scratch && !s.has_spheres)
    return closest_split<STACK>(s, rays, n, t, p, status, work, perm, rec_scratch, st);
  if (variant == 0) {  // fast, not exact
    const int64_t grid = (n + 127) / 128;
    if (s.has_spheres) {
      k_closest_fast<STACK, true><<<(unsigned)grid, 128, 0, st>>>(view_of(s), rays, n, t, p, status);
    } else {
      static int blocks = 0;
      if (!blocks) blocks = persistent_blocks(k_closest_fast_persistent<STACK>);
      cudaError_t e = cudaMemsetAsync(work, 0, sizeof(unsigned long long), st);
      if (e != cudaSuccess) return e;
      const int g = (int)std::min<int64_t>(blocks, grid);
      k_closest_fast_persistent<STACK><<<g, 128, 0, st>>>(view_of(s), rays, n, t, p, status, work, perm);
    }
    return cudaGetLastError();
  }
  switch (variant) {
    case 6: return closest_stack<STACK, 6>(s, rays, n, t, p, status, work, perm, st);
    case 8: return closest_stack<STACK, 8>(s, rays, n, t, p, status, work, perm, st);
    default: return closest_stack<STACK, 1>(s, rays, n, t, p, status, work, perm, st);
  }
}

template <int STACK>
cudaError_t any_var(const DeviceScene& s, const float4* rays, int64_t n, uint8_t* out, unsigned* status, int variant,
                    unsigned long long* work, void* rec_scratch, const int32_t* perm, cudaStream_t st) {
  if (rec_scratch && work && !s.has_spheres)
    return any_split<STACK>(s, rays, n, out, status, work, rec_scratch, perm, st);
  switch (variant) {
    case 6: return any_stack<STACK, 6>(s, rays, n, out, status, st);
    case 8: return any_stack<STACK, 8>(s, rays, n, out, status, st);
    default: return any_stack<STACK, 1>(s, rays, n, out, status, st);
  }
}

}  // namespace

size_t any_record_bytes(int64_t n) {
  return 256 + up256((size_t)n * 8) + up256((size_t)n * 4) + up256((size_t)n * 4 * kPending);
}

size_t exact_record_bytes(int64_t n) {
  return 256 + 3 * up256((size_t)n * 4) + 2 * up256((size_t)n * 4 * kPending) + up256((size_t)n * 8);
}

size_t ray_order_bytes(int64_t n) {
  return (size_t)kKeyBins * 4 + (size_t)(kKeyBins / kScanBlock) * 4 + (size_t)n * 8 + 4 * 256;
}

// Spatially coherent ray order (see k_ray_keys) into order_scratch; *perm is
// left NULL when the batch is not ordered (no scratch, fewer than
// kMinOrderedRays rays, 2^31 rays or more: the order holds 32-bit indices, or a
// scene with spheres, whose kernels read rays in order).
static cudaError_t order_rays(const DeviceScene& s, const float4* rays, int64_t n, void* order_scratch,
                              const int32_t** perm, cudaStream_t st) {
  *perm = nullptr;
  if (!order_scratch || n < kMinOrderedRays || n >= (int64_t(1) << 31) || s.has_spheres) return cudaSuccess;
  char* q = (char*)order_scratch;
  int32_t* bins = (int32_t*)q;
  int32_t* totals = (int32_t*)(q + (size_t)kKeyBins * 4);
  uint32_t* keys = (uint32_t*)(q + (size_t)kKeyBins * 4 + ((kKeyBins / kScanBlock) * 4 + 255) / 256 * 256);
  int32_t* pm = (int32_t*)((char*)keys + ((size_t)n * 4 + 255) / 256 * 256);
  cudaError_t e = cudaMemsetAsync(bins, 0, (size_t)kKeyBins * 4, st);
  if (e) return e;
  const float3 lo = make_float3(s.lo[0], s.lo[1], s.lo[2]);
  auto sc = [](float a, float b) { return b > a ? 64.0f / (b - a) : 0.0f; };
  const float3 scale = make_float3(sc(s.lo[0], s.hi[0]), sc(s.lo[1], s.hi[1]), sc(s.lo[2], s.hi[2]));
  const unsigned g = (unsigned)((n + 255) / 256);
  k_ray_keys<<<g, 256, 0, st>>>(rays, n, lo, scale, keys, bins);
  k_scan_bins<<<kKeyBins / kScanBlock, kScanBlock, 0, st>>>(bins, totals);
  k_scan_totals<<<1, kScanBlock, 0, st>>>(totals);
  k_ray_scatter<<<g, 256, 0, st>>>(n, keys, bins, totals, pm);
  if ((e = cudaGetLastError())) return e;
  *perm = pm;
  return cudaSuccess;
}

cudaError_t launch_raycast_closest(const DeviceScene& s, const float4* rays, int64_t n, float* t_out,
                                   int32_t* prim_out, unsigned* status, unsigned long long* work, int variant,
                                   void* order_scratch, void* rec_scratch, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int32_t* perm = nullptr;
  cudaError_t e = order_rays(s, rays, n, order_scratch, &perm, st);
  if (e) return e;
  switch (stack_variant(s.stack_need)) {
    case 64: e = closest_var<64>(s, rays, n, t_out, prim_out, status, work, variant, perm, rec_scratch, st); break;
    case 128: e = closest_var<128>(s, rays, n, t_out, prim_out, status, work, variant, perm, rec_scratch, st); break;
    case 256: e = closest_var<256>(s, rays, n, t_out, prim_out, status, work, variant, perm, rec_scratch, st); break;
    default: return cudaErrorInvalidValue;
  }
  if (e || variant == 0) return e;  // the plain fp32 form makes no tie promise
  if (!s.bin) return cudaErrorInvalidValue;  // every uploaded scene carries its binary tree
  // exact ties: rays the passes above marked are walked again as the reference walks them
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms < 1) sms = 1;
  }
  k_tie_replay<<<(int)std::min<int64_t>((int64_t)sms * 4, (n + 127) / 128), 128, 0, st>>>(view_of(s), s.bin, rays, n,
                                                                                        t_out, prim_out, status);
  return cudaGetLastError();
}

cudaError_t launch_raycast_any(const DeviceScene& s, const float4* rays, int64_t n, uint8_t* out, unsigned* status,
                               int variant, unsigned long long* work, void* rec_scratch, void* order_scratch,
                               cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int32_t* perm = nullptr;
  if (rec_scratch) {  // only the split walk reads rays through the order
    cudaError_t e = order_rays(s, rays, n, order_scratch, &perm, st);
    if (e) return e;
  }
  switch (stack_variant(s.stack_need)) {
    case 64: return any_var<64>(s, rays, n, out, status, variant, work, rec_scratch, perm, st);
    case 128: return any_var<128>(s, rays, n, out, status, variant, work, rec_scratch, perm, st);
    case 256: return any_var<256>(s, rays, n, out, status, variant, work, rec_scratch, perm, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace bcgx

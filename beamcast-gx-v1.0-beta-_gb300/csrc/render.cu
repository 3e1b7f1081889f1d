// Wavefront path tracer: the reference CPU integrator (trace, renderer.go:1484-1563;
// directLight 1427-1465; adaptivePixel's sample loop 1928-1970) as separate
// kernels over compacted queues of path slots, for one view or a batch of
// views over a resident scene set:
//
//   generate  -> the wave's paths: global path index -> (view, sample, pixel);
//                Halton jitter with the per-pixel rotation, float-float primary
//                ray (rounded to fp32), one PCG32 stream per (pixel, sample)
//   extend    -> closest hit of every queued path from its view's scene root
//                (persistent: idle lanes take the next paths once a few of the
//                warp's lanes are idle)
//   shade     -> miss / emissive (MIS weight) / diffuse (NEE shadow ray + cosine
//                bounce) / metal / glass, Russian roulette; survivors are pushed
//                with block-level compaction (one atomic per block), shadow rays
//                with warp-ballot compaction (one atomic per warp)
//   connect   -> any hit for the shadow queue; unoccluded contributions are added
//   accumulate-> per pixel, the firefly-clamped sample radiance of the wave,
//                summed in sample order (no atomics: one thread per pixel)
//   advance   -> moves the device-side wave start
//
// Every view's paths are sample-major (path = sample * npix + pixel) in one
// global index space; a wave is the next `cap` indices, read from device
// memory, so the same launch sequence (or one CUDA graph of it) is replayed
// until the batch is done. Each (pixel, sample) draws from its own seeded
// stream, so an image does not depend on the wave split or the launch shape.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "context.h"
#include "photon.cuh"
#include "sampling.cuh"
#include "trace_core.cuh"
#include "wave.h"

namespace bcgx {

struct PathSoA {
  float *ox, *oy, *oz, *dx, *dy, *dz;
  float *tx, *ty, *tz;     // throughput
  float *lx, *ly, *lz;     // radiance of the path so far
  float *px, *py, *pz;     // prevPoint
  uint32_t* prev;          // prevBSDFPDF (fp32, >= 0) in bits 0-30, prevWasDiffuse in bit 31
  uint64_t *rs, *ri;       // PCG32 state and increment
  float* hit_t;
  int32_t* hit_slot;
  int32_t* view;           // view of the path
  int32_t* pix;            // pixel within the view's rows
  int32_t* samp;           // sample index
};

struct ShadowSoA {
  float4* o;  // origin, tmax
  float4* d;  // direction
  float4* c;  // contribution (already multiplied by the path throughput)
  int32_t* path;
};

// Path replay records of a gradient render: for every path and bounce, the
// material whose parameter the vertex depends on and the value the adjoint
// needs (diffuse: radiance gathered before the albedo multiplied the
// throughput; emitter: throughput times MIS weight). m < 0: no record.
constexpr int kEmitTag = 1 << 30;
struct GradRec {
  int32_t* m;   // [bounce * cap + path]
  float4* v;    // [bounce * cap + path]
  int32_t* nb;  // bounces shaded per path
  int cap;
};

// Vertex records of the recursive integrator (traceRecursiveInner,
// renderer.go:1569-1621). The reference samples directLight at a diffuse vertex
// after tracing the subtree below it, so a path draws all its light samples
// after its last bounce, deepest vertex first. A diffuse vertex records its
// point, material, facing normal and the weight its directLight term carries;
// when the path ends, the records are unwound in that order (each draws its
// light sample and queues its shadow ray) and overwritten with the sample's
// contribution and a visibility flag, which the accumulation adds up.
struct RecurRec {
  float4* a;    // [bounce * cap + path]: (point, material bits; < 0: no light sample), then (contribution, visible)
  float4* n;    // (facing normal, 0)
  float4* w;    // (weight of the vertex's directLight term, 0)
  int32_t* nb;  // vertices shaded per path
  int cap;
};

// Device counters of a wave. cur/next alternate between [0] and [1].
struct WaveCounters {
  int q[2];
  int shadow;
  int work_ext;
  int work_con;
  int pad[3];
  unsigned long long rays;
  unsigned long long shadow_rays;
};

// One view of a batch (or the single view of a frame / row chunk).
struct ViewGPU {
  double origin[3], lower[3], horiz[3], vert[3];
  // primary-ray constants as float-float pairs (hi, lo), from the fp64 basis on
  // the host: the lower-left corner relative to the origin (no cancellation on
  // the device), the two spans, the reciprocals of max(W - 1, 1) and
  // max(H - 1, 1); and the origin rounded to fp32
  float2 base[3], span_u[3], span_v[3], inv_w1, inv_h1;
  float o32[3];
  long long path_off;  // first global path index of the view
  long long pix_off;   // first pixel of the view's rows in the frame buffers
  int W, H, y0, rows, npix;
  int spp, bounces, rr_depth, sampler, mis, power;
  int nseq, seq_off;   // Halton table slice
  int n_lights, light_off, root;
  int want_guides;
  float clamp;
  int adaptive;       // adaptivePixel's early stop (renderer.go:1961-1968)
  float adapt_thr;    // max(1e-8, AdaptiveThreshold)
  int min_samples;    // min(8, spp)
  int integrator;     // BC_INTEGRATOR_* (pixelRadiance, renderer.go:1833-1842)
  unsigned long long seed;
  PhotonView pm;      // photon integrator: the frame's photon map (null table: empty map)
};

// Per-pixel state of the adaptive stop: samples accumulated, luminance sums.
struct AdaptState {
  int32_t* n;       // samples accumulated; bit 31: the pixel has stopped
  float2* lum;      // (sum of luminance, sum of squared luminance)
};
constexpr int32_t kPixDone = int32_t(0x80000000u);

// luminance (renderer.go:2142)
__device__ __forceinline__ float luminance3(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }

// One sample of an adaptive pixel: updates the luminance sums and the count;
// true when the pixel stops after this sample (renderer.go:1957-1968).
__device__ __forceinline__ bool adaptive_step(const ViewGPU& V, float3 c, int* n, float* sl, float* ssl) {
  const float l = luminance3(c);
  *sl += l;
  *ssl += l * l;
  *n += 1;
  if (*n >= V.min_samples && (*n & 1) == 0) {
    const float nn = (float)*n;
    const float mean = *sl / nn;
    const float var = fmaxf(0.0f, *ssl / nn - mean * mean);
    return var < V.adapt_thr;
  }
  return false;
}

// Device-side wave cursor of a batch.
struct BatchState {
  long long w0;     // first global path index of the current wave
  long long total;  // paths of the batch
  int cap;          // paths per wave
  int n_views;
};

constexpr float kPi = 3.14159265358979323846f;
constexpr int kMaxBounces = 1024;  // a wave is one launch sequence of max(bounces) steps

// The path state streams through L2 once per kernel (tens of bytes per path,
// gigabytes per wave), so its loads and stores are marked evict-first
// (ld.global.cs / st.global.cs): L2 stays with the BVH nodes and triangle
// records the walks reuse.
__device__ __forceinline__ float sld(const float* p) { return __ldcs(p); }
__device__ __forceinline__ int32_t sld(const int32_t* p) { return __ldcs(p); }
__device__ __forceinline__ uint32_t sld(const uint32_t* p) { return __ldcs(p); }
__device__ __forceinline__ uint64_t sld(const uint64_t* p) {
  return __ldcs(reinterpret_cast<const unsigned long long*>(p));
}
__device__ __forceinline__ void sst(float* p, float v) { __stcs(p, v); }
__device__ __forceinline__ void sst(int32_t* p, int32_t v) { __stcs(p, v); }
__device__ __forceinline__ void sst(uint32_t* p, uint32_t v) { __stcs(p, v); }
__device__ __forceinline__ void sst(uint64_t* p, uint64_t v) {
  __stcs(reinterpret_cast<unsigned long long*>(p), (unsigned long long)v);
}

__device__ __forceinline__ int warp_reserve(int* counter, bool pred) {
  const unsigned lane = threadIdx.x & 31u;
  const unsigned mask = __ballot_sync(0xffffffffu, pred);
  int base = 0;
  if (mask) {
    const int leader = __ffs(mask) - 1;
    if ((int)lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
  }
  return base + __popc(mask & ((1u << lane) - 1u));
}

// Queue slots for a block's surviving paths, in thread order, with one atomic
// per block on the queue counter (per warp, the shading kernel's grid would
// put hundreds of thousands of atomics on that one word every bounce). Every
// thread of the block calls it; returns -1 where `alive` is false.
template <int BLOCK>
__device__ __forceinline__ int block_reserve(int* counter, bool alive) {
  constexpr int kWarps = BLOCK / 32;
  __shared__ int wbase[kWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned m = __ballot_sync(0xffffffffu, alive);
  if (lane == 0) wbase[warp] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < kWarps; w++) {
      const int c = wbase[w];
      wbase[w] = s;
      s += c;
    }
    const int base = s ? atomicAdd(counter, s) : 0;
    for (int w = 0; w < kWarps; w++) wbase[w] += base;
  }
  __syncthreads();
  const int pos = alive ? wbase[warp] + __popc(m & ((1u << lane) - 1u)) : -1;
  __syncthreads();  // the next call rewrites wbase
  return pos;
}

__device__ __forceinline__ int view_of(const ViewGPU* __restrict__ views, int n_views, long long g) {
  int lo = 0, hi = n_views - 1;  // last view with path_off <= g
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (views[mid].path_off <= g) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ---- float-float arithmetic (primary rays) ------------------------------------
// A value is hi + lo with |lo| <= ulp(hi) / 2. TwoSum (Knuth, TAOCP vol. 2,
// 4.2.2) and the FMA form of Dekker's TwoProduct give exact rounding errors;
// sums use Dekker's add2 ("A floating-point technique for extending the
// available precision", Numer. Math. 18, 1971), whose error stays below 2^-44 of
// the larger operand. The _rn intrinsics keep the compiler from contracting or
// reassociating the error terms.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_of(float2 v) { return FF{v.x, v.y}; }
__device__ __forceinline__ FF ff_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return FF{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ FF ff_fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = __fadd_rn(a, b);
  return FF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const FF s = ff_two_sum(a.hi, b.hi);
  return ff_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return ff_fast_two_sum(p, e);
}

// ---- generate --------------------------------------------------------------
// Primary ray of sample s of pixel (x, y) and the path's stream (adaptivePixel's
// sample loop, renderer.go:1940-1950): Halton / R2 jitter rotated per pixel, or
// random jitter; the camera arithmetic in float-float (about 48 significant
// bits, from the host's fp64 basis), rounded to fp32 once. GB300's fp64 pipe
// runs at a small fraction of its fp32 rate, and the fp64 form of this
// arithmetic (some 25 fp64 operations a sample) bounded k_generate. The pixel
// coordinate is scaled by a reciprocal, and the direction is
// (lower - origin) + u horiz + v vert with the first term from the host; against
// the reference's fp64 operation order the direction moves by ~2^-44 of the
// camera vectors' size before the fp32 rounding, which it changes only when the
// fp64 value lies that close to a rounding boundary.
// seq: per sample (x hi, x lo, y hi, y lo) of the view's sample table.
__device__ __forceinline__ void primary_ray(const ViewGPU& V, int x, int y, int s, const float4* __restrict__ seq,
                                            float3* o, float3* d, Pcg32* rng, float* jx_out, float* jy_out) {
  *rng = make_path_rng(V.seed, (uint64_t)y * (uint64_t)V.W + (uint64_t)x, (uint64_t)s);
  FF jx, jy;
  if (V.sampler != BC_SAMPLER_RANDOM && s < V.nseq) {
    // the per-pixel rotation h * 2^-32 split exactly into 24 + 8 bits
    uint32_t h1, h2;
    pixel_rotation_bits(x, y, &h1, &h2);
    const float k24 = 1.0f / 16777216.0f, k32 = 1.0f / 4294967296.0f;
    const FF rx{(float)(h1 >> 8) * k24, (float)(h1 & 255u) * k32};
    const FF ry{(float)(h2 >> 8) * k24, (float)(h2 & 255u) * k32};
    const float4 q = __ldg(seq + V.seq_off + s);
    // fract(q + r) with q, r in [0, 1): the sum lies in [0, 2); hi - 1 is exact
    // (Sterbenz) when the sum is at least 1
    const FF a = ff_add(FF{q.x, q.y}, rx), b = ff_add(FF{q.z, q.w}, ry);
    jx = (a.hi > 1.0f || (a.hi == 1.0f && a.lo >= 0.0f)) ? ff_fast_two_sum(a.hi - 1.0f, a.lo) : a;
    jy = (b.hi > 1.0f || (b.hi == 1.0f && b.lo >= 0.0f)) ? ff_fast_two_sum(b.hi - 1.0f, b.lo) : b;
  } else {
    jx = FF{rng->uniform(), 0.0f};
    jy = FF{rng->uniform(), 0.0f};
  }
  const FF u = ff_mul(ff_add(FF{(float)x, 0.0f}, jx), ff_of(V.inv_w1));
  const FF vv = ff_mul(ff_add(FF{(float)(V.H - 1 - y), 0.0f}, jy), ff_of(V.inv_h1));
  float dd[3];
#pragma unroll
  for (int k = 0; k < 3; k++)
    dd[k] = ff_add(ff_add(ff_of(V.base[k]), ff_mul(ff_of(V.span_u[k]), u)), ff_mul(ff_of(V.span_v[k]), vv)).hi;
  *o = f3(V.o32[0], V.o32[1], V.o32[2]);
  *d = f3(dd[0], dd[1], dd[2]);
  *jx_out = jx.hi;
  *jy_out = jy.hi;
}

__device__ __forceinline__ uint32_t jitter_word(float jx, float jy) {
  uint32_t a = (uint32_t)rintf(fminf(fmaxf(jx, 0.0f), 1.0f) * 65535.0f);
  uint32_t b = (uint32_t)rintf(fminf(fmaxf(jy, 0.0f), 1.0f) * 65535.0f);
  return (b << 16) | a;
}

// seq: the views' sample tables, (x, y) pairs
// The wave's paths of pixels that have not stopped (adaptive sampling) enter
// the first queue (warp-aggregated append; cnt->q[0] is zero on entry).
__global__ void k_generate(const BatchState* __restrict__ bs, const ViewGPU* __restrict__ views, PathSoA ps,
                           int* __restrict__ queue, const float4* __restrict__ seq,
                           uint32_t* __restrict__ guide_jit, WaveCounters* cnt, AdaptState ad) {
  const long long w0 = bs->w0;
  const int n = (int)min((long long)bs->cap, bs->total - w0);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) cnt->work_ext = 0;
  int v = 0, s = 0, p = 0;
  bool live = i < n;
  if (live) {
    const long long g = w0 + i;
    v = view_of(views, bs->n_views, g);
    const long long local = g - views[v].path_off;
    s = (int)(local / views[v].npix);
    p = (int)(local - (long long)s * views[v].npix);
    if (views[v].adaptive && (ad.n[views[v].pix_off + p] & kPixDone)) live = false;
  }
  const int slot = block_reserve<256>(&cnt->q[0], live);  // launched with 256-thread blocks
  if (!live) return;
  const ViewGPU& V = views[v];
  const int x = p % V.W, y = V.y0 + p / V.W;
  float3 o, d;
  Pcg32 rng;
  float jx, jy;
  primary_ray(V, x, y, s, seq, &o, &d, &rng, &jx, &jy);
  sst(ps.ox + i, o.x); sst(ps.oy + i, o.y); sst(ps.oz + i, o.z);
  sst(ps.dx + i, d.x); sst(ps.dy + i, d.y); sst(ps.dz + i, d.z);
  sst(ps.tx + i, 1.0f); sst(ps.ty + i, 1.0f); sst(ps.tz + i, 1.0f);
  sst(ps.lx + i, 0.0f); sst(ps.ly + i, 0.0f); sst(ps.lz + i, 0.0f);
  sst(ps.prev + i, 0u);
  sst(ps.rs + i, rng.state);
  sst(ps.ri + i, rng.inc);
  sst(ps.view + i, (int32_t)v);
  sst(ps.pix + i, (int32_t)p);
  sst(ps.samp + i, (int32_t)s);
  queue[slot] = i;
  if (s == 0 && V.want_guides) guide_jit[V.pix_off + p] = jitter_word(jx, jy);
}

// ---- extend ----------------------------------------------------------------
// Persistent: idle lanes take the next queue entries once kRefillLanes of the
// warp's lanes are idle (one atomic per warp for all of them). The walk is latency-bound, so
// resident warps matter; three variants trade registers against them
// (bc_set_option "render_extend", chosen per workload by bc_autotune_render):
//   0: the ray in registers, no register budget (56 registers, nine 128-thread
//      blocks per SM);
//   1: the ray in registers, 48 registers (ten blocks; ptxas spills 26 bytes);
//   2: each thread's ray in shared memory, which the triangle tests read (the
//      node test keeps its per-ray constants in registers): 40 registers
//      (82 bytes spilled), twelve blocks.
// All three compute the same hits.
constexpr int kExtendVariants = 3;

template <int STACK, bool SPH, int VAR>
__device__ __forceinline__ void extend_body(SceneView sv, const ViewGPU* __restrict__ views, PathSoA ps,
                                            const int* __restrict__ queue, WaveCounters* cnt, int cur,
                                            unsigned* status) {
  const int n = *((volatile int*)&cnt->q[cur]);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    atomicAdd(&cnt->rays, (unsigned long long)n);
    cnt->q[cur ^ 1] = 0;  // the queue and shadow list this bounce's shade fills
    cnt->shadow = 0;
  }
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  int path = -1;
  bool exhausted = false;
  __shared__ Ray32 ray_sh[VAR == 2 ? 128 : 1];
  Ray32 ray_reg;
  Ray32& r = VAR == 2 ? ray_sh[threadIdx.x] : ray_reg;
  r = make_ray(0, 0, 0, 0, 0, 0, 0);
  FastClosestLeaf<SPH> leaf(sv, r, 1e30f);
  FastWalker<STACK, kLeafVote> w;
  w.reset(r);
  for (;;) {
    const bool need = path < 0 && !exhausted;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m && (__popc(m) >= kRefillLanes || !__any_sync(0xffffffffu, path >= 0))) {
      const int leader = __ffs(m) - 1;
      int base = 0;
      if ((int)lane == leader) base = atomicAdd(&cnt->work_ext, __popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const int my = base + __popc(m & below);
        if (my < n) {
          path = queue[my];
          r = make_ray(sld(ps.ox + path), sld(ps.oy + path), sld(ps.oz + path), sld(ps.dx + path),
                       sld(ps.dy + path), sld(ps.dz + path), 1e-4f);
          leaf.reset(1e30f);
          w.reset(r, views[sld(ps.view + path)].root);
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, path >= 0)) break;
    if (path >= 0 && w.step(sv, r, leaf, status)) {
      sst(ps.hit_t + path, leaf.best_t);
      sst(ps.hit_slot + path, (int32_t)leaf.best_slot);
      path = -1;
    }
  }
}

// The variants differ only in their launch bounds (variant 0 leaves the
// register count to the compiler's default heuristic).
template <int STACK, bool SPH>
__global__ void __launch_bounds__(128) k_extend(SceneView sv, const ViewGPU* __restrict__ views, PathSoA ps,
                                                const int* __restrict__ queue, WaveCounters* cnt, int cur,
                                                unsigned* status) {
  extend_body<STACK, SPH, 0>(sv, views, ps, queue, cnt, cur, status);
}
template <int STACK, bool SPH>
__global__ void __launch_bounds__(128, 10) k_extend_10(SceneView sv, const ViewGPU* __restrict__ views, PathSoA ps,
                                                       const int* __restrict__ queue, WaveCounters* cnt, int cur,
                                                       unsigned* status) {
  extend_body<STACK, SPH, 1>(sv, views, ps, queue, cnt, cur, status);
}
template <int STACK, bool SPH>
__global__ void __launch_bounds__(128, 12) k_extend_12(SceneView sv, const ViewGPU* __restrict__ views, PathSoA ps,
                                                       const int* __restrict__ queue, WaveCounters* cnt, int cur,
                                                       unsigned* status) {
  extend_body<STACK, SPH, 2>(sv, views, ps, queue, cnt, cur, status);
}

// ---- shade -----------------------------------------------------------------
struct ShadeScene {
  SceneView sv;
  const MatGPU* __restrict__ mats;
  const LightGPU* __restrict__ lights;
  const float* __restrict__ lpdf_by_prim;
};

// lightDirectionalPDF (renderer.go:1404-1425) for a sphere light hit.
__device__ __forceinline__ float light_dir_pdf(const ShadeScene& sc, int n_lights, int power, int prim, float radius,
                                               float3 from, float3 lp, float3 ln) {
  if (!(radius > 0.0f)) return 0.0f;
  float3 to = lp - from;
  float dist2 = dot3(to, to);
  if (dist2 <= 1e-12f) return 0.0f;
  float3 ld = unit3(to);
  float cosL = fmaxf(0.0f, dot3(ln, ld * -1.0f));
  if (cosL <= 1e-12f) return 0.0f;
  float area = 4.0f * kPi * radius * radius;
  float sel = n_lights == 0 ? 0.0f : (power ? __ldg(sc.lpdf_by_prim + prim) : 1.0f / (float)n_lights);
  return sel * dist2 / (cosL * area);
}

// Path state between bounces as the shading step sees it. The wavefront
// kernels keep it in the SoA arrays (SoAPath loads what a vertex needs and
// stores what changes); the one-kernel renderer keeps it in registers (RegPath).
// LAZY: the path's radiance L is read on its first addition at a vertex and
// written back only if something was added; most vertices (a diffuse or metal
// bounce without a light sample) leave it as it was, and the additions keep
// their order. The kernel with the other integrators' code keeps L in
// registers from the start: at its register budget the lazy form spills.
template <bool LAZY>
struct SoAPath {
  const PathSoA& ps;
  int path;
  float3 o, d, tp, L;
  bool l_read, l_added;
  Pcg32 rng;
  uint32_t flags;
  float ppdf;
  __device__ SoAPath(const PathSoA& p, int i) : ps(p), path(i), l_read(false), l_added(false) {
    o = f3(sld(ps.ox + i), sld(ps.oy + i), sld(ps.oz + i));
    d = f3(sld(ps.dx + i), sld(ps.dy + i), sld(ps.dz + i));
    tp = f3(sld(ps.tx + i), sld(ps.ty + i), sld(ps.tz + i));
    if (!LAZY) get_L();
  }
  __device__ __forceinline__ float3 get_L() {
    if (!l_read) {
      L = f3(sld(ps.lx + path), sld(ps.ly + path), sld(ps.lz + path));
      l_read = true;
    }
    return L;
  }
  __device__ __forceinline__ void add_L(float3 v) {
    L = get_L() + v;
    l_added = true;
  }
  __device__ __forceinline__ void flush_L() {
    if (!LAZY || l_added) {
      sst(ps.lx + path, L.x); sst(ps.ly + path, L.y); sst(ps.lz + path, L.z);
    }
  }
  __device__ __forceinline__ void load_vertex() {  // only a path that hit a valid material needs these
    rng.state = sld(ps.rs + path);
    rng.inc = sld(ps.ri + path);
    const uint32_t w = sld(ps.prev + path);
    flags = w >> 31;
    ppdf = __uint_as_float(w & 0x7fffffffu);
  }
  __device__ __forceinline__ float3 prev() const {
    return f3(sld(ps.px + path), sld(ps.py + path), sld(ps.pz + path));
  }
  __device__ __forceinline__ void set_prev(float3 p) {
    sst(ps.px + path, p.x); sst(ps.py + path, p.y); sst(ps.pz + path, p.z);
  }
  __device__ __forceinline__ void store_continuation(float3 no, float3 nd) {
    sst(ps.ox + path, no.x); sst(ps.oy + path, no.y); sst(ps.oz + path, no.z);
    sst(ps.dx + path, nd.x); sst(ps.dy + path, nd.y); sst(ps.dz + path, nd.z);
    sst(ps.tx + path, tp.x); sst(ps.ty + path, tp.y); sst(ps.tz + path, tp.z);
    sst(ps.prev + path, (__float_as_uint(ppdf) & 0x7fffffffu) | (flags & 1u) << 31);  // ppdf >= 0 (or -0)
    sst(ps.rs + path, rng.state);
  }
};

struct RegPath {
  float3 o, d, tp, L, pv;
  Pcg32 rng;
  uint32_t flags;
  float ppdf;
  __device__ __forceinline__ float3 get_L() const { return L; }
  __device__ __forceinline__ void add_L(float3 v) { L = L + v; }
  __device__ __forceinline__ void load_vertex() {}
  __device__ __forceinline__ float3 prev() const { return pv; }
  __device__ __forceinline__ void set_prev(float3 p) { pv = p; }
  __device__ __forceinline__ void store_continuation(float3 no, float3 nd) {
    o = no;
    d = nd;
  }
};

// What a vertex asks of the caller: continue (state already advanced), trace
// a shadow ray, keep a path replay record.
struct VertexOut {
  bool alive, shadow;
  float4 so, sd, scon;  // shadow ray: origin + tmax, direction + scene root, contribution
  int rec_m;
  float3 rec_v;
};

// Guide outputs of a path's first vertex (sample 0 only).
struct GuideOut {
  float4* nd;
  uint32_t* c;
  const uint32_t* jit;
  long long px;  // frame pixel, < 0: no guide
};

// Guide outputs of a first vertex: normal and depth, and the compact guide
// words (gpu_opencl_windows.go:791-797): Euclidean depth, octahedral normal
// 10:10, material 11 bits, valid bit, jitter.
__device__ __forceinline__ void write_guides(const GuideOut& gd, float3 N, float t, float3 d, int m) {
  gd.nd[gd.px] = make_float4(N.x, N.y, N.z, t);
  const float dl = sqrtf(dot3(d, d));
  float3 q = N * (1.0f / (fabsf(N.x) + fabsf(N.y) + fabsf(N.z) + 1e-20f));
  float px = q.x, py = q.y;
  if (q.z < 0.0f) {
    float ax = 1.0f - fabsf(q.y), ay = 1.0f - fabsf(q.x);
    px = copysignf(ax, q.x);
    py = copysignf(ay, q.y);
  }
  px = fminf(fmaxf(px * 0.5f + 0.5f, 0.0f), 1.0f);
  py = fminf(fmaxf(py * 0.5f + 0.5f, 0.0f), 1.0f);
  const uint32_t qx = (uint32_t)rintf(px * 1023.0f), qy = (uint32_t)rintf(py * 1023.0f);
  const uint32_t mm = (uint32_t)min(max(m, 0), 2047);
  uint32_t* g = gd.c + 3 * (size_t)gd.px;
  g[0] = __float_as_uint(t * dl);
  g[1] = 0x80000000u | (mm << 20) | (qy << 10) | qx;
  g[2] = gd.jit[gd.px];
}

// directLight (renderer.go:1427-1465) at a diffuse vertex (p, N) of material
// M: draws the light sample and returns 0 (no contribution), 1 (contribution
// that needs no shadow ray: the light point is within 1e-6 of the offset
// origin, where visible() returns true) or 2 (shadow ray so/sd to trace).
// `weight` multiplies the contribution.
__device__ __forceinline__ int sample_direct(const ViewGPU& wp, const ShadeScene& sc, Pcg32& rng, float3 p, float3 N,
                                             const MatGPU& M, float3 weight, float4* so, float4* sd, float3* contrib) {
  if (wp.n_lights <= 0) return 0;
  int li;
  float sel;
  if (!wp.power) {  // rng.Intn
    li = draw_index(rng, wp.n_lights);
    sel = 1.0f / (float)wp.n_lights;
  } else {  // sort.Search over LightCDF
    const float r = rng.uniform();
    int lo = 0, hi = wp.n_lights;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (!(__ldg(&sc.lights[wp.light_off + mid].cdf_dn) >= r)) lo = mid + 1; else hi = mid;
    }
    li = min(lo, wp.n_lights - 1);
    sel = __ldg(&sc.lights[wp.light_off + li].select_pdf);
  }
  const LightGPU Lg = sc.lights[wp.light_off + li];
  const float3 ln = sel > 0.0f ? rand_unit_vector(rng) : f3(0, 0, 1);
  const float3 q = f3(Lg.cx, Lg.cy, Lg.cz) + ln * Lg.r;
  const float3 to = q - p;
  const float dist2 = dot3(to, to);
  if (!(dist2 >= 1e-8f && sel > 0.0f)) return 0;
  const float3 ld = unit3(to);
  const float ndl = fmaxf(0.0f, dot3(N, ld));
  const float cosL = fmaxf(0.0f, dot3(ln * -1.0f, ld));
  if (!(ndl > 0.0f && cosL > 0.0f)) return 0;
  const float area = 4.0f * kPi * Lg.r * Lg.r;
  const float lightPDF = sel * dist2 / (cosL * area);
  if (!(lightPDF > 0.0f)) return 0;
  const float bsdfPDF = ndl / kPi;
  const float w = wp.mis ? power_heuristic(lightPDF, bsdfPDF) : 1.0f;
  const float3 f = f3(M.cr, M.cg, M.cb) * (1.0f / kPi);
  *contrib = had(weight, had(f, f3(Lg.er, Lg.eg, Lg.eb)) * (ndl * w / lightPDF));
  const float3 from = p + N * 2e-4f;  // visible (renderer.go:1333-1341)
  const float3 sdv = q - from;
  const float sd2 = dot3(sdv, sdv);
  if (sd2 < 1e-12f) return 1;
  const float dist = sqrtf(sd2);
  const float3 dirn = sdv * (1.0f / dist);
  *so = make_float4(from.x, from.y, from.z, dist - 1e-4f);
  *sd = make_float4(dirn.x, dirn.y, dirn.z, __int_as_float(wp.root));
  return 2;
}

// One vertex of trace() (renderer.go:1497-1560), or of tracePhotonMapped
// (1763-1831: a photon gather at diffuse vertices, emitters without an MIS
// weight), for a path whose extension ray hit `slot` at fp32 distance t
// (slot < 0: miss). Updates s.L / s.tp and, when the path continues, its next
// ray (store_continuation). ALT: the batch has views of the other integrators
// (the path-only kernels compile without their code).
template <bool ALT, class P>
__device__ __forceinline__ void shade_vertex(const ViewGPU& wp, int n_mats, const ShadeScene& sc, P& s, float t,
                                             int slot, int bounce, const GuideOut& gd, VertexOut& out,
                                             bool want_rec) {
  out.alive = false;
  out.shadow = false;
  out.rec_m = -1;
  out.rec_v = f3(0, 0, 0);
  const int rr_depth = wp.rr_depth < 1 ? 4 : wp.rr_depth;
  const float3 o = s.o, d = s.d;
  float3 tp = s.tp;
  if (slot < 0) {
    s.add_L(had(tp, background(d)));
  } else {
    const float4 nrm = __ldg(sc.sv.snorm + slot);
    const int m = __float_as_int(nrm.w);
    if (m >= 0 && m < n_mats) {
      s.load_vertex();
      Pcg32 rng = s.rng;
      uint32_t flags = s.flags;
      float ppdf = s.ppdf;
      const Surface S = hit_surface(sc.sv, slot, nrm, o, d, t);
      const float3 p = S.p, N = S.N;
      const MatGPU M = sc.mats[m];
      const int kind = (int)M.kind;
      if (gd.px >= 0) write_guides(gd, N, t, d, m);
      if (kind == BC_MAT_EMISSIVE) {
        float w = 1.0f;
        if ((!ALT || wp.integrator == BC_INTEGRATOR_PATH) && wp.mis && (flags & 1u)) {  // 0 for triangles
          float lpdf = 0.0f;
          if (S.sphere) {
            const int prim = __ldg(sc.sv.slot_prim + slot);
            lpdf = light_dir_pdf(sc, wp.n_lights, wp.power, prim, S.radius, s.prev(), p, N);
          }
          w = power_heuristic(ppdf, lpdf);
        }
        s.add_L(had(tp, f3(M.er, M.eg, M.eb)) * w);
        out.rec_m = m | kEmitTag;
        out.rec_v = tp * w;
      } else {
        bool cont = true;
        float3 nd_dir = d, no = o;
        if (kind == BC_MAT_DIFFUSE) {
          out.rec_m = m;
          if (want_rec) out.rec_v = s.get_L();  // everything added from here on carries this albedo once more
          if (ALT && wp.integrator == BC_INTEGRATOR_PHOTON) s.add_L(had(tp, photon_gather(wp.pm, p, N)));
          float3 contrib;
          const int k = sample_direct(wp, sc, rng, p, N, M, tp, &out.so, &out.sd, &contrib);
          if (k == 1) {
            s.add_L(contrib);
          } else if (k == 2) {
            out.shadow = true;
            out.scon = make_float4(contrib.x, contrib.y, contrib.z, 0.0f);
          }
          tp = had(tp, f3(M.cr, M.cg, M.cb));
          nd_dir = rand_cos_hemisphere(N, rng);
          flags |= 1u;
          ppdf = fmaxf(0.0f, dot3(N, nd_dir)) / kPi;
          // prevPoint feeds only lightDirectionalPDF of a sphere light hit,
          // which is 0 for a view without sphere lights
          if (wp.n_lights > 0) s.set_prev(p);
          no = p + N * 2e-4f;
        } else if (kind == BC_MAT_METAL) {
          const float rough = fminf(fmaxf(M.rough, 0.0f), 1.0f);
          nd_dir = unit3(reflect3(unit3(d), N) + rand_in_unit_sphere(rng) * rough);
          if (dot3(nd_dir, N) <= 0.0f) {
            cont = false;
          } else {
            flags &= ~1u;
            tp = had(tp, f3(M.cr, M.cg, M.cb));
            no = p + N * 2e-4f;
          }
        } else {  // glass
          float eta = M.ior;
          if (eta <= 1.0f) eta = 1.5f;
          const float ratio = S.front ? 1.0f / eta : eta;
          const float3 un = unit3(d);
          const float cosT = fminf(dot3(un * -1.0f, N), 1.0f);
          const float sinT = sqrtf(fmaxf(0.0f, 1.0f - cosT * cosT));
          if (ratio * sinT > 1.0f || schlick(cosT, ratio) > rng.uniform())
            nd_dir = reflect3(un, N);
          else
            nd_dir = refract3(un, N, ratio);
          flags &= ~1u;
          tp = had(tp, f3(M.cr, M.cg, M.cb));
          no = p + nd_dir * 2e-4f;
        }
        if (cont && bounce >= rr_depth) {  // Russian roulette (renderer.go:1550-1560)
          const float pr = fminf(fmaxf(maxcomp(tp), 0.08f), 0.95f);
          if (rng.uniform() > pr) cont = false;
          else tp = tp * (1.0f / pr);
        }
        if (cont && bounce + 1 < wp.bounces) {
          out.alive = true;
          s.tp = tp;
          s.flags = flags;
          s.ppdf = ppdf;
          s.rng = rng;
          s.store_continuation(no, nd_dir);
        }
      }
    }
  }
}

// One vertex of traceRecursiveInner (renderer.go:1569-1621). s.tp is the weight
// of the vertex's value and s.L gathers the emitted and background radiance.
// A diffuse vertex is recorded (its light sample comes when the path ends) and
// the subtree below it weighs weight * color / p while depth < 8
// (renderer.go:1591-1596). Returns true when the path ends at this vertex;
// s.rng then holds the stream the unwinding continues.
template <class P>
__device__ __forceinline__ bool shade_recursive(const ViewGPU& wp, int n_mats, const ShadeScene& sc, P& s, float t,
                                                int slot, int bounce, const GuideOut& gd, const RecurRec& rr,
                                                int path) {
  s.load_vertex();  // the unwinding needs the stream even after a miss
  Pcg32 rng = s.rng;
  const float3 o = s.o, d = s.d;
  float3 W = s.tp;
  bool cont = false;
  float3 nd_dir = d, no = o;
  float4 rec = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
  const size_t r = (size_t)bounce * rr.cap + path;
  if (slot < 0) {
    s.add_L(had(W, background(d)));
  } else {
    const float4 nrm = __ldg(sc.sv.snorm + slot);
    const int m = __float_as_int(nrm.w);
    if (m >= 0 && m < n_mats) {
      const Surface S = hit_surface(sc.sv, slot, nrm, o, d, t);
      const float3 p = S.p, N = S.N;
      const MatGPU M = sc.mats[m];
      const int kind = (int)M.kind;
      const float3 col = f3(M.cr, M.cg, M.cb);
      if (gd.px >= 0) write_guides(gd, N, t, d, m);
      if (kind == BC_MAT_EMISSIVE) {
        s.add_L(had(W, f3(M.er, M.eg, M.eb)));
      } else if (kind == BC_MAT_DIFFUSE) {
        const float scale = (wp.bounces - bounce < 8) ? 1.0f / fminf(fmaxf(maxcomp(col), 0.1f), 0.95f) : 1.0f;
        const float3 Wv = W * scale;
        rec = make_float4(p.x, p.y, p.z, __int_as_float(m));
        rr.n[r] = make_float4(N.x, N.y, N.z, 0.0f);
        rr.w[r] = make_float4(Wv.x, Wv.y, Wv.z, 0.0f);
        W = had(Wv, col);
        nd_dir = rand_cos_hemisphere(N, rng);
        no = p + N * 2e-4f;
        cont = true;
      } else if (kind == BC_MAT_METAL) {
        const float rough = fminf(fmaxf(M.rough, 0.0f), 1.0f);
        nd_dir = unit3(reflect3(unit3(d), N) + rand_in_unit_sphere(rng) * rough);
        if (dot3(nd_dir, N) > 0.0f) {
          W = had(W, col);
          no = p + N * 2e-4f;
          cont = true;
        }
      } else {  // glass and any other kind
        float eta = M.ior;
        if (eta <= 1.0f) eta = 1.5f;
        const float ratio = S.front ? 1.0f / eta : eta;
        const float3 un = unit3(d);
        const float cosT = fminf(dot3(un * -1.0f, N), 1.0f);
        const float sinT = sqrtf(fmaxf(0.0f, 1.0f - cosT * cosT));
        if (ratio * sinT > 1.0f || schlick(cosT, ratio) > rng.uniform())
          nd_dir = reflect3(un, N);
        else
          nd_dir = refract3(un, N, ratio);
        W = had(W, col);
        no = p + nd_dir * 2e-4f;
        cont = true;
      }
    }
  }
  rr.a[r] = rec;
  s.rng = rng;
  if (cont && bounce + 1 < wp.bounces) {  // depth - 1 > 0: the subtree is traced
    s.tp = W;
    s.store_continuation(no, nd_dir);
    return false;
  }
  return true;
}

// The end of a recursive path whose last vertex is `last`: the recorded
// diffuse vertices draw their light samples deepest first, as the reference's
// recursion returns; each record becomes (contribution, visible) and each
// shadow ray is queued with its record's bounce + 1 in the contribution's w.
__device__ __forceinline__ void unwind_recursive(const ViewGPU& wp, const ShadeScene& sc, Pcg32 rng,
                                                 const RecurRec& rr, int path, int last, ShadowSoA sh,
                                                 WaveCounters* cnt, long long sh_cap, unsigned* status) {
  for (int b = last; b >= 0; b--) {
    const size_t r = (size_t)b * rr.cap + path;
    const float4 A = rr.a[r];
    const int m = __float_as_int(A.w);
    float4 res = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (m >= 0) {
      const float4 Nn = rr.n[r], Wv = rr.w[r];
      const MatGPU M = sc.mats[m];
      float4 so, sd;
      float3 c;
      const int k = sample_direct(wp, sc, rng, f3(A.x, A.y, A.z), f3(Nn.x, Nn.y, Nn.z), M, f3(Wv.x, Wv.y, Wv.z),
                                  &so, &sd, &c);
      if (k == 1) {
        res = make_float4(c.x, c.y, c.z, 1.0f);
      } else if (k == 2) {
        res = make_float4(c.x, c.y, c.z, 0.0f);
        const int q = atomicAdd(&cnt->shadow, 1);
        if (q < sh_cap) {
          sh.o[q] = so;
          sh.d[q] = sd;
          sh.c[q] = make_float4(c.x, c.y, c.z, __int_as_float(b + 1));
          sh.path[q] = path;
        } else {
          atomicOr(status, kStatusCapacity);
        }
      }
    }
    rr.a[r] = res;
  }
  rr.nb[path] = last + 1;
}

template <bool ALT, int BLOCK>
__device__ __forceinline__ void shade_body(const ViewGPU* __restrict__ views, int n_mats, ShadeScene sc,
                                               PathSoA ps, const int* __restrict__ qcur, int* __restrict__ qnext,
                                               ShadowSoA sh, WaveCounters* cnt, int cur, int bounce,
                                               float4* __restrict__ guide_nd, uint32_t* __restrict__ guide_c,
                                               const uint32_t* __restrict__ guide_jit, GradRec rec, RecurRec rr,
                                               long long sh_cap, unsigned* status) {
  const int n = *((volatile int*)&cnt->q[cur]);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    cnt->work_ext = 0;  // the next bounce's extend and this bounce's connect start from zero
    cnt->work_con = 0;
  }
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int idx = base + threadIdx.x;
    const int path = idx < n ? __ldcs(qcur + idx) : -1;
    VertexOut out;
    out.alive = false;
    out.shadow = false;
    if (path >= 0) {
      const ViewGPU& wp = views[sld(ps.view + path)];
      SoAPath<!ALT> s(ps, path);
      GuideOut gd{guide_nd, guide_c, guide_jit, -1};
      if (bounce == 0 && wp.want_guides && ps.samp[path] == 0) gd.px = wp.pix_off + ps.pix[path];
      const float hit_t = sld(ps.hit_t + path);
      const int hit_slot = sld(ps.hit_slot + path);
      if (ALT && wp.integrator == BC_INTEGRATOR_RECURSIVE) {
        const bool ended = shade_recursive(wp, n_mats, sc, s, hit_t, hit_slot, bounce, gd, rr, path);
        out.alive = !ended;
        if (ended) unwind_recursive(wp, sc, s.rng, rr, path, bounce, sh, cnt, sh_cap, status);
      } else {
        shade_vertex<ALT>(wp, n_mats, sc, s, hit_t, hit_slot, bounce, gd, out, rec.m != nullptr);
      }
      s.flush_L();
      if (rec.m) {
        const size_t r = (size_t)bounce * rec.cap + path;
        rec.m[r] = out.rec_m;
        rec.v[r] = make_float4(out.rec_v.x, out.rec_v.y, out.rec_v.z, 0.0f);
        rec.nb[path] = bounce + 1;
      }
    }
    const int qn = block_reserve<BLOCK>(&cnt->q[cur ^ 1], out.alive);
    if (out.alive) __stcs(qnext + qn, path);
    const int qs = warp_reserve(&cnt->shadow, out.shadow);
    if (out.shadow) {
      if (qs < sh_cap) {
        sh.o[qs] = out.so;
        sh.d[qs] = out.sd;
        sh.c[qs] = out.scon;
        sh.path[qs] = path;
      } else {
        atomicOr(status, kStatusCapacity);
      }
    }
  }
}

// Block shape of the shading kernel (bc_set_option "render_shade_block", chosen
// per workload by bc_autotune_render): 256 threads at four blocks per SM, or
// 128 threads at eight; the same 64-register budget and resident threads, a
// different scheduling granularity of the grid-stride loop.
#define BC_SHADE_ARGS                                                                                       \
  const ViewGPU *__restrict__ views, int n_mats, ShadeScene sc, PathSoA ps, const int *__restrict__ qcur,  \
      int *__restrict__ qnext, ShadowSoA sh, WaveCounters *cnt, int cur, int bounce,                       \
      float4 *__restrict__ guide_nd, uint32_t *__restrict__ guide_c, const uint32_t *__restrict__ guide_jit, \
      GradRec rec, RecurRec rr, long long sh_cap, unsigned *status
#define BC_SHADE_PASS views, n_mats, sc, ps, qcur, qnext, sh, cnt, cur, bounce, guide_nd, guide_c, guide_jit, rec, rr, sh_cap, status
template <bool ALT>
__global__ void __launch_bounds__(256, 4) k_shade(BC_SHADE_ARGS) { shade_body<ALT, 256>(BC_SHADE_PASS); }
template <bool ALT>
__global__ void __launch_bounds__(128, 8) k_shade_128(BC_SHADE_ARGS) { shade_body<ALT, 128>(BC_SHADE_PASS); }
#undef BC_SHADE_ARGS
#undef BC_SHADE_PASS

// ---- connect -----------------------------------------------------------------
template <int STACK, bool SPH>
__global__ void __launch_bounds__(128) k_connect(SceneView sv, PathSoA ps, ShadowSoA sh, WaveCounters* cnt,
                                                 RecurRec rr, long long sh_cap, unsigned* status) {
  // entries past the queue were never written (the shading step flagged them)
  const int n = (int)min((long long)*((volatile int*)&cnt->shadow), sh_cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&cnt->shadow_rays, (unsigned long long)n);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  int i = -1;
  bool exhausted = false;
  Ray32 r = make_ray(0, 0, 0, 0, 0, 0, 0);
  FastAnyLeaf<SPH> leaf(sv, r, 0.0f);
  FastWalker<STACK, kAnyLeafVote> w;
  w.reset(r);
  for (;;) {
    const bool need = i < 0 && !exhausted;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m && (__popc(m) >= kRefillLanes || !__any_sync(0xffffffffu, i >= 0))) {
      const int leader = __ffs(m) - 1;
      int base = 0;
      if ((int)lane == leader) base = atomicAdd(&cnt->work_con, __popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const int my = base + __popc(m & below);
        if (my < n) {
          i = my;
          const float4 o = sh.o[i], d = sh.d[i];
          r = make_ray(o.x, o.y, o.z, d.x, d.y, d.z, 1e-4f);
          leaf.reset(o.w);
          w.reset(r, (uint32_t)__float_as_int(d.w));  // the scene root rides in d.w
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, i >= 0)) break;
    if (i >= 0 && w.step(sv, r, leaf, status)) {
      if (!leaf.done) {  // no occluder: the light sample counts
        const int path = sh.path[i];
        const float4 c = sh.c[i];
        const int tag = __float_as_int(c.w);  // 0, or the recursive record's bounce + 1
        if (tag == 0) {
          ps.lx[path] += c.x;
          ps.ly[path] += c.y;
          ps.lz[path] += c.z;
        } else {
          rr.a[(size_t)(tag - 1) * rr.cap + path].w = 1.0f;
        }
      }
      i = -1;
    }
  }
}

// clampFirefly (renderer.go:1917-1926)
__device__ __forceinline__ float3 clamp_sample(float3 c, float limit) {
  if (limit > 0.0f) {
    const float mx = maxcomp(c);
    if (!(mx <= limit || mx <= 0.0f)) c = c * (limit / mx);
  }
  return c;
}

// ---- accumulate --------------------------------------------------------------
// For every view the wave touches, each pixel adds its samples of the wave in
// sample order (path = view.path_off + s * npix + p): no atomics, and the sum
// does not depend on thread scheduling.
__global__ void k_accumulate(const BatchState* __restrict__ bs, const ViewGPU* __restrict__ views, PathSoA ps,
                             float* __restrict__ sum, float* __restrict__ sumsq, AdaptState ad, RecurRec rr) {
  const long long w0 = bs->w0;
  const long long w1 = min(bs->total, w0 + (long long)bs->cap);
  if (w1 <= w0) return;
  const int v0 = view_of(views, bs->n_views, w0), v1 = view_of(views, bs->n_views, w1 - 1);
  const int stride = gridDim.x * blockDim.x;
  for (int v = v0; v <= v1; v++) {
    const ViewGPU& V = views[v];
    const long long a = max(w0, V.path_off);
    const long long b = min(w1, V.path_off + (long long)V.npix * V.spp);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < V.npix; p += stride) {
      const long long lo = a - V.path_off - p, hi = b - V.path_off - p;  // >= -(npix-1)
      const int s_lo = (int)max(0LL, (lo + V.npix - 1) / V.npix);
      const int s_hi = (int)((hi + V.npix - 1) / V.npix);
      if (s_hi <= s_lo) continue;
      // continue the stored running sum sample by sample: the rounding sequence is
      // that of one pass over samples 0..spp-1, whatever the wave boundaries
      float* sp = sum + 3 * (size_t)(V.pix_off + p);
      float* qp = sumsq ? sumsq + 3 * (size_t)(V.pix_off + p) : nullptr;
      int an = 0;
      float sl = 0.0f, ssl = 0.0f;
      if (V.adaptive) {
        an = ad.n[V.pix_off + p];
        if (an & kPixDone) continue;  // stopped in an earlier wave
        const float2 l = ad.lum[V.pix_off + p];
        sl = l.x;
        ssl = l.y;
      }
      float3 acc = f3(sp[0], sp[1], sp[2]);
      float3 acc2 = qp ? f3(qp[0], qp[1], qp[2]) : f3(0, 0, 0);
      bool stop = false;
      for (int s = s_lo; s < s_hi && !stop; s++) {
        const long long i = V.path_off + (long long)s * V.npix + p - w0;
        float3 L = f3(sld(ps.lx + i), sld(ps.ly + i), sld(ps.lz + i));
        if (V.integrator == BC_INTEGRATOR_RECURSIVE)  // the visible light samples, deepest vertex first
          for (int b = rr.nb[i] - 1; b >= 0; b--) {
            const float4 A = rr.a[(size_t)b * rr.cap + i];
            if (A.w == 1.0f) L = L + f3(A.x, A.y, A.z);
          }
        const float3 c = clamp_sample(L, V.clamp);
        acc = acc + c;
        acc2 = acc2 + had(c, c);
        if (V.adaptive) stop = adaptive_step(V, c, &an, &sl, &ssl);
      }
      if (V.adaptive) {
        ad.n[V.pix_off + p] = stop ? (an | kPixDone) : an;
        ad.lum[V.pix_off + p] = make_float2(sl, ssl);
      }
      sp[0] = acc.x;
      sp[1] = acc.y;
      sp[2] = acc.z;
      if (qp) {
        qp[0] = acc2.x;
        qp[1] = acc2.y;
        qp[2] = acc2.z;
      }
    }
  }
}

// ---- gradient (path replay) --------------------------------------------------------
// After the last bounce of a wave every path knows its final radiance Lf. With
// the adjoint d = dLoss/dImage(pixel) / spp of its pixel:
//   diffuse vertex on material m : dL/d albedo_m = (Lf - L_before) / albedo_m
//   emitter hit on material e    : dL/d emission_e = throughput * MIS weight
// (everything a path gathers after the albedo of m multiplied its throughput is
// linear in that albedo; Russian roulette probabilities are held fixed).
// Per block sums in fp64 shared memory, one row of `partial` per block.
__global__ void __launch_bounds__(256) k_gradient(const BatchState* __restrict__ bs, const ViewGPU* __restrict__ views,
                                                  PathSoA ps, GradRec rec, GradArgs ga,
                                                  const MatGPU* __restrict__ mats) {
  extern __shared__ double sg[];
  const int np3 = 3 * ga.n_params;
  for (int k = threadIdx.x; k < np3; k += blockDim.x) sg[k] = 0.0;
  __syncthreads();
  const long long w0 = bs->w0;
  const int n = (int)min((long long)bs->cap, bs->total - w0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const ViewGPU& V = views[ps.view[i]];
    const float* dp = ga.dimg + 3 * (size_t)(V.pix_off + ps.pix[i]);
    const float inv = 1.0f / (float)V.spp;
    const float3 dl = f3(dp[0] * inv, dp[1] * inv, dp[2] * inv);
    if (dl.x == 0.0f && dl.y == 0.0f && dl.z == 0.0f) continue;
    const float3 Lf = f3(ps.lx[i], ps.ly[i], ps.lz[i]);
    const int nb = rec.nb[i];
    for (int b = 0; b < nb; b++) {
      const size_t r = (size_t)b * rec.cap + i;
      const int m = rec.m[r];
      if (m < 0) continue;
      const int mm = m & ~kEmitTag;
      const int k = ga.mat2param[mm];
      if (k < 0) continue;
      const float4 v = rec.v[r];
      float gx, gy, gz;
      if (m & kEmitTag) {
        gx = dl.x * v.x;
        gy = dl.y * v.y;
        gz = dl.z * v.z;
      } else {
        const MatGPU M = mats[mm];
        gx = M.cr > 0.0f ? dl.x * ((Lf.x - v.x) / M.cr) : 0.0f;
        gy = M.cg > 0.0f ? dl.y * ((Lf.y - v.y) / M.cg) : 0.0f;
        gz = M.cb > 0.0f ? dl.z * ((Lf.z - v.z) / M.cb) : 0.0f;
      }
      atomicAdd(&sg[3 * k], (double)gx);
      atomicAdd(&sg[3 * k + 1], (double)gy);
      atomicAdd(&sg[3 * k + 2], (double)gz);
    }
  }
  __syncthreads();
  double* row = ga.partial + (size_t)blockIdx.x * np3;
  for (int k = threadIdx.x; k < np3; k += blockDim.x) row[k] += sg[k];
}

__global__ void k_advance(BatchState* bs, WaveCounters* cnt) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    bs->w0 = min(bs->total, bs->w0 + (long long)bs->cap);
    cnt->q[0] = 0;  // the next wave's generate appends to it
  }
}

__global__ void k_clear_guides(int n, float4* __restrict__ nd, uint32_t* __restrict__ c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  nd[i] = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
  c[3 * i] = 0u;
  c[3 * i + 1] = 0u;
  c[3 * i + 2] = 0u;
}

// mean = sum / spp for every pixel of every view
// mean = sum / spp for every pixel of every view (sum / samples taken for an
// adaptive view, renderer.go:1965)
__global__ void k_finish_views(const ViewGPU* __restrict__ views, int n_views, const float* __restrict__ sum,
                               float* __restrict__ out, const int32_t* __restrict__ pix_n) {
  const int stride = gridDim.x * blockDim.x;
  for (int v = 0; v < n_views; v++) {
    const ViewGPU& V = views[v];
    const float inv = 1.0f / (float)V.spp;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < 3 * V.npix; k += stride) {
      float f = inv;
      if (V.adaptive) {
        const int n = pix_n[V.pix_off + k / 3] & 0x7fffffff;
        f = 1.0f / (float)max(n, 1);
      }
      out[3 * (size_t)V.pix_off + k] = sum[3 * (size_t)V.pix_off + k] * f;
    }
  }
}

// ---- one-kernel form ----------------------------------------------------------------
// The reference's OpenCL design (one work-item per pixel looping over samples
// and bounces, gpu_opencl_windows.go:800-822), on the same primary rays,
// traversal, shading and accumulation code as the wave engine: the plain
// one-view-per-launch form the wave engine is measured against. Shadow rays are
// traced in place; a lane idles once its path ends until the warp's longest
// path of that sample is done.
template <int STACK, bool SPH, bool ALT>
__global__ void __launch_bounds__(128) k_render_plain(const ViewGPU* __restrict__ views, int v, int n_mats,
                                                      ShadeScene sc, const float4* __restrict__ seq,
                                                      float* __restrict__ sum, float* __restrict__ sumsq,
                                                      float4* __restrict__ guide_nd, uint32_t* __restrict__ guide_c,
                                                      uint32_t* __restrict__ guide_jit, WaveCounters* cnt,
                                                      unsigned* status, AdaptState ad) {
  const ViewGPU& V = views[v];
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long segs = 0, shadows = 0;
  if (p < V.npix) {
    const int x = p % V.W, y = V.y0 + p / V.W;
    float* sp = sum + 3 * (size_t)(V.pix_off + p);
    float* qp = sumsq ? sumsq + 3 * (size_t)(V.pix_off + p) : nullptr;
    float3 acc = f3(sp[0], sp[1], sp[2]);
    float3 acc2 = qp ? f3(qp[0], qp[1], qp[2]) : f3(0, 0, 0);
    FastWalker<STACK, kLeafVote> w;
    int an = 0;
    float sl = 0.0f, ssl = 0.0f;
    for (int s = 0; s < V.spp; s++) {
      RegPath st;
      float jx, jy;
      primary_ray(V, x, y, s, seq, &st.o, &st.d, &st.rng, &jx, &jy);
      st.tp = f3(1.0f, 1.0f, 1.0f);
      st.L = f3(0.0f, 0.0f, 0.0f);
      st.pv = f3(0.0f, 0.0f, 0.0f);
      st.flags = 0u;
      st.ppdf = 0.0f;
      const bool guide = s == 0 && V.want_guides;
      if (guide) guide_jit[V.pix_off + p] = jitter_word(jx, jy);
      for (int b = 0; b < V.bounces; b++) {
        const Ray32 r = make_ray(st.o.x, st.o.y, st.o.z, st.d.x, st.d.y, st.d.z, 1e-4f);
        FastClosestLeaf<SPH> leaf(sc.sv, r, 1e30f);
        w.reset(r, V.root);
        while (!w.step(sc.sv, r, leaf, status)) {
        }
        segs++;
        const GuideOut gd{guide_nd, guide_c, guide_jit, (b == 0 && guide) ? V.pix_off + p : -1};
        VertexOut out;
        shade_vertex<ALT>(V, n_mats, sc, st, leaf.best_t, leaf.best_slot, b, gd, out, false);
        if (out.shadow) {
          shadows++;
          const Ray32 sr = make_ray(out.so.x, out.so.y, out.so.z, out.sd.x, out.sd.y, out.sd.z, 1e-4f);
          FastAnyLeaf<SPH> any(sc.sv, sr, out.so.w);
          w.reset(sr, V.root);
          while (!w.step(sc.sv, sr, any, status)) {
          }
          if (!any.done) st.L = st.L + f3(out.scon.x, out.scon.y, out.scon.z);
        }
        if (!out.alive) break;
      }
      const float3 c = clamp_sample(st.L, V.clamp);
      acc = acc + c;
      acc2 = acc2 + had(c, c);
      if (V.adaptive && adaptive_step(V, c, &an, &sl, &ssl)) {
        an |= kPixDone;
        break;
      }
    }
    if (V.adaptive) {
      ad.n[V.pix_off + p] = an;
      ad.lum[V.pix_off + p] = make_float2(sl, ssl);
    }
    sp[0] = acc.x;
    sp[1] = acc.y;
    sp[2] = acc.z;
    if (qp) {
      qp[0] = acc2.x;
      qp[1] = acc2.y;
      qp[2] = acc2.z;
    }
  }
  // one atomic per warp for the ray counters
  for (int o = 16; o > 0; o >>= 1) {
    segs += __shfl_down_sync(0xffffffffu, segs, o);
    shadows += __shfl_down_sync(0xffffffffu, shadows, o);
  }
  if ((threadIdx.x & 31u) == 0) {
    if (segs) atomicAdd(&cnt->rays, segs);
    if (shadows) atomicAdd(&cnt->shadow_rays, shadows);
  }
}

// ---- host orchestration ----------------------------------------------------------
template <class T>
T* carve(char*& p, size_t n) {
  T* r = reinterpret_cast<T*>(p);
  p += ((n * sizeof(T) + 255) / 256) * 256;
  return r;
}

// Kernel classes of the per-launch device timing (bc_last_timing); kTimeEnd
// marks the end of the last timed launch.
enum { kTimeEnd = -1, kTimeGenerate = 0, kTimeExtend, kTimeShade, kTimeConnect, kTimeAccumulate, kTimePost, kTimeOther };

}  // namespace bcgx

struct RenderBuffers {
  int cap = 0;          // path slots
  long long sh_cap = 0; // shadow queue entries
  size_t frame_px = 0;  // pixels of the frame buffers
  bcgx::DevBuf paths, shadow, queues, counters, seq, frame, table;
  bcgx::HostBuf staging;
  bcgx::PathSoA ps{};
  bcgx::ShadowSoA sh{};
  int* q[2] = {nullptr, nullptr};
  bcgx::WaveCounters* cnt = nullptr;
  bcgx::BatchState* bs = nullptr;
  bcgx::ViewGPU* views = nullptr;
  float4* seq_xy = nullptr;  // per sample: (x hi, x lo, y hi, y lo)
  float* sum = nullptr;        // 3 per pixel
  float* sumsq = nullptr;      // 3 per pixel (sample second moments, on request)
  bool want_sumsq = false;
  float* out = nullptr;        // 3 per pixel (mean, then post)
  float* post_tmp = nullptr;   // 3 per pixel
  float* post_tmp2 = nullptr;  // 3 per pixel
  float4* guide_nd = nullptr;  // N, depth (<0: invalid)
  uint32_t* guide_c = nullptr; // compact guide
  uint32_t* guide_jit = nullptr;
  uint32_t* rgba = nullptr;
  bcgx::AdaptState adapt{};    // per-pixel adaptive-sampling state
  // path replay records (gradient renders)
  bcgx::DevBuf rec;
  bcgx::GradRec grec{};
  int rec_bounces = 0, rec_cap = 0;
  // vertex records of the recursive integrator
  bcgx::DevBuf rrec;
  bcgx::RecurRec rr{};
  int rr_bounces = 0, rr_cap = 0;
  // one wave as an instantiated CUDA graph, and the launch arguments it was captured with
  cudaGraphExec_t graph = nullptr;
  std::vector<uintptr_t> graph_key;
  std::vector<uintptr_t> single_key;  // last single-wave render launched without a graph
  // Device time of the last render call: CUDA events on the context's stream
  // around its device work; with render_timing on, one event before every
  // launch (and one after the last), each interval charged to its launch's class.
  cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
  std::vector<cudaEvent_t> kev;
  std::vector<int> kcls;
  size_t kused = 0;
  bool ktiming = false;
  int64_t launches = 0, extend_launches = 0;
  // marks the start of a launch of class `cls` (kTimeEnd: the end of the last one)
  void mark(cudaStream_t st, int cls) {
    if (!ktiming) return;
    if (kused == kev.size()) {
      cudaEvent_t e = nullptr;
      if (cudaEventCreate(&e) != cudaSuccess) {
        ktiming = false;  // timing is best effort; the render itself goes on
        return;
      }
      kev.push_back(e);
    }
    cudaEventRecord(kev[kused++], st);
    kcls.push_back(cls);
  }
};

namespace bcgx {

void destroy_render_buffers(bc_context* ctx) {
  if (!ctx->rb) return;
  RenderBuffers* rb = ctx->rb;
  if (rb->graph) cudaGraphExecDestroy(rb->graph);
  if (rb->ev_begin) cudaEventDestroy(rb->ev_begin);
  if (rb->ev_end) cudaEventDestroy(rb->ev_end);
  for (cudaEvent_t e : rb->kev) cudaEventDestroy(e);
  rb->paths.release();
  rb->shadow.release();
  rb->queues.release();
  rb->counters.release();
  rb->seq.release();
  rb->frame.release();
  rb->table.release();
  rb->staging.release();
  rb->rec.release();
  rb->rrec.release();
  delete rb;
  ctx->rb = nullptr;
}

// Device timing of a render call (bc_last_timing): events on the context's
// stream before the call's first and after its last device work.
static void timing_begin(bc_context* ctx) {
  RenderBuffers* rb = ctx->rb;
  if (!rb->ev_begin) cudaEventCreate(&rb->ev_begin);
  if (!rb->ev_end) cudaEventCreate(&rb->ev_end);
  rb->ktiming = ctx->render_timing != 0;
  rb->kused = 0;
  rb->kcls.clear();
  rb->launches = rb->extend_launches = 0;
  if (rb->ev_begin) cudaEventRecord(rb->ev_begin, ctx->stream);
  rb->mark(ctx->stream, kTimeOther);
}

static void timing_end(bc_context* ctx) {
  RenderBuffers* rb = ctx->rb;
  rb->mark(ctx->stream, kTimeEnd);
  if (rb->ev_end) cudaEventRecord(rb->ev_end, ctx->stream);
}

// After the stream has drained: elapsed times into ctx->last_timing.
static void timing_collect(bc_context* ctx) {
  RenderBuffers* rb = ctx->rb;
  bc_timing t;
  std::memset(&t, 0, sizeof(t));
  float ms = 0.0f;
  if (rb->ev_begin && rb->ev_end && cudaEventElapsedTime(&ms, rb->ev_begin, rb->ev_end) == cudaSuccess)
    t.device_ms = ms;
  t.launches = rb->launches;
  t.extend_launches = rb->extend_launches;
  if (rb->ktiming) {
    double cls_ms[kTimeOther + 1] = {0, 0, 0, 0, 0, 0, 0};
    for (size_t i = 0; i + 1 < rb->kused; i++) {
      const int c = rb->kcls[i];
      if (c < 0) continue;
      if (cudaEventElapsedTime(&ms, rb->kev[i], rb->kev[i + 1]) == cudaSuccess) cls_ms[c] += ms;
    }
    t.kernel_timing = 1;
    t.generate_ms = cls_ms[kTimeGenerate];
    t.extend_ms = cls_ms[kTimeExtend];
    t.shade_ms = cls_ms[kTimeShade];
    t.connect_ms = cls_ms[kTimeConnect];
    t.accumulate_ms = cls_ms[kTimeAccumulate];
    t.post_ms = cls_ms[kTimePost];
    t.other_ms = cls_ms[kTimeOther];
  }
  cudaGetLastError();  // timing is best effort: a failed event query is not the render's error
  ctx->last_timing = t;
}

// Path slots, queues and a shadow queue of sh_cap entries (one per path and
// bounce for the one-shadow-ray integrators; a recursive path can queue one per
// recorded vertex when it ends).
static bc_status ensure_paths(bc_context* ctx, int cap, long long sh_cap) {
  RenderBuffers* rb = ctx->rb;
  if (rb->cap < cap) {
    size_t per = 15 * sizeof(float) + sizeof(uint32_t) + 2 * sizeof(uint64_t) + sizeof(float) + 4 * sizeof(int32_t);
    cudaError_t e = rb->paths.ensure((size_t)cap * per + 64 * 256);
    if (e == cudaSuccess) e = rb->queues.ensure((size_t)cap * 2 * sizeof(int) + 4 * 256);
    if (e != cudaSuccess) {
      rb->cap = 0;
      return cuda_status(ctx, e, "path buffers");
    }
    char* p = (char*)rb->paths.p;
    PathSoA& s = rb->ps;
    float** fl[] = {&s.ox, &s.oy, &s.oz, &s.dx, &s.dy, &s.dz, &s.tx, &s.ty, &s.tz, &s.lx, &s.ly, &s.lz, &s.px, &s.py, &s.pz};
    for (float** f : fl) *f = carve<float>(p, cap);
    s.prev = carve<uint32_t>(p, cap);
    s.rs = carve<uint64_t>(p, cap);
    s.ri = carve<uint64_t>(p, cap);
    s.hit_t = carve<float>(p, cap);
    s.hit_slot = carve<int32_t>(p, cap);
    s.view = carve<int32_t>(p, cap);
    s.pix = carve<int32_t>(p, cap);
    s.samp = carve<int32_t>(p, cap);
    char* qq = (char*)rb->queues.p;
    rb->q[0] = carve<int>(qq, cap);
    rb->q[1] = carve<int>(qq, cap);
    rb->cap = cap;
  }
  if (rb->sh_cap < sh_cap) {
    cudaError_t e = rb->shadow.ensure((size_t)sh_cap * (3 * sizeof(float4) + sizeof(int32_t)) + 8 * 256);
    if (e != cudaSuccess) {
      rb->sh_cap = 0;
      return cuda_status(ctx, e, "shadow queue");
    }
    char* q = (char*)rb->shadow.p;
    rb->sh.o = carve<float4>(q, sh_cap);
    rb->sh.d = carve<float4>(q, sh_cap);
    rb->sh.c = carve<float4>(q, sh_cap);
    rb->sh.path = carve<int32_t>(q, sh_cap);
    rb->sh_cap = sh_cap;
  }
  return BC_OK;
}

static bc_status ensure_frame(bc_context* ctx, size_t px) {
  RenderBuffers* rb = ctx->rb;
  if (rb->frame_px >= px) return BC_OK;
  size_t bytes = px * (5 * 3 * sizeof(float) + sizeof(float4) + 5 * sizeof(uint32_t) + sizeof(int32_t) +
                       sizeof(float2)) + 16 * 256;
  cudaError_t e = rb->frame.ensure(bytes);
  if (e != cudaSuccess) {
    rb->frame_px = 0;
    return cuda_status(ctx, e, "frame buffers");
  }
  char* p = (char*)rb->frame.p;
  rb->sum = carve<float>(p, 3 * px);
  rb->sumsq = carve<float>(p, 3 * px);
  rb->out = carve<float>(p, 3 * px);
  rb->post_tmp = carve<float>(p, 3 * px);
  rb->post_tmp2 = carve<float>(p, 3 * px);
  rb->guide_nd = carve<float4>(p, px);
  rb->guide_c = carve<uint32_t>(p, 3 * px);
  rb->guide_jit = carve<uint32_t>(p, px);
  rb->rgba = carve<uint32_t>(p, px);
  rb->adapt.n = carve<int32_t>(p, px);
  rb->adapt.lum = carve<float2>(p, px);
  rb->frame_px = px;
  return BC_OK;
}

int effective_spp(const bc_settings& s) {  // renderer.go:2395-2417
  int msaa = (s.msaa == 2 || s.msaa == 4 || s.msaa == 8) ? s.msaa : 1;
  int tsaa = s.tsaa == 1 ? 2 : s.tsaa == 2 ? 3 : s.tsaa == 3 ? 4 : 1;
  long v = (long)s.spp * msaa * tsaa;
  return v < 1 ? 1 : (v > 4096 ? 4096 : (int)v);
}

// Halton table (buildSampleSequence, renderer.go:1883-1904), computed on the
// host in fp64 exactly as the reference does; appended to X, Y.
// fp64 value as a float-float pair (hi, lo): hi = fp32(v), lo = fp32(v - hi)
static float2 ff_split(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}

static void sample_sequence(const bc_settings& s, std::vector<double>* X, std::vector<double>* Y) {
  if (s.sampler == BC_SAMPLER_RANDOM) return;
  const int n = effective_spp(s);
  if (s.sampler == BC_SAMPLER_R2) {
    const double g = 1.324717957244746;
    const double a1 = 1.0 / g, a2 = 1.0 / (g * g);
    for (int i = 0; i < n; i++) {
      double a = 0.5 + (double)(i + 1) * a1, b = 0.5 + (double)(i + 1) * a2;
      X->push_back(a - std::floor(a));
      Y->push_back(b - std::floor(b));
    }
    return;
  }
  for (int i = 0; i < n; i++) {
    uint64_t m = (uint64_t)(i + 1), r = 0;
    for (int k = 0; k < 64; k++) { r = (r << 1) | (m & 1); m >>= 1; }
    X->push_back((double)r * 5.421010862427522e-20);
    uint64_t n3 = (uint64_t)(i + 1);
    double invBase = 1.0 / 3.0, inv = invBase, res = 0;
    while (n3 > 0) {
      res += (double)(n3 % 3) * inv;
      n3 /= 3;
      inv *= invBase;
    }
    Y->push_back(res);
  }
}

// Camera.basis (renderer.go:947-960) in fp64.
static void camera_basis(const bc_camera& c, double aspect, double o[3], double lower[3], double horiz[3],
                         double vert[3]) {
  auto unit = [](double v[3]) {
    double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (l < 1e-12) { v[0] = v[1] = v[2] = 0; return; }
    double s = 1 / l;
    v[0] *= s; v[1] *= s; v[2] *= s;
  };
  auto cross = [](const double a[3], const double b[3], double r[3]) {
    r[0] = a[1] * b[2] - a[2] * b[1];
    r[1] = a[2] * b[0] - a[0] * b[2];
    r[2] = a[0] * b[1] - a[1] * b[0];
  };
  double theta = c.fov_deg * M_PI / 180;
  double h = std::tan(theta / 2);
  double vh = 2 * h, vw = aspect * vh;
  double w[3] = {c.position[0] - c.target[0], c.position[1] - c.target[1], c.position[2] - c.target[2]};
  unit(w);
  double u[3];
  cross(c.up, w, u);
  unit(u);
  double v[3];
  cross(w, u, v);
  for (int k = 0; k < 3; k++) {
    o[k] = c.position[k];
    horiz[k] = u[k] * vw;
    vert[k] = v[k] * vh;
    lower[k] = ((o[k] - horiz[k] * .5) - vert[k] * .5) - w[k];
  }
}

static int sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms < 1) sms = 1;
  }
  return sms;
}

int gradient_grid() { return sm_count() * 2; }

static int persistent_grid(const void* fn, int block) {
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, 0);
  return sm_count() * std::max(1, per);
}

// Launch shape of one wave; computed before any stream capture.
struct WaveShape {
  int ext;          // k_extend variant (render_extend)
  int shade_block;  // k_shade block size (render_shade_block)
  int gen_grid, ext_grid, con_grid, shade_grid, acc_grid;
  int bounces;
  bool lights;
  const GradArgs* grad;  // non-null: gradient render
  bool recursive;        // the batch has views of the recursive integrator
  bool alt;              // the batch has views of the recursive or photon integrator
};

template <int STACK, bool SPH>
static const void* extend_kernel(int var) {
  switch (var) {
    case 0: return (const void*)k_extend<STACK, SPH>;
    case 2: return (const void*)k_extend_12<STACK, SPH>;
    default: return (const void*)k_extend_10<STACK, SPH>;
  }
}

template <int STACK, bool SPH>
static WaveShape wave_shape(int cap, int bounces, bool lights, const GradArgs* grad, int ext_var, int shade_block) {
  static int ext[kExtendVariants] = {0, 0, 0}, con = 0;
  const int var = ext_var >= 0 && ext_var < kExtendVariants ? ext_var : 1;
  if (!ext[var]) ext[var] = persistent_grid(extend_kernel<STACK, SPH>(var), 128);
  if (!con) con = persistent_grid((const void*)k_connect<STACK, SPH>, 128);
  WaveShape w;
  w.ext = var;
  w.gen_grid = (cap + 255) / 256;
  w.ext_grid = ext[var];
  w.con_grid = con;
  // grid-stride kernels at their resident blocks per SM (four of 256 threads,
  // eight of 128: their register budget): one wave of blocks, no partial last wave
  w.shade_block = shade_block == 128 ? 128 : 256;
  w.shade_grid = sm_count() * (w.shade_block == 128 ? 8 : 4);
  w.acc_grid = sm_count() * 3;
  w.bounces = bounces;
  w.lights = lights;
  w.grad = grad;
  w.recursive = false;
  w.alt = false;
  return w;
}

// Enqueues one wave: generate, the bounces, accumulate, advance.
template <int STACK, bool SPH>
static cudaError_t enqueue_wave(bc_context* ctx, const WaveShape& w, const ShadeScene& sc, cudaStream_t st) {
  RenderBuffers* rb = ctx->rb;
  WaveCounters* c = rb->cnt;
  const RecurRec rr = w.recursive ? rb->rr : RecurRec{nullptr, nullptr, nullptr, nullptr, 0};
  rb->mark(st, kTimeGenerate);
  k_generate<<<w.gen_grid, 256, 0, st>>>(rb->bs, rb->views, rb->ps, rb->q[0], rb->seq_xy, rb->guide_jit, c,
                                         rb->adapt);
  int cur = 0;
  // Counter resets ride in the kernels: generate zeroes the first extend's work
  // counter, extend zeroes the queue and shadow list its shade fills, shade
  // zeroes the work counters of the next extend and of its connect.
  for (int b = 0; b < w.bounces; b++) {
    rb->mark(st, kTimeExtend);
    if (w.ext == 0)
      k_extend<STACK, SPH><<<w.ext_grid, 128, 0, st>>>(sc.sv, rb->views, rb->ps, rb->q[cur], c, cur, ctx->d_status);
    else if (w.ext == 2)
      k_extend_12<STACK, SPH><<<w.ext_grid, 128, 0, st>>>(sc.sv, rb->views, rb->ps, rb->q[cur], c, cur, ctx->d_status);
    else
      k_extend_10<STACK, SPH><<<w.ext_grid, 128, 0, st>>>(sc.sv, rb->views, rb->ps, rb->q[cur], c, cur, ctx->d_status);
    const GradRec rec = w.grad ? rb->grec : GradRec{nullptr, nullptr, nullptr, 0};
    rb->mark(st, kTimeShade);
#define BC_SHADE_LAUNCH(KERNEL, BLOCK)                                                                         \
  KERNEL<<<w.shade_grid, BLOCK, 0, st>>>(rb->views, ctx->ds.n_mats, sc, rb->ps, rb->q[cur], rb->q[cur ^ 1], rb->sh, \
                                        c, cur, b, rb->guide_nd, rb->guide_c, rb->guide_jit, rec, rr, rb->sh_cap,   \
                                        ctx->d_status)
    if (w.shade_block == 128) {
      if (w.alt) BC_SHADE_LAUNCH(k_shade_128<true>, 128);
      else BC_SHADE_LAUNCH(k_shade_128<false>, 128);
    } else {
      if (w.alt) BC_SHADE_LAUNCH(k_shade<true>, 256);
      else BC_SHADE_LAUNCH(k_shade<false>, 256);
    }
#undef BC_SHADE_LAUNCH
    if (w.lights) rb->mark(st, kTimeConnect);
    if (w.lights)
      k_connect<STACK, SPH><<<w.con_grid, 128, 0, st>>>(sc.sv, rb->ps, rb->sh, c, rr, rb->sh_cap, ctx->d_status);
    cur ^= 1;
  }
  if (w.grad) rb->mark(st, kTimeOther);
  if (w.grad)
    k_gradient<<<gradient_grid(), 256, 3 * w.grad->n_params * sizeof(double), st>>>(rb->bs, rb->views, rb->ps,
                                                                                  rb->grec, *w.grad, sc.mats);
  rb->mark(st, kTimeAccumulate);
  k_accumulate<<<w.acc_grid, 256, 0, st>>>(rb->bs, rb->views, rb->ps, rb->sum, rb->want_sumsq ? rb->sumsq : nullptr,
                                           rb->adapt, rr);
  rb->mark(st, kTimeOther);
  k_advance<<<1, 32, 0, st>>>(rb->bs, c);
  return cudaGetLastError();
}

// Runs `n_waves` waves, through one captured CUDA graph when the option allows.
template <int STACK, bool SPH>
static bc_status run_waves(bc_context* ctx, int bounces, bool lights, const ShadeScene& sc, int64_t n_waves,
                           int wave_paths, const GradArgs* grad, bool recursive, bool alt) {
  RenderBuffers* rb = ctx->rb;
  cudaStream_t st = ctx->stream;
  // generate's grid covers this render's wave, not the slots a larger earlier
  // render left allocated
  WaveShape w = wave_shape<STACK, SPH>(wave_paths, bounces, lights, grad, ctx->render_extend, ctx->render_shade_block);
  w.recursive = recursive;
  w.alt = alt;
  // A wave graph pays for its capture when a render has several waves, or when
  // a single-wave render repeats with the same launches (a frame loop at fixed
  // settings): such a render is captured the second time its key is seen.
  bool use_graph = ctx->render_graph != 0 && !rb->ktiming;  // per-launch events need direct launches
  rb->launches += n_waves * (3 + (int64_t)bounces * (2 + (lights ? 1 : 0)) + (grad ? 1 : 0));
  rb->extend_launches += n_waves * (int64_t)bounces;
  if (use_graph) {
    // every value the captured launches were given
    std::vector<uintptr_t> key = {(uintptr_t)STACK, (uintptr_t)SPH, (uintptr_t)w.ext, (uintptr_t)w.ext_grid,
                                  (uintptr_t)w.shade_block, (uintptr_t)w.shade_grid,
                                  (uintptr_t)bounces, (uintptr_t)lights,
                                  (uintptr_t)rb->cap, (uintptr_t)w.gen_grid, (uintptr_t)rb->q[0], (uintptr_t)rb->q[1],
                                  (uintptr_t)rb->cnt, (uintptr_t)rb->bs, (uintptr_t)rb->views, (uintptr_t)rb->seq_xy,
                                  (uintptr_t)rb->sum, (uintptr_t)(rb->want_sumsq ? rb->sumsq : nullptr),
                                  (uintptr_t)rb->guide_nd, (uintptr_t)rb->guide_c, (uintptr_t)rb->guide_jit,
                                  (uintptr_t)rb->adapt.n, (uintptr_t)rb->adapt.lum,
                                  (uintptr_t)ctx->ds.n_mats, (uintptr_t)ctx->d_status};
    auto add_bytes = [&key](const void* p, size_t n) {
      const size_t k = key.size();
      key.resize(k + (n + sizeof(uintptr_t) - 1) / sizeof(uintptr_t), 0);
      std::memcpy(key.data() + k, p, n);
    };
    add_bytes(&rb->ps, sizeof(rb->ps));
    add_bytes(&rb->sh, sizeof(rb->sh));
    key.push_back((uintptr_t)rb->sh_cap);
    key.push_back((uintptr_t)recursive);
    key.push_back((uintptr_t)alt);
    if (recursive) add_bytes(&rb->rr, sizeof(rb->rr));
    add_bytes(&sc, sizeof(sc));
    key.push_back((uintptr_t)(grad != nullptr));
    if (grad) {
      add_bytes(grad, sizeof(*grad));
      add_bytes(&rb->grec, sizeof(rb->grec));
    }
    if (n_waves == 1 && !(rb->graph && rb->graph_key == key) && rb->single_key != key) {
      rb->single_key = key;  // first sighting: launch directly
      use_graph = false;
    } else if (!rb->graph || rb->graph_key != key) {
      if (rb->graph) cudaGraphExecDestroy(rb->graph);
      rb->graph = nullptr;
      rb->graph_key.clear();
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
      if (e) return cuda_status(ctx, e, "wave capture");
      cudaError_t le = enqueue_wave<STACK, SPH>(ctx, w, sc, st);
      e = cudaStreamEndCapture(st, &g);
      if (le) e = le;
      if (!e) e = cudaGraphInstantiate(&rb->graph, g, 0);
      if (g) cudaGraphDestroy(g);
      if (e) {
        rb->graph = nullptr;
        return cuda_status(ctx, e, "wave graph");
      }
      rb->graph_key = key;
    }
  }
  for (int64_t k = 0; k < n_waves; k++) {
    if (*(volatile int*)ctx->h_cancel || ctx->cancel.load()) {
      cudaStreamSynchronize(st);
      return set_error(ctx, BC_ERR_CANCELLED, "render cancelled");
    }
    cudaError_t e = use_graph ? cudaGraphLaunch(rb->graph, st) : enqueue_wave<STACK, SPH>(ctx, w, sc, st);
    if (e) return cuda_status(ctx, e, "wavefront launch");
  }
  return BC_OK;
}

static bc_status check_view(bc_context* ctx, const ViewRequest& r) {
  const bc_settings& s = r.s;
  if (r.scene < 0 || r.scene >= (int)ctx->ranges.size())
    return set_error(ctx, BC_ERR_INVALID_ARG, "view names a scene outside the resident set");
  if (s.width < 1 || s.height < 1 || s.bounces < 1 || s.spp < 1 || r.y0 < 0 || r.rows < 1 || r.y0 + r.rows > s.height)
    return set_error(ctx, BC_ERR_INVALID_ARG, "invalid render size, rows, spp or bounces");
  if ((int64_t)s.width * s.height > (1 << 26)) return set_error(ctx, BC_ERR_INVALID_ARG, "frame too large");
  if (s.bounces > kMaxBounces) return set_error(ctx, BC_ERR_INVALID_ARG, "bounces above 1024");
  if (s.integrator < BC_INTEGRATOR_PATH || s.integrator > BC_INTEGRATOR_PHOTON)
    return set_error(ctx, BC_ERR_INVALID_ARG, "unknown integrator");
  if (s.integrator == BC_INTEGRATOR_RECURSIVE && ctx->render_engine == 1)
    return set_error(ctx, BC_ERR_INVALID_ARG, "the one-kernel form renders the path and photon integrators");
  return BC_OK;
}

// Renders the requested views into rb->sum (and guides); `frame_px` pixels of
// frame buffers are kept. Leaves the per-view table in rb->views.
// The one-kernel form: one launch per view.
template <int STACK, bool SPH>
static bc_status run_plain(bc_context* ctx, const ShadeScene& sc, const std::vector<ViewGPU>& views, bool alt) {
  RenderBuffers* rb = ctx->rb;
  for (int v = 0; v < (int)views.size(); v++) {
    if (*(volatile int*)ctx->h_cancel || ctx->cancel.load()) {
      cudaStreamSynchronize(ctx->stream);
      return set_error(ctx, BC_ERR_CANCELLED, "render cancelled");
    }
    const int grid = (views[v].npix + 127) / 128;
    rb->mark(ctx->stream, kTimeOther);
    rb->launches++;
    if (alt)
      k_render_plain<STACK, SPH, true><<<grid, 128, 0, ctx->stream>>>(
          rb->views, v, ctx->ds.n_mats, sc, rb->seq_xy, rb->sum, rb->want_sumsq ? rb->sumsq : nullptr, rb->guide_nd,
          rb->guide_c, rb->guide_jit, rb->cnt, ctx->d_status, rb->adapt);
    else
      k_render_plain<STACK, SPH, false><<<grid, 128, 0, ctx->stream>>>(
          rb->views, v, ctx->ds.n_mats, sc, rb->seq_xy, rb->sum, rb->want_sumsq ? rb->sumsq : nullptr, rb->guide_nd,
          rb->guide_c, rb->guide_jit, rb->cnt, ctx->d_status, rb->adapt);
    cudaError_t e = cudaGetLastError();
    if (e) return cuda_status(ctx, e, "one-kernel render launch");
  }
  return BC_OK;
}

bc_status render_views(bc_context* ctx, const std::vector<ViewRequest>& req, size_t frame_px, int64_t* rays,
                       const GradArgs* grad) {
  if (!ctx->has_scene) return set_error(ctx, BC_ERR_NO_SCENE, "no scene uploaded");
  if (req.empty()) return set_error(ctx, BC_ERR_INVALID_ARG, "no views");
  bc_status bst;
  for (const ViewRequest& r : req) {
    if ((bst = check_view(ctx, r))) return bst;
    if (grad && r.s.integrator != BC_INTEGRATOR_PATH)
      return set_error(ctx, BC_ERR_INVALID_ARG, "gradient renders use the path integrator");
  }
  if (!ctx->rb) ctx->rb = new RenderBuffers();
  RenderBuffers* rb = ctx->rb;
  const int n = (int)req.size();
  std::vector<ViewGPU> views(n);
  std::vector<double> X, Y;
  long long total = 0;
  int max_bounces = 0, rec_bounces = 0;
  bool lights = false, alt = false;
  std::vector<const unsigned long long*> photon_rays;  // ray counters of photon maps built for this call
  const uint64_t photon_pin = photon_clock(ctx);
  for (int v = 0; v < n; v++) {
    const ViewRequest& r = req[v];
    const SceneRange& sr = ctx->ranges[r.scene];
    ViewGPU& V = views[v];
    std::memset(&V, 0, sizeof(V));
    V.W = r.s.width;
    V.H = r.s.height;
    V.y0 = r.y0;
    V.rows = r.rows;
    V.npix = r.s.width * r.rows;
    V.pix_off = r.pix_off;
    V.spp = effective_spp(r.s);
    V.bounces = r.s.bounces;
    V.rr_depth = r.s.rr_depth;
    V.sampler = r.s.sampler;
    V.mis = r.s.mis != 0;
    V.power = r.s.power_light_sampling != 0;
    V.seq_off = (int)X.size();
    sample_sequence(r.s, &X, &Y);
    V.nseq = (int)X.size() - V.seq_off;
    V.n_lights = sr.n_lights;
    V.light_off = sr.light_off;
    V.root = sr.root;
    V.want_guides = r.want_guides ? 1 : 0;
    V.clamp = (float)r.s.firefly_clamp;
    V.adaptive = (r.s.adaptive_sampling != 0 && !grad) ? 1 : 0;  // gradient renders take every sample
    V.adapt_thr = (float)std::max(1e-8, r.s.adaptive_threshold);
    V.min_samples = std::min(8, V.spp);
    V.seed = r.s.seed;
    V.integrator = r.s.integrator;
    alt = alt || V.integrator != BC_INTEGRATOR_PATH;
    if (V.integrator == BC_INTEGRATOR_RECURSIVE) rec_bounces = std::max(rec_bounces, V.bounces);
    if (V.integrator == BC_INTEGRATOR_PHOTON) {  // built once per frame (renderer.go:2728-2734), then cached
      const unsigned long long* built = nullptr;
      if ((bst = photon_map_for(ctx, r.scene, r.s, photon_pin, &V.pm, &built))) return bst;
      if (built) photon_rays.push_back(built);
    }
    camera_basis(r.cam, (double)V.W / (double)V.H, V.origin, V.lower, V.horiz, V.vert);
    for (int k = 0; k < 3; k++) {
      V.base[k] = ff_split(V.lower[k] - V.origin[k]);
      V.span_u[k] = ff_split(V.horiz[k]);
      V.span_v[k] = ff_split(V.vert[k]);
      V.o32[k] = (float)V.origin[k];
    }
    V.inv_w1 = ff_split(1.0 / (double)std::max(V.W - 1, 1));
    V.inv_h1 = ff_split(1.0 / (double)std::max(V.H - 1, 1));
    V.path_off = total;
    total += (long long)V.npix * V.spp;
    max_bounces = std::max(max_bounces, V.bounces);
    lights = lights || sr.n_lights > 0;
  }
  long long cap_limit = ctx->render_wave_cap;
  if (grad)  // path replay records cost 20 bytes per path and bounce: keep them under 8 GB
    cap_limit = std::min<long long>(cap_limit, std::max<long long>(4096, (8LL << 30) / (20LL * max_bounces)));
  if (rec_bounces)  // a recursive path queues up to one shadow ray per vertex when it ends
    cap_limit = std::max<long long>(4096, cap_limit / rec_bounces);
  const int cap = (int)std::max<long long>(1, std::min<long long>(total, cap_limit));
  const long long sh_cap = (long long)cap * std::max(1, rec_bounces);
  if ((bst = ensure_paths(ctx, cap, sh_cap))) return bst;
  if ((bst = ensure_frame(ctx, frame_px))) return bst;
  if (rec_bounces && (rb->rr_bounces < rec_bounces || rb->rr_cap < cap)) {  // stride: this render's wave size
    const size_t nrec = (size_t)rec_bounces * cap;
    cudaError_t e = rb->rrec.ensure(nrec * 3 * sizeof(float4) + (size_t)cap * sizeof(int32_t) + 8 * 256);
    if (e) {
      rb->rr_bounces = rb->rr_cap = 0;
      return cuda_status(ctx, e, "recursive vertex records");
    }
    char* p = (char*)rb->rrec.p;
    rb->rr.a = carve<float4>(p, nrec);
    rb->rr.n = carve<float4>(p, nrec);
    rb->rr.w = carve<float4>(p, nrec);
    rb->rr.nb = carve<int32_t>(p, cap);
    rb->rr.cap = cap;
    rb->rr_bounces = rec_bounces;
    rb->rr_cap = cap;
  }
  if (grad) {  // path replay records: one per path and bounce
    if (max_bounces > kMaxGradBounces) return set_error(ctx, BC_ERR_INVALID_ARG, "gradient renders allow 64 bounces");
    // stride: this render's wave size (path slots >= cap are never used by it)
    if (rb->rec_bounces < max_bounces || rb->rec_cap < cap) {
      const size_t per = sizeof(int32_t) + sizeof(float4);
      cudaError_t e = rb->rec.ensure((size_t)max_bounces * cap * per + (size_t)cap * sizeof(int32_t) + 4 * 256);
      if (e) {
        rb->rec_bounces = rb->rec_cap = 0;
        return cuda_status(ctx, e, "path replay records");
      }
      char* p = (char*)rb->rec.p;
      rb->grec.v = carve<float4>(p, (size_t)max_bounces * cap);
      rb->grec.m = carve<int32_t>(p, (size_t)max_bounces * cap);
      rb->grec.nb = carve<int32_t>(p, cap);
      rb->grec.cap = cap;
      rb->rec_bounces = max_bounces;
      rb->rec_cap = cap;
    }
  }
  BatchState bsh;
  bsh.w0 = 0;
  bsh.total = total;
  bsh.cap = std::min(cap, rb->cap);
  bsh.n_views = n;
  // device tables: views, batch cursor, counters; the sample tables
  // device tables at fixed offsets (a captured wave keeps these addresses):
  // [BatchState | WaveCounters | views], and the (x, y) sample pairs
  const size_t tbytes = 512 + n * sizeof(ViewGPU);
  const size_t sbytes = std::max<size_t>(16, X.size() * sizeof(float4));
  cudaError_t e = cudaStreamSynchronize(ctx->stream);  // the staging buffer may still be in flight
  if (!e) e = rb->table.ensure(tbytes);
  if (!e) e = rb->seq.ensure(sbytes);
  if (!e) e = rb->staging.ensure(tbytes + 16 + sbytes);
  if (e) return cuda_status(ctx, e, "render tables");
  rb->bs = rb->table.as<BatchState>();
  rb->cnt = reinterpret_cast<WaveCounters*>((char*)rb->table.p + 256);
  rb->views = reinterpret_cast<ViewGPU*>((char*)rb->table.p + 512);
  rb->seq_xy = rb->seq.as<float4>();
  char* hs = (char*)rb->staging.p;
  std::memset(hs, 0, 512);
  std::memcpy(hs, &bsh, sizeof(bsh));
  std::memcpy(hs + 512, views.data(), n * sizeof(ViewGPU));
  float4* hq = reinterpret_cast<float4*>(hs + tbytes + ((16 - (tbytes & 15)) & 15));
  for (size_t i = 0; i < X.size(); i++) {
    const float2 a = ff_split(X[i]), b = ff_split(Y[i]);
    hq[i] = make_float4(a.x, a.y, b.x, b.y);
  }
  timing_begin(ctx);
  e = cudaMemcpyAsync(rb->table.p, hs, tbytes, cudaMemcpyHostToDevice, ctx->stream);
  if (!e && !X.empty())
    e = cudaMemcpyAsync(rb->seq.p, hq, X.size() * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream);
  for (int v = 0; v < n && !e; v++) {
    const ViewGPU& V = views[v];
    e = cudaMemsetAsync(rb->sum + 3 * (size_t)V.pix_off, 0, 3 * sizeof(float) * (size_t)V.npix, ctx->stream);
    if (!e && V.adaptive) e = cudaMemsetAsync(rb->adapt.n + V.pix_off, 0, sizeof(int32_t) * (size_t)V.npix, ctx->stream);
    if (!e && V.adaptive)
      e = cudaMemsetAsync(rb->adapt.lum + V.pix_off, 0, sizeof(float2) * (size_t)V.npix, ctx->stream);
    if (!e && rb->want_sumsq)
      e = cudaMemsetAsync(rb->sumsq + 3 * (size_t)V.pix_off, 0, 3 * sizeof(float) * (size_t)V.npix, ctx->stream);
    if (!e && V.want_guides) {  // invalid guides: depth -1, compact words 0
      rb->launches++;
      k_clear_guides<<<(V.npix + 255) / 256, 256, 0, ctx->stream>>>(V.npix, rb->guide_nd + V.pix_off,
                                                                    rb->guide_c + 3 * (size_t)V.pix_off);
      e = cudaGetLastError();
    }
  }
  if (e) return cuda_status(ctx, e, "render setup");

  ShadeScene sc;
  sc.sv.nodes = ctx->ds.nodes;
  sc.sv.tri = ctx->ds.tri;
  sc.sv.slot64 = ctx->ds.slot64;
  sc.sv.snorm = ctx->ds.snorm;
  sc.sv.slot_prim = ctx->ds.slot_prim;
  sc.mats = ctx->ds.mats;
  sc.lights = ctx->ds.lights;
  sc.lpdf_by_prim = ctx->ds.light_pdf_by_prim;
  const int64_t n_waves = (total + bsh.cap - 1) / bsh.cap;
  const int stack = stack_variant(ctx->ds.stack_need);
  const bool sph = ctx->ds.has_spheres;
  if (ctx->render_engine == 1 && !grad) {
    if (stack == 64) bst = sph ? run_plain<64, true>(ctx, sc, views, alt) : run_plain<64, false>(ctx, sc, views, alt);
    else if (stack == 128) bst = sph ? run_plain<128, true>(ctx, sc, views, alt) : run_plain<128, false>(ctx, sc, views, alt);
    else bst = sph ? run_plain<256, true>(ctx, sc, views, alt) : run_plain<256, false>(ctx, sc, views, alt);
  } else if (stack == 64)
    bst = sph ? run_waves<64, true>(ctx, max_bounces, lights, sc, n_waves, bsh.cap, grad, rec_bounces > 0, alt)
              : run_waves<64, false>(ctx, max_bounces, lights, sc, n_waves, bsh.cap, grad, rec_bounces > 0, alt);
  else if (stack == 128)
    bst = sph ? run_waves<128, true>(ctx, max_bounces, lights, sc, n_waves, bsh.cap, grad, rec_bounces > 0, alt)
              : run_waves<128, false>(ctx, max_bounces, lights, sc, n_waves, bsh.cap, grad, rec_bounces > 0, alt);
  else
    bst = sph ? run_waves<256, true>(ctx, max_bounces, lights, sc, n_waves, bsh.cap, grad, rec_bounces > 0, alt)
              : run_waves<256, false>(ctx, max_bounces, lights, sc, n_waves, bsh.cap, grad, rec_bounces > 0, alt);
  if (bst) return bst;
  rb->mark(ctx->stream, kTimeOther);
  k_finish_views<<<sm_count() * 8, 256, 0, ctx->stream>>>(rb->views, n, rb->sum, rb->out, rb->adapt.n);
  if (rb->want_sumsq)
    k_finish_views<<<sm_count() * 8, 256, 0, ctx->stream>>>(rb->views, n, rb->sumsq, rb->post_tmp, rb->adapt.n);
  rb->launches += rb->want_sumsq ? 2 : 1;
  timing_end(ctx);
  e = cudaGetLastError();
  unsigned long long r = 0;
  std::vector<unsigned long long> pr(photon_rays.size(), 0);
  if (!e) e = cudaMemcpyAsync(&r, &rb->cnt->rays, sizeof(r), cudaMemcpyDeviceToHost, ctx->stream);
  for (size_t k = 0; k < photon_rays.size() && !e; k++)
    e = cudaMemcpyAsync(&pr[k], photon_rays[k], sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  if (e) return cuda_status(ctx, e, "render");
  for (unsigned long long v : pr) r += v;  // Start counts the photon map's rays (renderer.go:2809)
  if (rays) *rays = (int64_t)r;
  timing_collect(ctx);
  return check_kernel_status(ctx);
}

static bc_status render_rows_device(bc_context* ctx, const bc_camera& cam, const bc_settings& s, int y0, int rows,
                                    bool want_guides, int64_t* rays) {
  ViewRequest r;
  r.scene = 0;
  r.cam = cam;
  r.s = s;
  r.y0 = y0;
  r.rows = rows;
  r.pix_off = (long long)y0 * s.width;
  r.want_guides = want_guides;
  if (s.width < 1 || s.height < 1 || (int64_t)s.width * s.height > (1 << 26))
    return set_error(ctx, BC_ERR_INVALID_ARG, "invalid render size, rows, spp or bounces");
  return render_views(ctx, std::vector<ViewRequest>{r}, (size_t)s.width * s.height, rays, nullptr);
}

float* render_mean(bc_context* ctx) { return ctx->rb ? ctx->rb->out : nullptr; }

bc_status run_post(bc_context* ctx, const bc_settings& s);  // post.cu

struct PostTargets {
  float* img;
  const float4* guide;
  float* tmp;
  float* tmp2;
  uint32_t* rgba;
};

PostTargets post_targets(bc_context* ctx) {
  RenderBuffers* rb = ctx->rb;
  return PostTargets{rb->out, rb->guide_nd, rb->post_tmp, rb->post_tmp2, rb->rgba};
}

bc_status ensure_post_scratch(bc_context* ctx, int px, PostTargets* t) {
  if (!ctx->rb) ctx->rb = new RenderBuffers();
  bc_status st = ensure_frame(ctx, (size_t)px);
  if (st) return st;
  *t = post_targets(ctx);
  return BC_OK;
}

// The whole-frame requests of a batch of views, laid out one after another in
// the frame buffers; *px = pixels of the batch.
bc_status batch_requests(bc_context* ctx, const bc_view* views, int32_t n_views, std::vector<ViewRequest>* req,
                         long long* px) {
  req->assign(n_views, ViewRequest());
  *px = 0;
  for (int v = 0; v < n_views; v++) {
    ViewRequest& r = (*req)[v];
    r.scene = views[v].scene;
    r.cam = views[v].camera;
    r.s = views[v].settings;
    r.y0 = 0;
    r.rows = r.s.height;
    r.pix_off = *px;
    r.want_guides = false;
    if (r.s.width < 1 || r.s.height < 1 || (int64_t)r.s.width * r.s.height > (1 << 26))
      return set_error(ctx, BC_ERR_INVALID_ARG, "invalid render size in view " + std::to_string(v));
    *px += (long long)r.s.width * r.s.height;
  }
  if (*px > (1LL << 30)) return set_error(ctx, BC_ERR_INVALID_ARG, "batch holds more than 2^30 pixels");
  return BC_OK;
}

}  // namespace bcgx

using namespace bcgx;

extern "C" {

bc_status bc_render_rows(bc_context* ctx, const bc_camera* cam, const bc_settings* settings, int32_t y0,
                         int32_t rows, float* linear_out, uint32_t* guide_out, int64_t* rays_out) {
  if (!ctx || !cam || !settings || !linear_out) return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument");
  cudaSetDevice(ctx->device);
  int64_t rays = 0;
  bc_status st = render_rows_device(ctx, *cam, *settings, y0, rows, guide_out != nullptr, &rays);
  if (st) return st;
  RenderBuffers* rb = ctx->rb;
  const int W = settings->width, npix = W * rows;
  cudaError_t e = cudaMemcpyAsync(linear_out, rb->out + 3 * (size_t)y0 * W, 3 * sizeof(float) * (size_t)npix,
                                  cudaMemcpyDeviceToHost, ctx->stream);
  if (!e && guide_out)
    e = cudaMemcpyAsync(guide_out, rb->guide_c + 3 * (size_t)y0 * W, 3 * sizeof(uint32_t) * (size_t)npix,
                        cudaMemcpyDeviceToHost, ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  if (e) return cuda_status(ctx, e, "render readback");
  if (rays_out) *rays_out = rays;
  return BC_OK;
}

bc_status bc_render_frame(bc_context* ctx, const bc_camera* cam, const bc_settings* settings, float* linear_out,
                          uint32_t* guide_out, uint32_t* rgba_out, int64_t* rays_out) {
  if (!ctx || !cam || !settings) return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument");
  cudaSetDevice(ctx->device);
  const bool need_guides = settings->denoise || guide_out;
  int64_t rays = 0;
  bc_status st = render_rows_device(ctx, *cam, *settings, 0, settings->height, need_guides, &rays);
  if (st) return st;
  RenderBuffers* rb = ctx->rb;
  const int npix = settings->width * settings->height;
  rb->mark(ctx->stream, kTimePost);
  if ((st = run_post(ctx, *settings))) return st;
  // the frame's device time runs to the end of the post stack
  rb->launches += (settings->denoise ? std::max(0, 2 + std::min(3, std::max(settings->taa, settings->txaa))) : 0) +
                  (settings->bloom > 0 ? 2 : 0) + 1;
  timing_end(ctx);
  cudaError_t e = cudaSuccess;
  if (linear_out)
    e = cudaMemcpyAsync(linear_out, rb->out, 3 * sizeof(float) * (size_t)npix, cudaMemcpyDeviceToHost, ctx->stream);
  if (!e && guide_out)
    e = cudaMemcpyAsync(guide_out, rb->guide_c, 3 * sizeof(uint32_t) * (size_t)npix, cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (!e && rgba_out)
    e = cudaMemcpyAsync(rgba_out, rb->rgba, sizeof(uint32_t) * (size_t)npix, cudaMemcpyDeviceToHost, ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  if (e) return cuda_status(ctx, e, "frame readback");
  timing_collect(ctx);
  if (rays_out) *rays_out = rays;
  return BC_OK;
}

bc_status bc_render_moments(bc_context* ctx, const bc_camera* cam, const bc_settings* settings, float* mean_out,
                            float* meansq_out, int64_t* rays_out) {
  if (!ctx || !cam || !settings || !mean_out || !meansq_out)
    return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument");
  cudaSetDevice(ctx->device);
  if (!ctx->rb) ctx->rb = new RenderBuffers();
  ctx->rb->want_sumsq = true;
  int64_t rays = 0;
  bc_status st = render_rows_device(ctx, *cam, *settings, 0, settings->height, false, &rays);
  ctx->rb->want_sumsq = false;
  if (st) return st;
  RenderBuffers* rb = ctx->rb;
  const int npix = settings->width * settings->height;
  cudaError_t e =
      cudaMemcpyAsync(mean_out, rb->out, 3 * sizeof(float) * (size_t)npix, cudaMemcpyDeviceToHost, ctx->stream);
  if (!e)
    e = cudaMemcpyAsync(meansq_out, rb->post_tmp, 3 * sizeof(float) * (size_t)npix, cudaMemcpyDeviceToHost, ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  if (e) return cuda_status(ctx, e, "moments readback");
  if (rays_out) *rays_out = rays;
  return BC_OK;
}

bc_status bc_render_batch(bc_context* ctx, const bc_view* views, int32_t n_views, float* const* linear_out,
                          int64_t* rays_out) {
  if (!ctx || !views || n_views < 1) return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument or no views");
  cudaSetDevice(ctx->device);
  std::vector<ViewRequest> req;
  long long px = 0;
  bc_status bst = batch_requests(ctx, views, n_views, &req, &px);
  if (bst) return bst;
  int64_t rays = 0;
  bc_status st = render_views(ctx, req, (size_t)px, &rays, nullptr);
  if (st) return st;
  RenderBuffers* rb = ctx->rb;
  cudaError_t e = cudaSuccess;
  for (int v = 0; v < n_views && !e; v++)
    if (linear_out && linear_out[v])
      e = cudaMemcpyAsync(linear_out[v], rb->out + 3 * (size_t)req[v].pix_off,
                          3 * sizeof(float) * (size_t)req[v].s.width * req[v].s.height, cudaMemcpyDeviceToHost,
                          ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  if (e) return cuda_status(ctx, e, "batch readback");
  if (rays_out) *rays_out = rays;
  return BC_OK;
}

}  // extern "C"

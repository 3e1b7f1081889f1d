// Wavefront path tracer: the reference CPU integrator (trace, renderer.go:1484-1563;
// directLight 1427-1465; adaptivePixel's sample loop 1928-1970) as separate
// kernels over compacted queues of path slots:
//
//   generate  -> one path per (pixel, sample) of the wave: Halton jitter with the
//                per-pixel rotation, fp64 primary ray (rounded to fp32), PCG32 stream
//   extend    -> closest hit for every queued path (persistent warps fetch 32 rays
//                at a time from an atomic work counter)
//   shade     -> miss / emissive (MIS weight) / diffuse (NEE shadow ray + cosine
//                bounce) / metal / glass, Russian roulette; survivors and shadow
//                rays are pushed with warp-ballot compaction (one atomic per warp)
//   connect   -> any hit for the shadow queue; unoccluded contributions are added
//   accumulate-> per pixel, the firefly-clamped sample radiance summed in sample order
//
// Path state is structure-of-arrays indexed by path slot; queues hold slot
// indices. Waves are sample-major (slot = sample_in_wave * npix + pixel), so
// accumulation is a deterministic per-pixel loop and every (pixel, sample)
// draws from its own seeded stream: the image does not depend on the wave
// split, the chunking into rows, or the launch shape.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"
#include "sampling.cuh"
#include "trace_core.cuh"

namespace bcgx {

struct PathSoA {
  float *ox, *oy, *oz, *dx, *dy, *dz;
  float *tx, *ty, *tz;     // throughput
  float *lx, *ly, *lz;     // radiance of the path so far
  float *px, *py, *pz;     // prevPoint
  float *ppdf;             // prevBSDFPDF
  uint64_t *rs, *ri;       // PCG32 state and increment
  uint32_t* flags;         // bit 0: prevWasDiffuse
  float* hit_t;
  int32_t* hit_slot;
};

struct ShadowSoA {
  float4* o;  // origin, tmax
  float4* d;  // direction
  float4* c;  // contribution (already multiplied by the path throughput)
  int32_t* path;
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

struct WaveParams {
  int W, H, y0, rows, npix;
  int S, s0, bounces, rr_depth;
  int mis, power, sampler, nseq;
  int n_mats, n_lights, want_guides;
  float clamp;
  uint64_t seed;
  double origin[3], lower[3], horiz[3], vert[3];
};

constexpr float kPi = 3.14159265358979323846f;

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

// ---- generate --------------------------------------------------------------
__global__ void k_generate(WaveParams wp, PathSoA ps, int* __restrict__ queue, const double* __restrict__ seqX,
                           const double* __restrict__ seqY, uint32_t* __restrict__ guide_jit, WaveCounters* cnt) {
  const int n = wp.npix * wp.S;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) cnt->q[0] = n;  // the first bounce's queue holds every path of the wave
  if (i >= n) return;
  const int p = i % wp.npix, sl = i / wp.npix;
  const int x = p % wp.W, y = wp.y0 + p / wp.W;
  const int s = wp.s0 + sl;
  Pcg32 rng = make_path_rng(wp.seed, (uint64_t)y * (uint64_t)wp.W + (uint64_t)x, (uint64_t)s);
  double jx, jy;
  if (wp.sampler != BC_SAMPLER_RANDOM && s < wp.nseq) {
    double rx, ry;
    pixel_rotation(x, y, &rx, &ry);
    double a = seqX[s] + rx, b = seqY[s] + ry;
    jx = a - floor(a);
    jy = b - floor(b);
  } else {
    jx = (double)rng.uniform();
    jy = (double)rng.uniform();
  }
  const double u = ((double)x + jx) / (double)max(wp.W - 1, 1);
  const double v = ((double)(wp.H - 1 - y) + jy) / (double)max(wp.H - 1, 1);
  float d[3];
#pragma unroll
  for (int k = 0; k < 3; k++) d[k] = (float)(((wp.lower[k] + wp.horiz[k] * u) + wp.vert[k] * v) - wp.origin[k]);
  ps.ox[i] = (float)wp.origin[0]; ps.oy[i] = (float)wp.origin[1]; ps.oz[i] = (float)wp.origin[2];
  ps.dx[i] = d[0]; ps.dy[i] = d[1]; ps.dz[i] = d[2];
  ps.tx[i] = 1.0f; ps.ty[i] = 1.0f; ps.tz[i] = 1.0f;
  ps.lx[i] = 0.0f; ps.ly[i] = 0.0f; ps.lz[i] = 0.0f;
  ps.ppdf[i] = 0.0f;
  ps.flags[i] = 0u;
  ps.rs[i] = rng.state;
  ps.ri[i] = rng.inc;
  queue[i] = i;
  if (s == 0 && wp.want_guides) {
    uint32_t a = (uint32_t)rintf(fminf(fmaxf((float)jx, 0.0f), 1.0f) * 65535.0f);
    uint32_t b = (uint32_t)rintf(fminf(fmaxf((float)jy, 0.0f), 1.0f) * 65535.0f);
    guide_jit[p] = (b << 16) | a;
  }
}

// ---- extend ----------------------------------------------------------------
// Persistent: a lane whose ray is done takes the next queue entry at once (one
// atomic per warp for all lanes that need work).
template <int STACK, bool SPH>
__global__ void __launch_bounds__(128) k_extend(SceneView sv, PathSoA ps, const int* __restrict__ queue,
                                                WaveCounters* cnt, int cur, unsigned* status) {
  const int n = *((volatile int*)&cnt->q[cur]);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&cnt->rays, (unsigned long long)n);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  int path = -1;
  bool exhausted = false;
  Ray32 r = make_ray(0, 0, 0, 0, 0, 0, 0);
  FastClosestLeaf<SPH> leaf(sv, r, 1e30f);
  Walker<STACK> w;
  w.reset();
  for (;;) {
    const bool need = path < 0 && !exhausted;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m) {
      const int leader = __ffs(m) - 1;
      int base = 0;
      if ((int)lane == leader) base = atomicAdd(&cnt->work_ext, __popc(m));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (need) {
        const int my = base + __popc(m & below);
        if (my < n) {
          path = queue[my];
          r = make_ray(ps.ox[path], ps.oy[path], ps.oz[path], ps.dx[path], ps.dy[path], ps.dz[path], 1e-4f);
          leaf.reset(1e30f);
          w.reset();
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(0xffffffffu, path >= 0)) break;
    if (path >= 0 && w.step(sv, r, leaf, status)) {
      ps.hit_t[path] = leaf.best_t;
      ps.hit_slot[path] = leaf.best_slot;
      path = -1;
    }
  }
}

// ---- shade -----------------------------------------------------------------
struct ShadeScene {
  SceneView sv;
  const MatGPU* __restrict__ mats;
  const LightGPU* __restrict__ lights;
  const float* __restrict__ lpdf_by_prim;
};

// lightDirectionalPDF (renderer.go:1404-1425) for a sphere light hit.
__device__ __forceinline__ float light_dir_pdf(const ShadeScene& sc, const WaveParams& wp, int prim, float radius,
                                               float3 from, float3 lp, float3 ln) {
  if (!(radius > 0.0f)) return 0.0f;
  float3 to = lp - from;
  float dist2 = dot3(to, to);
  if (dist2 <= 1e-12f) return 0.0f;
  float3 ld = unit3(to);
  float cosL = fmaxf(0.0f, dot3(ln, ld * -1.0f));
  if (cosL <= 1e-12f) return 0.0f;
  float area = 4.0f * kPi * radius * radius;
  float sel = wp.n_lights == 0 ? 0.0f : (wp.power ? __ldg(sc.lpdf_by_prim + prim) : 1.0f / (float)wp.n_lights);
  return sel * dist2 / (cosL * area);
}

__global__ void __launch_bounds__(256) k_shade(WaveParams wp, ShadeScene sc, PathSoA ps, const int* __restrict__ qcur,
                                               int* __restrict__ qnext, ShadowSoA sh, WaveCounters* cnt, int cur,
                                               int bounce, float4* __restrict__ guide_nd,
                                               uint32_t* __restrict__ guide_c,
                                               const uint32_t* __restrict__ guide_jit) {
  const int n = *((volatile int*)&cnt->q[cur]);
  const int stride = gridDim.x * blockDim.x;
  const int rr_depth = wp.rr_depth < 1 ? 4 : wp.rr_depth;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int idx = base + threadIdx.x;
    const int path = idx < n ? qcur[idx] : -1;
    bool alive = false, shadow = false;
    float4 so = make_float4(0, 0, 0, 0), sd = so, scon = so;
    if (path >= 0) {
      float3 o = f3(ps.ox[path], ps.oy[path], ps.oz[path]);
      float3 d = f3(ps.dx[path], ps.dy[path], ps.dz[path]);
      float3 tp = f3(ps.tx[path], ps.ty[path], ps.tz[path]);
      float3 L = f3(ps.lx[path], ps.ly[path], ps.lz[path]);
      const float t = ps.hit_t[path];
      const int slot = ps.hit_slot[path];
      if (slot < 0) {
        L = L + had(tp, background(d));
      } else {
        const float4 nrm = __ldg(sc.sv.snorm + slot);
        const int m = __float_as_int(nrm.w);
        if (m >= 0 && m < wp.n_mats) {
          Pcg32 rng;
          rng.state = ps.rs[path];
          rng.inc = ps.ri[path];
          uint32_t flags = ps.flags[path];
          float ppdf = ps.ppdf[path];
          const float3 p = o + d * t;
          const float4 r2 = __ldg(sc.sv.tri + 3 * slot + 2);
          const bool sphere = r2.w < 0.0f;
          float3 N;
          bool front;
          float radius = 0.0f;
          if (sphere) {  // sphereHitAccel normal (renderer.go:670-676)
            const float4 c = __ldg(sc.sv.tri + 3 * slot);
            radius = c.w;
            float3 outward = (p - f3(c.x, c.y, c.z)) * (1.0f / c.w);
            front = dot3(d, outward) < 0.0f;
            N = front ? outward : outward * -1.0f;
          } else {
            N = f3(nrm.x, nrm.y, nrm.z);
            front = dot3(d, N) < 0.0f;
            if (!front) N = N * -1.0f;
          }
          const MatGPU M = sc.mats[m];
          const int kind = (int)M.kind;
          if (bounce == 0 && wp.want_guides && wp.s0 == 0 && path < wp.npix) {
            guide_nd[wp.y0 * wp.W + path] = make_float4(N.x, N.y, N.z, t);
            // compact guide (gpu_opencl_windows.go:791-797): Euclidean depth,
            // octahedral normal 10:10, material 11 bits, valid bit, jitter
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
            uint32_t* g = guide_c + 3 * (size_t)(wp.y0 * wp.W + path);
            g[0] = __float_as_uint(t * dl);
            g[1] = 0x80000000u | (mm << 20) | (qy << 10) | qx;
            g[2] = guide_jit[path];
          }
          if (kind == BC_MAT_EMISSIVE) {
            float w = 1.0f;
            if (wp.mis && (flags & 1u)) {  // lightDirectionalPDF is 0 for triangles
              float lpdf = 0.0f;
              if (sphere) {
                const int prim = __ldg(sc.sv.slot_prim + slot);
                lpdf = light_dir_pdf(sc, wp, prim, radius, f3(ps.px[path], ps.py[path], ps.pz[path]), p, N);
              }
              w = power_heuristic(ppdf, lpdf);
            }
            L = L + had(tp, f3(M.er, M.eg, M.eb)) * w;
          } else {
            bool cont = true;
            float3 nd_dir = d, no = o;
            if (kind == BC_MAT_DIFFUSE) {
              if (wp.n_lights > 0) {  // directLight (renderer.go:1427-1465)
                int li;
                float sel;
                if (!wp.power) {  // rng.Intn (in fp64 so the index matches the CPU draw)
                  li = min((int)((double)rng.uniform() * (double)wp.n_lights), wp.n_lights - 1);
                  sel = 1.0f / (float)wp.n_lights;
                } else {  // sort.Search over LightCDF
                  const double r = (double)rng.uniform();
                  int lo = 0, hi = wp.n_lights;
                  while (lo < hi) {
                    int mid = (lo + hi) >> 1;
                    if (!(__ldg(&sc.lights[mid].cdf) >= r)) lo = mid + 1; else hi = mid;
                  }
                  li = min(lo, wp.n_lights - 1);
                  sel = __ldg(&sc.lights[li].select_pdf);
                }
                const LightGPU Lg = sc.lights[li];
                const float3 ln = sel > 0.0f ? rand_unit_vector(rng) : f3(0, 0, 1);
                const float3 q = f3(Lg.cx, Lg.cy, Lg.cz) + ln * Lg.r;
                const float3 to = q - p;
                const float dist2 = dot3(to, to);
                if (dist2 >= 1e-8f && sel > 0.0f) {
                  const float3 ld = unit3(to);
                  const float ndl = fmaxf(0.0f, dot3(N, ld));
                  const float cosL = fmaxf(0.0f, dot3(ln * -1.0f, ld));
                  if (ndl > 0.0f && cosL > 0.0f) {
                    const float area = 4.0f * kPi * Lg.r * Lg.r;
                    const float lightPDF = sel * dist2 / (cosL * area);
                    if (lightPDF > 0.0f) {
                      const float bsdfPDF = ndl / kPi;
                      const float w = wp.mis ? power_heuristic(lightPDF, bsdfPDF) : 1.0f;
                      const float3 f = f3(M.cr, M.cg, M.cb) * (1.0f / kPi);
                      const float3 contrib = had(tp, had(f, f3(Lg.er, Lg.eg, Lg.eb)) * (ndl * w / lightPDF));
                      const float3 from = p + N * 2e-4f;  // visible (renderer.go:1333-1341)
                      const float3 sdv = q - from;
                      const float sd2 = dot3(sdv, sdv);
                      if (sd2 < 1e-12f) {
                        L = L + contrib;
                      } else {
                        const float dist = sqrtf(sd2);
                        const float3 dirn = sdv * (1.0f / dist);
                        shadow = true;
                        so = make_float4(from.x, from.y, from.z, dist - 1e-4f);
                        sd = make_float4(dirn.x, dirn.y, dirn.z, 0.0f);
                        scon = make_float4(contrib.x, contrib.y, contrib.z, 0.0f);
                      }
                    }
                  }
                }
              }
              tp = had(tp, f3(M.cr, M.cg, M.cb));
              nd_dir = rand_cos_hemisphere(N, rng);
              flags |= 1u;
              ppdf = fmaxf(0.0f, dot3(N, nd_dir)) / kPi;
              ps.px[path] = p.x; ps.py[path] = p.y; ps.pz[path] = p.z;
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
              const float ratio = front ? 1.0f / eta : eta;
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
              alive = true;
              ps.ox[path] = no.x; ps.oy[path] = no.y; ps.oz[path] = no.z;
              ps.dx[path] = nd_dir.x; ps.dy[path] = nd_dir.y; ps.dz[path] = nd_dir.z;
              ps.tx[path] = tp.x; ps.ty[path] = tp.y; ps.tz[path] = tp.z;
              ps.flags[path] = flags;
              ps.ppdf[path] = ppdf;
              ps.rs[path] = rng.state;
            }
          }
        }
      }
      ps.lx[path] = L.x; ps.ly[path] = L.y; ps.lz[path] = L.z;
    }
    const int qn = warp_reserve(&cnt->q[cur ^ 1], alive);
    if (alive) qnext[qn] = path;
    const int qs = warp_reserve(&cnt->shadow, shadow);
    if (shadow) {
      sh.o[qs] = so;
      sh.d[qs] = sd;
      sh.c[qs] = scon;
      sh.path[qs] = path;
    }
  }
}

// ---- connect -----------------------------------------------------------------
template <int STACK, bool SPH>
__global__ void __launch_bounds__(128) k_connect(SceneView sv, PathSoA ps, ShadowSoA sh, WaveCounters* cnt,
                                                 unsigned* status) {
  const int n = *((volatile int*)&cnt->shadow);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&cnt->shadow_rays, (unsigned long long)n);
  const unsigned lane = threadIdx.x & 31u;
  const unsigned below = (1u << lane) - 1u;
  int i = -1;
  bool exhausted = false;
  Ray32 r = make_ray(0, 0, 0, 0, 0, 0, 0);
  FastAnyLeaf<SPH> leaf(sv, r, 0.0f);
  Walker<STACK> w;
  w.reset();
  for (;;) {
    const bool need = i < 0 && !exhausted;
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m) {
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
          w.reset();
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
        ps.lx[path] += c.x;
        ps.ly[path] += c.y;
        ps.lz[path] += c.z;
      }
      i = -1;
    }
  }
}

// ---- accumulate ----------------------------------------------------------------
__global__ void k_accumulate(WaveParams wp, PathSoA ps, float* __restrict__ sum, float* __restrict__ sumsq) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= wp.npix) return;
  float3 acc = f3(0, 0, 0), acc2 = f3(0, 0, 0);
  for (int sl = 0; sl < wp.S; sl++) {
    const int i = sl * wp.npix + p;
    float3 c = f3(ps.lx[i], ps.ly[i], ps.lz[i]);
    if (wp.clamp > 0.0f) {  // clampFirefly (renderer.go:1917-1926)
      const float m = maxcomp(c);
      if (!(m <= wp.clamp || m <= 0.0f)) c = c * (wp.clamp / m);
    }
    acc = acc + c;
    acc2 = acc2 + had(c, c);
  }
  float* s = sum + 3 * (size_t)(wp.y0 * wp.W + p);
  s[0] += acc.x;
  s[1] += acc.y;
  s[2] += acc.z;
  if (sumsq) {
    float* q = sumsq + 3 * (size_t)(wp.y0 * wp.W + p);
    q[0] += acc2.x;
    q[1] += acc2.y;
    q[2] += acc2.z;
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

__global__ void k_finish(int n, int spp, const float* __restrict__ sum, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * n) return;
  out[i] = sum[i] * (1.0f / (float)spp);
}

// ---- host orchestration ----------------------------------------------------------
template <class T>
T* carve(char*& p, size_t n) {
  T* r = reinterpret_cast<T*>(p);
  p += ((n * sizeof(T) + 255) / 256) * 256;
  return r;
}

}  // namespace bcgx

struct RenderBuffers {
  int cap = 0;        // path slots
  int frame_px = 0;   // pixels of the frame buffers
  bcgx::DevBuf paths, shadow, queues, counters, seq, frame;
  bcgx::PathSoA ps{};
  bcgx::ShadowSoA sh{};
  int* q[2] = {nullptr, nullptr};
  bcgx::WaveCounters* cnt = nullptr;
  double* seqX = nullptr;
  double* seqY = nullptr;
  int nseq = 0;
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
  int ext_grid = 0, con_grid = 0, shade_grid = 0;
};

namespace bcgx {

void destroy_render_buffers(bc_context* ctx) {
  if (!ctx->rb) return;
  ctx->rb->paths.release();
  ctx->rb->shadow.release();
  ctx->rb->queues.release();
  ctx->rb->counters.release();
  ctx->rb->seq.release();
  ctx->rb->frame.release();
  delete ctx->rb;
  ctx->rb = nullptr;
}

static bc_status ensure_paths(bc_context* ctx, int cap) {
  RenderBuffers* rb = ctx->rb;
  if (rb->cap >= cap) return BC_OK;
  size_t per = 16 * sizeof(float) + 2 * sizeof(uint64_t) + sizeof(uint32_t) + sizeof(float) + sizeof(int32_t);
  cudaError_t e = rb->paths.ensure((size_t)cap * per + 64 * 256);
  if (e == cudaSuccess) e = rb->shadow.ensure((size_t)cap * (3 * sizeof(float4) + sizeof(int32_t)) + 8 * 256);
  if (e == cudaSuccess) e = rb->queues.ensure((size_t)cap * 2 * sizeof(int) + 4 * 256);
  if (e != cudaSuccess) return cuda_status(ctx, e, "path buffers");
  char* p = (char*)rb->paths.p;
  PathSoA& s = rb->ps;
  float** fl[] = {&s.ox, &s.oy, &s.oz, &s.dx, &s.dy, &s.dz, &s.tx, &s.ty, &s.tz, &s.lx, &s.ly, &s.lz, &s.px, &s.py, &s.pz, &s.ppdf};
  for (float** f : fl) *f = carve<float>(p, cap);
  s.rs = carve<uint64_t>(p, cap);
  s.ri = carve<uint64_t>(p, cap);
  s.flags = carve<uint32_t>(p, cap);
  s.hit_t = carve<float>(p, cap);
  s.hit_slot = carve<int32_t>(p, cap);
  char* q = (char*)rb->shadow.p;
  rb->sh.o = carve<float4>(q, cap);
  rb->sh.d = carve<float4>(q, cap);
  rb->sh.c = carve<float4>(q, cap);
  rb->sh.path = carve<int32_t>(q, cap);
  char* qq = (char*)rb->queues.p;
  rb->q[0] = carve<int>(qq, cap);
  rb->q[1] = carve<int>(qq, cap);
  rb->cap = cap;
  return BC_OK;
}

static bc_status ensure_frame(bc_context* ctx, int px) {
  RenderBuffers* rb = ctx->rb;
  if (rb->frame_px >= px) return BC_OK;
  size_t bytes = (size_t)px * (5 * 3 * sizeof(float) + sizeof(float4) + 5 * sizeof(uint32_t)) + 16 * 256;
  cudaError_t e = rb->frame.ensure(bytes);
  if (e != cudaSuccess) return cuda_status(ctx, e, "frame buffers");
  char* p = (char*)rb->frame.p;
  rb->sum = carve<float>(p, 3 * (size_t)px);
  rb->sumsq = carve<float>(p, 3 * (size_t)px);
  rb->out = carve<float>(p, 3 * (size_t)px);
  rb->post_tmp = carve<float>(p, 3 * (size_t)px);
  rb->post_tmp2 = carve<float>(p, 3 * (size_t)px);
  rb->guide_nd = carve<float4>(p, px);
  rb->guide_c = carve<uint32_t>(p, 3 * (size_t)px);
  rb->guide_jit = carve<uint32_t>(p, px);
  rb->rgba = carve<uint32_t>(p, px);
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
// host in fp64 exactly as the reference does.
static void sample_sequence(const bc_settings& s, std::vector<double>* X, std::vector<double>* Y) {
  X->clear();
  Y->clear();
  if (s.sampler == BC_SAMPLER_RANDOM) return;
  const int n = effective_spp(s);
  X->resize(n);
  Y->resize(n);
  if (s.sampler == BC_SAMPLER_R2) {
    const double g = 1.324717957244746;
    const double a1 = 1.0 / g, a2 = 1.0 / (g * g);
    for (int i = 0; i < n; i++) {
      double a = 0.5 + (double)(i + 1) * a1, b = 0.5 + (double)(i + 1) * a2;
      (*X)[i] = a - std::floor(a);
      (*Y)[i] = b - std::floor(b);
    }
    return;
  }
  for (int i = 0; i < n; i++) {
    uint64_t m = (uint64_t)(i + 1), r = 0;
    for (int k = 0; k < 64; k++) { r = (r << 1) | (m & 1); m >>= 1; }
    (*X)[i] = (double)r * 5.421010862427522e-20;
    uint64_t n3 = (uint64_t)(i + 1);
    double invBase = 1.0 / 3.0, inv = invBase, res = 0;
    while (n3 > 0) {
      res += (double)(n3 % 3) * inv;
      n3 /= 3;
      inv *= invBase;
    }
    (*Y)[i] = res;
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

template <int STACK, bool SPH>
static int persistent_grid(const void* fn, int block) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, block, 0);
  return std::max(1, sms * std::max(1, per));
}

template <int STACK, bool SPH>
static cudaError_t launch_bounce(bc_context* ctx, const WaveParams& wp, const ShadeScene& sc, int bounce, int cur) {
  RenderBuffers* rb = ctx->rb;
  cudaStream_t st = ctx->stream;
  static int ext_grid = 0, con_grid = 0;
  if (!ext_grid) ext_grid = persistent_grid<STACK, SPH>((const void*)k_extend<STACK, SPH>, 128);
  if (!con_grid) con_grid = persistent_grid<STACK, SPH>((const void*)k_connect<STACK, SPH>, 128);
  WaveCounters* c = rb->cnt;
  cudaError_t e = cudaMemsetAsync(&c->work_ext, 0, sizeof(int) * 2, st);
  if (e) return e;
  e = cudaMemsetAsync(&c->q[cur ^ 1], 0, sizeof(int), st);
  if (e) return e;
  e = cudaMemsetAsync(&c->shadow, 0, sizeof(int), st);
  if (e) return e;
  k_extend<STACK, SPH><<<ext_grid, 128, 0, st>>>(sc.sv, rb->ps, rb->q[cur], c, cur, ctx->d_status);
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  k_shade<<<sms * 8, 256, 0, st>>>(wp, sc, rb->ps, rb->q[cur], rb->q[cur ^ 1], rb->sh, c, cur, bounce, rb->guide_nd,
                                   rb->guide_c, rb->guide_jit);
  if (wp.n_lights > 0)
    k_connect<STACK, SPH><<<con_grid, 128, 0, st>>>(sc.sv, rb->ps, rb->sh, c, ctx->d_status);
  return cudaGetLastError();
}

template <int STACK, bool SPH>
static cudaError_t run_wave(bc_context* ctx, const WaveParams& wp, const ShadeScene& sc) {
  RenderBuffers* rb = ctx->rb;
  cudaStream_t st = ctx->stream;
  const int n = wp.npix * wp.S;
  WaveCounters* c = rb->cnt;
  cudaError_t e = cudaSuccess;
  k_generate<<<(n + 255) / 256, 256, 0, st>>>(wp, rb->ps, rb->q[0], rb->seqX, rb->seqY, rb->guide_jit, c);
  int cur = 0;
  for (int b = 0; b < wp.bounces; b++) {
    e = launch_bounce<STACK, SPH>(ctx, wp, sc, b, cur);
    if (e) return e;
    cur ^= 1;
  }
  k_accumulate<<<(wp.npix + 255) / 256, 256, 0, st>>>(wp, rb->ps, rb->sum, rb->want_sumsq ? rb->sumsq : nullptr);
  return cudaGetLastError();
}

// Renders rows [y0, y0 + rows) into rb->sum (and guides). Returns rays traced.
static bc_status render_rows_device(bc_context* ctx, const bc_camera& cam, const bc_settings& s, int y0, int rows,
                                    bool want_guides, int64_t* rays) {
  if (!ctx->has_scene) return set_error(ctx, BC_ERR_NO_SCENE, "no scene uploaded");
  if (s.width < 1 || s.height < 1 || s.bounces < 1 || s.spp < 1 || y0 < 0 || rows < 1 || y0 + rows > s.height)
    return set_error(ctx, BC_ERR_INVALID_ARG, "invalid render size, rows, spp or bounces");
  if ((int64_t)s.width * s.height > (1 << 26)) return set_error(ctx, BC_ERR_INVALID_ARG, "frame too large");
  if (!ctx->rb) ctx->rb = new RenderBuffers();
  RenderBuffers* rb = ctx->rb;
  const int W = s.width, H = s.height;
  const int npix = W * rows;
  const int spp = effective_spp(s);
  const int cap_target = 1 << 22;
  int S = std::max(1, std::min(spp, cap_target / std::max(1, npix)));
  int cap = std::max(npix * S, 1 << 16);
  bc_status bst = ensure_paths(ctx, std::min(cap, std::max(cap_target, npix)));
  if (bst) return bst;
  if ((bst = ensure_frame(ctx, W * H))) return bst;
  if (npix > rb->cap) return set_error(ctx, BC_ERR_CAPACITY, "row chunk exceeds path capacity");
  S = std::max(1, std::min(S, rb->cap / npix));
  cudaError_t e = rb->counters.ensure(sizeof(WaveCounters));
  if (e) return cuda_status(ctx, e, "counters");
  rb->cnt = rb->counters.as<WaveCounters>();
  std::vector<double> X, Y;
  sample_sequence(s, &X, &Y);
  e = rb->seq.ensure(std::max<size_t>(16, 2 * X.size() * sizeof(double)));
  if (e) return cuda_status(ctx, e, "sample table");
  rb->seqX = rb->seq.as<double>();
  rb->seqY = rb->seqX + X.size();
  rb->nseq = (int)X.size();
  if (!X.empty()) {
    e = cudaMemcpyAsync(rb->seqX, X.data(), X.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    if (!e) e = cudaMemcpyAsync(rb->seqY, Y.data(), Y.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
  }
  if (!e) e = cudaMemsetAsync(rb->cnt, 0, sizeof(WaveCounters), ctx->stream);
  if (!e) e = cudaMemsetAsync(rb->sum + 3 * (size_t)y0 * W, 0, 3 * sizeof(float) * (size_t)npix, ctx->stream);
  if (!e && rb->want_sumsq)
    e = cudaMemsetAsync(rb->sumsq + 3 * (size_t)y0 * W, 0, 3 * sizeof(float) * (size_t)npix, ctx->stream);
  if (!e && want_guides) {  // invalid guides: depth -1, compact words 0
    k_clear_guides<<<(npix + 255) / 256, 256, 0, ctx->stream>>>(npix, rb->guide_nd + (size_t)y0 * W,
                                                                rb->guide_c + 3 * (size_t)y0 * W);
    e = cudaGetLastError();
  }
  if (e) return cuda_status(ctx, e, "render setup");

  WaveParams wp;
  std::memset(&wp, 0, sizeof(wp));
  wp.W = W; wp.H = H; wp.y0 = y0; wp.rows = rows; wp.npix = npix;
  wp.bounces = s.bounces;
  wp.rr_depth = s.rr_depth;
  wp.mis = s.mis != 0;
  wp.power = s.power_light_sampling != 0;
  wp.sampler = s.sampler;
  wp.nseq = rb->nseq;
  wp.n_mats = ctx->ds.n_mats;
  wp.n_lights = ctx->ds.n_lights;
  wp.want_guides = want_guides ? 1 : 0;
  wp.clamp = (float)s.firefly_clamp;
  wp.seed = s.seed;
  camera_basis(cam, (double)W / (double)H, wp.origin, wp.lower, wp.horiz, wp.vert);
  ShadeScene sc;
  sc.sv.nodes = ctx->ds.nodes;
  sc.sv.tri = ctx->ds.tri;
  sc.sv.slot64 = ctx->ds.slot64;
  sc.sv.snorm = ctx->ds.snorm;
  sc.sv.slot_prim = ctx->ds.slot_prim;
  sc.mats = ctx->ds.mats;
  sc.lights = ctx->ds.lights;
  sc.lpdf_by_prim = ctx->ds.light_pdf_by_prim;
  const int stack = stack_variant(ctx->ds.stack_need);
  for (int s0 = 0; s0 < spp; s0 += S) {
    if (*(volatile int*)ctx->h_cancel || ctx->cancel.load()) {
      cudaStreamSynchronize(ctx->stream);
      return set_error(ctx, BC_ERR_CANCELLED, "render cancelled");
    }
    wp.s0 = s0;
    wp.S = std::min(S, spp - s0);
    const bool sph = ctx->ds.has_spheres;
    if (stack == 64) e = sph ? run_wave<64, true>(ctx, wp, sc) : run_wave<64, false>(ctx, wp, sc);
    else if (stack == 128) e = sph ? run_wave<128, true>(ctx, wp, sc) : run_wave<128, false>(ctx, wp, sc);
    else e = sph ? run_wave<256, true>(ctx, wp, sc) : run_wave<256, false>(ctx, wp, sc);
    if (e) return cuda_status(ctx, e, "wavefront launch");
  }
  unsigned long long r = 0;
  e = cudaMemcpyAsync(&r, &rb->cnt->rays, sizeof(r), cudaMemcpyDeviceToHost, ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  if (e) return cuda_status(ctx, e, "render");
  if (rays) *rays = (int64_t)r;
  return check_kernel_status(ctx);
}

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
  bc_status st = ensure_frame(ctx, px);
  if (st) return st;
  *t = post_targets(ctx);
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
  const int spp = effective_spp(*settings);
  k_finish<<<(3 * npix + 255) / 256, 256, 0, ctx->stream>>>(npix, spp, rb->sum + 3 * (size_t)y0 * W,
                                                            rb->out + 3 * (size_t)y0 * W);
  cudaError_t e = cudaGetLastError();
  if (!e) e = cudaMemcpyAsync(linear_out, rb->out + 3 * (size_t)y0 * W, 3 * sizeof(float) * (size_t)npix,
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
  const int spp = effective_spp(*settings);
  k_finish<<<(3 * npix + 255) / 256, 256, 0, ctx->stream>>>(npix, spp, rb->sum, rb->out);
  cudaError_t e = cudaGetLastError();
  if (e) return cuda_status(ctx, e, "finish");
  if ((st = run_post(ctx, *settings))) return st;
  if (linear_out)
    e = cudaMemcpyAsync(linear_out, rb->out, 3 * sizeof(float) * (size_t)npix, cudaMemcpyDeviceToHost, ctx->stream);
  if (!e && guide_out)
    e = cudaMemcpyAsync(guide_out, rb->guide_c, 3 * sizeof(uint32_t) * (size_t)npix, cudaMemcpyDeviceToHost,
                        ctx->stream);
  if (!e && rgba_out)
    e = cudaMemcpyAsync(rgba_out, rb->rgba, sizeof(uint32_t) * (size_t)npix, cudaMemcpyDeviceToHost, ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  if (e) return cuda_status(ctx, e, "frame readback");
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
  const int spp = effective_spp(*settings);
  k_finish<<<(3 * npix + 255) / 256, 256, 0, ctx->stream>>>(npix, spp, rb->sum, rb->out);
  k_finish<<<(3 * npix + 255) / 256, 256, 0, ctx->stream>>>(npix, spp, rb->sumsq, rb->post_tmp);
  cudaError_t e = cudaGetLastError();
  if (!e) e = cudaMemcpyAsync(mean_out, rb->out, 3 * sizeof(float) * (size_t)npix, cudaMemcpyDeviceToHost, ctx->stream);
  if (!e)
    e = cudaMemcpyAsync(meansq_out, rb->post_tmp, 3 * sizeof(float) * (size_t)npix, cudaMemcpyDeviceToHost, ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  if (e) return cuda_status(ctx, e, "moments readback");
  if (rays_out) *rays_out = rays;
  return BC_OK;
}

}  // extern "C"

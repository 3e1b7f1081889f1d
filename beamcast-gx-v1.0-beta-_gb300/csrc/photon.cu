// Photon map of the photon-mapping integrator, built on the device
// (buildPhotonMap, renderer.go:1642-1728).
//
// The reference emits photons one after another from one generator and stops
// before an emission once the map holds `budget` photons. Here emission k draws
// from its own stream (seed, k), so the emissions run in parallel, in two passes
// of one kernel: the first counts each emission's deposits, an exclusive scan
// of the counts gives every emission its first photon index, and the second pass
// re-traces the emissions whose first index is below the budget and writes
// their photons there. The result is the reference's photon list in its append
// order, the last emission's overshoot past the budget included. One block
// then sorts the photons by (cell key, append index) and builds the table that
// the gather looks keys up in.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"
#include "photon.cuh"
#include "trace_core.cuh"
#include "wave.h"

namespace bcgx {

constexpr float kPhotonPi = 3.14159265358979323846f;

int photon_budget(int level) {  // renderer.go:1148-1161
  switch (level) {
    case 1: return 512;
    case 2: return 2048;
    case 3: return 8192;
    case 4: return 16384;
    default: return 0;
  }
}

double photon_radius(double diag, int level) {  // renderer.go:1163-1182
  if (diag < 1e-3) diag = 10;
  const double base = diag * 0.03;
  switch (level) {
    case 1: return base * 1.8;
    case 2: return base * 1.2;
    case 3: return base * 0.85;
    case 4: return base * 0.6;
    default: return base;
  }
}

struct PhotonTraceArgs {
  SceneView sv;
  const MatGPU* __restrict__ mats;
  const LightGPU* __restrict__ lights;
  int n_mats, n_lights, light_off, root;
  int budget, attempts, max_bounces;
  unsigned long long seed;
  float cell;
  int* count;                      // deposits per emission (written by the counting pass, read by the second)
  const int* start;                // second pass: first photon index of each emission; null: counting pass
  float4 *pos, *nrm, *flux;        // second pass: photons in append order (pos.w: emission index)
  unsigned long long* key;         // second pass: cell key of each photon
  unsigned long long* rays;        // second pass: rays of the emissions that ran
};

// One photon emission per thread (renderer.go:1656-1718). Both passes run this
// kernel; the second writes at most the deposits the first counted.
template <int STACK, bool SPH>
__global__ void __launch_bounds__(128) k_photon_trace(PhotonTraceArgs a, unsigned* status) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const bool store = a.start != nullptr;
  unsigned long long rays = 0;
  if (k < a.attempts) {
    int base = 0, limit = 0;
    bool run = true;
    if (store) {
      base = a.start[k];
      limit = a.count[k];
      run = base < a.budget;
    }
    int out = 0;
    if (run) {
      Pcg32 rng = make_path_rng(a.seed, (uint64_t)k, kPhotonStream);
      const int li = draw_index(rng, a.n_lights);  // rng.Intn
      const LightGPU Lg = a.lights[a.light_off + li];
      const float3 surf = rand_unit_vector(rng);
      float3 o = f3(Lg.cx, Lg.cy, Lg.cz) + surf * (Lg.r + 2e-4f);
      float3 d = rand_cos_hemisphere(surf, rng);
      float3 tp = f3(Lg.er, Lg.eg, Lg.eb) * ((4.0f * kPhotonPi * Lg.r * Lg.r) / (float)a.budget);
      FastWalker<STACK, kLeafVote> w;
      for (int b = 0; b < a.max_bounces; b++) {
        rays++;
        const Ray32 r = make_ray(o.x, o.y, o.z, d.x, d.y, d.z, 1e-4f);
        FastClosestLeaf<SPH> leaf(a.sv, r, 1e30f);
        w.reset(r, (uint32_t)a.root);
        while (!w.step(a.sv, r, leaf, status)) {
        }
        const int slot = leaf.best_slot;
        if (slot < 0) break;
        const float4 nrm = __ldg(a.sv.snorm + slot);
        const int m = __float_as_int(nrm.w);
        if (m < 0 || m >= a.n_mats) break;
        const Surface S = hit_surface(a.sv, slot, nrm, o, d, leaf.best_t);
        const MatGPU M = a.mats[m];
        const int kind = (int)M.kind;
        if (kind == BC_MAT_EMISSIVE) break;
        const float3 col = f3(M.cr, M.cg, M.cb);
        if (kind == BC_MAT_DIFFUSE) {
          tp = had(tp, col);
          if (store && out < limit) {
            const int i = base + out;
            a.pos[i] = make_float4(S.p.x, S.p.y, S.p.z, (float)k);
            a.nrm[i] = make_float4(S.N.x, S.N.y, S.N.z, 0.0f);
            a.flux[i] = make_float4(tp.x, tp.y, tp.z, 0.0f);
            a.key[i] = photon_cell_key((long long)floorf(S.p.x / a.cell), (long long)floorf(S.p.y / a.cell),
                                       (long long)floorf(S.p.z / a.cell));
          }
          out++;
          d = rand_cos_hemisphere(S.N, rng);
          o = S.p + S.N * 2e-4f;
        } else if (kind == BC_MAT_METAL) {
          const float rough = fminf(fmaxf(M.rough, 0.0f), 1.0f);
          const float3 nd = unit3(reflect3(unit3(d), S.N) + rand_in_unit_sphere(rng) * rough);
          if (dot3(nd, S.N) <= 0.0f) break;
          tp = had(tp, col);
          o = S.p + S.N * 2e-4f;
          d = nd;
        } else {  // glass and any other kind (renderer.go:1695-1710)
          float eta = M.ior;
          if (eta <= 1.0f) eta = 1.5f;
          const float ratio = S.front ? 1.0f / eta : eta;
          const float3 un = unit3(d);
          const float cosT = fminf(dot3(un * -1.0f, S.N), 1.0f);
          const float sinT = sqrtf(fmaxf(0.0f, 1.0f - cosT * cosT));
          const float3 nd = (ratio * sinT > 1.0f || schlick(cosT, ratio) > rng.uniform()) ? reflect3(un, S.N)
                                                                                          : refract3(un, S.N, ratio);
          tp = had(tp, col);
          o = S.p + nd * 2e-4f;
          d = nd;
        }
        if (b >= 2) {  // renderer.go:1711-1717
          const float pr = fminf(fmaxf(maxcomp(tp), 0.1f), 0.95f);
          if (rng.uniform() > pr) break;
          tp = tp * (1.0f / pr);
        }
      }
      if (store)  // a path that deposited fewer photons than counted leaves far-away, flux-free ones
        for (int j = out; j < limit; j++) {
          a.pos[base + j] = make_float4(3.0e38f, 3.0e38f, 3.0e38f, (float)k);
          a.nrm[base + j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          a.flux[base + j] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          a.key[base + j] = 0ull;
        }
    }
    if (!store) a.count[k] = out;
  }
  if (store) {
    for (int o = 16; o > 0; o >>= 1) rays += __shfl_down_sync(0xffffffffu, rays, o);
    if ((threadIdx.x & 31u) == 0 && rays) atomicAdd(a.rays, rays);
  }
}

// Exclusive scan over one block of 1024 threads: returns the sum of v over
// the threads below, and the block total in *total.
__device__ __forceinline__ int block_scan_1024(int v, int* sm, int* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int s = sm[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    sm[lane] = s;  // inclusive warp totals
  }
  __syncthreads();
  *total = sm[31];
  const int below = (warp ? sm[warp - 1] : 0) + x - v;
  __syncthreads();  // sm is reused by the caller's next scan
  return below;
}

// First photon index of every emission; header[0] = photons in the map (the
// deposits of the emissions that start below the budget), header[1] = those emissions.
__global__ void __launch_bounds__(1024) k_photon_scan(const int* __restrict__ count, int attempts, int budget,
                                                      int* __restrict__ start, int* __restrict__ header) {
  __shared__ int sm[32];
  __shared__ int first;
  if (threadIdx.x == 0) first = attempts;
  const int per = (attempts + 1023) / 1024;
  const int lo = min(attempts, (int)threadIdx.x * per), hi = min(attempts, lo + per);
  int local = 0;
  for (int k = lo; k < hi; k++) local += count[k];
  int total = 0;
  int run = block_scan_1024(local, sm, &total);
  int mine = attempts;
  for (int k = lo; k < hi; k++) {
    start[k] = run;
    if (run >= budget && mine == attempts) mine = k;
    run += count[k];
  }
  atomicMin(&first, mine);
  __syncthreads();
  if (threadIdx.x == 0) {
    header[0] = first < attempts ? start[first] : total;
    header[1] = first;
  }
}

// Sorts the photons by (cell key, append index) (bitonic sort of the padded
// power of two), lists the distinct keys with their runs, gathers the photons
// into sorted order, fills the lookup table and writes the dense table's box
// (the photons' cells and two more each side; no dense table when it would
// hold more than max_cells cells). One block.
__global__ void __launch_bounds__(1024) k_photon_grid(const int* __restrict__ header, int p2max,
                                                      const unsigned long long* __restrict__ key,
                                                      const float4* __restrict__ pos_u, const float4* __restrict__ nrm_u,
                                                      const float4* __restrict__ flux_u, unsigned long long* skey,
                                                      int* sidx, unsigned long long* ukey, int2* span, float4* pos,
                                                      float4* nrm, float4* flux, int* table, int tsize, float cell,
                                                      long long max_cells, PhotonGrid* grid, unsigned* status) {
  __shared__ int sm[32];
  __shared__ long long cmin[3], cmax[3];
  const int t = threadIdx.x;
  const int n = header[0];
  if (t < 3) {
    cmin[t] = LLONG_MAX;
    cmax[t] = LLONG_MIN;
  }
  int P2 = 2;
  while (P2 < n) P2 <<= 1;
  if (P2 > p2max) {  // cannot happen: n <= budget + max_bounces - 1 <= p2max
    if (t == 0) atomicOr(status, kStatusCapacity);
    return;
  }
  for (int i = t; i < P2; i += 1024) {
    skey[i] = i < n ? key[i] : ~0ull;
    sidx[i] = i < n ? i : 0x7fffffff;
  }
  __syncthreads();
  for (int k = 2; k <= P2; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = t; i < P2; i += 1024) {
        const int l = i ^ j;
        if (l > i) {
          const unsigned long long ka = skey[i], kb = skey[l];
          const int ia = sidx[i], ib = sidx[l];
          const bool greater = ka > kb || (ka == kb && ia > ib);
          if (greater == ((i & k) == 0)) {
            skey[i] = kb;
            skey[l] = ka;
            sidx[i] = ib;
            sidx[l] = ia;
          }
        }
      }
      __syncthreads();
    }
  const int per = (n + 1023) / 1024;
  const int lo = min(n, t * per), hi = min(n, lo + per);
  int local = 0;
  for (int i = lo; i < hi; i++) local += (i == 0 || skey[i] != skey[i - 1]) ? 1 : 0;
  int n_keys = 0;
  int u = block_scan_1024(local, sm, &n_keys);
  for (int i = lo; i < hi; i++)
    if (i == 0 || skey[i] != skey[i - 1]) {
      ukey[u] = skey[i];
      span[u] = make_int2(i, 0);
      u++;
    }
  for (int i = t; i < n; i += 1024) {
    const int s = sidx[i];
    pos[i] = pos_u[s];
    nrm[i] = nrm_u[s];
    flux[i] = flux_u[s];
  }
  for (int s = t; s < tsize; s += 1024) table[s] = 0;
  long long clo[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, chi[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
  for (int i = t; i < n; i += 1024) {  // cells of the photons, as the keys were formed
    const float4 P = pos_u[i];
    const long long c[3] = {(long long)floorf(P.x / cell), (long long)floorf(P.y / cell), (long long)floorf(P.z / cell)};
    for (int a = 0; a < 3; a++) {
      clo[a] = min(clo[a], c[a]);
      chi[a] = max(chi[a], c[a]);
    }
  }
  for (int a = 0; a < 3; a++) {
    atomicMin(&cmin[a], clo[a]);
    atomicMax(&cmax[a], chi[a]);
  }
  __syncthreads();
  if (t == 0) {
    bool ok = n > 0 && max_cells > 0;
    double cells = 1.0;
    for (int a = 0; a < 3 && ok; a++) {
      const long long d = cmax[a] - cmin[a] + 5;
      ok = d > 0 && d < (1LL << 30);
      cells *= (double)d;
      grid->g0[a] = cmin[a] - 2;
      grid->dim[a] = ok ? (int)d : 0;
    }
    if (!ok || cells > (double)max_cells) grid->dim[0] = 0;
  }
  for (int v = t; v < n_keys; v += 1024) {
    const int first = span[v].x;
    span[v].y = (v + 1 < n_keys ? span[v + 1].x : n) - first;
  }
  for (int v = t; v < n_keys; v += 1024) {
    uint32_t h = photon_slot_hash(ukey[v]) & (uint32_t)(tsize - 1);
    for (int probe = 0; probe < tsize; probe++) {  // the table has at least twice as many slots as keys
      if (atomicCAS(&table[h], 0, v + 1) == 0) break;
      h = (h + 1) & (uint32_t)(tsize - 1);
    }
  }
}

}  // namespace bcgx

namespace bcgx {

// The dense table: the run of every cell of the box, looked up in the hash
// table exactly as a gather would look the cell up.
__global__ void k_photon_dense(PhotonView pm, const PhotonGrid* __restrict__ grid, int* __restrict__ dense) {
  const int gx = grid->dim[0];
  if (gx == 0) return;
  const int gy = grid->dim[1], gz = grid->dim[2];
  const long long total = (long long)gx * gy * gz;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (long long)gridDim.x * blockDim.x) {
    const long long x = i % gx, y = (i / gx) % gy, z = i / ((long long)gx * gy);
    dense[i] = photon_cell_lookup(pm, photon_cell_key(grid->g0[0] + x, grid->g0[1] + y, grid->g0[2] + z));
  }
}

}  // namespace bcgx

// ---- host ----------------------------------------------------------------------
struct PhotonEntry {
  uint64_t gen = 0, seed = 0, stamp = 0;
  int scene = 0, level = 0, max_bounces = 0;
  void* mem = nullptr;
  int attempts = 0, np = 0;
  int* header = nullptr;
  unsigned long long* rays = nullptr;
  const float4 *pos_u = nullptr, *nrm_u = nullptr, *flux_u = nullptr;
  bcgx::PhotonView view{};
};

struct PhotonCache {
  std::vector<PhotonEntry> e;
  uint64_t clock = 0;
};

namespace bcgx {

constexpr size_t kPhotonCacheEntries = 16;

static void free_entry(PhotonEntry& p) {
  if (p.mem) cudaFree(p.mem);
  p.mem = nullptr;
}

void destroy_photon_state(bc_context* ctx) {
  if (!ctx->photons) return;
  for (PhotonEntry& p : ctx->photons->e) free_entry(p);
  delete ctx->photons;
  ctx->photons = nullptr;
}

template <class T>
static T* take(char*& p, size_t n) {
  T* r = reinterpret_cast<T*>(p);
  p += ((n * sizeof(T) + 255) / 256) * 256;
  return r;
}

template <int STACK, bool SPH>
static cudaError_t launch_trace(const PhotonTraceArgs& a, unsigned* status, cudaStream_t st) {
  k_photon_trace<STACK, SPH><<<(a.attempts + 127) / 128, 128, 0, st>>>(a, status);
  return cudaGetLastError();
}

static cudaError_t trace_pass(bc_context* ctx, const PhotonTraceArgs& a) {
  const int stack = stack_variant(ctx->ds.stack_need);
  const bool sph = ctx->ds.has_spheres;
  cudaStream_t st = ctx->stream;
  if (stack == 64) return sph ? launch_trace<64, true>(a, ctx->d_status, st) : launch_trace<64, false>(a, ctx->d_status, st);
  if (stack == 128)
    return sph ? launch_trace<128, true>(a, ctx->d_status, st) : launch_trace<128, false>(a, ctx->d_status, st);
  return sph ? launch_trace<256, true>(a, ctx->d_status, st) : launch_trace<256, false>(a, ctx->d_status, st);
}

// Builds the map of `scene` for (seed, level, max_bounces) into a new entry.
static bc_status build_entry(bc_context* ctx, int scene, const bc_settings& s, PhotonEntry* out) {
  const SceneRange& sr = ctx->ranges[scene];
  PhotonEntry& p = *out;
  p.gen = ctx->scene_gen;
  p.scene = scene;
  p.seed = s.seed;
  p.level = s.photon_mapping;
  p.max_bounces = std::max(2, s.bounces);
  const int budget = photon_budget(s.photon_mapping);
  if (budget <= 0 || sr.n_lights == 0) return BC_OK;  // an empty map: gathers return zero
  double radius = photon_radius(sr.diag, s.photon_mapping);
  if (radius <= 1e-4) radius = 0.25;
  p.attempts = budget * 6;
  p.np = budget + p.max_bounces;  // the last emission may overshoot the budget by max_bounces - 1
  // dense table: photons lie in the scene bounds (a cell of slack per side for
  // fp32 hit points); larger than 2^22 cells, the hash serves alone
  double cells = 1.0;
  for (int a = 0; a < 3; a++)
    cells *= std::floor(sr.hi[a] / radius) - std::floor(sr.lo[a] / radius) + 7.0;
  const long long max_cells = (cells >= 1.0 && cells <= (double)(1 << 22)) ? (long long)cells : 0;
  int p2max = 2;
  while (p2max < p.np) p2max <<= 1;
  const int tsize = 2 * p2max;
  const size_t a = (size_t)p.attempts, np = (size_t)p.np, p2 = (size_t)p2max;
  const size_t bytes = 4 * 256 + ((a * 4 + 255) / 256) * 256 * 2 + ((np * 16 + 255) / 256) * 256 * 6 +
                       ((np * 8 + 255) / 256) * 256 * 2 + ((p2 * 8 + 255) / 256) * 256 +
                       ((p2 * 4 + 255) / 256) * 256 + ((np * 8 + 255) / 256) * 256 + ((tsize * 4 + 255) / 256) * 256 +
                       256 + (((size_t)max_cells * 4 + 255) / 256) * 256;
  cudaError_t e = cudaMalloc(&p.mem, bytes);
  if (e) {
    p.mem = nullptr;
    return cuda_status(ctx, e, "photon map");
  }
  char* c = (char*)p.mem;
  p.header = take<int>(c, 4);
  p.rays = take<unsigned long long>(c, 1);
  int* count = take<int>(c, a);
  int* start = take<int>(c, a);
  float4* pos_u = take<float4>(c, np);
  float4* nrm_u = take<float4>(c, np);
  float4* flux_u = take<float4>(c, np);
  unsigned long long* key = take<unsigned long long>(c, np);
  unsigned long long* skey = take<unsigned long long>(c, p2);
  int* sidx = take<int>(c, p2);
  unsigned long long* ukey = take<unsigned long long>(c, np);
  int2* span = take<int2>(c, np);
  float4* pos = take<float4>(c, np);
  float4* nrm = take<float4>(c, np);
  float4* flux = take<float4>(c, np);
  int* table = take<int>(c, tsize);
  PhotonGrid* grid = take<PhotonGrid>(c, 1);
  int* dense = max_cells ? take<int>(c, (size_t)max_cells) : nullptr;
  p.pos_u = pos_u;
  p.nrm_u = nrm_u;
  p.flux_u = flux_u;

  PhotonTraceArgs ta;
  std::memset(&ta, 0, sizeof(ta));
  ta.sv = SceneView{ctx->ds.nodes, ctx->ds.tri, ctx->ds.slot64, ctx->ds.snorm, ctx->ds.slot_prim};
  ta.mats = ctx->ds.mats;
  ta.lights = ctx->ds.lights;
  ta.n_mats = ctx->ds.n_mats;
  ta.n_lights = sr.n_lights;
  ta.light_off = sr.light_off;
  ta.root = sr.root;
  ta.budget = budget;
  ta.attempts = p.attempts;
  ta.max_bounces = p.max_bounces;
  ta.seed = s.seed;
  ta.cell = (float)radius;
  ta.count = count;
  ta.rays = p.rays;
  cudaStream_t st = ctx->stream;
  e = cudaMemsetAsync(p.mem, 0, 512, st);  // header and ray counter
  if (!e) e = trace_pass(ctx, ta);  // counting pass
  if (!e) {
    k_photon_scan<<<1, 1024, 0, st>>>(count, p.attempts, budget, start, p.header);
    e = cudaGetLastError();
  }
  if (!e) {
    ta.start = start;
    ta.pos = pos_u;
    ta.nrm = nrm_u;
    ta.flux = flux_u;
    ta.key = key;
    e = trace_pass(ctx, ta);
  }
  if (!e) {
    k_photon_grid<<<1, 1024, 0, st>>>(p.header, p2max, key, pos_u, nrm_u, flux_u, skey, sidx, ukey, span, pos, nrm,
                                      flux, table, tsize, (float)radius, max_cells, grid, ctx->d_status);
    e = cudaGetLastError();
  }
  PhotonView hv{};
  hv.ukey = ukey;
  hv.table = table;
  hv.mask = tsize - 1;
  if (!e && dense) {
    const int blocks = (int)std::min<long long>(1024, (max_cells + 255) / 256);
    k_photon_dense<<<blocks, 256, 0, st>>>(hv, grid, dense);
    e = cudaGetLastError();
  }
  if (e) {
    free_entry(p);
    return cuda_status(ctx, e, "photon map build");
  }
  p.view.pos = pos;
  p.view.nrm = nrm;
  p.view.flux = flux;
  p.view.ukey = ukey;
  p.view.span = span;
  p.view.table = table;
  p.view.mask = tsize - 1;
  p.view.cell = (float)radius;
  p.view.r2 = (float)(radius * radius);
  p.view.pir2 = (float)(M_PI * radius * radius);
  p.view.grid = dense ? grid : nullptr;
  p.view.dense = dense;
  return BC_OK;
}

uint64_t photon_clock(bc_context* ctx) { return ctx->photons ? ctx->photons->clock : 0; }

// The cached map for (scene, seed, PhotonMapping level, max(2, bounces)) or a
// newly built one; *built_rays is the new map's device ray counter, or null.
// Maps used after the clock read `pin` (by views of the same render) stay.
static bc_status photon_entry(bc_context* ctx, int scene, const bc_settings& s, uint64_t pin, PhotonEntry** out,
                              const unsigned long long** built_rays) {
  if (!ctx->photons) ctx->photons = new PhotonCache();
  PhotonCache& c = *ctx->photons;
  if (built_rays) *built_rays = nullptr;
  bool synced = false;
  for (size_t i = 0; i < c.e.size();) {  // maps of an older scene can never be used again
    if (c.e[i].gen != ctx->scene_gen) {
      if (!synced) cudaStreamSynchronize(ctx->stream);
      synced = true;
      free_entry(c.e[i]);
      c.e.erase(c.e.begin() + i);
    } else {
      i++;
    }
  }
  const int mb = std::max(2, s.bounces);
  for (PhotonEntry& p : c.e)
    if (p.scene == scene && p.seed == s.seed && p.level == s.photon_mapping && p.max_bounces == mb) {
      p.stamp = ++c.clock;
      *out = &p;
      return BC_OK;
    }
  if (c.e.size() >= kPhotonCacheEntries) {  // evict the least recently used map not pinned
    size_t lru = c.e.size();
    for (size_t i = 0; i < c.e.size(); i++)
      if (c.e[i].stamp <= pin && (lru == c.e.size() || c.e[i].stamp < c.e[lru].stamp)) lru = i;
    if (lru < c.e.size()) {
      cudaStreamSynchronize(ctx->stream);
      free_entry(c.e[lru]);
      c.e.erase(c.e.begin() + lru);
    }
  }
  PhotonEntry p;
  bc_status st = build_entry(ctx, scene, s, &p);
  if (st) return st;
  p.stamp = ++c.clock;
  c.e.push_back(p);
  *out = &c.e.back();
  if (built_rays && p.mem) *built_rays = p.rays;
  return BC_OK;
}

bc_status photon_map_for(bc_context* ctx, int scene, const bc_settings& s, uint64_t pin, PhotonView* view,
                         const unsigned long long** built_rays) {
  PhotonEntry* p = nullptr;
  bc_status st = photon_entry(ctx, scene, s, pin, &p, built_rays);
  if (st) return st;
  *view = p->view;  // an empty map has a null table
  if (!ctx->photon_grid) {
    view->grid = nullptr;
    view->dense = nullptr;
  }
  return BC_OK;
}

}  // namespace bcgx

using namespace bcgx;

extern "C" bc_status bc_photon_map(bc_context* ctx, int32_t scene, const bc_settings* settings, int32_t capacity,
                                   float* photons_out, int32_t* n_out, int64_t* rays_out) {
  if (!ctx || !settings || capacity < 0 || (capacity > 0 && !photons_out))
    return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument");
  if (!ctx->has_scene) return set_error(ctx, BC_ERR_NO_SCENE, "no scene uploaded");
  if (scene < 0 || scene >= (int32_t)ctx->ranges.size())
    return set_error(ctx, BC_ERR_INVALID_ARG, "scene outside the resident set");
  cudaSetDevice(ctx->device);
  PhotonEntry* p = nullptr;
  const unsigned long long* built = nullptr;
  bc_status st = photon_entry(ctx, scene, *settings, photon_clock(ctx), &p, &built);
  if (st) return st;
  int header[2] = {0, 0};
  unsigned long long rays = 0;
  cudaError_t e = cudaSuccess;
  if (p->mem) {
    e = cudaMemcpyAsync(header, p->header, sizeof(header), cudaMemcpyDeviceToHost, ctx->stream);
    if (!e) e = cudaMemcpyAsync(&rays, p->rays, sizeof(rays), cudaMemcpyDeviceToHost, ctx->stream);
    if (!e) e = cudaStreamSynchronize(ctx->stream);
  }
  if (e) return cuda_status(ctx, e, "photon map");
  const int n = header[0];
  const int take_n = std::min(n, capacity);
  if (take_n > 0) {
    std::vector<float4> buf(3 * (size_t)take_n);
    e = cudaMemcpy(buf.data(), p->pos_u, take_n * sizeof(float4), cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(buf.data() + take_n, p->nrm_u, take_n * sizeof(float4), cudaMemcpyDeviceToHost);
    if (!e) e = cudaMemcpy(buf.data() + 2 * (size_t)take_n, p->flux_u, take_n * sizeof(float4), cudaMemcpyDeviceToHost);
    if (e) return cuda_status(ctx, e, "photon map");
    for (int i = 0; i < take_n; i++) {
      const float4 P = buf[i], N = buf[take_n + i], F = buf[2 * (size_t)take_n + i];
      float* q = photons_out + 10 * (size_t)i;
      q[0] = P.x; q[1] = P.y; q[2] = P.z;
      q[3] = N.x; q[4] = N.y; q[5] = N.z;
      q[6] = F.x; q[7] = F.y; q[8] = F.z;
      q[9] = P.w;
    }
  }
  if (n_out) *n_out = n;
  if (rays_out) *rays_out = (int64_t)rays;
  return check_kernel_status(ctx);
}

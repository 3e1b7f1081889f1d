// Test infrastructure only (see bc_oracle.h): a flat C interface over the
// oracle for ctypes. Ray batches run on a thread pool; every result is
// independent of the thread count.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>

#include "bc_oracle.h"

using namespace orc;

namespace {
template <class F>
void parallel_for(int64_t n, int threads, F&& fn) {
  if (threads < 1) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  if (n < 256 || threads == 1) { fn(0, n, 0); return; }
  std::atomic<int64_t> next{0};
  const int64_t chunk = 1024;
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++)
    pool.emplace_back([&, t] {
      for (;;) {
        int64_t s = next.fetch_add(chunk);
        if (s >= n) return;
        fn(s, std::min(n, s + chunk), t);
      }
    });
  for (auto& th : pool) th.join();
}
inline V3 ld3(const double* p) { return v3(p[0], p[1], p[2]); }
inline void st3(double* p, V3 v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }
}  // namespace

extern "C" {

struct orc_settings {
  int32_t width, height, spp, bounces, msaa, tsaa, sampler, mis, power_light;
  double firefly_clamp;
  int32_t rr_depth, adaptive;
  double adaptive_threshold;
  int32_t tile;
  int32_t integrator, photon_mapping;
  int64_t photon_seed;
};

static Settings load_settings(const orc_settings* cs) {
  Settings st;
  st.width = cs->width; st.height = cs->height; st.spp = cs->spp; st.bounces = cs->bounces;
  st.msaa = cs->msaa; st.tsaa = cs->tsaa; st.sampler = cs->sampler; st.mis = cs->mis != 0;
  st.power_light = cs->power_light != 0; st.firefly_clamp = cs->firefly_clamp; st.rr_depth = cs->rr_depth;
  st.adaptive = cs->adaptive != 0; st.adaptive_threshold = cs->adaptive_threshold; st.tile = cs->tile;
  st.integrator = cs->integrator; st.photon_mapping = cs->photon_mapping; st.photon_seed = cs->photon_seed;
  return st;
}

void* orc_scene_new() { return new Scene(); }
void orc_scene_free(void* s) { delete (Scene*)s; }
void orc_scene_set_bvh(void* sp, const char* mode, int bins, int leaf) {
  Scene* s = (Scene*)sp;
  s->bvh_mode = mode ? mode : "SAH";
  s->bvh_bins = bins;
  s->bvh_leaf = leaf;
}
int orc_add_material(void* sp, int kind, const double* color, double rough, double ior, const double* emission) {
  Material m;
  m.kind = kind;
  m.color = ld3(color);
  m.roughness = rough;
  m.ior = ior;
  m.emission = ld3(emission);
  return ((Scene*)sp)->add_material(m);
}
// Replaces the color and/or emission of material idx in place (the Go Scene's
// Materials slice is mutable, renderer.go:94-101, 242-245). The sphere-light CDF
// of build() is not recomputed. Returns 0, or -1 for an index out of range.
int orc_set_material(void* sp, int idx, const double* color, const double* emission) {
  Scene* s = (Scene*)sp;
  if (idx < 0 || idx >= (int)s->materials.size()) return -1;
  if (color) s->materials[idx].color = ld3(color);
  if (emission) s->materials[idx].emission = ld3(emission);
  return 0;
}
void orc_add_sphere(void* sp, const double* c, double r, int mat) { ((Scene*)sp)->add_sphere(ld3(c), r, mat); }
void orc_add_triangles(void* sp, int64_t n, const double* v9, const int32_t* mats) {
  Scene* s = (Scene*)sp;
  s->prims.reserve(s->prims.size() + n);
  for (int64_t i = 0; i < n; i++) s->add_triangle(ld3(v9 + 9 * i), ld3(v9 + 9 * i + 3), ld3(v9 + 9 * i + 6), mats[i]);
}
void orc_build(void* sp) { ((Scene*)sp)->build(); }
void orc_refit(void* sp) { ((Scene*)sp)->refit(); }

// translatePrimitive (renderer.go:310-330)
void orc_translate_prim(void* sp, int idx, const double* d3) {
  Scene* s = (Scene*)sp;
  Primitive& p = s->prims[idx];
  V3 d = ld3(d3);
  if (p.kind == PrimSphere) {
    p.center = add(p.center, d);
    p.centroid = p.center;
    V3 rv = v3(p.radius, p.radius, p.radius);
    p.box = AABB{sub(p.center, rv), add(p.center, rv)};
    return;
  }
  p.a = add(p.a, d); p.b = add(p.b, d); p.c = add(p.c, d);
  p.e1 = sub(p.b, p.a); p.e2 = sub(p.c, p.a);
  p.normal = unit(cross(p.e1, p.e2));
  p.centroid = mul(add(add(p.a, p.b), p.c), 1.0 / 3.0);
  AABB box = expand_point(expand_point(expand_point(empty_aabb(), p.a), p.b), p.c);
  double eps = 1e-6;
  box.mn = sub(box.mn, v3(eps, eps, eps));
  box.mx = add(box.mx, v3(eps, eps, eps));
  p.box = box;
}

void orc_counts(void* sp, int64_t* out) {
  Scene* s = (Scene*)sp;
  out[0] = (int64_t)s->prims.size();
  out[1] = (int64_t)s->nodes.size();
  out[2] = (int64_t)s->light_spheres.size();
  out[3] = (int64_t)s->materials.size();
  out[4] = (int64_t)s->topo_rev;
  out[5] = (int64_t)s->geom_rev;
}
void orc_get_nodes(void* sp, double* box6, int32_t* left, int32_t* right, int32_t* start, int32_t* count) {
  Scene* s = (Scene*)sp;
  for (size_t i = 0; i < s->nodes.size(); i++) {
    const Node& n = s->nodes[i];
    st3(box6 + 6 * i, n.box.mn);
    st3(box6 + 6 * i + 3, n.box.mx);
    left[i] = n.left; right[i] = n.right; start[i] = n.start; count[i] = n.count;
  }
}
void orc_get_order(void* sp, int32_t* out) {
  Scene* s = (Scene*)sp;
  for (size_t i = 0; i < s->order.size(); i++) out[i] = s->order[i];
}
void orc_get_escapes(void* sp, int32_t* out) {
  std::vector<int32_t> e = threaded_escapes(((Scene*)sp)->nodes);
  std::memcpy(out, e.data(), e.size() * sizeof(int32_t));
}
void orc_get_lights(void* sp, int32_t* spheres, double* cdf, double* pdf_by_prim) {
  Scene* s = (Scene*)sp;
  for (size_t i = 0; i < s->light_spheres.size(); i++) { spheres[i] = s->light_spheres[i]; cdf[i] = s->light_cdf[i]; }
  for (size_t i = 0; i < s->light_pdf_by_prim.size(); i++) pdf_by_prim[i] = s->light_pdf_by_prim[i];
}
void orc_get_prims(void* sp, int32_t* kind, int32_t* mat, double* center, double* radius, double* a, double* e1,
                   double* e2, double* normal, double* box6) {
  Scene* s = (Scene*)sp;
  for (size_t i = 0; i < s->prims.size(); i++) {
    const Primitive& p = s->prims[i];
    kind[i] = p.kind; mat[i] = p.material;
    st3(center + 3 * i, p.center); radius[i] = p.radius;
    st3(a + 3 * i, p.a); st3(e1 + 3 * i, p.e1); st3(e2 + 3 * i, p.e2); st3(normal + 3 * i, p.normal);
    st3(box6 + 6 * i, p.box.mn); st3(box6 + 6 * i + 3, p.box.mx);
  }
}
void orc_get_materials(void* sp, int32_t* kind, double* color, double* rough, double* ior, double* emission) {
  Scene* s = (Scene*)sp;
  for (size_t i = 0; i < s->materials.size(); i++) {
    const Material& m = s->materials[i];
    kind[i] = m.kind; st3(color + 3 * i, m.color); rough[i] = m.roughness; ior[i] = m.ior;
    st3(emission + 3 * i, m.emission);
  }
}

int orc_aabb_hit(const double* box6, const double* ray6, double tmin, double tmax, double* near_out) {
  AABB b{ld3(box6), ld3(box6 + 3)};
  RayAccel ar = prepare_ray(Ray{ld3(ray6), ld3(ray6 + 3)});
  return aabb_hit(b, ar, tmin, tmax, near_out) ? 1 : 0;
}

// Closest hit over fp64 rays (o, d) with one (tmin, tmax) for the batch.
// mode 0: Scene.Hit; 1: stackless escape traversal.
void orc_hit_batch(void* sp, int64_t n, const double* rays6, double tmin, double tmax, int mode, double* t_out,
                   int32_t* prim_out, int64_t* counters, int threads) {
  Scene* s = (Scene*)sp;
  std::vector<int32_t> esc;
  if (mode == 1) esc = threaded_escapes(s->nodes);
  int T = threads < 1 ? (int)std::max(1u, std::thread::hardware_concurrency()) : threads;
  std::vector<Counters> per(T + 1);
  parallel_for(n, T, [&](int64_t a, int64_t b, int tid) {
    for (int64_t i = a; i < b; i++) {
      Ray r{ld3(rays6 + 6 * i), ld3(rays6 + 6 * i + 3)};
      Hit h;
      bool ok = mode == 1 ? s->hit_threaded(r, tmin, tmax, esc, &h) : s->hit(r, tmin, tmax, &h, &per[tid]);
      t_out[i] = ok ? h.t : -1.0;
      prim_out[i] = ok ? h.primitive : -1;
    }
  });
  if (counters) {
    counters[0] = counters[1] = counters[2] = 0;
    for (auto& c : per) { counters[0] += c.boxes; counters[1] += c.tris; counters[2] += c.spheres; }
  }
}

// Closest hit / any hit over fp32 ray records (ox, oy, oz, tmin, dx, dy, dz, tmax),
// the ray-cast format of the C-ABI. The fp32 values widen exactly to fp64.
void orc_hit_batch_f32(void* sp, int64_t n, const float* rays8, double* t_out, int32_t* prim_out, int64_t* counters,
                       int threads) {
  Scene* s = (Scene*)sp;
  int T = threads < 1 ? (int)std::max(1u, std::thread::hardware_concurrency()) : threads;
  std::vector<Counters> per(T + 1);
  parallel_for(n, T, [&](int64_t a, int64_t b, int tid) {
    for (int64_t i = a; i < b; i++) {
      const float* r8 = rays8 + 8 * i;
      Ray r{v3(r8[0], r8[1], r8[2]), v3(r8[4], r8[5], r8[6])};
      Hit h;
      bool ok = s->hit(r, (double)r8[3], (double)r8[7], &h, &per[tid]);
      t_out[i] = ok ? h.t : -1.0;
      prim_out[i] = ok ? h.primitive : -1;
    }
  });
  if (counters) {
    counters[0] = counters[1] = counters[2] = 0;
    for (auto& c : per) { counters[0] += c.boxes; counters[1] += c.tris; counters[2] += c.spheres; }
  }
}
// Brute force over every primitive (small scenes): the number of primitives
// whose fp64 test gives exactly the minimal distance, and up to `k` of them.
// Distinct primitives at bit-identical distances are resolved by the
// reference's traversal order, which this tie set makes visible to tests.
void orc_tie_sets_f32(void* sp, int64_t n, const float* rays8, int k, int32_t* count_out, int32_t* members) {
  Scene* s = (Scene*)sp;
  parallel_for(n, 0, [&](int64_t a, int64_t b, int) {
    for (int64_t i = a; i < b; i++) {
      const float* r8 = rays8 + 8 * i;
      RayAccel ar = prepare_ray(Ray{v3(r8[0], r8[1], r8[2]), v3(r8[4], r8[5], r8[6])});
      double best = (double)r8[7];
      int cnt = 0;
      for (int p = 0; p < (int)s->prims.size(); p++) {
        Hit h;
        if (!prim_hit(s->prims[p], ar, (double)r8[3], (double)r8[7], &h)) continue;
        if (h.t < best || cnt == 0) { best = h.t; cnt = 0; }
        if (h.t == best) {
          if (cnt < k) members[i * k + cnt] = p;
          cnt++;
        }
      }
      count_out[i] = cnt;
    }
  });
}

void orc_occluded_batch_f32(void* sp, int64_t n, const float* rays8, uint8_t* out, int64_t* counters, int threads) {
  Scene* s = (Scene*)sp;
  int T = threads < 1 ? (int)std::max(1u, std::thread::hardware_concurrency()) : threads;
  std::vector<Counters> per(T + 1);
  parallel_for(n, T, [&](int64_t a, int64_t b, int tid) {
    for (int64_t i = a; i < b; i++) {
      const float* r8 = rays8 + 8 * i;
      Ray r{v3(r8[0], r8[1], r8[2]), v3(r8[4], r8[5], r8[6])};
      out[i] = s->occluded(r, (double)r8[3], (double)r8[7], &per[tid]) ? 1 : 0;
    }
  });
  if (counters) {
    counters[0] = counters[1] = counters[2] = 0;
    for (auto& c : per) { counters[0] += c.boxes; counters[1] += c.tris; counters[2] += c.spheres; }
  }
}
void orc_occluded_batch(void* sp, int64_t n, const double* rays6, const double* tmax_per_ray, double tmin,
                        uint8_t* out, int threads) {
  Scene* s = (Scene*)sp;
  parallel_for(n, threads, [&](int64_t a, int64_t b, int) {
    for (int64_t i = a; i < b; i++) {
      Ray r{ld3(rays6 + 6 * i), ld3(rays6 + 6 * i + 3)};
      out[i] = s->occluded(r, tmin, tmax_per_ray[i], nullptr) ? 1 : 0;
    }
  });
}

double orc_radical_inverse(uint64_t n, uint64_t base) { return radical_inverse(n, base); }
void orc_pixel_sample_rotation(int x, int y, double* out2) { pixel_sample_rotation(x, y, out2, out2 + 1); }
int orc_effective_spp(int spp, int msaa, int tsaa) {
  Settings s;
  s.spp = spp; s.msaa = msaa; s.tsaa = tsaa;
  return effective_spp(s);
}
int orc_build_sample_sequence(int sampler, int spp, int msaa, int tsaa, double* X, double* Y) {
  Settings s;
  s.sampler = sampler; s.spp = spp; s.msaa = msaa; s.tsaa = tsaa;
  std::vector<double> x, y;
  build_sample_sequence(s, &x, &y);
  if (X) std::memcpy(X, x.data(), x.size() * sizeof(double));
  if (Y) std::memcpy(Y, y.data(), y.size() * sizeof(double));
  return (int)x.size();
}
void orc_cos_hemisphere(const double* n3, uint64_t seed, int64_t count, double* out) {
  Rng r = make_path_rng(seed, 0, 0);
  for (int64_t i = 0; i < count; i++) st3(out + 3 * i, rand_cos_hemisphere(ld3(n3), r));
}
void orc_unit_vectors(uint64_t seed, int64_t count, double* out) {
  Rng r = make_path_rng(seed, 0, 0);
  for (int64_t i = 0; i < count; i++) st3(out + 3 * i, rand_unit_vector(r));
}
void orc_rng_floats(uint64_t seed, uint64_t pixel, uint64_t sample, int64_t count, double* out) {
  Rng r = make_path_rng(seed, pixel, sample);
  for (int64_t i = 0; i < count; i++) out[i] = r.float64();
}
void orc_make_tile_order(int tx, int ty, const char* mode, int32_t* out) {
  std::vector<int> o = make_tile_order(tx, ty, mode ? mode : "Center");
  for (size_t i = 0; i < o.size(); i++) out[i] = o[i];
}
double orc_power_heuristic(double a, double b) { return power_heuristic(a, b); }
double orc_light_selection_pdf(void* sp, int prim, int power) {
  return light_selection_pdf(*(Scene*)sp, prim, power != 0);
}
void orc_clamp_firefly(const double* c3, double limit, double* out3) { st3(out3, clamp_firefly(ld3(c3), limit)); }
void orc_camera_basis(const double* cam10, double aspect, double* out12) {
  Camera c{ld3(cam10), ld3(cam10 + 3), ld3(cam10 + 6), cam10[9]};
  V3 o, l, h, v;
  camera_basis(c, aspect, &o, &l, &h, &v);
  st3(out12, o); st3(out12 + 3, l); st3(out12 + 6, h); st3(out12 + 9, v);
}

// Render: linear3 = per-pixel mean, sumsq3 = per-pixel mean of squares,
// guides11 = (p3, n3, albedo3, depth, valid) or NULL,
// stats6 = (segments, shadow rays, box tests, tri tests, sphere tests, photon map rays).
static int render_to(void* sp, const double* cam10, const Settings& st, uint64_t seed, int threads, double* linear3,
                     double* sumsq3, double* guides11, int64_t* stats6) {
  Scene* s = (Scene*)sp;
  Camera cam{ld3(cam10), ld3(cam10 + 3), ld3(cam10 + 6), cam10[9]};
  RenderOut out;
  render(*s, cam, st, seed, threads, &out, nullptr);
  size_t np = out.linear.size();
  for (size_t i = 0; i < np; i++) {
    st3(linear3 + 3 * i, out.linear[i]);
    if (sumsq3) st3(sumsq3 + 3 * i, out.sumsq[i]);
    if (guides11) {
      const Guide& g = out.guides[i];
      double* q = guides11 + 11 * i;
      st3(q, g.p); st3(q + 3, g.n); st3(q + 6, g.albedo); q[9] = g.depth; q[10] = g.valid ? 1 : 0;
    }
  }
  if (stats6) {
    stats6[0] = out.segments; stats6[1] = out.shadow; stats6[2] = out.c.boxes; stats6[3] = out.c.tris;
    stats6[4] = out.c.spheres; stats6[5] = out.photon_rays;
  }
  return 0;
}
int orc_render(void* sp, const double* cam10, const orc_settings* cs, uint64_t seed, int threads, double* linear3,
               double* sumsq3, double* guides11, int64_t* stats6) {
  return render_to(sp, cam10, load_settings(cs), seed, threads, linear3, sumsq3, guides11, stats6);
}
// The pixels [x0, x0 + w) x [y0, y0 + h) of the frame, each as the whole-frame
// render would give it (outputs hold w*h pixels, row-major). Returns -1 for a
// window outside the frame.
int orc_render_window(void* sp, const double* cam10, const orc_settings* cs, int x0, int y0, int w, int h,
                      uint64_t seed, int threads, double* linear3, double* sumsq3, double* guides11, int64_t* stats6) {
  Settings st = load_settings(cs);
  if (x0 < 0 || y0 < 0 || w <= 0 || h <= 0 || x0 + w > st.width || y0 + h > st.height) return -1;
  st.win_x = x0; st.win_y = y0; st.win_w = w; st.win_h = h;
  return render_to(sp, cam10, st, seed, threads, linear3, sumsq3, guides11, stats6);
}

int orc_photon_budget(int level) { return photon_budget(level); }
uint64_t orc_photon_cell_key(int64_t x, int64_t y, int64_t z) { return photon_cell_key(x, y, z); }
double orc_photon_radius(void* sp, int level) { return photon_radius(*(Scene*)sp, level); }

// buildPhotonMap: photons in append order, 10 doubles each (P, N, flux,
// emission index) up to `cap`; returns the photon count. out3 = (radius, rays, 0).
int64_t orc_photon_map(void* sp, const orc_settings* cs, uint64_t seed, int64_t cap, double* photons10,
                       double* out3) {
  Settings st = load_settings(cs);
  int64_t rays = 0;
  PhotonMap pm = build_photon_map(*(Scene*)sp, st, seed, &rays);
  const int64_t n = (int64_t)pm.photons.size();
  for (int64_t i = 0; i < n && i < cap; i++) {
    const Photon& ph = pm.photons[i];
    double* q = photons10 + 10 * i;
    st3(q, ph.p); st3(q + 3, ph.n); st3(q + 6, ph.flux); q[9] = ph.emission;
  }
  if (out3) { out3[0] = pm.radius; out3[1] = (double)rays; out3[2] = 0; }
  return n;
}

// PhotonMap.gather at n points (3 + 3 doubles each) over the map built from
// (settings, seed); out3 per point.
void orc_photon_gather(void* sp, const orc_settings* cs, uint64_t seed, int64_t n, const double* pn6, double* out3) {
  Settings st = load_settings(cs);
  PhotonMap pm = build_photon_map(*(Scene*)sp, st, seed, nullptr);
  for (int64_t i = 0; i < n; i++) st3(out3 + 3 * i, photon_gather(pm, ld3(pn6 + 6 * i), ld3(pn6 + 6 * i + 3), 64));
}

static std::vector<Guide> load_guides(const double* g11, int n) {
  std::vector<Guide> g(n);
  for (int i = 0; i < n; i++) {
    const double* q = g11 + 11 * i;
    g[i].p = ld3(q); g[i].n = ld3(q + 3); g[i].albedo = ld3(q + 6); g[i].depth = q[9]; g[i].valid = q[10] != 0;
  }
  return g;
}
static std::vector<V3> load_img(const double* p, int n) {
  std::vector<V3> v(n);
  for (int i = 0; i < n; i++) v[i] = ld3(p + 3 * i);
  return v;
}
void orc_atrous(const double* img3, const double* guides11, int w, int h, int iters, double* out3) {
  std::vector<V3> o = atrous_denoise(load_img(img3, w * h), load_guides(guides11, w * h), w, h, iters);
  for (int i = 0; i < w * h; i++) st3(out3 + 3 * i, o[i]);
}
void orc_bloom(const double* img3, int w, int h, int level, double* out3) {
  std::vector<V3> o = apply_bloom(load_img(img3, w * h), w, h, level);
  for (int i = 0; i < w * h; i++) st3(out3 + 3 * i, o[i]);
}
void orc_tone_map(const double* img3, int64_t n, int hdr, double* out3) {
  for (int64_t i = 0; i < n; i++) st3(out3 + 3 * i, tone_map_hdr(ld3(img3 + 3 * i), hdr));
}
void orc_to_rgba(const double* img3, int64_t n, double exposure, double gamma, int hdr, uint32_t* out) {
  for (int64_t i = 0; i < n; i++) out[i] = to_rgba(ld3(img3 + 3 * i), exposure, gamma, hdr);
}

void orc_hbao(const double* img3, const double* guides11, int w, int h, int level, int plus, double* out3) {
  std::vector<V3> o = apply_hbao(load_img(img3, w * h), load_guides(guides11, w * h), w, h, level, plus != 0);
  for (int i = 0; i < w * h; i++) st3(out3 + 3 * i, o[i]);
}
void orc_temporal(const double* cur3, const double* guides11, int w, int h, const double* prev3,
                  const double* prev_guides11, const double* cam10, double weight, double* out3) {
  Camera cam{ld3(cam10), ld3(cam10 + 3), ld3(cam10 + 6), cam10[9]};
  std::vector<V3> o = temporal_accumulate(load_img(cur3, w * h), load_guides(guides11, w * h), w, h,
                                          load_img(prev3, w * h), load_guides(prev_guides11, w * h), cam, weight);
  for (int i = 0; i < w * h; i++) st3(out3 + 3 * i, o[i]);
}
double orc_temporal_weight(int taa, int tsaa, int txaa) { return temporal_weight(taa, tsaa, txaa); }
void orc_debug_view(const double* lin3, const double* guides11, int w, int h, int mode, int hbao, int hbao_plus,
                    double* out3) {
  std::vector<V3> o = make_debug_view(load_img(lin3, w * h), load_guides(guides11, w * h), w, h, mode, hbao, hbao_plus);
  for (int i = 0; i < w * h; i++) st3(out3 + 3 * i, o[i]);
}
void orc_upscale(const double* src3, int sw, int sh, int dw, int dh, int mode, double* out3) {
  std::vector<V3> o = upscale_basic(load_img(src3, sw * sh), sw, sh, dw, dh, mode);
  for (int i = 0; i < dw * dh; i++) st3(out3 + 3 * i, o[i]);
}
void orc_sharpen(const double* img3, int w, int h, double amount, double* out3) {
  std::vector<V3> o = edge_aware_sharpen(load_img(img3, w * h), w, h, amount);
  for (int i = 0; i < w * h; i++) st3(out3 + 3 * i, o[i]);
}
void orc_fxaa(const double* img3, int w, int h, int level, double* out3) {
  std::vector<V3> o = apply_fxaa(load_img(img3, w * h), w, h, level);
  for (int i = 0; i < w * h; i++) st3(out3 + 3 * i, o[i]);
}
void orc_txaa(const double* img3, int w, int h, int level, double* out3) {
  std::vector<V3> o = apply_txaa_resolve(load_img(img3, w * h), w, h, level);
  for (int i = 0; i < w * h; i++) st3(out3 + 3 * i, o[i]);
}
void orc_internal_size(int w, int h, int mode, int* out2) { internal_size(w, h, mode, out2, out2 + 1); }
int orc_project_point(const double* cam10, const double* p3, int w, int h, int* out2) {
  Camera cam{ld3(cam10), ld3(cam10 + 3), ld3(cam10 + 6), cam10[9]};
  return project_point(cam, ld3(p3), w, h, out2, out2 + 1) ? 1 : 0;
}

}  // extern "C"

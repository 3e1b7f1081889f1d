// Test infrastructure only (see bc_oracle.h): samplers, the path integrator,
// the pixel loop, the tile scheduler and the post passes restated from
// windows_portable/renderer.go in fp64.
#include "bc_oracle.h"

#include <algorithm>
#include <cmath>
#include <thread>

namespace orc {

// ---- PCG32 (O'Neill, "PCG: A Family of Simple Fast Space-Efficient
// Statistically Good Algorithms for Random Number Generation", 2014),
// seeded per (pixel, sample) through SplitMix64 finalisers. The GPU draws
// from the same generator, so CRN runs replay identical decisions.
static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
uint32_t Rng::next_u32() {
  uint64_t old = state;
  state = old * 6364136223846793005ull + inc;
  uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
  uint32_t rot = (uint32_t)(old >> 59);
  return (xs >> rot) | (xs << ((32u - rot) & 31u));
}
double Rng::float64() { return (double)(next_u32() >> 8) * (1.0 / 16777216.0); }
int Rng::intn(int n) {
  int i = (int)(float64() * (double)n);
  return i >= n ? n - 1 : i;
}
Rng make_path_rng(uint64_t seed, uint64_t pixel_key, uint64_t sample) {
  uint64_t key = mix64(seed + 0x9E3779B97F4A7C15ull * (pixel_key + 1)) ^
                 mix64(sample * 0xD1B54A32D192ED03ull + 0x632BE59BD9B4E019ull);
  Rng r;
  r.state = 0;
  r.inc = (key << 1) | 1u;
  r.next_u32();
  r.state += mix64(key ^ 0xA0761D6478BD642Full);
  r.next_u32();
  return r;
}

// renderer.go:1262-1269
V3 rand_in_unit_sphere(Rng& r) {
  for (;;) {
    double x = r.float64() * 2 - 1;
    double y = r.float64() * 2 - 1;
    double z = r.float64() * 2 - 1;
    V3 p = v3(x, y, z);
    double l2 = dot(p, p);
    if (l2 < 1 && l2 > 1e-18) return p;
  }
}
// renderer.go:1273-1285
V3 rand_unit_vector(Rng& r) {
  for (;;) {
    double u = r.float64() * 2 - 1;
    double v = r.float64() * 2 - 1;
    double s = u * u + v * v;
    if (s >= 1 || s <= 1e-18) continue;
    double f = 2 * std::sqrt(1 - s);
    return v3(u * f, v * f, 1 - 2 * s);
  }
}
// renderer.go:1290-1311
V3 rand_cos_hemisphere(V3 n, Rng& r) {
  double x, y, s;
  for (;;) {
    x = r.float64() * 2 - 1;
    y = r.float64() * 2 - 1;
    s = x * x + y * y;
    if (s < 1) break;
  }
  double z = std::sqrt(gmax(0, 1 - s));
  double sign = 1.0;
  if (n.z < 0) sign = -1;
  double a = -1.0 / (sign + n.z);
  double b = n.x * n.y * a;
  V3 t = v3(1 + sign * n.x * n.x * a, sign * b, -sign * n.x);
  V3 bt = v3(b, sign + n.y * n.y * a, -n.y);
  return add(add(mul(t, x), mul(bt, y)), mul(n, z));
}
V3 reflect(V3 v, V3 n) { return sub(v, mul(n, 2 * dot(v, n))); }  // renderer.go:1312
V3 refract(V3 uv, V3 n, double eta) {                             // renderer.go:1313-1318
  double ct = gmin(dot(mul(uv, -1), n), 1);
  V3 perp = mul(add(uv, mul(n, ct)), eta);
  V3 par = mul(n, -std::sqrt(std::fabs(1 - dot(perp, perp))));
  return add(perp, par);
}
double schlick(double cosine, double ref) {  // renderer.go:1319-1326
  double r0 = (1 - ref) / (1 + ref);
  r0 *= r0;
  double x = 1 - cosine;
  double x2 = x * x;
  double x5 = x2 * x2 * x;
  return r0 + (1 - r0) * x5;
}
V3 background(V3 d) {  // renderer.go:1327-1331
  V3 u = unit(d);
  double t = .5 * (u.y + 1);
  return add(mul(v3(.06, .08, .12), 1 - t), mul(v3(.32, .48, .72), t));
}

static bool visible(const Scene& s, V3 from, V3 to, Counters* c) {  // renderer.go:1333-1341
  V3 d = sub(to, from);
  double dist2 = dot(d, d);
  if (dist2 < 1e-12) return true;
  double dist = std::sqrt(dist2);
  return !s.occluded(Ray{from, mul(d, 1 / dist)}, 1e-4, dist - 1e-4, c);
}

double light_selection_pdf(const Scene& s, int pi, bool power) {  // renderer.go:1358-1369
  if (s.light_spheres.empty()) return 0;
  if (!power) return 1 / (double)s.light_spheres.size();
  if (pi >= 0 && pi < (int)s.light_pdf_by_prim.size()) return s.light_pdf_by_prim[pi];
  return 0;
}

static int choose_light(const Scene& s, Rng& rng, bool power, double* pdf_out) {  // renderer.go:1371-1393
  int nl = (int)s.light_spheres.size();
  if (nl == 0) { *pdf_out = 0; return -1; }
  if (!power || (int)s.light_cdf.size() != nl) {
    int idx = rng.intn(nl);
    *pdf_out = 1 / (double)nl;
    return s.light_spheres[idx];
  }
  double r = rng.float64();
  // sort.Search: smallest i with cdf[i] >= r
  int lo = 0, hi = nl;
  while (lo < hi) {
    int mid = (int)((unsigned)(lo + hi) >> 1);
    if (!(s.light_cdf[mid] >= r)) lo = mid + 1; else hi = mid;
  }
  int idx = lo;
  if (idx >= nl) idx = nl - 1;
  int pi = s.light_spheres[idx];
  double pdf = 0;
  if (pi >= 0 && pi < (int)s.light_pdf_by_prim.size()) pdf = s.light_pdf_by_prim[pi];
  if (pdf <= 0) pdf = 1 / (double)nl;
  *pdf_out = pdf;
  return pi;
}

double power_heuristic(double a, double b) {  // renderer.go:1395-1402
  double a2 = a * a, b2 = b * b;
  if (a2 + b2 <= 1e-20) return 0;
  return a2 / (a2 + b2);
}

double light_directional_pdf(const Scene& s, int pi, V3 from, V3 lp, V3 ln, bool power) {  // renderer.go:1404-1425
  if (pi < 0 || pi >= (int)s.prims.size()) return 0;
  const Primitive& p = s.prims[pi];
  if (p.kind != PrimSphere || p.radius <= 0) return 0;
  V3 to = sub(lp, from);
  double dist2 = dot(to, to);
  if (dist2 <= 1e-12) return 0;
  V3 ld = unit(to);
  double cosL = gmax(0, dot(ln, mul(ld, -1)));
  if (cosL <= 1e-12) return 0;
  double area = 4 * M_PI * p.radius * p.radius;
  double sel = light_selection_pdf(s, pi, power);
  return sel * dist2 / (cosL * area);
}

V3 direct_light(const Scene& s, const Hit& h, V3 hitP, const Material& mat, Rng& rng,
                       const Settings& st, TraceStats* stats) {  // renderer.go:1427-1465
  if (mat.kind != MatDiffuse || s.light_spheres.empty()) return v3(0, 0, 0);
  double selectPDF;
  int li = choose_light(s, rng, st.power_light, &selectPDF);
  if (li < 0 || selectPDF <= 0) return v3(0, 0, 0);
  const Primitive& lp = s.prims[li];
  const Material& lm = s.materials[lp.material];
  V3 ln = rand_unit_vector(rng);
  V3 q = add(lp.center, mul(ln, lp.radius));
  V3 to = sub(q, hitP);
  double dist2 = dot(to, to);
  if (dist2 < 1e-8) return v3(0, 0, 0);
  V3 ld = unit(to);
  double nd = gmax(0, dot(h.n, ld));
  double cosL = gmax(0, dot(mul(ln, -1), ld));
  if (nd <= 0 || cosL <= 0) return v3(0, 0, 0);
  if (stats) stats->shadow++;
  if (!visible(s, add(hitP, mul(h.n, 2e-4)), q, stats ? &stats->c : nullptr)) return v3(0, 0, 0);
  double area = 4 * M_PI * lp.radius * lp.radius;
  double lightPDF = selectPDF * dist2 / (cosL * area);
  if (lightPDF <= 0) return v3(0, 0, 0);
  double bsdfPDF = nd / M_PI;
  double w = 1.0;
  if (st.mis) w = power_heuristic(lightPDF, bsdfPDF);
  V3 f = mul(mat.color, 1 / M_PI);
  return mul(had(f, lm.emission), nd * w / lightPDF);
}

V3 material_preview_color(const Material& m) {  // renderer.go:1467-1475
  if (m.kind == MatEmissive)
    return v3(clampd(m.emission.x / 8, 0, 1), clampd(m.emission.y / 8, 0, 1), clampd(m.emission.z / 8, 0, 1));
  if (dot(m.color, m.color) > 0) return m.color;
  return v3(0.8, 0.8, 0.8);
}

// renderer.go:1484-1563
V3 trace(const Scene& s, Ray ray, const Settings& st, Rng& rng, TraceStats* stats, Guide* guide) {
  V3 throughput = v3(1, 1, 1);
  V3 radiance = v3(0, 0, 0);
  bool prevWasDiffuse = false;
  double prevBSDFPDF = 0;
  V3 prevPoint = v3(0, 0, 0);
  Counters* cc = stats ? &stats->c : nullptr;
  for (int bounce = 0; bounce < st.bounces; bounce++) {
    if (stats) stats->segments++;
    Hit h;
    if (!s.hit(ray, 1e-4, 1e30, &h, cc)) return add(radiance, had(throughput, background(ray.d)));
    if (h.material < 0 || h.material >= (int)s.materials.size()) return radiance;
    const Material& m = s.materials[h.material];
    V3 p = add(ray.o, mul(ray.d, h.t));
    if (bounce == 0 && guide) {
      guide->p = p; guide->n = h.n; guide->albedo = material_preview_color(m);
      guide->depth = h.t; guide->valid = true;
    }
    if (m.kind == MatEmissive) {
      double w = 1.0;
      if (st.mis && prevWasDiffuse && h.primitive >= 0) {
        double lightPDF = light_directional_pdf(s, h.primitive, prevPoint, p, h.n, st.power_light);
        w = power_heuristic(prevBSDFPDF, lightPDF);
      }
      return add(radiance, mul(had(throughput, m.emission), w));
    }
    if (m.kind == MatDiffuse) {
      radiance = add(radiance, had(throughput, direct_light(s, h, p, m, rng, st, stats)));
      throughput = had(throughput, m.color);
      V3 d = rand_cos_hemisphere(h.n, rng);
      prevWasDiffuse = true;
      prevBSDFPDF = gmax(0, dot(h.n, d)) / M_PI;
      prevPoint = p;
      ray = Ray{add(p, mul(h.n, 2e-4)), d};
    } else if (m.kind == MatMetal) {
      V3 d = unit(add(reflect(unit(ray.d), h.n), mul(rand_in_unit_sphere(rng), clampd(m.roughness, 0, 1))));
      if (dot(d, h.n) <= 0) return radiance;
      prevWasDiffuse = false;
      throughput = had(throughput, m.color);
      ray = Ray{add(p, mul(h.n, 2e-4)), d};
    } else if (m.kind == MatGlass) {
      double eta = m.ior;
      if (eta <= 1) eta = 1.5;
      double ratio = eta;
      if (h.front) ratio = 1 / eta;
      V3 un = unit(ray.d);
      double cosTheta = gmin(dot(mul(un, -1), h.n), 1);
      double sinTheta = std::sqrt(gmax(0, 1 - cosTheta * cosTheta));
      V3 d;
      if (ratio * sinTheta > 1 || schlick(cosTheta, ratio) > rng.float64()) d = reflect(un, h.n);
      else d = refract(un, h.n, ratio);
      prevWasDiffuse = false;
      throughput = had(throughput, m.color);
      ray = Ray{add(p, mul(d, 2e-4)), d};
    }
    int rrDepth = st.rr_depth;
    if (rrDepth < 1) rrDepth = 4;
    if (bounce >= rrDepth) {
      double pr = clampd(maxcomp(throughput), .08, .95);
      if (rng.float64() > pr) return radiance;
      throughput = mul(throughput, 1 / pr);
    }
  }
  return radiance;
}

int effective_spp(const Settings& s) {  // renderer.go:2395-2417
  int msaa = s.msaa;
  if (msaa != 2 && msaa != 4 && msaa != 8) msaa = 1;
  int tsaa = 1;
  switch (s.tsaa) {
    case 1: tsaa = 2; break;
    case 2: tsaa = 3; break;
    case 3: tsaa = 4; break;
  }
  int v = s.spp * msaa * tsaa;
  if (v < 1) return 1;
  if (v > 4096) return 4096;
  return v;
}

double radical_inverse(uint64_t n, uint64_t base) {  // renderer.go:1844-1858
  if (base == 2) {
    uint64_t r = 0;
    for (int i = 0; i < 64; i++) { r = (r << 1) | (n & 1); n >>= 1; }
    return (double)r * 5.421010862427522e-20;
  }
  double invBase = 1.0 / (double)base;
  double inv = invBase;
  double result = 0;
  while (n > 0) {
    uint64_t digit = n % base;
    result += (double)digit * inv;
    n /= base;
    inv *= invBase;
  }
  return result;
}
double fractd(double x) { return x - std::floor(x); }  // renderer.go:1860

void build_sample_sequence(const Settings& s, std::vector<double>* X, std::vector<double>* Y) {  // renderer.go:1883-1904
  X->clear(); Y->clear();
  if (s.sampler == SamplerRandom) return;
  int n = effective_spp(s);
  X->resize(n); Y->resize(n);
  if (s.sampler == SamplerR2) {
    const double g = 1.324717957244746;
    double a1 = 1.0 / g, a2 = 1.0 / (g * g);
    for (int i = 0; i < n; i++) {
      (*X)[i] = fractd(0.5 + (double)(i + 1) * a1);
      (*Y)[i] = fractd(0.5 + (double)(i + 1) * a2);
    }
    return;
  }
  for (int i = 0; i < n; i++) {
    (*X)[i] = radical_inverse((uint64_t)(i + 1), 2);
    (*Y)[i] = radical_inverse((uint64_t)(i + 1), 3);
  }
}

void pixel_sample_rotation(int x, int y, double* rx, double* ry) {  // renderer.go:1906-1915
  uint32_t h1 = ((uint32_t)x * 0x9e3779b1u) ^ ((uint32_t)y * 0x85ebca77u);
  h1 ^= h1 >> 16;
  h1 *= 0x7feb352du;
  h1 ^= h1 >> 15;
  uint32_t h2 = h1 ^ 0x68bc21ebu;
  h2 ^= h2 >> 13;
  const double inv = 1.0 / 4294967296.0;
  *rx = (double)h1 * inv;
  *ry = (double)h2 * inv;
}

V3 clamp_firefly(V3 c, double limit) {  // renderer.go:1917-1926
  if (limit <= 0) return c;
  double m = maxcomp(c);
  if (m <= limit || m <= 0) return c;
  return mul(c, limit / m);
}

// renderer.go:2376-2393 (Go's sort.Slice is not stable; keys are distinct
// except for mirror-symmetric tiles, whose relative order the reference does
// not pin either).
std::vector<int> make_tile_order(int tx, int ty, const std::string& mode) {
  int total = tx * ty;
  std::vector<int> order(total);
  for (int i = 0; i < total; i++) order[i] = i;
  std::string m = mode;
  for (auto& ch : m) ch = (char)std::tolower((unsigned char)ch);
  if (m == "scanline" || total <= 2) return order;
  double cx = (double)(tx - 1) * 0.5, cy = (double)(ty - 1) * 0.5;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    double ax = (double)(a % tx) - cx, ay = (double)(a / tx) - cy;
    double bx = (double)(b % tx) - cx, by = (double)(b / tx) - cy;
    return ax * ax + ay * ay < bx * bx + by * by;
  });
  return order;
}

// renderer.go:1928-1970; each sample draws from its own PCG32 stream keyed by
// (seed, pixel, sample), which makes renders independent of thread count.
static V3 adaptive_pixel(const Scene& s, V3 origin, V3 lower, V3 horiz, V3 vert, int x, int y, int W, int H,
                         const Settings& st, uint64_t seed, const std::vector<double>& SX,
                         const std::vector<double>& SY, TraceStats* stats, Guide* guide, V3* sumsq_out,
                         const PhotonMap* pm) {
  int pixelSPP = effective_spp(st);
  V3 sum = v3(0, 0, 0), sq = v3(0, 0, 0);
  double sumLum = 0, sumSqLum = 0;
  int minSamples = std::min(8, pixelSPP);
  double rotX, rotY;
  pixel_sample_rotation(x, y, &rotX, &rotY);
  uint64_t pkey = (uint64_t)y * (uint64_t)W + (uint64_t)x;
  for (int sample = 0; sample < pixelSPP; sample++) {
    Rng rng = make_path_rng(seed, pkey, (uint64_t)sample);
    double jx, jy;
    if (!SX.empty() && sample < (int)SX.size()) {
      jx = fractd(SX[sample] + rotX);
      jy = fractd(SY[sample] + rotY);
    } else {
      jx = rng.float64();
      jy = rng.float64();
    }
    double u = ((double)x + jx) / (double)std::max(W - 1, 1);
    double v = ((double)(H - 1 - y) + jy) / (double)std::max(H - 1, 1);
    V3 dir = sub(add(add(lower, mul(horiz, u)), mul(vert, v)), origin);
    V3 c = clamp_firefly(pixel_radiance(s, Ray{origin, dir}, st, rng, stats, sample == 0 ? guide : nullptr, pm),
                         st.firefly_clamp);
    sum = add(sum, c);
    sq = add(sq, had(c, c));
    double lum = luminance(c);
    sumLum += lum;
    sumSqLum += lum * lum;
    if (st.adaptive && sample + 1 >= minSamples && (sample + 1) % 2 == 0) {
      double n = (double)(sample + 1);
      double mean = sumLum / n;
      double variance = gmax(0, sumSqLum / n - mean * mean);
      if (variance < gmax(1e-8, st.adaptive_threshold)) {
        *sumsq_out = mul(sq, 1 / n);
        return mul(sum, 1 / n);
      }
    }
  }
  *sumsq_out = mul(sq, 1 / (double)pixelSPP);
  return mul(sum, 1 / (double)pixelSPP);
}

void render(const Scene& s, const Camera& cam, const Settings& st, uint64_t seed, int threads, RenderOut* out,
            const std::atomic<bool>* cancel) {
  int W = st.width, H = st.height;
  // the rendered region: the whole frame or the window, clipped to the frame
  int rx0 = 0, ry0 = 0, RW = W, RH = H;
  if (st.win_w > 0 && st.win_h > 0) {
    rx0 = std::max(0, std::min(st.win_x, W));
    ry0 = std::max(0, std::min(st.win_y, H));
    RW = std::min(st.win_w, W - rx0);
    RH = std::min(st.win_h, H - ry0);
  }
  out->linear.assign((size_t)RW * RH, v3(0, 0, 0));
  out->sumsq.assign((size_t)RW * RH, v3(0, 0, 0));
  out->guides.assign((size_t)RW * RH, Guide{});
  V3 origin, lower, horiz, vert;
  camera_basis(cam, (double)W / (double)H, &origin, &lower, &horiz, &vert);
  int tile = st.tile > 0 ? st.tile : 16;
  int tx = (RW + tile - 1) / tile, ty = (RH + tile - 1) / tile, total = tx * ty;
  std::vector<int> order = make_tile_order(tx, ty, "Center");
  std::vector<double> SX, SY;
  build_sample_sequence(st, &SX, &SY);
  // renderer.go:2728-2734: the photon map is built once per frame, before the tiles
  PhotonMap pm;
  if (st.integrator == IntegratorPhoton)
    pm = build_photon_map(s, st, st.photon_seed >= 0 ? (uint64_t)st.photon_seed : seed, &out->photon_rays);
  if (threads < 1) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  threads = std::min(threads, std::max(1, total));
  std::atomic<int> next{0};
  std::vector<TraceStats> per(threads);
  auto worker = [&](int id) {
    for (;;) {
      int oi = next.fetch_add(1);
      if (oi >= total) return;
      if (cancel && cancel->load()) return;
      int ti = order[oi];
      int x0 = rx0 + (ti % tx) * tile, y0 = ry0 + (ti / tx) * tile;
      int x1 = std::min(x0 + tile, rx0 + RW), y1 = std::min(y0 + tile, ry0 + RH);
      for (int y = y0; y < y1; y++)
        for (int x = x0; x < x1; x++) {
          size_t i = (size_t)(y - ry0) * RW + (x - rx0);
          out->linear[i] = adaptive_pixel(s, origin, lower, horiz, vert, x, y, W, H, st, seed, SX, SY, &per[id],
                                          &out->guides[i], &out->sumsq[i], &pm);
        }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; t++) pool.emplace_back(worker, t);
  for (auto& t : pool) t.join();
  for (auto& p : per) {
    out->segments += p.segments;
    out->shadow += p.shadow;
    out->c.boxes += p.c.boxes;
    out->c.tris += p.c.tris;
    out->c.spheres += p.c.spheres;
  }
}

// renderer.go:2228-2287 (single-threaded: the reference pins that its
// parallel post stack is bit-identical to the serial one).
std::vector<V3> atrous_denoise(const std::vector<V3>& img, const std::vector<Guide>& guides, int w, int h, int iters) {
  if ((int)img.size() != w * h || (int)guides.size() != w * h || iters <= 0) return img;
  std::vector<V3> cur = img, next(img.size());
  for (int it = 0; it < iters; it++) {
    int step = 1 << it;
    for (int y = 0; y < h; y++)
      for (int x = 0; x < w; x++) {
        int i = y * w + x;
        V3 center = cur[i];
        const Guide& g0 = guides[i];
        double l0 = luminance(center);
        V3 sum = v3(0, 0, 0);
        double wsum = 0;
        for (int oy = -1; oy <= 1; oy++) {
          int yy = y + oy * step;
          if (yy < 0 || yy >= h) continue;
          for (int ox = -1; ox <= 1; ox++) {
            int xx = x + ox * step;
            if (xx < 0 || xx >= w) continue;
            int j = yy * w + xx;
            const Guide& g1 = guides[j];
            if (g0.valid != g1.valid) continue;
            V3 q = cur[j];
            double wgt = 1.0;
            if (g0.valid) {
              double nd = clampd(dot(g0.n, g1.n), -1, 1);
              wgt *= std::exp((nd - 1) * 48.0);
              double depthScale = gmax(0.15, 0.04 * gmax(g0.depth, 1.0));
              wgt *= std::exp(-std::fabs(g0.depth - g1.depth) / depthScale);
            }
            wgt *= std::exp(-std::fabs(l0 - luminance(q)) * 3.5);
            if (ox == 0 && oy == 0) wgt *= 1.5;
            sum = add(sum, mul(q, wgt));
            wsum += wgt;
          }
        }
        next[i] = wsum > 1e-12 ? mul(sum, 1 / wsum) : center;
      }
    std::swap(cur, next);
  }
  return cur;
}

std::vector<V3> box_blur(const std::vector<V3>& img, int w, int h, int radius) {  // renderer.go:2490-2529
  if (radius <= 0 || (int)img.size() != w * h) return img;
  std::vector<V3> tmp(img.size()), out(img.size());
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      V3 sum = v3(0, 0, 0);
      double count = 0;
      for (int ox = -radius; ox <= radius; ox++) {
        int xx = x + ox;
        if (xx >= 0 && xx < w) { sum = add(sum, img[y * w + xx]); count++; }
      }
      tmp[y * w + x] = mul(sum, 1 / gmax(count, 1));
    }
  for (int x = 0; x < w; x++)
    for (int y = 0; y < h; y++) {
      V3 sum = v3(0, 0, 0);
      double count = 0;
      for (int oy = -radius; oy <= radius; oy++) {
        int yy = y + oy;
        if (yy >= 0 && yy < h) { sum = add(sum, tmp[yy * w + x]); count++; }
      }
      out[y * w + x] = mul(sum, 1 / gmax(count, 1));
    }
  return out;
}

std::vector<V3> apply_bloom(const std::vector<V3>& img, int w, int h, int level) {  // renderer.go:2531-2555
  if (level <= 0 || (int)img.size() != w * h) return img;
  std::vector<V3> bright(img.size(), v3(0, 0, 0));
  double threshold = 1.25 - 0.2 * (double)level;
  for (size_t i = 0; i < img.size(); i++) {
    V3 c = img[i];
    double l = luminance(c);
    if (l > threshold) bright[i] = mul(c, (l - threshold) / gmax(l, 1e-6));
  }
  std::vector<V3> blur = box_blur(bright, w, h, 1 + level);
  double strength = 0.08 + 0.09 * (double)level;
  std::vector<V3> out(img.size());
  for (size_t i = 0; i < img.size(); i++) out[i] = add(img[i], mul(blur[i], strength));
  return out;
}

V3 tone_map_hdr(V3 c, int hdr) {  // renderer.go:2034-2053
  switch (hdr) {
    case 0: return v3(clampd(c.x, 0, 1), clampd(c.y, 0, 1), clampd(c.z, 0, 1));
    case 1: return v3(c.x / (1 + c.x), c.y / (1 + c.y), c.z / (1 + c.z));
    case 3: {
      auto aces = [](double x) {
        double a = 2.51, b = 0.03, cc = 2.43, d = 0.59, e = 0.14;
        return clampd((x * (a * x + b)) / (x * (cc * x + d) + e), 0, 1);
      };
      return v3(aces(c.x), aces(c.y), aces(c.z));
    }
    default: {
      auto filmic = [](double x) {
        x = gmax(0, x - 0.004);
        return clampd((x * (6.2 * x + 0.5)) / (x * (6.2 * x + 1.7) + 0.06), 0, 1);
      };
      return v3(filmic(c.x), filmic(c.y), filmic(c.z));
    }
  }
}

uint32_t to_rgba(V3 c, double exposure, double gamma, int hdr) {  // renderer.go:2055-2064
  double exposureScale = std::pow(2.0, exposure);
  c = tone_map_hdr(mul(c, exposureScale), hdr);
  double invGamma = 1.0 / gmax(0.1, gamma);
  c = v3(std::pow(gmax(0, c.x), invGamma), std::pow(gmax(0, c.y), invGamma), std::pow(gmax(0, c.z), invGamma));
  uint32_t r = (uint32_t)(clampd(c.x, 0, .999) * 256);
  uint32_t g = (uint32_t)(clampd(c.y, 0, .999) * 256);
  uint32_t b = (uint32_t)(clampd(c.z, 0, .999) * 256);
  return 0xff000000u | (b << 16) | (g << 8) | r;
}

}  // namespace orc

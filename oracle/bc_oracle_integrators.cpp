// Test infrastructure only (see bc_oracle.h): the recursive and the
// photon-mapping integrators of windows_portable/renderer.go (1565-1831),
// restated in fp64 with the reference's evaluation and draw order.
#include "bc_oracle.h"

namespace orc {

// Scene.Bounds (renderer.go:1137-1146): union of the primitive boxes.
AABB scene_bounds(const Scene& s) {
  AABB box = empty_aabb();
  for (const Primitive& p : s.prims) box = expand_box(box, p.box);
  if (std::isinf(box.mn.x) && box.mn.x > 0) return AABB{v3(-1, -1, -1), v3(1, 1, 1)};
  return box;
}

int photon_budget(int level) {  // renderer.go:1148-1161
  switch (level) {
    case 1: return 512;
    case 2: return 2048;
    case 3: return 8192;
    case 4: return 16384;
    default: return 0;
  }
}

double photon_radius(const Scene& s, int level) {  // renderer.go:1163-1182
  AABB box = scene_bounds(s);
  double diag = len(sub(box.mx, box.mn));
  if (diag < 1e-3) diag = 10;
  double base = diag * 0.03;
  switch (level) {
    case 1: return base * 1.8;
    case 2: return base * 1.2;
    case 3: return base * 0.85;
    case 4: return base * 0.6;
    default: return base;
  }
}

// photonCellKey (renderer.go:1636-1639): int64 products wrap, then XOR.
uint64_t photon_cell_key(int64_t x, int64_t y, int64_t z) {
  return ((uint64_t)x * 73856093ull) ^ ((uint64_t)y * 19349663ull) ^ ((uint64_t)z * 83492791ull);
}

static int64_t cell_of(double v, double cell) { return (int64_t)std::floor(v / cell); }

// buildPhotonMap (renderer.go:1642-1728). Emission k draws from its own
// stream; the loop, its stop rule (checked before each emission, so the last
// emission may push the count past the budget) and the grid are the reference's.
PhotonMap build_photon_map(const Scene& s, const Settings& st, uint64_t seed, int64_t* rays) {
  PhotonMap pm;
  const int budget = photon_budget(st.photon_mapping);
  if (budget <= 0 || s.light_spheres.empty()) return pm;
  double radius = photon_radius(s, st.photon_mapping);
  if (radius <= 1e-4) radius = 0.25;
  pm.cell = radius;
  pm.radius = radius;
  pm.photons.reserve(budget);
  const int max_bounces = std::max(2, st.bounces);
  const int attempts = budget * 6;
  int64_t nrays = 0;
  for (int emitted = 0; emitted < attempts && (int)pm.photons.size() < budget; emitted++) {
    Rng rng = make_path_rng(seed, (uint64_t)emitted, kPhotonStream);
    const int li = s.light_spheres[rng.intn((int)s.light_spheres.size())];
    const Primitive& lp = s.prims[li];
    const Material& lm = s.materials[lp.material];
    V3 surf = rand_unit_vector(rng);
    V3 origin = add(lp.center, mul(surf, lp.radius + 2e-4));
    V3 dir = rand_cos_hemisphere(surf, rng);
    V3 flux = mul(lm.emission, (4 * M_PI * lp.radius * lp.radius) / (double)budget);
    Ray ray{origin, dir};
    V3 throughput = flux;
    for (int bounce = 0; bounce < max_bounces; bounce++) {
      nrays++;
      Hit h;
      if (!s.hit(ray, 1e-4, 1e30, &h, nullptr) || h.material < 0 || h.material >= (int)s.materials.size()) break;
      const Material& m = s.materials[h.material];
      V3 p = add(ray.o, mul(ray.d, h.t));
      if (m.kind == MatEmissive) break;
      if (m.kind == MatDiffuse) {
        pm.photons.push_back(Photon{p, h.n, had(throughput, m.color), emitted});
        throughput = had(throughput, m.color);
        ray = Ray{add(p, mul(h.n, 2e-4)), rand_cos_hemisphere(h.n, rng)};
      } else if (m.kind == MatMetal) {
        V3 d = unit(add(reflect(unit(ray.d), h.n), mul(rand_in_unit_sphere(rng), clampd(m.roughness, 0, 1))));
        if (dot(d, h.n) <= 0) break;
        throughput = had(throughput, m.color);
        ray = Ray{add(p, mul(h.n, 2e-4)), d};
      } else {
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
        throughput = had(throughput, m.color);
        ray = Ray{add(p, mul(d, 2e-4)), d};
      }
      if (bounce >= 2) {
        double pr = clampd(maxcomp(throughput), .1, .95);
        if (rng.float64() > pr) break;
        throughput = mul(throughput, 1 / pr);
      }
    }
  }
  for (size_t i = 0; i < pm.photons.size(); i++) {
    const Photon& ph = pm.photons[i];
    uint64_t key = photon_cell_key(cell_of(ph.p.x, pm.cell), cell_of(ph.p.y, pm.cell), cell_of(ph.p.z, pm.cell));
    pm.grid[key].push_back((int)i);
  }
  if (rays) *rays = nrays;
  return pm;
}

// PhotonMap.gather (renderer.go:1730-1761): the 27 cells around p in
// (dz, dy, dx) order, each cell's photons in append order, stopping at
// max_photons accepted photons.
V3 photon_gather(const PhotonMap& pm, V3 p, V3 n, int max_photons) {
  if (pm.photons.empty() || pm.cell <= 0) return v3(0, 0, 0);
  const int64_t cx = cell_of(p.x, pm.cell), cy = cell_of(p.y, pm.cell), cz = cell_of(p.z, pm.cell);
  const double r2 = pm.radius * pm.radius;
  V3 sum = v3(0, 0, 0);
  int count = 0;
  for (int dz = -1; dz <= 1; dz++)
    for (int dy = -1; dy <= 1; dy++)
      for (int dx = -1; dx <= 1; dx++) {
        auto it = pm.grid.find(photon_cell_key(cx + dx, cy + dy, cz + dz));
        if (it == pm.grid.end()) continue;
        for (int idx : it->second) {
          const Photon& ph = pm.photons[idx];
          V3 d = sub(ph.p, p);
          double nd = dot(ph.n, n);
          if (dot(d, d) > r2 || nd <= 0.05) continue;
          sum = add(sum, mul(ph.flux, nd));
          count++;
          if (max_photons > 0 && count >= max_photons)
            return mul(sum, 1 / (M_PI * pm.radius * pm.radius * (double)count));
        }
      }
  if (count == 0) return v3(0, 0, 0);
  return mul(sum, 1 / (M_PI * pm.radius * pm.radius * (double)count));
}

static void set_guide(Guide* guide, V3 p, const Hit& h, const Material& m) {
  guide->p = p;
  guide->n = h.n;
  guide->albedo = material_preview_color(m);
  guide->depth = h.t;
  guide->valid = true;
}

// traceRecursiveInner (renderer.go:1569-1621). At a diffuse vertex the bounce
// direction is drawn, the subtree traced, and only then directLight sampled.
static V3 trace_recursive_inner(const Scene& s, Ray ray, int depth, const Settings& st, Rng& rng, TraceStats* stats,
                                Guide* guide, int bounce) {
  if (depth <= 0) return v3(0, 0, 0);
  if (stats) stats->segments++;
  Hit h;
  if (!s.hit(ray, 1e-4, 1e30, &h, stats ? &stats->c : nullptr)) return background(ray.d);
  if (h.material < 0 || h.material >= (int)s.materials.size()) return v3(0, 0, 0);
  const Material& m = s.materials[h.material];
  V3 p = add(ray.o, mul(ray.d, h.t));
  if (bounce == 0 && guide) set_guide(guide, p, h, m);
  if (m.kind == MatEmissive) return m.emission;
  if (m.kind == MatDiffuse) {
    V3 d = rand_cos_hemisphere(h.n, rng);
    V3 bc = trace_recursive_inner(s, Ray{add(p, mul(h.n, 2e-4)), d}, depth - 1, st, rng, stats, nullptr, bounce + 1);
    V3 dl = direct_light(s, h, p, m, rng, st, stats);
    V3 result = add(dl, had(m.color, bc));
    if (depth < 8) {
      double pr = clampd(maxcomp(m.color), .1, .95);
      return mul(result, 1 / pr);
    }
    return result;
  }
  if (m.kind == MatMetal) {
    V3 d = unit(add(reflect(unit(ray.d), h.n), mul(rand_in_unit_sphere(rng), clampd(m.roughness, 0, 1))));
    if (dot(d, h.n) <= 0) return v3(0, 0, 0);
    return had(m.color, trace_recursive_inner(s, Ray{add(p, mul(h.n, 2e-4)), d}, depth - 1, st, rng, stats, nullptr,
                                              bounce + 1));
  }
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
  return had(m.color,
             trace_recursive_inner(s, Ray{add(p, mul(d, 2e-4)), d}, depth - 1, st, rng, stats, nullptr, bounce + 1));
}

V3 trace_recursive(const Scene& s, Ray ray, const Settings& st, Rng& rng, TraceStats* stats, Guide* guide) {
  return trace_recursive_inner(s, ray, st.bounces, st, rng, stats, guide, 0);  // renderer.go:1565-1567
}

// tracePhotonMapped (renderer.go:1763-1831): the path loop with a photon
// gather at diffuse vertices and emitters counted without an MIS weight.
V3 trace_photon(const Scene& s, Ray ray, const Settings& st, Rng& rng, TraceStats* stats, Guide* guide,
                const PhotonMap& pm) {
  V3 throughput = v3(1, 1, 1);
  V3 radiance = v3(0, 0, 0);
  for (int bounce = 0; bounce < st.bounces; bounce++) {
    if (stats) stats->segments++;
    Hit h;
    if (!s.hit(ray, 1e-4, 1e30, &h, stats ? &stats->c : nullptr)) return add(radiance, had(throughput, background(ray.d)));
    if (h.material < 0 || h.material >= (int)s.materials.size()) return radiance;
    const Material& m = s.materials[h.material];
    V3 p = add(ray.o, mul(ray.d, h.t));
    if (bounce == 0 && guide) set_guide(guide, p, h, m);
    if (m.kind == MatEmissive) return add(radiance, had(throughput, m.emission));
    if (m.kind == MatDiffuse) {
      V3 phot = photon_gather(pm, p, h.n, 64);
      V3 dl = direct_light(s, h, p, m, rng, st, stats);
      radiance = add(radiance, had(throughput, add(dl, phot)));
      throughput = had(throughput, m.color);
      ray = Ray{add(p, mul(h.n, 2e-4)), rand_cos_hemisphere(h.n, rng)};
    } else if (m.kind == MatMetal) {
      V3 d = unit(add(reflect(unit(ray.d), h.n), mul(rand_in_unit_sphere(rng), clampd(m.roughness, 0, 1))));
      if (dot(d, h.n) <= 0) return radiance;
      throughput = had(throughput, m.color);
      ray = Ray{add(p, mul(h.n, 2e-4)), d};
    } else {
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

V3 pixel_radiance(const Scene& s, Ray ray, const Settings& st, Rng& rng, TraceStats* stats, Guide* guide,
                  const PhotonMap* pm) {
  if (st.integrator == IntegratorRecursive) return trace_recursive(s, ray, st, rng, stats, guide);
  if (st.integrator == IntegratorPhoton && pm) return trace_photon(s, ray, st, rng, stats, guide, *pm);
  return trace(s, ray, st, rng, stats, guide);
}

}  // namespace orc

// Test infrastructure only (see bc_oracle.h): scene, BVH and traversal
// restated from windows_portable/renderer.go in fp64.
#include "bc_oracle.h"

#include <algorithm>
#include <cmath>
#include <functional>
#include <limits>

namespace orc {

double len(V3 a) { return std::sqrt(dot(a, a)); }

// renderer.go:32-38
V3 unit(V3 a) {
  double l = len(a);
  if (l < 1e-12) return v3(0, 0, 0);
  return mul(a, 1 / l);
}

// renderer.go:59-81
RayAccel prepare_ray(const Ray& r) {
  RayAccel a;
  a.ray = r;
  a.dirLen2 = dot(r.d, r.d);
  if (a.dirLen2 > 1e-18) a.invDirLen2 = 1 / a.dirLen2;
  if (std::fabs(r.d.x) < 1e-15) a.zx = true; else a.inv.x = 1 / r.d.x;
  if (std::fabs(r.d.y) < 1e-15) a.zy = true; else a.inv.y = 1 / r.d.y;
  if (std::fabs(r.d.z) < 1e-15) a.zz = true; else a.inv.z = 1 / r.d.z;
  return a;
}

// renderer.go:122-139
AABB empty_aabb() {
  double inf = std::numeric_limits<double>::infinity();
  return AABB{v3(inf, inf, inf), v3(-inf, -inf, -inf)};
}
AABB expand_point(AABB b, V3 p) {
  b.mn.x = gmin(b.mn.x, p.x);
  b.mn.y = gmin(b.mn.y, p.y);
  b.mn.z = gmin(b.mn.z, p.z);
  b.mx.x = gmax(b.mx.x, p.x);
  b.mx.y = gmax(b.mx.y, p.y);
  b.mx.z = gmax(b.mx.z, p.z);
  return b;
}
AABB expand_box(AABB b, const AABB& c) {
  b = expand_point(b, c.mn);
  b = expand_point(b, c.mx);
  return b;
}
double surface_area(const AABB& b) {
  V3 e = sub(b.mx, b.mn);
  if (e.x < 0 || e.y < 0 || e.z < 0) return 0;
  return 2 * (e.x * e.y + e.y * e.z + e.z * e.x);
}

// One slab of AABB.HitAccel (renderer.go:147-210).
static inline bool slab(bool zero, double o, double inv, double mn, double mx, double* near, double* tmax) {
  if (zero) return !(o < mn || o > mx);
  double t0 = (mn - o) * inv;
  double t1 = (mx - o) * inv;
  if (inv < 0) std::swap(t0, t1);
  if (t0 > *near) *near = t0;
  if (t1 < *tmax) *tmax = t1;
  return !(*tmax <= *near);
}

bool aabb_hit(const AABB& b, const RayAccel& r, double tmin, double tmax, double* near_out) {
  double near = tmin;
  if (!slab(r.zx, r.ray.o.x, r.inv.x, b.mn.x, b.mx.x, &near, &tmax)) return false;
  if (!slab(r.zy, r.ray.o.y, r.inv.y, b.mn.y, b.mx.y, &near, &tmax)) return false;
  if (!slab(r.zz, r.ray.o.z, r.inv.z, b.mn.z, b.mx.z, &near, &tmax)) return false;
  if (near_out) *near_out = near;
  return true;
}

int Scene::add_material(const Material& m) {
  materials.push_back(m);
  return (int)materials.size() - 1;
}

// renderer.go:246-256
void Scene::add_sphere(V3 c, double r, int mat) {
  if (r <= 0) return;
  V3 rv = v3(r, r, r);
  Primitive p;
  p.kind = PrimSphere;
  p.material = mat;
  p.center = c;
  p.radius = r;
  p.centroid = c;
  p.box = AABB{sub(c, rv), add(c, rv)};
  prims.push_back(p);
  if (mat >= 0 && mat < (int)materials.size() && materials[mat].kind == MatEmissive)
    light_spheres.push_back((int)prims.size() - 1);
}

// renderer.go:257-269
void Scene::add_triangle(V3 a, V3 b, V3 c, int mat) {
  V3 e1 = sub(b, a), e2 = sub(c, a);
  V3 n = cross(e1, e2);
  if (dot(n, n) < 1e-18) return;
  AABB box = expand_point(expand_point(expand_point(empty_aabb(), a), b), c);
  double eps = 1e-6;
  box.mn = sub(box.mn, v3(eps, eps, eps));
  box.mx = add(box.mx, v3(eps, eps, eps));
  Primitive p;
  p.kind = PrimTriangle;
  p.material = mat;
  p.a = a; p.b = b; p.c = c;
  p.e1 = e1; p.e2 = e2;
  p.normal = unit(n);
  p.box = box;
  p.centroid = mul(add(add(a, b), c), 1.0 / 3.0);
  prims.push_back(p);
}

static double light_weight(const Scene& s, int pi) {  // renderer.go:1342-1356
  if (pi < 0 || pi >= (int)s.prims.size()) return 0;
  const Primitive& p = s.prims[pi];
  if (p.kind != PrimSphere || p.material < 0 || p.material >= (int)s.materials.size()) return 0;
  const Material& m = s.materials[p.material];
  if (m.kind != MatEmissive) return 0;
  double area = 4 * M_PI * p.radius * p.radius;
  return gmax(1e-9, luminance(m.emission) * area);
}

// renderer.go:363-407
void Scene::rebuild_light_distribution() {
  light_cdf.assign(light_spheres.size(), 0.0);
  light_pdf_by_prim.assign(prims.size(), 0.0);
  double total = 0;
  for (size_t i = 0; i < light_spheres.size(); i++) {
    total += light_weight(*this, light_spheres[i]);
    light_cdf[i] = total;
  }
  if (total <= 0) {
    if (light_spheres.empty()) return;
    double pdf = 1 / (double)light_spheres.size();
    for (size_t i = 0; i < light_spheres.size(); i++) {
      light_cdf[i] = (double)(i + 1) / (double)light_spheres.size();
      int pi = light_spheres[i];
      if (pi >= 0 && pi < (int)light_pdf_by_prim.size()) light_pdf_by_prim[pi] = pdf;
    }
    return;
  }
  double prev = 0;
  for (size_t i = 0; i < light_spheres.size(); i++) {
    double cdf = light_cdf[i] / total;
    light_cdf[i] = cdf;
    double pdf = cdf - prev;
    prev = cdf;
    int pi = light_spheres[i];
    if (pi >= 0 && pi < (int)light_pdf_by_prim.size()) light_pdf_by_prim[pi] = pdf;
  }
  if (!light_cdf.empty()) light_cdf.back() = 1;
}

static bool iequals(const std::string& a, const char* b) {
  std::string x = a, y = b;
  if (x.size() != y.size()) return false;
  for (size_t i = 0; i < x.size(); i++)
    if (std::tolower((unsigned char)x[i]) != std::tolower((unsigned char)y[i])) return false;
  return true;
}

// renderer.go:409-449
void Scene::build() {
  topo_rev++;
  geom_rev++;
  rebuild_light_distribution();
  if (bvh_mode.empty()) bvh_mode = "SAH";
  if (bvh_bins < 4) bvh_bins = 16;
  if (bvh_bins > 32) bvh_bins = 32;
  if (bvh_leaf < 1) bvh_leaf = 4;
  if (bvh_leaf > 16) bvh_leaf = 16;
  nodes.clear();
  nodes.reserve(prims.size() * 2);
  order.resize(prims.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
  if (!order.empty()) {
    if (iequals(bvh_mode, "median")) build_median(0, (int)order.size());
    else build_sah(0, (int)order.size());
  }
}

// renderer.go:451-473
void Scene::refit() {
  geom_rev++;
  if (nodes.empty()) { build(); return; }
  for (int ni = (int)nodes.size() - 1; ni >= 0; ni--) {
    Node& n = nodes[ni];
    if (n.count > 0) {
      AABB box = empty_aabb();
      for (int i = 0; i < n.count; i++) {
        int pi = order[n.start + i];
        if (pi >= 0 && pi < (int)prims.size()) box = expand_box(box, prims[pi].box);
      }
      n.box = box;
    } else if (n.left >= 0 && n.right >= 0) {
      n.box = expand_box(nodes[n.left].box, nodes[n.right].box);
    }
  }
  rebuild_light_distribution();
}

static inline double caxis(V3 v, int axis) { return axis == 0 ? v.x : (axis == 1 ? v.y : v.z); }
static inline int largest_axis(V3 e) {  // renderer.go:485-493
  if (e.y > e.x && e.y >= e.z) return 1;
  if (e.z > e.x && e.z > e.y) return 2;
  return 0;
}

void Scene::node_bounds(int start, int end, AABB* box, AABB* cb) const {  // renderer.go:495-504
  AABB b = empty_aabb(), c = empty_aabb();
  for (int i = start; i < end; i++) {
    const Primitive& p = prims[order[i]];
    b = expand_box(b, p.box);
    c = expand_point(c, p.centroid);
  }
  *box = b;
  *cb = c;
}

// renderer.go:506-524 (sort.Slice is unstable in Go; only hit distances of
// the resulting tree are pinned by the reference tests).
int Scene::build_median(int start, int end) {
  int idx = (int)nodes.size();
  nodes.push_back(Node{});
  AABB box, cb;
  node_bounds(start, end, &box, &cb);
  int count = end - start;
  if (count <= bvh_leaf) {
    Node n; n.box = box; n.start = start; n.count = count;
    nodes[idx] = n;
    return idx;
  }
  int axis = largest_axis(sub(cb.mx, cb.mn));
  std::stable_sort(order.begin() + start, order.begin() + end, [&](int a, int b) {
    return caxis(prims[a].centroid, axis) < caxis(prims[b].centroid, axis);
  });
  int mid = (start + end) / 2;
  int l = build_median(start, mid);
  int r = build_median(mid, end);
  Node n; n.box = box; n.left = l; n.right = r;
  nodes[idx] = n;
  return idx;
}

// renderer.go:526-633
int Scene::build_sah(int start, int end) {
  int idx = (int)nodes.size();
  nodes.push_back(Node{});
  AABB box, cb;
  node_bounds(start, end, &box, &cb);
  int count = end - start;
  auto make_leaf = [&]() {
    Node n; n.box = box; n.start = start; n.count = count;
    nodes[idx] = n;
    return idx;
  };
  if (count <= bvh_leaf) return make_leaf();
  V3 ext = sub(cb.mx, cb.mn);
  int axis = largest_axis(ext);
  double axisExtent = caxis(cb.mx, axis) - caxis(cb.mn, axis);
  if (axisExtent < 1e-12) return make_leaf();
  int binsN = bvh_bins;
  AABB bbox[32];
  int bcount[32];
  for (int i = 0; i < binsN; i++) { bbox[i] = empty_aabb(); bcount[i] = 0; }
  double minC = caxis(cb.mn, axis);
  double invExtent = 1 / axisExtent;
  auto bin_of = [&](const Primitive& p) {
    int b = (int)((caxis(p.centroid, axis) - minC) * invExtent * (double)binsN);
    if (b < 0) b = 0;
    if (b >= binsN) b = binsN - 1;
    return b;
  };
  for (int i = start; i < end; i++) {
    const Primitive& p = prims[order[i]];
    int b = bin_of(p);
    bcount[b]++;
    bbox[b] = expand_box(bbox[b], p.box);
  }
  int leftCount[31], rightCount[31];
  double leftArea[31], rightArea[31];
  AABB acc = empty_aabb();
  int accN = 0;
  for (int i = 0; i < binsN - 1; i++) {
    if (bcount[i] > 0) acc = expand_box(acc, bbox[i]);
    accN += bcount[i];
    leftCount[i] = accN;
    leftArea[i] = surface_area(acc);
  }
  acc = empty_aabb();
  accN = 0;
  for (int i = binsN - 1; i > 0; i--) {
    if (bcount[i] > 0) acc = expand_box(acc, bbox[i]);
    accN += bcount[i];
    rightCount[i - 1] = accN;
    rightArea[i - 1] = surface_area(acc);
  }
  int bestSplit = -1;
  double bestCost = std::numeric_limits<double>::infinity();
  for (int i = 0; i < binsN - 1; i++) {
    if (leftCount[i] == 0 || rightCount[i] == 0) continue;
    double cost = leftArea[i] * (double)leftCount[i] + rightArea[i] * (double)rightCount[i];
    if (cost < bestCost) { bestCost = cost; bestSplit = i; }
  }
  double leafCost = surface_area(box) * (double)count;
  if (bestSplit < 0 || (count <= bvh_leaf * 2 && bestCost >= leafCost * 0.98)) return make_leaf();
  int i = start, j = end - 1;
  while (i <= j) {
    int b = bin_of(prims[order[i]]);
    if (b <= bestSplit) {
      i++;
    } else {
      std::swap(order[i], order[j]);
      j--;
    }
  }
  int mid = i;
  if (mid <= start || mid >= end) {  // unreachable when the two binning passes agree
    std::stable_sort(order.begin() + start, order.begin() + end, [&](int a, int b) {
      return caxis(prims[a].centroid, axis) < caxis(prims[b].centroid, axis);
    });
    mid = (start + end) / 2;
  }
  int l = build_sah(start, mid);
  int r = build_sah(mid, end);
  Node n; n.box = box; n.left = l; n.right = r;
  nodes[idx] = n;
  return idx;
}

// renderer.go:650-678
static bool sphere_hit(const Primitive& p, const RayAccel& ar, double tmin, double tmax, Hit* h) {
  if (ar.invDirLen2 <= 0) return false;
  const Ray& r = ar.ray;
  V3 oc = sub(r.o, p.center);
  double hb = dot(oc, r.d);
  double c = dot(oc, oc) - p.radius * p.radius;
  double disc = hb * hb - ar.dirLen2 * c;
  if (disc < 0) return false;
  double sq = std::sqrt(disc);
  double root = (-hb - sq) * ar.invDirLen2;
  if (root < tmin || root > tmax) {
    root = (-hb + sq) * ar.invDirLen2;
    if (root < tmin || root > tmax) return false;
  }
  V3 pos = add(r.o, mul(r.d, root));
  V3 outward = mul(sub(pos, p.center), 1 / p.radius);
  bool front = dot(r.d, outward) < 0;
  V3 n = front ? outward : mul(outward, -1);
  h->t = root; h->n = n; h->material = p.material; h->primitive = -1; h->front = front;
  return true;
}

// renderer.go:684-711
static bool tri_hit(const Primitive& p, const Ray& r, double tmin, double tmax, Hit* out) {
  V3 h = cross(r.d, p.e2);
  double det = dot(p.e1, h);
  if (std::fabs(det) < 1e-10) return false;
  double f = 1 / det;
  V3 ss = sub(r.o, p.a);
  double u = f * dot(ss, h);
  if (u < 0 || u > 1) return false;
  V3 q = cross(ss, p.e1);
  double v = f * dot(r.d, q);
  if (v < 0 || u + v > 1) return false;
  double t = f * dot(p.e2, q);
  if (t < tmin || t > tmax) return false;
  V3 n = p.normal;
  bool front = dot(r.d, n) < 0;
  if (!front) n = mul(n, -1);
  out->t = t; out->n = n; out->material = p.material; out->primitive = -1; out->front = front;
  return true;
}

bool prim_hit(const Primitive& p, const RayAccel& ar, double tmin, double tmax, Hit* h) {
  if (p.kind == PrimSphere) return sphere_hit(p, ar, tmin, tmax, h);
  return tri_hit(p, ar.ray, tmin, tmax, h);
}

// renderer.go:724-770
bool prim_any_hit(const Primitive& p, const RayAccel& ar, double tmin, double tmax) {
  if (p.kind == PrimSphere) {
    if (ar.invDirLen2 <= 0) return false;
    V3 oc = sub(ar.ray.o, p.center);
    double hb = dot(oc, ar.ray.d);
    double c = dot(oc, oc) - p.radius * p.radius;
    double disc = hb * hb - ar.dirLen2 * c;
    if (disc < 0) return false;
    double sq = std::sqrt(disc);
    double root = (-hb - sq) * ar.invDirLen2;
    if (root >= tmin && root <= tmax) return true;
    root = (-hb + sq) * ar.invDirLen2;
    return root >= tmin && root <= tmax;
  }
  const Ray& r = ar.ray;
  V3 h = cross(r.d, p.e2);
  double det = dot(p.e1, h);
  if (det > -1e-10 && det < 1e-10) return false;
  double f = 1 / det;
  V3 ss = sub(r.o, p.a);
  double u = f * dot(ss, h);
  if (u < 0 || u > 1) return false;
  V3 q = cross(ss, p.e1);
  double v = f * dot(r.d, q);
  if (v < 0 || u + v > 1) return false;
  double t = f * dot(p.e2, q);
  return t >= tmin && t <= tmax;
}

static inline void count_prim(const Primitive& p, Counters* c) {
  if (!c) return;
  if (p.kind == PrimSphere) c->spheres++; else c->tris++;
}

// renderer.go:777-849
bool Scene::hit(const Ray& r, double tmin, double tmax, Hit* out, Counters* c) const {
  if (nodes.empty()) return false;
  RayAccel ar = prepare_ray(r);
  double rootNear;
  if (c) c->boxes++;
  if (!aabb_hit(nodes[0].box, ar, tmin, tmax, &rootNear)) return false;
  struct Entry { int node; double near; };
  Entry stack[16];
  int sp = 1;
  stack[0] = Entry{0, rootNear};
  double closest = tmax;
  Hit best;
  bool found = false;
  while (sp > 0) {
    sp--;
    Entry e = stack[sp];
    if (e.near >= closest) continue;
    const Node& n = nodes[e.node];
    if (n.count > 0) {
      for (int i = 0; i < n.count; i++) {
        int pi = order[n.start + i];
        Hit h;
        count_prim(prims[pi], c);
        if (prim_hit(prims[pi], ar, tmin, closest, &h)) {
          h.primitive = pi;
          closest = h.t; best = h; found = true;
        }
      }
      continue;
    }
    double ln = 0, rn = 0;
    if (c) c->boxes += 2;
    bool lok = aabb_hit(nodes[n.left].box, ar, tmin, closest, &ln);
    bool rok = aabb_hit(nodes[n.right].box, ar, tmin, closest, &rn);
    if (!lok && !rok) continue;
    if (sp + 2 > 16) {
      Hit h;
      if (lok && hit_recursive(n.left, ar, tmin, closest, &h, c)) { closest = h.t; best = h; found = true; }
      if (rok && hit_recursive(n.right, ar, tmin, closest, &h, c)) { closest = h.t; best = h; found = true; }
      continue;
    }
    if (lok && rok) {
      if (ln <= rn) {
        stack[sp++] = Entry{n.right, rn};
        stack[sp++] = Entry{n.left, ln};
      } else {
        stack[sp++] = Entry{n.left, ln};
        stack[sp++] = Entry{n.right, rn};
      }
    } else if (lok) {
      stack[sp++] = Entry{n.left, ln};
    } else {
      stack[sp++] = Entry{n.right, rn};
    }
  }
  if (found) *out = best;
  return found;
}

// renderer.go:914-939
bool Scene::hit_recursive(int ni, const RayAccel& ar, double tmin, double tmax, Hit* out, Counters* c) const {
  const Node& n = nodes[ni];
  if (c) c->boxes++;
  if (!aabb_hit(n.box, ar, tmin, tmax, nullptr)) return false;
  double closest = tmax;
  Hit best;
  bool found = false;
  if (n.count > 0) {
    for (int i = 0; i < n.count; i++) {
      int pi = order[n.start + i];
      Hit h;
      count_prim(prims[pi], c);
      if (prim_hit(prims[pi], ar, tmin, closest, &h)) {
        h.primitive = pi;
        closest = h.t; best = h; found = true;
      }
    }
    if (found) *out = best;
    return found;
  }
  Hit h;
  if (hit_recursive(n.left, ar, tmin, closest, &h, c)) { closest = h.t; best = h; found = true; }
  if (hit_recursive(n.right, ar, tmin, closest, &h, c)) { best = h; found = true; }
  if (found) *out = best;
  return found;
}

// renderer.go:851-895
bool Scene::occluded(const Ray& r, double tmin, double tmax, Counters* c) const {
  if (nodes.empty()) return false;
  RayAccel ar = prepare_ray(r);
  if (c) c->boxes++;
  if (!aabb_hit(nodes[0].box, ar, tmin, tmax, nullptr)) return false;
  int stack[16];
  stack[0] = 0;
  int sp = 1;
  while (sp > 0) {
    sp--;
    const Node& n = nodes[stack[sp]];
    if (n.count > 0) {
      for (int i = 0; i < n.count; i++) {
        int pi = order[n.start + i];
        count_prim(prims[pi], c);
        if (prim_any_hit(prims[pi], ar, tmin, tmax)) return true;
      }
      continue;
    }
    if (c) c->boxes += 2;
    bool lok = aabb_hit(nodes[n.left].box, ar, tmin, tmax, nullptr);
    bool rok = aabb_hit(nodes[n.right].box, ar, tmin, tmax, nullptr);
    if (sp + 2 > 16) {
      if (lok && occluded_recursive(n.left, ar, tmin, tmax, c)) return true;
      if (rok && occluded_recursive(n.right, ar, tmin, tmax, c)) return true;
      continue;
    }
    if (lok) stack[sp++] = n.left;
    if (rok) stack[sp++] = n.right;
  }
  return false;
}

// renderer.go:897-912
bool Scene::occluded_recursive(int ni, const RayAccel& ar, double tmin, double tmax, Counters* c) const {
  const Node& n = nodes[ni];
  if (c) c->boxes++;
  if (!aabb_hit(n.box, ar, tmin, tmax, nullptr)) return false;
  if (n.count > 0) {
    for (int i = 0; i < n.count; i++) {
      int pi = order[n.start + i];
      count_prim(prims[pi], c);
      if (prim_any_hit(prims[pi], ar, tmin, tmax)) return true;
    }
    return false;
  }
  return occluded_recursive(n.left, ar, tmin, tmax, c) || occluded_recursive(n.right, ar, tmin, tmax, c);
}

// renderer_test.go:797-830: stackless traversal over the escape table.
bool Scene::hit_threaded(const Ray& r, double tmin, double tmax, const std::vector<int32_t>& esc, Hit* out) const {
  if (nodes.empty()) return false;
  RayAccel ar = prepare_ray(r);
  double bestT = tmax;
  Hit best;
  bool found = false;
  for (int ni = 0; ni >= 0 && ni < (int)nodes.size();) {
    const Node& n = nodes[ni];
    if (!aabb_hit(n.box, ar, tmin, bestT, nullptr)) { ni = esc[ni]; continue; }
    if (n.count > 0) {
      for (int j = 0; j < n.count; j++) {
        int pi = order[n.start + j];
        Hit h;
        if (prim_hit(prims[pi], ar, tmin, bestT, &h)) {
          h.primitive = pi;
          best = h; bestT = h.t; found = true;
        }
      }
      ni = esc[ni];
    } else {
      ni = n.left;
    }
  }
  if (found) *out = best;
  return found;
}

// renderer.go:3251-3276
std::vector<int32_t> threaded_escapes(const std::vector<Node>& nodes) {
  std::vector<int32_t> esc(nodes.size(), -1);
  if (nodes.empty()) return esc;
  std::function<void(int, int32_t)> assign = [&](int idx, int32_t next) {
    if (idx < 0 || idx >= (int)nodes.size()) return;
    esc[idx] = next;
    const Node& n = nodes[idx];
    if (n.count > 0) return;
    if (n.left >= 0 && n.right >= 0) {
      assign(n.left, (int32_t)n.right);
      assign(n.right, next);
    }
  };
  assign(0, -1);
  return esc;
}

// renderer.go:947-960
void camera_basis(const Camera& c, double aspect, V3* origin, V3* lower, V3* horiz, V3* vert) {
  double theta = c.fov * M_PI / 180;
  double h = std::tan(theta / 2);
  double vh = 2 * h;
  double vw = aspect * vh;
  V3 w = unit(sub(c.position, c.target));
  V3 u = unit(cross(c.up, w));
  V3 v = cross(w, u);
  *origin = c.position;
  *horiz = mul(u, vw);
  *vert = mul(v, vh);
  *lower = sub(sub(sub(*origin, mul(*horiz, .5)), mul(*vert, .5)), w);
}

}  // namespace orc

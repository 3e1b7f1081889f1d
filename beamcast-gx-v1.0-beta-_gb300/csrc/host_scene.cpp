// Host-side scene builder: the fp64 scene model and binned-SAH / median BVH
// of the portable Go renderer (renderer.go:242-633), for callers that do not
// run the Go renderer. The tree, its node numbering (pre-order, left subtree
// first) and the Order permutation are identical to Scene.Build's.
//
// Storage is structure-of-arrays; the builder is iterative with an explicit
// task stack and keeps each primitive's bin next to its Order entry, so the
// partition pass reuses the bins of the binning pass instead of recomputing
// them (the reference computes the same expression twice, renderer.go:555, 608).
//
// Compiled with -ffp-contract=off: every fp64 product and sum rounds on its
// own, like the reference's Go code on amd64.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "../../include/bc_host_scene.h"

namespace {

struct Box {
  double mn[3], mx[3];
};

inline double go_min(double a, double b) {  // math.Min incl. signed zeros
  if (a < b) return a;
  if (b < a) return b;
  if (a == 0 && b == 0) return std::signbit(a) ? a : b;
  return a;
}
inline double go_max(double a, double b) {  // math.Max incl. signed zeros
  if (a > b) return a;
  if (b > a) return b;
  if (a == 0 && b == 0) return std::signbit(a) ? b : a;
  return a;
}
inline Box empty_box() {
  const double inf = std::numeric_limits<double>::infinity();
  return Box{{inf, inf, inf}, {-inf, -inf, -inf}};
}
inline void grow_point(Box& b, const double* p) {
  for (int k = 0; k < 3; k++) {
    b.mn[k] = go_min(b.mn[k], p[k]);
    b.mx[k] = go_max(b.mx[k], p[k]);
  }
}
inline void grow_box(Box& b, const Box& c) {
  grow_point(b, c.mn);
  grow_point(b, c.mx);
}
inline double area(const Box& b) {  // AABB.SurfaceArea, renderer.go:133-139
  double ex = b.mx[0] - b.mn[0], ey = b.mx[1] - b.mn[1], ez = b.mx[2] - b.mn[2];
  if (ex < 0 || ey < 0 || ez < 0) return 0;
  return 2 * (ex * ey + ey * ez + ez * ex);
}
inline double lum(const double* c) { return 0.2126 * c[0] + 0.7152 * c[1] + 0.0722 * c[2]; }

}  // namespace

struct bc_hscene {
  // materials
  std::vector<int32_t> mkind;
  std::vector<double> mcolor, mrough, mior, memission;
  // primitives (SoA)
  std::vector<int32_t> kind, mat;
  std::vector<double> center, radius, A, B, C, E1, E2, N, cent;
  std::vector<Box> pbox;
  // BVH (SoA)
  std::vector<double> nbox;  // 6 per node
  std::vector<int32_t> left, right, start, count;
  std::vector<int32_t> order;
  // lights
  std::vector<int32_t> lights;
  std::vector<double> lcdf, lpdf;
  std::string mode = "SAH";
  int32_t bins = 16, leaf = 4;
  uint64_t topo = 0, geom = 0;

  int32_t nprims() const { return (int32_t)kind.size(); }
  void push_prim(int32_t k, int32_t m) {
    kind.push_back(k);
    mat.push_back(m);
    for (auto* v : {&center, &A, &B, &C, &E1, &E2, &N, &cent}) v->insert(v->end(), 3, 0.0);
    radius.push_back(0);
    pbox.push_back(Box{});
  }
  void set_tri_geometry(int32_t i, const double* a, const double* b, const double* c);
  void rebuild_lights();
  void build_tree();
  int32_t new_node() {
    int32_t idx = (int32_t)left.size();
    nbox.insert(nbox.end(), 6, 0.0);
    left.push_back(-1);
    right.push_back(-1);
    start.push_back(0);
    count.push_back(0);
    return idx;
  }
  void set_node_box(int32_t idx, const Box& b) {
    std::memcpy(&nbox[6 * (size_t)idx], b.mn, 3 * sizeof(double));
    std::memcpy(&nbox[6 * (size_t)idx + 3], b.mx, 3 * sizeof(double));
  }
};

// Triangle derived fields (renderer.go:258-268 and 318-329).
void bc_hscene::set_tri_geometry(int32_t i, const double* a, const double* b, const double* c) {
  double* e1 = &E1[3 * (size_t)i];
  double* e2 = &E2[3 * (size_t)i];
  for (int k = 0; k < 3; k++) {
    A[3 * (size_t)i + k] = a[k];
    B[3 * (size_t)i + k] = b[k];
    C[3 * (size_t)i + k] = c[k];
    e1[k] = b[k] - a[k];
    e2[k] = c[k] - a[k];
  }
  double nx = e1[1] * e2[2] - e1[2] * e2[1];
  double ny = e1[2] * e2[0] - e1[0] * e2[2];
  double nz = e1[0] * e2[1] - e1[1] * e2[0];
  double l = std::sqrt(nx * nx + ny * ny + nz * nz);
  double* n = &N[3 * (size_t)i];
  if (l < 1e-12) {
    n[0] = n[1] = n[2] = 0;
  } else {
    double s = 1 / l;
    n[0] = nx * s; n[1] = ny * s; n[2] = nz * s;
  }
  Box bx = empty_box();
  grow_point(bx, a);
  grow_point(bx, b);
  grow_point(bx, c);
  const double eps = 1e-6;
  for (int k = 0; k < 3; k++) {
    bx.mn[k] = bx.mn[k] - eps;
    bx.mx[k] = bx.mx[k] + eps;
  }
  pbox[i] = bx;
  for (int k = 0; k < 3; k++) cent[3 * (size_t)i + k] = ((a[k] + b[k]) + c[k]) * (1.0 / 3.0);
}

// Scene.rebuildLightDistribution (renderer.go:363-407) with lightWeight (1342-1356).
void bc_hscene::rebuild_lights() {
  const size_t nl = lights.size();
  lcdf.assign(nl, 0.0);
  lpdf.assign((size_t)nprims(), 0.0);
  double total = 0;
  for (size_t i = 0; i < nl; i++) {
    int32_t pi = lights[i];
    double w = 0;
    if (pi >= 0 && pi < nprims() && kind[pi] == BC_PRIM_SPHERE && mat[pi] >= 0 && mat[pi] < (int32_t)mkind.size() &&
        mkind[mat[pi]] == BC_MAT_EMISSIVE) {
      double r = radius[pi];
      double ar = 4 * M_PI * r * r;
      w = go_max(1e-9, lum(&memission[3 * (size_t)mat[pi]]) * ar);
    }
    total += w;
    lcdf[i] = total;
  }
  if (total <= 0) {
    if (nl == 0) return;
    double pdf = 1 / (double)nl;
    for (size_t i = 0; i < nl; i++) {
      lcdf[i] = (double)(i + 1) / (double)nl;
      if (lights[i] >= 0 && lights[i] < nprims()) lpdf[lights[i]] = pdf;
    }
    return;
  }
  double prev = 0;
  for (size_t i = 0; i < nl; i++) {
    double cdf = lcdf[i] / total;
    lcdf[i] = cdf;
    if (lights[i] >= 0 && lights[i] < nprims()) lpdf[lights[i]] = cdf - prev;
    prev = cdf;
  }
  lcdf[nl - 1] = 1;
}

// buildNodeSAH / buildNodeMedian (renderer.go:506-633), iteratively.
void bc_hscene::build_tree() {
  const int32_t n = nprims();
  left.clear(); right.clear(); start.clear(); count.clear(); nbox.clear();
  left.reserve(2 * (size_t)n); right.reserve(2 * (size_t)n); start.reserve(2 * (size_t)n);
  count.reserve(2 * (size_t)n); nbox.reserve(12 * (size_t)n);
  order.resize(n);
  for (int32_t i = 0; i < n; i++) order[i] = i;
  if (n == 0) return;
  std::string lower = mode;
  for (auto& ch : lower) ch = (char)std::tolower((unsigned char)ch);
  const bool median = lower == "median";
  std::vector<uint8_t> bin(n);

  struct Task { int32_t s, e, parent; bool is_right; };
  std::vector<Task> stack;
  stack.push_back(Task{0, n, -1, false});
  while (!stack.empty()) {
    Task t = stack.back();
    stack.pop_back();
    const int32_t idx = new_node();
    if (t.parent >= 0) (t.is_right ? right : left)[t.parent] = idx;
    Box box = empty_box(), cb = empty_box();
    for (int32_t i = t.s; i < t.e; i++) {
      int32_t p = order[i];
      grow_box(box, pbox[p]);
      grow_point(cb, &cent[3 * (size_t)p]);
    }
    set_node_box(idx, box);
    const int32_t cnt = t.e - t.s;
    auto leafify = [&]() { start[idx] = t.s; count[idx] = cnt; };
    if (cnt <= leaf) { leafify(); continue; }
    double ext[3] = {cb.mx[0] - cb.mn[0], cb.mx[1] - cb.mn[1], cb.mx[2] - cb.mn[2]};
    int axis = 0;  // largestAxis, renderer.go:485-493
    if (ext[1] > ext[0] && ext[1] >= ext[2]) axis = 1;
    else if (ext[2] > ext[0] && ext[2] > ext[1]) axis = 2;
    int32_t mid;
    if (median) {
      std::stable_sort(order.begin() + t.s, order.begin() + t.e, [&](int32_t a, int32_t b) {
        return cent[3 * (size_t)a + axis] < cent[3 * (size_t)b + axis];
      });
      mid = (t.s + t.e) / 2;
    } else {
      const double axisExtent = cb.mx[axis] - cb.mn[axis];
      if (axisExtent < 1e-12) { leafify(); continue; }
      const int nb = bins;
      const double minC = cb.mn[axis];
      const double invExtent = 1 / axisExtent;
      Box bb[32];
      int32_t bn[32];
      for (int i = 0; i < nb; i++) { bb[i] = empty_box(); bn[i] = 0; }
      for (int32_t i = t.s; i < t.e; i++) {
        int32_t p = order[i];
        int b = (int)((cent[3 * (size_t)p + axis] - minC) * invExtent * (double)nb);
        b = b < 0 ? 0 : (b >= nb ? nb - 1 : b);
        bin[i] = (uint8_t)b;
        bn[b]++;
        grow_box(bb[b], pbox[p]);
      }
      double lArea[31], rArea[31];
      int32_t lCnt[31], rCnt[31];
      Box acc = empty_box();
      int32_t accN = 0;
      for (int i = 0; i < nb - 1; i++) {
        if (bn[i] > 0) grow_box(acc, bb[i]);
        accN += bn[i];
        lCnt[i] = accN;
        lArea[i] = area(acc);
      }
      acc = empty_box();
      accN = 0;
      for (int i = nb - 1; i > 0; i--) {
        if (bn[i] > 0) grow_box(acc, bb[i]);
        accN += bn[i];
        rCnt[i - 1] = accN;
        rArea[i - 1] = area(acc);
      }
      int best = -1;
      double bestCost = std::numeric_limits<double>::infinity();
      for (int i = 0; i < nb - 1; i++) {
        if (lCnt[i] == 0 || rCnt[i] == 0) continue;
        double cost = lArea[i] * (double)lCnt[i] + rArea[i] * (double)rCnt[i];
        if (cost < bestCost) { bestCost = cost; best = i; }
      }
      const double leafCost = area(box) * (double)cnt;
      if (best < 0 || (cnt <= leaf * 2 && bestCost >= leafCost * 0.98)) { leafify(); continue; }
      int32_t i = t.s, j = t.e - 1;
      while (i <= j) {
        if (bin[i] <= best) {
          i++;
        } else {
          std::swap(order[i], order[j]);
          std::swap(bin[i], bin[j]);
          j--;
        }
      }
      mid = i;
      if (mid <= t.s || mid >= t.e) {  // unreachable: both sides of the chosen split are non-empty
        std::stable_sort(order.begin() + t.s, order.begin() + t.e, [&](int32_t a, int32_t b) {
          return cent[3 * (size_t)a + axis] < cent[3 * (size_t)b + axis];
        });
        mid = (t.s + t.e) / 2;
      }
    }
    // Right pushed first so the left subtree is numbered next (pre-order).
    stack.push_back(Task{mid, t.e, idx, true});
    stack.push_back(Task{t.s, mid, idx, false});
  }
}

extern "C" {

bc_hscene* bc_hscene_create(void) { return new (std::nothrow) bc_hscene(); }
void bc_hscene_destroy(bc_hscene* s) { delete s; }

int32_t bc_hscene_add_material(bc_hscene* s, int32_t kind, const double color[3], double roughness, double ior,
                               const double emission[3]) {
  s->mkind.push_back(kind);
  s->mcolor.insert(s->mcolor.end(), color, color + 3);
  s->mrough.push_back(roughness);
  s->mior.push_back(ior);
  s->memission.insert(s->memission.end(), emission, emission + 3);
  return (int32_t)s->mkind.size() - 1;
}

void bc_hscene_add_sphere(bc_hscene* s, const double c[3], double r, int32_t material) {
  if (!(r > 0)) return;
  s->push_prim(BC_PRIM_SPHERE, material);
  int32_t i = s->nprims() - 1;
  Box bx;
  for (int k = 0; k < 3; k++) {
    s->center[3 * (size_t)i + k] = c[k];
    s->cent[3 * (size_t)i + k] = c[k];
    bx.mn[k] = c[k] - r;
    bx.mx[k] = c[k] + r;
  }
  s->radius[i] = r;
  s->pbox[i] = bx;
  if (material >= 0 && material < (int32_t)s->mkind.size() && s->mkind[material] == BC_MAT_EMISSIVE)
    s->lights.push_back(i);
}

void bc_hscene_add_triangles(bc_hscene* s, int64_t n, const double* v, const int32_t* materials) {
  for (int64_t t = 0; t < n; t++) {
    const double* a = v + 9 * t;
    const double* b = a + 3;
    const double* c = a + 6;
    double e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    double e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    double nx = e1[1] * e2[2] - e1[2] * e2[1];
    double ny = e1[2] * e2[0] - e1[0] * e2[2];
    double nz = e1[0] * e2[1] - e1[1] * e2[0];
    if (nx * nx + ny * ny + nz * nz < 1e-18) continue;  // renderer.go:261
    s->push_prim(BC_PRIM_TRIANGLE, materials[t]);
    s->set_tri_geometry(s->nprims() - 1, a, b, c);
  }
}

bc_status bc_hscene_translate_prim(bc_hscene* s, int32_t i, const double d[3]) {
  if (!s || i < 0 || i >= s->nprims()) return BC_ERR_INVALID_ARG;
  if (s->kind[i] == BC_PRIM_SPHERE) {
    double r = s->radius[i];
    Box bx;
    for (int k = 0; k < 3; k++) {
      double c = s->center[3 * (size_t)i + k] + d[k];
      s->center[3 * (size_t)i + k] = c;
      s->cent[3 * (size_t)i + k] = c;
      bx.mn[k] = c - r;
      bx.mx[k] = c + r;
    }
    s->pbox[i] = bx;
    return BC_OK;
  }
  double a[3], b[3], c[3];
  for (int k = 0; k < 3; k++) {
    a[k] = s->A[3 * (size_t)i + k] + d[k];
    b[k] = s->B[3 * (size_t)i + k] + d[k];
    c[k] = s->C[3 * (size_t)i + k] + d[k];
  }
  s->set_tri_geometry(i, a, b, c);
  return BC_OK;
}

void bc_hscene_set_bvh(bc_hscene* s, const char* mode, int32_t bins, int32_t leaf_size) {
  s->mode = mode ? mode : "";
  s->bins = bins;
  s->leaf = leaf_size;
}

bc_status bc_hscene_build(bc_hscene* s) {
  if (!s) return BC_ERR_INVALID_ARG;
  s->topo++;
  s->geom++;
  s->rebuild_lights();
  if (s->mode.empty()) s->mode = "SAH";  // renderer.go:413-427
  if (s->bins < 4) s->bins = 16;
  if (s->bins > 32) s->bins = 32;
  if (s->leaf < 1) s->leaf = 4;
  if (s->leaf > 16) s->leaf = 16;
  try {
    s->build_tree();
  } catch (const std::bad_alloc&) {
    return BC_ERR_OOM;
  }
  return BC_OK;
}

bc_status bc_hscene_refit(bc_hscene* s) {
  if (!s) return BC_ERR_INVALID_ARG;
  s->geom++;
  if (s->left.empty()) {
    s->geom--;
    return bc_hscene_build(s);
  }
  for (int64_t ni = (int64_t)s->left.size() - 1; ni >= 0; ni--) {
    if (s->count[ni] > 0) {
      Box b = empty_box();
      for (int32_t i = 0; i < s->count[ni]; i++) {
        int32_t p = s->order[s->start[ni] + i];
        if (p >= 0 && p < s->nprims()) grow_box(b, s->pbox[p]);
      }
      s->set_node_box((int32_t)ni, b);
    } else if (s->left[ni] >= 0 && s->right[ni] >= 0) {
      Box b;
      std::memcpy(b.mn, &s->nbox[6 * (size_t)s->left[ni]], 3 * sizeof(double));
      std::memcpy(b.mx, &s->nbox[6 * (size_t)s->left[ni] + 3], 3 * sizeof(double));
      Box r;
      std::memcpy(r.mn, &s->nbox[6 * (size_t)s->right[ni]], 3 * sizeof(double));
      std::memcpy(r.mx, &s->nbox[6 * (size_t)s->right[ni] + 3], 3 * sizeof(double));
      grow_box(b, r);
      s->set_node_box((int32_t)ni, b);
    }
  }
  s->rebuild_lights();
  return BC_OK;
}

void bc_hscene_counts(const bc_hscene* s, int64_t out[6]) {
  out[0] = s->nprims();
  out[1] = (int64_t)s->left.size();
  out[2] = (int64_t)s->lights.size();
  out[3] = (int64_t)s->mkind.size();
  out[4] = (int64_t)s->topo;
  out[5] = (int64_t)s->geom;
}

bc_status bc_hscene_describe(const bc_hscene* s, bc_scene_desc* d) {
  if (!s || !d) return BC_ERR_INVALID_ARG;
  std::memset(d, 0, sizeof(*d));
  d->n_materials = (int32_t)s->mkind.size();
  d->mat_kind = s->mkind.data();
  d->mat_color = s->mcolor.data();
  d->mat_roughness = s->mrough.data();
  d->mat_ior = s->mior.data();
  d->mat_emission = s->memission.data();
  d->n_prims = s->nprims();
  d->prim_kind = s->kind.data();
  d->prim_material = s->mat.data();
  d->prim_center = s->center.data();
  d->prim_radius = s->radius.data();
  d->prim_a = s->A.data();
  d->prim_e1 = s->E1.data();
  d->prim_e2 = s->E2.data();
  d->prim_normal = s->N.data();
  d->n_nodes = (int32_t)s->left.size();
  d->node_box = s->nbox.data();
  d->node_left = s->left.data();
  d->node_right = s->right.data();
  d->node_start = s->start.data();
  d->node_count = s->count.data();
  d->order = s->order.data();
  d->n_lights = (int32_t)s->lights.size();
  d->light_spheres = s->lights.data();
  d->light_cdf = s->lcdf.data();
  d->light_pdf_by_prim = s->lpdf.data();
  return BC_OK;
}

}  // extern "C"

namespace bcgx {

// Scene.Build in SAH mode with the tree produced by an external builder (the
// device build): the clamps, revisions and light distribution of
// bc_hscene_build, then `fn` fills the node arrays and Order.
using TreeBuildFn = bc_status (*)(void* user, int32_t n, const double* pbox, const double* cent, int32_t bins,
                                  int32_t leaf, int32_t* n_nodes, double* box, int32_t* left, int32_t* right,
                                  int32_t* start, int32_t* count, int32_t* order);
bc_status hscene_build_external(bc_hscene* s, TreeBuildFn fn, void* user) {
  if (!s || !fn) return BC_ERR_INVALID_ARG;
  std::string lower = s->mode.empty() ? std::string("sah") : s->mode;
  for (auto& ch : lower) ch = (char)std::tolower((unsigned char)ch);
  if (lower == "median" || s->nprims() == 0) return bc_hscene_build(s);
  s->topo++;
  s->geom++;
  s->rebuild_lights();
  if (s->mode.empty()) s->mode = "SAH";  // the clamps of bc_hscene_build (renderer.go:413-427)
  if (s->bins < 4) s->bins = 16;
  if (s->bins > 32) s->bins = 32;
  if (s->leaf < 1) s->leaf = 4;
  if (s->leaf > 16) s->leaf = 16;
  const int32_t n = s->nprims();
  const size_t cap = 2 * (size_t)n - 1;
  try {
    s->nbox.assign(6 * cap, 0.0);
    s->left.assign(cap, -1);
    s->right.assign(cap, -1);
    s->start.assign(cap, 0);
    s->count.assign(cap, 0);
    s->order.assign(n, 0);
  } catch (const std::bad_alloc&) {
    return BC_ERR_OOM;
  }
  int32_t nn = 0;
  const bc_status st = fn(user, n, reinterpret_cast<const double*>(s->pbox.data()), s->cent.data(), s->bins, s->leaf,
                          &nn, s->nbox.data(), s->left.data(), s->right.data(), s->start.data(), s->count.data(),
                          s->order.data());
  if (st != BC_OK) {
    s->left.clear(); s->right.clear(); s->start.clear(); s->count.clear(); s->nbox.clear();
    return st;
  }
  s->nbox.resize(6 * (size_t)nn);
  s->left.resize(nn);
  s->right.resize(nn);
  s->start.resize(nn);
  s->count.resize(nn);
  return BC_OK;
}

}  // namespace bcgx


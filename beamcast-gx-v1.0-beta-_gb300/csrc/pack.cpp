// Host packer (see pack.h). Validation mirrors validateGPUSceneEncoding
// (gpu_opencl_windows.go:470-482) and adds the structural checks a device
// kernel needs to stay in bounds: child indices, leaf ranges, the Order
// permutation and material indices are all checked here, once, on the host.
#include "pack.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <system_error>
#include <thread>

#include "quantize.h"

namespace bcgx {

void scene_extent(const bc_scene_desc& d, SceneRange* r) {
  const bool some = d.n_prims > 0 && d.n_nodes > 0 && d.node_box;
  double e[3];
  for (int k = 0; k < 3; k++) {
    r->lo[k] = some ? d.node_box[k] : -1.0;
    r->hi[k] = some ? d.node_box[3 + k] : 1.0;
    e[k] = r->hi[k] - r->lo[k];
  }
  const double dd = e[0] * e[0] + e[1] * e[1];
  r->diag = std::sqrt(dd + e[2] * e[2]);
}

float round_down_f32(double x) { return rd_f32(x); }
float round_up_f32(double x) { return ru_f32(x); }

namespace {

// f(lo, hi) over [0, n) in contiguous chunks of at least min_chunk items, on up
// to 16 host threads; the chunks write disjoint outputs. Where no thread can be
// started, the rest runs on the calling thread.
template <class F>
void parallel_chunks(int64_t n, int64_t min_chunk, const F& f) {
  const int64_t hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const int64_t chunks = std::min<int64_t>(hw, (n + min_chunk - 1) / std::max<int64_t>(1, min_chunk));
  if (chunks <= 1) {
    if (n > 0) f((int64_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  th.reserve((size_t)chunks - 1);
  int64_t c = 1;
  try {
    for (; c < chunks; c++) th.emplace_back(f, n * c / chunks, n * (c + 1) / chunks);
  } catch (const std::system_error&) {
    for (int64_t k = c; k < chunks; k++) f(n * k / chunks, n * (k + 1) / chunks);
  }
  f((int64_t)0, n / chunks);
  for (std::thread& t : th) t.join();
}

double box_area(const double* b) {
  double ex = b[3] - b[0], ey = b[4] - b[1], ez = b[5] - b[2];
  if (ex < 0 || ey < 0 || ez < 0) return 0;
  return 2 * (ex * ey + ey * ez + ez * ex);
}

bc_status fail(std::string* err, const std::string& m) {
  if (err) *err = m;
  return BC_ERR_BAD_SCENE;
}

bc_status validate(const bc_scene_desc& d, std::string* err) {
  if (d.n_prims <= 0 || d.n_nodes <= 0)
    return fail(err, "scene requires a non-empty built scene (primitives and BVH nodes)");
  if (d.n_nodes >= kMaxIndex || d.n_prims >= kMaxIndex)
    return fail(err, "compact BVH supports fewer than 134217728 nodes/primitives");
  if (!d.prim_kind || !d.prim_material || !d.node_box || !d.node_left || !d.node_right || !d.node_start ||
      !d.node_count || !d.order)
    return fail(err, "scene descriptor is missing primitive or node arrays");
  if (d.n_materials < 1 || !d.mat_kind || !d.mat_color || !d.mat_emission)
    return fail(err, "scene requires at least one material");
  for (int32_t i = 0; i < d.n_materials; i++)
    if (d.mat_kind[i] < BC_MAT_DIFFUSE || d.mat_kind[i] > BC_MAT_EMISSIVE)
      return fail(err, "material " + std::to_string(i) + " has an unknown kind");
  bool any_sphere = false, any_tri = false;
  for (int32_t i = 0; i < d.n_prims; i++) {
    if (d.prim_kind[i] == BC_PRIM_SPHERE) any_sphere = true;
    else if (d.prim_kind[i] == BC_PRIM_TRIANGLE) any_tri = true;
    else return fail(err, "primitive " + std::to_string(i) + " has an unknown kind");
  }
  if (any_sphere && (!d.prim_center || !d.prim_radius)) return fail(err, "sphere arrays missing");
  if (any_tri && (!d.prim_a || !d.prim_e1 || !d.prim_e2 || !d.prim_normal)) return fail(err, "triangle arrays missing");
  for (int32_t i = 0; i < d.n_nodes; i++) {
    int32_t c = d.node_count[i];
    if (c < 0 || c > 16)
      return fail(err, "compact BVH leaf " + std::to_string(i) + " has unsupported count " + std::to_string(c));
    if (c > 0) {
      if (d.node_start[i] < 0 || (int64_t)d.node_start[i] + c > d.n_prims)
        return fail(err, "leaf " + std::to_string(i) + " range outside Order");
    } else {
      int32_t l = d.node_left[i], r = d.node_right[i];
      if (l <= i || r <= i || l >= d.n_nodes || r >= d.n_nodes || l == r)
        return fail(err, "inner node " + std::to_string(i) + " has invalid children");
    }
  }
  // Each node reachable exactly once from the root (children always follow
  // their parent, so the walk terminates).
  std::vector<uint8_t> seen(d.n_nodes, 0);
  std::vector<int32_t> st{0};
  while (!st.empty()) {
    int32_t i = st.back();
    st.pop_back();
    if (seen[i]) return fail(err, "node " + std::to_string(i) + " is shared by two parents");
    seen[i] = 1;
    if (d.node_count[i] == 0) {
      st.push_back(d.node_left[i]);
      st.push_back(d.node_right[i]);
    }
  }
  std::vector<uint8_t> used(d.n_prims, 0);
  for (int32_t i = 0; i < d.n_prims; i++) {
    int32_t p = d.order[i];
    if (p < 0 || p >= d.n_prims || used[p]) return fail(err, "Order is not a permutation of the primitives");
    used[p] = 1;
  }
  if (d.n_lights < 0 || (d.n_lights > 0 && (!d.light_spheres || !d.light_cdf)))
    return fail(err, "light arrays missing");
  for (int32_t i = 0; i < d.n_lights; i++) {
    int32_t p = d.light_spheres[i];
    if (p < 0 || p >= d.n_prims || d.prim_kind[p] != BC_PRIM_SPHERE)
      return fail(err, "light " + std::to_string(i) + " is not a sphere primitive");
  }
  return BC_OK;
}

void pack_slots(const bc_scene_desc& d, PackedScene* ps) {
  const int32_t n = d.n_prims;
  ps->tri.resize(3 * (size_t)n);
  ps->slot64.assign(9 * (size_t)n, 0.0);
  ps->snorm.resize(n);
  ps->slot_prim.resize(n);
  ps->has_spheres = false;
  for (int32_t p = 0; p < n && !ps->has_spheres; p++) ps->has_spheres = d.prim_kind[p] == BC_PRIM_SPHERE;
  parallel_chunks(n, 1 << 16, [&](int64_t lo, int64_t hi) {
    for (int32_t s = (int32_t)lo; s < (int32_t)hi; s++) {
      const int32_t p = d.order[s];
      ps->slot_prim[s] = p;
      int32_t mat = d.prim_material[p];
      float matbits;
      std::memcpy(&matbits, &mat, 4);
      const bool sphere = d.prim_kind[p] == BC_PRIM_SPHERE;
      const double zero[3] = {0.0, 0.0, 0.0};
      const size_t k3 = 3 * (size_t)p;
      float nrm[3];
      pack_slot(sphere, sphere ? d.prim_center + k3 : zero, sphere ? d.prim_radius[p] : 0.0,
                sphere ? zero : d.prim_a + k3, sphere ? zero : d.prim_e1 + k3, sphere ? zero : d.prim_e2 + k3,
                sphere ? zero : d.prim_normal + k3, &ps->tri[3 * (size_t)s], &ps->slot64[9 * (size_t)s], nrm);
      ps->snorm[s] = F4{nrm[0], nrm[1], nrm[2], matbits};
    }
  });
}

void quantize_node(Node8& n, const double* boxes, int nk) {
  quantize_children(n, boxes, nk);
  n.nchild = (uint8_t)nk;
}

uint32_t leaf_ref(const bc_scene_desc& d, int32_t i) {
  return kLeafBit | ((uint32_t)(d.node_count[i] - 1) & 0xfu) << 27 | ((uint32_t)d.node_start[i] & kSlotMask);
}

// Which binary subtrees become the children of each BVH8 node, and which
// become leaves. The surface-area heuristic charges each BVH8 node its box's
// area A and each leaf tri_cost * A * (its primitives). A dynamic program over
// the binary tree (after Ylitie, Karras and Laine, "Efficient Incoherent Ray
// Traversal on GPUs Through Compressed Wide BVHs", HPG 2017) minimises the
// total: cost(i, k) is the least cost that binary node i's subtree adds when
// it takes at most k child slots of its parent. One slot makes i itself a
// child: a leaf if it is one; if it is inner, its own BVH8 node (A(i) + the
// best split of 8 slots between its children) or, when its subtree holds at
// most max_leaf primitives in one contiguous slot range, a leaf of all of them.
// More slots may open it into its children's slots. Every binary leaf's slots
// stay in one BVH8 leaf, and the hits are the same whatever the choice.
// Without merging the binary leaves stay exactly as they are; the node area is
// then 10% below that of opening the largest child greedily on the
// Ultra-shaped scene.
class WideCollapse {
 public:
  WideCollapse(const bc_scene_desc& d, const CollapseParams& cp) : d_(d), n_(d.n_nodes) {
    cost_.assign((size_t)n_ * 9, 0.0);
    split_.assign((size_t)n_ * 9, 0);
    open_.assign((size_t)n_ * 9, 0);
    merged_.assign(n_, 0);
    start_.assign(n_, 0);
    count_.assign(n_, 0);
    max_leaf_ = cp.merges(d.n_prims) && cp.max_leaf > 0 && leaves_partition(d) ? std::min(cp.max_leaf, 16) : 0;
    tri_cost_ = max_leaf_ > 0 ? cp.tri_cost : 0.0;  // 0: the node-area-only collapse
    // A node needs only its children's results: the levels of the tree are
    // solved deepest first, the nodes of a level in parallel (children follow
    // their parent, so one forward pass gives the depths).
    std::vector<int32_t> depth(n_, 0);
    int32_t max_depth = 0;
    for (int32_t i = 0; i < n_; i++)
      if (d.node_count[i] == 0) {
        depth[d.node_left[i]] = depth[d.node_right[i]] = depth[i] + 1;
        max_depth = std::max(max_depth, depth[i] + 1);
      }
    std::vector<int32_t> at((size_t)max_depth + 2, 0), order(n_);
    for (int32_t i = 0; i < n_; i++) at[depth[i] + 1]++;
    for (int32_t k = 0; k <= max_depth; k++) at[k + 1] += at[k];
    {
      std::vector<int32_t> fill(at.begin(), at.end() - 1);
      for (int32_t i = 0; i < n_; i++) order[fill[depth[i]]++] = i;
    }
    for (int32_t k = max_depth; k >= 0; k--) {
      const int32_t* lvl = order.data() + at[k];
      parallel_chunks(at[k + 1] - at[k], 1 << 14, [&](int64_t lo, int64_t hi) {
        for (int64_t j = lo; j < hi; j++) solve(lvl[j]);
      });
    }
  }
  // The DP entries of binary node i from its children's.
  void solve(int32_t i) {
    const bc_scene_desc& d = d_;
    const int max_leaf = max_leaf_;
    const double tri_cost = tri_cost_;
    {
      if (d.node_count[i] > 0) {
        start_[i] = d.node_start[i];
        count_[i] = d.node_count[i];
        const double c = tri_cost * box_area(d.node_box + 6 * (size_t)i) * d.node_count[i];
        for (int k = 1; k <= 8; k++) cost_[(size_t)i * 9 + k] = c;
        return;
      }
      const int32_t l = d.node_left[i], r = d.node_right[i];
      // the subtree's slots: one range when the children's ranges abut
      const int32_t lo = std::min(start_[l], start_[r]);
      const int64_t n = (int64_t)count_[l] + count_[r];
      const bool run = count_[l] > 0 && count_[r] > 0 && n <= 16 &&
                       (start_[l] + count_[l] == start_[r] || start_[r] + count_[r] == start_[l]);
      start_[i] = run ? lo : 0;
      count_[i] = run ? (int32_t)n : 0;  // 0: not one range of at most 16 slots
      double dist[9];  // dist[k]: the best split of k slots between the two children
      for (int k = 2; k <= 8; k++) {
        dist[k] = 0.0;
        int at = 0;
        for (int a = 1; a < k; a++) {
          const double c = cost(l, a) + cost(r, k - a);
          if (at == 0 || c < dist[k]) {
            dist[k] = c;
            at = a;
          }
        }
        split_[(size_t)i * 9 + k] = (uint8_t)at;
      }
      const double area = box_area(d.node_box + 6 * (size_t)i);
      cost_[(size_t)i * 9 + 1] = area + dist[8];
      if (count_[i] > 0 && count_[i] <= max_leaf) {
        const double as_leaf = tri_cost * area * count_[i];
        if (as_leaf < cost_[(size_t)i * 9 + 1]) {
          cost_[(size_t)i * 9 + 1] = as_leaf;
          merged_[i] = 1;
        }
      }
      for (int k = 2; k <= 8; k++) {
        const double fewer = cost_[(size_t)i * 9 + k - 1];
        const bool open = dist[k] < fewer;
        open_[(size_t)i * 9 + k] = open ? 1 : 0;
        cost_[(size_t)i * 9 + k] = open ? dist[k] : fewer;
      }
    }
  }
  // The children of the BVH8 node made from inner binary node w, in binary order.
  int children(int32_t w, int32_t kids[8]) const {
    int nk = 0;
    const int a = split_[(size_t)w * 9 + 8];
    expand(d_.node_left[w], a, kids, &nk);
    expand(d_.node_right[w], 8 - a, kids, &nk);
    return nk;
  }
  // A child that is a BVH8 leaf: a binary leaf, or an inner node merged into one.
  bool is_leaf(int32_t i) const { return d_.node_count[i] > 0 || merged_[i]; }
  uint32_t leaf_ref(int32_t i) const {
    return kLeafBit | ((uint32_t)(count_[i] - 1) & 0xfu) << 27 | ((uint32_t)start_[i] & kSlotMask);
  }

 private:
  // Every slot lies in exactly one binary leaf (a builder's tree always; a
  // caller's tree is only checked for bounds), so merged ranges are exact.
  static bool leaves_partition(const bc_scene_desc& d) {
    std::vector<uint8_t> seen(d.n_prims, 0);
    for (int32_t i = 0; i < d.n_nodes; i++)
      for (int32_t s = d.node_start[i]; d.node_count[i] > 0 && s < d.node_start[i] + d.node_count[i]; s++) {
        if (seen[s]) return false;
        seen[s] = 1;
      }
    for (int32_t s = 0; s < d.n_prims; s++)
      if (!seen[s]) return false;
    return true;
  }
  double cost(int32_t i, int k) const { return cost_[(size_t)i * 9 + k]; }
  void expand(int32_t i, int k, int32_t kids[8], int* nk) const {
    while (k > 1 && d_.node_count[i] == 0 && !open_[(size_t)i * 9 + k]) k--;  // fewer slots were as good
    if (k == 1 || d_.node_count[i] > 0) {
      kids[(*nk)++] = i;
      return;
    }
    const int a = split_[(size_t)i * 9 + k];
    expand(d_.node_left[i], a, kids, nk);
    expand(d_.node_right[i], k - a, kids, nk);
  }
  const bc_scene_desc& d_;
  int32_t n_;
  std::vector<double> cost_;   // [node][k], k = 1..8
  std::vector<uint8_t> split_; // [node][k]: slots of the left child in the best split of k
  std::vector<uint8_t> open_;  // [node][k]: k slots open the node (else k - 1 were as good)
  std::vector<uint8_t> merged_; // inner node that is a leaf when it takes one slot
  std::vector<int32_t> start_, count_;  // the subtree's slot range (count 0: not one range)
  int max_leaf_ = 0;
  double tri_cost_ = 0.0;
};

void collapse(const bc_scene_desc& d, const CollapseParams& cp, PackedScene* ps) {
  ps->nodes.clear();
  const WideCollapse wide(d, cp);
  struct Job { int32_t bin, parent, slot, depth, acc; };
  std::vector<Job> jobs{Job{0, -1, 0, 1, 0}};
  ps->depth = 0;
  ps->stack_need = 1;
  while (!jobs.empty()) {
    Job j = jobs.back();
    jobs.pop_back();
    const int32_t idx = (int32_t)ps->nodes.size();
    ps->nodes.emplace_back();
    if (j.parent >= 0) ps->nodes[j.parent].child[j.slot] = (uint32_t)idx;
    int32_t kids[8];
    int nk = 0;
    if (d.node_count[j.bin] > 0) {
      kids[nk++] = j.bin;  // single-leaf scene: the root holds one leaf child
    } else {
      nk = wide.children(j.bin, kids);
    }
    Node8& n = ps->nodes[idx];
    std::memset(&n, 0, sizeof(n));
    double boxes[48];
    for (int k = 0; k < nk; k++) std::memcpy(boxes + 6 * k, d.node_box + 6 * (size_t)kids[k], 6 * sizeof(double));
    quantize_node(n, boxes, nk);
    ps->kids8.resize(8 * ps->nodes.size(), -1);
    for (int k = 0; k < nk; k++) ps->kids8[8 * (size_t)idx + k] = kids[k];
    ps->depth = std::max(ps->depth, j.depth);
    ps->stack_need = std::max(ps->stack_need, j.acc + nk + 1);
    for (int k = nk - 1; k >= 0; k--) {
      if (d.node_count[kids[k]] > 0) {
        ps->nodes[idx].child[k] = leaf_ref(d, kids[k]);
      } else if (wide.is_leaf(kids[k])) {
        ps->nodes[idx].child[k] = wide.leaf_ref(kids[k]);
      } else {
        jobs.push_back(Job{kids[k], idx, k, j.depth + 1, j.acc + nk - 1});
      }
    }
  }
}

void pack_materials(const bc_scene_desc& d, PackedScene* ps) {
  ps->mats.resize(d.n_materials);
  for (int32_t i = 0; i < d.n_materials; i++) {
    const double* c = d.mat_color + 3 * (size_t)i;
    const double* e = d.mat_emission + 3 * (size_t)i;
    MatGPU& m = ps->mats[i];
    m.cr = (float)c[0]; m.cg = (float)c[1]; m.cb = (float)c[2];
    m.rough = d.mat_roughness ? (float)d.mat_roughness[i] : 0.0f;
    m.er = (float)e[0]; m.eg = (float)e[1]; m.eb = (float)e[2];
    m.kind = (float)d.mat_kind[i];
    m.ior = d.mat_ior ? (float)d.mat_ior[i] : 0.0f;
    // materialPreviewColor (renderer.go:1467-1475)
    if (d.mat_kind[i] == BC_MAT_EMISSIVE) {
      auto cl = [](double x) { return (float)std::min(1.0, std::max(0.0, x / 8)); };
      m.preview_r = cl(e[0]); m.preview_g = cl(e[1]); m.preview_b = cl(e[2]);
    } else if (c[0] * c[0] + c[1] * c[1] + c[2] * c[2] > 0) {
      m.preview_r = (float)c[0]; m.preview_g = (float)c[1]; m.preview_b = (float)c[2];
    } else {
      m.preview_r = m.preview_g = m.preview_b = 0.8f;
    }
  }
}

void pack_lights(const bc_scene_desc& d, PackedScene* ps) {
  ps->lights.resize(d.n_lights);
  ps->light_pdf_by_prim.assign(d.n_prims, 0.0f);
  if (d.light_pdf_by_prim)
    for (int32_t i = 0; i < d.n_prims; i++) ps->light_pdf_by_prim[i] = (float)d.light_pdf_by_prim[i];
  for (int32_t i = 0; i < d.n_lights; i++) {
    int32_t p = d.light_spheres[i];
    LightGPU& L = ps->lights[i];
    const double* c = d.prim_center + 3 * (size_t)p;
    L.cx = (float)c[0]; L.cy = (float)c[1]; L.cz = (float)c[2];
    L.r = (float)d.prim_radius[p];
    int32_t m = d.prim_material[p];
    const double* e = (m >= 0 && m < d.n_materials) ? d.mat_emission + 3 * (size_t)m : nullptr;
    L.er = e ? (float)e[0] : 0.0f; L.eg = e ? (float)e[1] : 0.0f; L.eb = e ? (float)e[2] : 0.0f;
    double pdf = d.light_pdf_by_prim ? d.light_pdf_by_prim[p] : 0.0;
    if (pdf <= 0) pdf = 1.0 / (double)d.n_lights;  // chooseLight fallback, renderer.go:1389-1391
    L.select_pdf = (float)pdf;
    L.cdf = d.light_cdf[i];
    L.cdf_dn = (float)L.cdf;
    if ((double)L.cdf_dn > L.cdf) L.cdf_dn = std::nextafter(L.cdf_dn, -INFINITY);
    L.prim = p;
  }
}

}  // namespace

void pack_binary(const bc_scene_desc& d, std::vector<BinNode>* out) {
  out->resize(d.n_nodes);
  for (int32_t i = 0; i < d.n_nodes; i++) {
    BinNode& b = (*out)[i];
    for (int k = 0; k < 3; k++) {
      b.lo[k] = d.node_box[6 * (size_t)i + k];
      b.hi[k] = d.node_box[6 * (size_t)i + 3 + k];
    }
    const bool leaf = d.node_count[i] > 0;
    b.left = leaf ? -1 : d.node_left[i];
    b.right = leaf ? -1 : d.node_right[i];
    b.start = leaf ? d.node_start[i] : 0;
    b.count = leaf ? d.node_count[i] : 0;
  }
}

bc_status pack_scene(const bc_scene_desc& d, PackedScene* out, std::string* err, const CollapseParams& cp) {
  bc_status st = validate(d, err);
  if (st != BC_OK) return st;
  try {
    out->n_prims = d.n_prims;
    out->n_binary = d.n_nodes;
    pack_slots(d, out);
    collapse(d, cp, out);
    pack_binary(d, &out->bin);
    pack_materials(d, out);
    pack_lights(d, out);
    for (int k = 0; k < 3; k++) {
      out->scene_lo[k] = round_down_f32(d.node_box[k]);
      out->scene_hi[k] = round_up_f32(d.node_box[3 + k]);
    }
  } catch (const std::bad_alloc&) {
    if (err) *err = "host allocation failed while packing the scene";
    return BC_ERR_OOM;
  }
  return BC_OK;
}

bc_status pack_scene_set(const bc_scene_desc* d, int n, PackedScene* out, std::vector<SceneRange>* ranges,
                         std::string* err, const CollapseParams& cp) {
  if (n < 1 || !d) {
    if (err) *err = "a scene set needs at least one scene";
    return BC_ERR_INVALID_ARG;
  }
  *out = PackedScene();
  ranges->assign(n, SceneRange());
  for (int k = 0; k < n; k++) {
    PackedScene ps;
    bc_status st = pack_scene(d[k], &ps, err, cp);
    if (st != BC_OK) {
      if (err) *err = "scene " + std::to_string(k) + ": " + *err;
      return st;
    }
    SceneRange& r = (*ranges)[k];
    r.root = (int32_t)out->nodes.size();
    r.slot_off = out->n_prims;
    r.n_slots = ps.n_prims;
    r.prim_off = out->n_prims;  // primitive indices and slots share one numbering per scene
    r.mat_off = (int32_t)out->mats.size();
    scene_extent(d[k], &r);
    r.light_off = (int32_t)out->lights.size();
    r.n_lights = (int32_t)ps.lights.size();
    if ((int64_t)out->nodes.size() + ps.nodes.size() >= kMaxIndex || (int64_t)out->n_prims + ps.n_prims >= kMaxIndex) {
      if (err) *err = "scene set exceeds 2^27 nodes or primitives";
      return BC_ERR_BAD_SCENE;
    }
    for (Node8 nd : ps.nodes) {
      for (int c = 0; c < nd.nchild; c++) {
        if (nd.child[c] & kLeafBit) nd.child[c] += (uint32_t)r.slot_off;  // start field: low 27 bits
        else nd.child[c] += (uint32_t)r.root;
      }
      out->nodes.push_back(nd);
    }
    out->tri.insert(out->tri.end(), ps.tri.begin(), ps.tri.end());
    out->slot64.insert(out->slot64.end(), ps.slot64.begin(), ps.slot64.end());
    if (k == 0) out->bin = std::move(ps.bin);  // the ray-cast entry points trace scene 0
    const int32_t n_mats = (int32_t)ps.mats.size();
    for (F4 f : ps.snorm) {
      int32_t m;
      std::memcpy(&m, &f.w, 4);
      // an index outside the scene's own table ends the path; keep it outside the set's
      m = (m >= 0 && m < n_mats) ? m + r.mat_off : -1;
      std::memcpy(&f.w, &m, 4);
      out->snorm.push_back(f);
    }
    for (int32_t p : ps.slot_prim) out->slot_prim.push_back(p + r.prim_off);
    out->mats.insert(out->mats.end(), ps.mats.begin(), ps.mats.end());
    for (LightGPU L : ps.lights) {
      L.prim += r.prim_off;
      out->lights.push_back(L);
    }
    out->light_pdf_by_prim.insert(out->light_pdf_by_prim.end(), ps.light_pdf_by_prim.begin(),
                                  ps.light_pdf_by_prim.end());
    out->n_prims += ps.n_prims;
    out->n_binary += ps.n_binary;
    out->depth = std::max(out->depth, ps.depth);
    out->stack_need = std::max(out->stack_need, ps.stack_need);
    out->has_spheres = out->has_spheres || ps.has_spheres;
    for (int a = 0; a < 3; a++) {  // bounds of the whole set
      out->scene_lo[a] = k == 0 ? ps.scene_lo[a] : std::min(out->scene_lo[a], ps.scene_lo[a]);
      out->scene_hi[a] = k == 0 ? ps.scene_hi[a] : std::max(out->scene_hi[a], ps.scene_hi[a]);
    }
  }
  return BC_OK;
}

void pack_scene_lights(const bc_scene_desc& d, PackedScene* out) { pack_lights(d, out); }

}  // namespace bcgx

// Host check of the BVH8 packer (compiled and run by tests/test_pack_native.py):
// every quantized child box, decoded the way the device decodes it (round-down
// lower bound, round-up upper bound of p + q * 2^e), must strictly contain the
// fp64 box of the binary node it stands for; without leaf merging the BVH8
// leaves must be exactly the binary tree's leaves, and with it every leaf must
// hold the slots of one binary subtree and every slot lie in exactly one leaf.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <random>
#include <vector>

#include "bc_host_scene.h"
#include "pack.h"

using namespace bcgx;

static float rd(double x) { return round_down_f32(x); }
static float ru(double x) { return round_up_f32(x); }

// slot range [lo, hi) and primitive count of binary node i's subtree
static void subtree_range(const bc_scene_desc& d, int i, int64_t* lo, int64_t* hi, int64_t* n) {
  if (d.node_count[i] > 0) {
    *lo = d.node_start[i];
    *hi = (int64_t)d.node_start[i] + d.node_count[i];
    *n = d.node_count[i];
    return;
  }
  int64_t l0, h0, n0, l1, h1, n1;
  subtree_range(d, d.node_left[i], &l0, &h0, &n0);
  subtree_range(d, d.node_right[i], &l1, &h1, &n1);
  *lo = std::min(l0, l1);
  *hi = std::max(h0, h1);
  *n = n0 + n1;
}

static int check_merged(const bc_scene_desc& d) {
  PackedScene ps;
  std::string err;
  CollapseParams cp;
  cp.merge = 1;
  if (pack_scene(d, &ps, &err, cp) != BC_OK) { std::printf("pack failed: %s\n", err.c_str()); return 1; }
  std::vector<int> cover(d.n_prims, 0);
  int merged = 0, bad = 0;
  for (size_t i = 0; i < ps.nodes.size(); i++) {
    const Node8& n = ps.nodes[i];
    for (int k = 0; k < n.nchild; k++) {
      const int b = ps.kids8[8 * i + k];
      const double* box = d.node_box + 6 * (size_t)b;
      const float p[3] = {n.px, n.py, n.pz};
      const uint8_t e[3] = {n.ex, n.ey, n.ez};
      const uint8_t ql[3] = {n.qlox[k], n.qloy[k], n.qloz[k]};
      const uint8_t qh[3] = {n.qhix[k], n.qhiy[k], n.qhiz[k]};
      for (int a = 0; a < 3; a++) {
        const double sc = std::ldexp(1.0, (int)e[a] - 127);
        const float lo = rd((double)p[a] + ql[a] * sc), hi = ru((double)p[a] + qh[a] * sc);
        if (!((double)lo < box[a]) || !((double)hi > box[3 + a])) bad++;
      }
      if (!(n.child[k] & kLeafBit)) continue;
      const int64_t start = n.child[k] & kSlotMask, cnt = ((n.child[k] >> 27) & 15u) + 1;
      int64_t lo, hi, np;
      subtree_range(d, b, &lo, &hi, &np);
      if (lo != start || hi != start + cnt || np != cnt) { std::printf("leaf range differs from its subtree\n"); return 1; }
      if (d.node_count[b] == 0) merged++;
      for (int64_t s = start; s < start + cnt; s++) cover[s]++;
    }
  }
  for (int32_t s = 0; s < d.n_prims; s++)
    if (cover[s] != 1) { std::printf("slot %d in %d leaves\n", s, cover[s]); return 1; }
  if (bad) { std::printf("%d non-conservative child bounds (merged)\n", bad); return 1; }
  if (merged == 0) { std::printf("no merged leaf\n"); return 1; }
  std::printf("ok merged nodes=%zu merged_leaves=%d\n", ps.nodes.size(), merged);
  return 0;
}

// A caller's tree whose leaf ranges overlap passes the bounds checks but is no
// partition of the slots: leaf merging then stays off, and every BVH8 leaf is
// one of the caller's leaves.
static int check_overlapping_leaves(const bc_scene_desc& d0) {
  std::vector<int32_t> start(d0.node_start, d0.node_start + d0.n_nodes);
  int first = -1, second = -1;
  for (int i = 0; i < d0.n_nodes; i++)
    if (d0.node_count[i] > 0) {
      if (first < 0) first = i;
      else if (second < 0 && start[i] != start[first]) second = i;
    }
  if (first < 0 || second < 0) { std::printf("fewer than two leaves\n"); return 1; }
  start[second] = start[first];  // the two leaves now share slots
  bc_scene_desc d = d0;
  d.node_start = start.data();
  PackedScene ps;
  std::string err;
  CollapseParams cp;
  cp.merge = 1;
  if (pack_scene(d, &ps, &err, cp) != BC_OK) { std::printf("pack failed: %s\n", err.c_str()); return 1; }
  for (size_t i = 0; i < ps.nodes.size(); i++)
    for (int k = 0; k < ps.nodes[i].nchild; k++) {
      const int b = ps.kids8[8 * i + k];
      if ((ps.nodes[i].child[k] & kLeafBit) && d.node_count[b] == 0) {
        std::printf("merged leaf over overlapping ranges\n");
        return 1;
      }
    }
  std::printf("ok overlapping leaves unmerged\n");
  return 0;
}

static int check_scene(bc_hscene* s) {
  bc_scene_desc d;
  if (bc_hscene_describe(s, &d) != BC_OK) return 1;
  if (check_merged(d)) return 1;
  if (check_overlapping_leaves(d)) return 1;
  PackedScene ps;
  std::string err;
  if (pack_scene(d, &ps, &err) != BC_OK) { std::printf("pack failed: %s\n", err.c_str()); return 1; }
  // map leaf ref -> binary leaf box, and count leaves
  std::map<uint32_t, int> leaf_of;
  int binary_leaves = 0;
  for (int i = 0; i < d.n_nodes; i++)
    if (d.node_count[i] > 0) {
      binary_leaves++;
      uint32_t ref = kLeafBit | ((uint32_t)(d.node_count[i] - 1) & 0xfu) << 27 | ((uint32_t)d.node_start[i] & kSlotMask);
      leaf_of[ref] = i;
    }
  int leaves = 0, bad = 0;
  // walk BVH8 and the binary boxes in parallel: record for each Node8 child the binary node box
  // by re-deriving the box from the referenced subtree (leaf: its box; inner: union of descendants)
  // compute union box of each Node8 subtree bottom-up (children indices are larger than parents)
  std::vector<std::array<double, 6>> sub(ps.nodes.size());
  for (int i = (int)ps.nodes.size() - 1; i >= 0; i--) {
    std::array<double, 6> u = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    const Node8& n = ps.nodes[i];
    for (int k = 0; k < n.nchild; k++) {
      const double* b;
      std::array<double, 6> cb;
      if (n.child[k] & kLeafBit) {
        auto it = leaf_of.find(n.child[k]);
        if (it == leaf_of.end()) { std::printf("unknown leaf ref\n"); return 1; }
        b = d.node_box + 6 * (size_t)it->second;
        leaves++;
      } else {
        cb = sub[n.child[k]];
        b = cb.data();
      }
      for (int a = 0; a < 3; a++) { u[a] = std::min(u[a], b[a]); u[3 + a] = std::max(u[3 + a], b[3 + a]); }
      const float p[3] = {n.px, n.py, n.pz};
      const uint8_t e[3] = {n.ex, n.ey, n.ez};
      const uint8_t ql[3] = {n.qlox[k], n.qloy[k], n.qloz[k]};
      const uint8_t qh[3] = {n.qhix[k], n.qhiy[k], n.qhiz[k]};
      for (int a = 0; a < 3; a++) {
        const double sc = std::ldexp(1.0, (int)e[a] - 127);
        const float lo = rd((double)p[a] + ql[a] * sc), hi = ru((double)p[a] + qh[a] * sc);
        if (!((double)lo < b[a]) || !((double)hi > b[3 + a])) bad++;
      }
    }
    sub[i] = u;
  }
  if (leaves != binary_leaves) { std::printf("leaf count %d vs binary %d\n", leaves, binary_leaves); return 1; }
  if (bad) { std::printf("%d non-conservative child bounds\n", bad); return 1; }
  std::printf("ok nodes=%zu leaves=%d\n", ps.nodes.size(), leaves);
  return 0;
}

// The light records' fp32 CDF copy is the largest fp32 value <= the fp64 CDF
// entry, so the device's fp32 comparison with an fp32 draw takes the fp64
// comparison's branch for every draw.
static int check_light_cdf() {
  std::mt19937_64 rng(777);
  std::uniform_real_distribution<double> U(0, 1);
  bc_hscene* s = bc_hscene_create();
  const double c0[3] = {0.5, 0.5, 0.5}, e0[3] = {0, 0, 0};
  const int diffuse = bc_hscene_add_material(s, BC_MAT_DIFFUSE, c0, 0, 0, e0);
  for (int k = 0; k < 300; k++) {
    const double em[3] = {0.1 + 10 * U(rng), 0.1 + U(rng), 0.1 + 3 * U(rng)};
    const int m = bc_hscene_add_material(s, BC_MAT_EMISSIVE, c0, 0, 0, em);
    const double c[3] = {U(rng), U(rng), U(rng)};
    bc_hscene_add_sphere(s, c, 0.001 + 0.05 * U(rng), k % 7 ? m : diffuse);
  }
  bc_hscene_set_bvh(s, "SAH", 32, 4);
  bc_hscene_build(s);
  bc_scene_desc d;
  int rc = bc_hscene_describe(s, &d) != BC_OK;
  PackedScene ps;
  std::string err;
  if (!rc && pack_scene(d, &ps, &err) != BC_OK) rc = 1;
  int exact = 0;
  for (size_t i = 0; !rc && i < ps.lights.size(); i++) {
    const double cdf = ps.lights[i].cdf;
    const float dn = ps.lights[i].cdf_dn;
    if (!((double)dn <= cdf) || !((double)std::nextafter(dn, INFINITY) > cdf)) {
      std::printf("light %zu: cdf_dn %.9g not the largest fp32 <= %.17g\n", i, dn, cdf);
      rc = 1;
    }
    exact += (double)dn == cdf;
  }
  if (!rc && ps.lights.size() < 200) {
    std::printf("only %zu lights\n", ps.lights.size());
    rc = 1;
  }
  if (!rc) std::printf("ok light cdf lights=%zu exact=%d\n", ps.lights.size(), exact);
  bc_hscene_destroy(s);
  return rc;
}

// A scene large enough for the packer's threads (slot records in chunks of
// 65,536, tree levels of more than 16,384 nodes): two packs of it are
// byte-identical, with and without leaf merging.
static int check_threaded_pack() {
  std::mt19937_64 rng(99);
  std::uniform_real_distribution<double> U(0, 1);
  bc_hscene* s = bc_hscene_create();
  const double c0[3] = {0.5, 0.5, 0.5}, e0[3] = {0, 0, 0};
  const int m = bc_hscene_add_material(s, BC_MAT_DIFFUSE, c0, 0, 0, e0);
  const int n = 300000;
  std::vector<double> v(9 * (size_t)n);
  for (int t = 0; t < n; t++) {
    const double c[3] = {U(rng), U(rng), U(rng)};
    for (int j = 0; j < 3; j++)
      for (int a = 0; a < 3; a++) v[9 * (size_t)t + 3 * j + a] = c[a] + (U(rng) - 0.5) * 0.01;
  }
  std::vector<int32_t> mats(n, m);
  bc_hscene_add_triangles(s, n, v.data(), mats.data());
  bc_hscene_set_bvh(s, "SAH", 32, 4);
  bc_hscene_build(s);
  bc_scene_desc d;
  int rc = bc_hscene_describe(s, &d) != BC_OK;
  for (int merge = 0; merge <= 1 && !rc; merge++) {
    CollapseParams cp;
    cp.merge = merge;
    PackedScene a, b;
    std::string err;
    if (pack_scene(d, &a, &err, cp) != BC_OK || pack_scene(d, &b, &err, cp) != BC_OK) {
      std::printf("pack failed: %s\n", err.c_str());
      rc = 1;
      break;
    }
    auto same = [](const auto& x, const auto& y) {
      return x.size() == y.size() && std::memcmp(x.data(), y.data(), x.size() * sizeof(x[0])) == 0;
    };
    if (!same(a.nodes, b.nodes) || !same(a.tri, b.tri) || !same(a.slot64, b.slot64) || !same(a.snorm, b.snorm) ||
        !same(a.slot_prim, b.slot_prim) || !same(a.kids8, b.kids8) || a.stack_need != b.stack_need) {
      std::printf("two packs differ (merge %d)\n", merge);
      rc = 1;
    }
  }
  if (!rc) rc = check_scene(s);
  if (!rc) std::printf("ok threaded pack\n");
  bc_hscene_destroy(s);
  return rc;
}

int main() {
  std::mt19937_64 rng(12345);
  int rc = check_light_cdf();
  rc |= check_threaded_pack();
  for (int trial = 0; trial < 6; trial++) {
    bc_hscene* s = bc_hscene_create();
    double c0[3] = {0.5, 0.5, 0.5}, e0[3] = {0, 0, 0};
    int m = bc_hscene_add_material(s, BC_MAT_DIFFUSE, c0, 0, 0, e0);
    const double scale = trial < 2 ? 1.0 : (trial < 4 ? 1000.0 : 1e-2);
    const double offset = trial % 2 ? 5e5 : 0.0;
    std::uniform_real_distribution<double> U(0, 1);
    std::lognormal_distribution<double> LN(-5, 0.5);
    const int n = 20000;
    std::vector<double> v(9 * n);
    std::vector<int32_t> mats(n, m);
    for (int t = 0; t < n; t++) {
      double c[3] = {U(rng) * scale + offset, U(rng) * scale, U(rng) * scale};
      for (int j = 0; j < 3; j++)
        for (int a = 0; a < 3; a++) v[9 * t + 3 * j + a] = c[a] + (U(rng) - 0.5) * LN(rng) * scale;
    }
    // axis-aligned and degenerate-extent triangles
    for (int t = 0; t < 200; t++) {
      // axis-aligned triangles on a few shared planes (flat boxes, exact coordinates)
      double y = std::floor(U(rng) * 8) * 0.125 * scale;
      double x = offset + std::floor(U(rng) * 64) / 64 * scale, z = std::floor(U(rng) * 64) / 64 * scale;
      double tri[9] = {x, y, z, x + scale * 0.01, y, z, x, y, z + scale * 0.01};
      std::memcpy(&v[9 * t], tri, sizeof(tri));
    }
    bc_hscene_add_triangles(s, n, v.data(), mats.data());
    for (int k = 0; k < 50; k++) {
      double c[3] = {U(rng) * scale + offset, U(rng) * scale, U(rng) * scale};
      bc_hscene_add_sphere(s, c, 0.01 * scale, m);
    }
    bc_hscene_set_bvh(s, trial % 3 == 0 ? "Median" : "SAH", 32, 1 + trial);
    bc_hscene_build(s);
    rc |= check_scene(s);
    bc_hscene_destroy(s);
  }
  return rc;
}

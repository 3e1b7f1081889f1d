// Host packer: validates a bc_scene_desc and converts the reference's binary
// BVH into the device layout of layout.h (BVH8 collapse, outward-rounded fp32
// boxes, Order-sorted primitive slots).
#pragma once
#include <string>
#include <vector>

#include "../../include/bc_gx.h"
#include "layout.h"

namespace bcgx {

struct PackedScene {
  std::vector<Node8> nodes;
  std::vector<F4> tri;           // 3 per slot
  std::vector<double> slot64;    // 9 per slot
  std::vector<F4> snorm;         // 1 per slot
  std::vector<int32_t> slot_prim;
  std::vector<int32_t> kids8;    // 8 per node: binary node index of each child (-1: empty slot)
  std::vector<BinNode> bin;      // the caller's binary BVH (scene 0 of a set), for exact-tie replay
  std::vector<MatGPU> mats;
  std::vector<LightGPU> lights;
  std::vector<float> light_pdf_by_prim;
  int32_t n_prims = 0, n_binary = 0;
  int32_t depth = 0, stack_need = 0;
  bool has_spheres = false;
  float scene_lo[3] = {0, 0, 0}, scene_hi[3] = {0, 0, 0};
};

// One scene of a resident scene set: where its records start in the
// concatenated arrays.
struct SceneRange {
  int32_t root = 0;                    // Node8 index of its root
  int32_t light_off = 0, n_lights = 0; // its sphere lights in `lights`
  int32_t slot_off = 0, n_slots = 0;
  int32_t prim_off = 0;                // added to its primitive indices (slot_prim, light prims)
  int32_t mat_off = 0;
  double diag = 0;                     // length of the scene's bounds diagonal (photon radius)
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // the scene's bounds (photon grid extent)
};

// Leaf merging in the BVH8 collapse: inner binary subtrees of at most max_leaf
// primitives (one contiguous slot range) may become one leaf, which the
// collapse charges tri_cost * (its box's area) * (its primitives) against a
// node's area. merge: 1 on, 0 off (the binary leaves stay as they are), -1 on
// for scenes of at most kAutoMergePrims primitives. Measured: on the 36-triangle
// Cornell box, whose triangles stay in L1, merging at tri_cost 0.2 leaves most
// rays one node visit (frame +8.6%); on scenes of 1-2M triangles, whose
// triangle records come from L2 and HBM while the nodes stay in L2, the same
// merges cost 1.6% (render) and 2.4% (ray cast).
struct CollapseParams {
  static constexpr int32_t kAutoMergePrims = 1024;
  double tri_cost = 0.2;
  int max_leaf = 8;
  int merge = -1;
  bool merges(int32_t n_prims) const { return merge == 1 || (merge < 0 && n_prims <= kAutoMergePrims); }
};

// Fills `out`; returns BC_OK or BC_ERR_BAD_SCENE / BC_ERR_INVALID_ARG with a message.
bc_status pack_scene(const bc_scene_desc& d, PackedScene* out, std::string* err,
                     const CollapseParams& cp = CollapseParams());
// Packs several scenes into one set of arrays: node references, slots,
// materials and light primitives of scene k are offset past scenes 0..k-1, and
// `ranges[k]` tells where each scene starts. stack_need is the maximum.
bc_status pack_scene_set(const bc_scene_desc* d, int n, PackedScene* out, std::vector<SceneRange>* ranges,
                         std::string* err, const CollapseParams& cp = CollapseParams());
// The caller's binary BVH as BinNode records (validated descriptor).
void pack_binary(const bc_scene_desc& d, std::vector<BinNode>* out);
// Sphere-light records and per-primitive light selection pdfs of a scene.
void pack_scene_lights(const bc_scene_desc& d, PackedScene* out);

// Scene.Bounds() (renderer.go:1137-1146) into r->lo / r->hi and the length of its
// diagonal (1164-1165) into r->diag: the root node box is the union of the
// primitive boxes; a scene without primitives has [-1, 1]^3.
void scene_extent(const bc_scene_desc& d, SceneRange* r);

float round_down_f32(double x);
float round_up_f32(double x);

}  // namespace bcgx

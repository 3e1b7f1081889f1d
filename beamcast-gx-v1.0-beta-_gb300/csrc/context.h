// bc_context internals shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <vector>

#include "../../include/bc_gx.h"
#include "kernels.h"
#include "pack.h"

namespace bcgx {

// Growable device buffer owned by a context.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e == cudaSuccess) cap = bytes;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  template <class T>
  T* as() const { return static_cast<T*>(p); }
};

// Growable pinned host buffer.
struct HostBuf {
  void* p = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    cudaError_t e = cudaHostAlloc(&p, bytes, cudaHostAllocDefault);
    if (e == cudaSuccess) cap = bytes;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
  }
};

// What the geometry-only update needs to know about the resident scene.
struct GeomInfo {
  bool valid = false;  // the resident scene came from bc_scene_upload and kept its BVH8 child map
  int32_t n_binary = 0, n_lights = 0, n_materials = 0, n_node8 = 0;
  bool has_tris = false;
};

}  // namespace bcgx

struct bc_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t aux_stream = nullptr;  // second stream of the pipelined host-buffer ray cast
  std::string err;
  std::string name;
  // resident scene
  bool has_scene = false;
  uint64_t scene_id = 0, topo_rev = 0, geom_rev = 0;
  bcgx::DeviceScene ds;
  bcgx::DevBuf d_nodes, d_tri, d_slot64, d_snorm, d_slot_prim, d_mats, d_lights, d_lpdf, d_bin;
  std::vector<bcgx::SceneRange> ranges;  // scenes of the resident set (one for bc_scene_upload)
  bool is_set = false;                    // resident scenes came from bc_scene_set_upload
  bcgx::GeomInfo geom;                    // geometry-only updates (refit.cu)
  bcgx::DevBuf d_kids8, d_geom;           // Node8 -> binary child map; fp64 geometry staging
  bcgx::DevBuf d_build, d_build_out;      // device SAH build (build.cu)
  bcgx::DevBuf d_post_stack, d_post_hist; // bc_post_stack buffers and temporal history (post.cu)
  struct PostHistory* post_hist = nullptr;
  std::vector<int8_t> mat_kind;           // host copy of the resident materials' kinds
  std::vector<int8_t> mat_is_light;       // 1: material of a sphere light (its emission feeds NEE records)
  int64_t stats[7] = {0, 0, 0, 0, 0, 0, 0};  // bc_scene_stats; [6] counts geometry-only updates
  int raycast_minblocks = 6;  // register budget of the exact ray-cast kernels (bc_set_option)
  int raycast_exact = 1;      // 0: plain fp32 closest hit (bc_set_option "raycast_exact")
  int raycast_variant = 6;    // 0 = fast kernel, else the exact kernel's minblocks
  int raycast_sort = 1;       // trace rays in a spatially coherent order (bc_set_option "raycast_sort")
  long long raycast_chunk = 1 << 21;  // rays per pipelined chunk of bc_raycast (bc_set_option "raycast_chunk")
  bcgx::DevBuf d_order[3];    // ray order scratch: [0], [1] the two streams of bc_raycast, [2] bc_raycast_device
  int raycast_split = 1;      // exact closest hit as walk + settlement passes (bc_set_option "raycast_split")
  bcgx::DevBuf d_rec[3];      // per-ray records of the split passes, indexed as d_order
  bcgx::DevBuf d_rec_any;     // listed rays of the split any-hit passes
  // ray-cast staging
  bcgx::DevBuf d_rays, d_t, d_prim, d_occ;
  unsigned* d_status = nullptr;
  // status word of the device-pointer calls (bc_raycast_device, bc_occluded_device),
  // read and cleared only by bc_sync, so their kernel status reaches their caller
  unsigned* d_status_async = nullptr;
  unsigned test_status_bits = 0;  // bc_set_option "test_status_bits": raised by the next device-pointer call
  // work counters of the persistent ray-cast kernels: [0], [1] the two streams of
  // bc_raycast, [2] bc_raycast_device
  unsigned long long* d_work = nullptr;
  long long render_wave_cap = 1 << 27;  // paths per wave (bc_set_option "render_wave_cap")
  int scene_leaf_merge = -1;            // BVH8 leaf merging of the next upload (bc_set_option "scene_leaf_merge")
  int packed_merge = -1;                // the leaf merging the resident scene was packed with
  int render_graph = 1;                 // replay a captured wave graph (bc_set_option "render_graph")
  int render_engine = 0;                // 0: wave engine, 1: one kernel per view (bc_set_option "render_engine")
  int render_extend = 1;                // k_extend variant 0..2 (bc_set_option "render_extend")
  int render_shade_block = 256;         // k_shade block size, 128 or 256 (bc_set_option "render_shade_block")
  int render_timing = 0;                // per-kernel events in renders (bc_set_option "render_timing")
  bc_timing last_timing{};              // bc_last_timing
  struct DiffState* diff = nullptr;  // differentiable rendering (diff.cu)
  struct PhotonCache* photons = nullptr;  // photon maps of the photon-mapping integrator (photon.cu)
  int photon_grid = 1;                    // gathers read the dense cell table (bc_set_option "photon_grid")
  uint64_t scene_gen = 0;                 // bumped by every scene or geometry upload
  // rendering state (render.cu)
  struct RenderBuffers* rb = nullptr;
  std::atomic<int> cancel{0};
  int* h_cancel = nullptr;  // host-mapped cancel flag read by device loops
  int* d_cancel = nullptr;
};

namespace bcgx {
bc_status set_error(bc_context* ctx, bc_status st, const std::string& msg);
bc_status cuda_status(bc_context* ctx, cudaError_t e, const char* what);
bc_status check_kernel_status(bc_context* ctx);
bc_status check_status_word(bc_context* ctx, unsigned* d_word, cudaStream_t stream);
void destroy_render_buffers(bc_context* ctx);
void destroy_diff_state(bc_context* ctx);
void destroy_post_state(bc_context* ctx);
void destroy_photon_state(bc_context* ctx);
bc_status update_geometry(bc_context* ctx, const bc_scene_desc& d);  // refit.cu
}  // namespace bcgx

// C-ABI: context lifetime, scene upload and the ray-cast entry points.
// Mirrors the call sequence of renderOpenCL (gpu_opencl_windows.go:565-720):
// init once, ensure the scene by revision, then launch and read back.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>

#include "context.h"

namespace bcgx {

static thread_local std::string g_tls_error;

bc_status set_error(bc_context* ctx, bc_status st, const std::string& msg) {
  if (ctx) ctx->err = msg;
  g_tls_error = msg;
  return st;
}

bc_status cuda_status(bc_context* ctx, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return BC_OK;
  std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  cudaGetLastError();  // clear a non-sticky error
  return set_error(ctx, e == cudaErrorMemoryAllocation ? BC_ERR_OOM : BC_ERR_DEVICE, m);
}

// Reads and clears a kernel status word once `stream` has drained.
bc_status check_status_word(bc_context* ctx, unsigned* d_word, cudaStream_t stream) {
  unsigned h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, d_word, sizeof(unsigned), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_status(ctx, e, "reading kernel status");
  if (h == 0) return BC_OK;
  cudaMemsetAsync(d_word, 0, sizeof(unsigned), stream);
  cudaStreamSynchronize(stream);
  if (h & kStatusStackOverflow)
    return set_error(ctx, BC_ERR_CAPACITY, "traversal stack overflow (scene deeper than the compiled stack)");
  if (h & kStatusTimeout) return set_error(ctx, BC_ERR_TIMEOUT, "a bounded device wait gave up");
  if (h & kStatusCapacity) return set_error(ctx, BC_ERR_CAPACITY, "a device queue exceeded its capacity");
  if (h & kStatusBound) return set_error(ctx, BC_ERR_DEVICE, "fp32 error bound violated by an fp64 re-test");
  return set_error(ctx, BC_ERR_DEVICE, "unknown kernel status");
}

// Status of the host-buffer calls and renders (their own word, on the context's stream).
bc_status check_kernel_status(bc_context* ctx) { return check_status_word(ctx, ctx->d_status, ctx->stream); }

// Test hook of the device-pointer calls: ORs bits into their status word on
// their stream, as a kernel that hit a stack or queue limit would.
static __global__ void k_raise_status(unsigned* word, unsigned bits) { atomicOr(word, bits); }

static cudaError_t raise_test_status(bc_context* ctx, cudaStream_t st) {
  if (!ctx->test_status_bits) return cudaSuccess;
  k_raise_status<<<1, 1, 0, st>>>(ctx->d_status_async, ctx->test_status_bits);
  ctx->test_status_bits = 0;
  return cudaGetLastError();
}

static bc_status upload(bc_context* ctx, DevBuf& b, const void* src, size_t bytes, const char* what) {
  cudaError_t e = b.ensure(bytes ? bytes : 16);
  if (e != cudaSuccess) return cuda_status(ctx, e, what);
  if (bytes) {
    e = cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_status(ctx, e, what);
  }
  return BC_OK;
}

}  // namespace bcgx

using namespace bcgx;

extern "C" {

int bc_gpu_available(char* reason, size_t reason_len) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  std::string msg;
  int ok = 0;
  if (e != cudaSuccess) {
    msg = std::string("CUDA unavailable: ") + cudaGetErrorString(e);
    cudaGetLastError();
  } else if (n == 0) {
    msg = "no CUDA device";
  } else {
    cudaDeviceProp p;
    cudaGetDeviceProperties(&p, 0);
    if (p.major == 10 && p.minor == 3) {
      ok = 1;
      msg = std::string("CUDA GPU: ") + p.name;
    } else {
      msg = std::string("device 0 (") + p.name + ") is sm_" + std::to_string(p.major) + std::to_string(p.minor) +
            "; the library is compiled for sm_103a";
    }
  }
  if (reason && reason_len) {
    std::snprintf(reason, reason_len, "%s", msg.c_str());
  }
  return ok;
}

bc_status bc_create(int device_ordinal, bc_context** out) {
  if (!out) return set_error(nullptr, BC_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0 || device_ordinal < 0 || device_ordinal >= n) {
    cudaGetLastError();
    return set_error(nullptr, BC_ERR_NO_DEVICE, "no usable CUDA device at that ordinal");
  }
  cudaDeviceProp p;
  e = cudaGetDeviceProperties(&p, device_ordinal);
  if (e != cudaSuccess) return set_error(nullptr, BC_ERR_NO_DEVICE, cudaGetErrorString(e));
  if (!(p.major == 10 && p.minor == 3))
    return set_error(nullptr, BC_ERR_NO_DEVICE, std::string("device is not sm_103: ") + p.name);
  bc_context* ctx = new (std::nothrow) bc_context();
  if (!ctx) return set_error(nullptr, BC_ERR_OOM, "host allocation failed");
  ctx->device = device_ordinal;
  ctx->name = p.name;
  e = cudaSetDevice(device_ordinal);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_status, 2 * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(ctx->d_status, 0, 2 * sizeof(unsigned));
  if (e == cudaSuccess) ctx->d_status_async = ctx->d_status + 1;
  if (e == cudaSuccess) e = cudaMalloc(&ctx->d_work, 64);
  if (e == cudaSuccess) {
    e = cudaMemset(ctx->d_work, 0, 64);
  }
  if (e == cudaSuccess) e = cudaHostAlloc((void**)&ctx->h_cancel, sizeof(int), cudaHostAllocMapped);
  if (e == cudaSuccess) {
    *ctx->h_cancel = 0;
    e = cudaHostGetDevicePointer((void**)&ctx->d_cancel, ctx->h_cancel, 0);
  }
  if (e != cudaSuccess) {
    bc_status st = cuda_status(nullptr, e, "context creation");
    bc_destroy(ctx);
    return st;
  }
  *out = ctx;
  return BC_OK;
}

void bc_destroy(bc_context* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  destroy_render_buffers(ctx);
  destroy_diff_state(ctx);
  destroy_post_state(ctx);
  destroy_photon_state(ctx);
  for (DevBuf* b : {&ctx->d_nodes, &ctx->d_tri, &ctx->d_slot64, &ctx->d_snorm, &ctx->d_slot_prim, &ctx->d_mats,
                    &ctx->d_lights, &ctx->d_lpdf, &ctx->d_bin, &ctx->d_rays, &ctx->d_t, &ctx->d_prim, &ctx->d_occ,
                    &ctx->d_kids8, &ctx->d_geom, &ctx->d_build, &ctx->d_build_out, &ctx->d_order[0],
                    &ctx->d_order[1], &ctx->d_order[2], &ctx->d_rec[0], &ctx->d_rec[1], &ctx->d_rec[2],
                    &ctx->d_rec_any})
    b->release();
  if (ctx->d_status) cudaFree(ctx->d_status);
  if (ctx->d_work) cudaFree(ctx->d_work);
  if (ctx->h_cancel) cudaFreeHost(ctx->h_cancel);
  if (ctx->aux_stream) cudaStreamDestroy(ctx->aux_stream);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

bc_status bc_last_error(const bc_context* ctx, char* buf, size_t len) {
  if (!buf || !len) return BC_ERR_INVALID_ARG;
  const std::string& m = ctx ? ctx->err : g_tls_error;
  std::snprintf(buf, len, "%s", m.c_str());
  return BC_OK;
}

bc_status bc_device_name(const bc_context* ctx, char* buf, size_t len) {
  if (!ctx || !buf || !len) return BC_ERR_INVALID_ARG;
  std::snprintf(buf, len, "%s", ctx->name.c_str());
  return BC_OK;
}

}  // extern "C"

namespace bcgx {

// Makes `ps` the resident scene set.
static bc_status install_scene(bc_context* ctx, const PackedScene& ps, const std::vector<SceneRange>& ranges) {
  if (stack_variant(ps.stack_need) == 0)
    return set_error(ctx, BC_ERR_BAD_SCENE,
                     "BVH too deep for the compiled traversal stack (needs " + std::to_string(ps.stack_need) + ")");
  // The stream may still be reading the previous scene.
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(ctx, e, "scene upload");
  ctx->has_scene = false;
  ctx->ranges.clear();
  ctx->geom.valid = false;
  ctx->scene_gen++;
  const size_t slots = (size_t)ps.n_prims;
  bc_status st;
  if ((st = upload(ctx, ctx->d_nodes, ps.nodes.data(), ps.nodes.size() * sizeof(Node8), "BVH8 upload")) ||
      (st = upload(ctx, ctx->d_tri, ps.tri.data(), ps.tri.size() * sizeof(F4), "primitive upload")) ||
      (st = upload(ctx, ctx->d_slot64, ps.slot64.data(), ps.slot64.size() * sizeof(double), "fp64 upload")) ||
      (st = upload(ctx, ctx->d_snorm, ps.snorm.data(), ps.snorm.size() * sizeof(F4), "normal upload")) ||
      (st = upload(ctx, ctx->d_slot_prim, ps.slot_prim.data(), slots * sizeof(int32_t), "order upload")) ||
      (st = upload(ctx, ctx->d_mats, ps.mats.data(), ps.mats.size() * sizeof(MatGPU), "material upload")) ||
      (st = upload(ctx, ctx->d_lights, ps.lights.data(), ps.lights.size() * sizeof(LightGPU), "light upload")) ||
      (st = upload(ctx, ctx->d_lpdf, ps.light_pdf_by_prim.data(), ps.light_pdf_by_prim.size() * sizeof(float),
                   "light pdf upload")) ||
      (st = upload(ctx, ctx->d_bin, ps.bin.data(), ps.bin.size() * sizeof(BinNode), "binary BVH upload")))
    return st;
  // The host arrays of `ps` may die once this returns: drain the copies first.
  e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(ctx, e, "scene upload");
  DeviceScene& ds = ctx->ds;
  ds.nodes = ctx->d_nodes.as<Node8>();
  ds.tri = ctx->d_tri.as<float4>();
  ds.slot64 = ctx->d_slot64.as<double>();
  ds.snorm = ctx->d_snorm.as<float4>();
  ds.slot_prim = ctx->d_slot_prim.as<int32_t>();
  ds.mats = ctx->d_mats.as<MatGPU>();
  ds.lights = ctx->d_lights.as<LightGPU>();
  ds.light_pdf_by_prim = ctx->d_lpdf.as<float>();
  ds.bin = ctx->d_bin.as<BinNode>();
  ds.n_bin = (int32_t)ps.bin.size();
  ds.n_mats = (int32_t)ps.mats.size();
  ds.n_lights = ranges.empty() ? 0 : ranges[0].n_lights;  // the single-view calls see scene 0
  ds.n_prims = ps.n_prims;
  ds.stack_need = ps.stack_need;
  ds.has_spheres = ps.has_spheres;
  for (int k = 0; k < 3; k++) {
    ds.lo[k] = ps.scene_lo[k];
    ds.hi[k] = ps.scene_hi[k];
  }
  ctx->stats[0] = (int64_t)ps.nodes.size();
  ctx->stats[1] = ps.n_prims;
  ctx->stats[2] = ps.n_binary;
  ctx->stats[3] = ps.depth;
  ctx->stats[4] = ps.stack_need;
  ctx->stats[5] = (int64_t)(ps.nodes.size() * sizeof(Node8) + ps.tri.size() * sizeof(F4) +
                            ps.slot64.size() * sizeof(double) + ps.snorm.size() * sizeof(F4) +
                            slots * sizeof(int32_t) + ps.mats.size() * sizeof(MatGPU) +
                            ps.lights.size() * sizeof(LightGPU) + ps.light_pdf_by_prim.size() * sizeof(float) +
                            ps.bin.size() * sizeof(BinNode));
  ctx->mat_kind.assign(ps.mats.size(), 0);
  for (size_t i = 0; i < ps.mats.size(); i++) ctx->mat_kind[i] = (int8_t)ps.mats[i].kind;
  ctx->mat_is_light.assign(ps.mats.size(), 0);
  if (!ps.lights.empty()) {
    std::vector<int32_t> slot_of(ps.n_prims, -1);
    for (int32_t sl = 0; sl < ps.n_prims; sl++)
      if (ps.slot_prim[sl] >= 0 && ps.slot_prim[sl] < ps.n_prims) slot_of[ps.slot_prim[sl]] = sl;
    for (const LightGPU& L : ps.lights) {
      const int32_t sl = (L.prim >= 0 && L.prim < ps.n_prims) ? slot_of[L.prim] : -1;
      if (sl < 0) continue;
      int32_t m;
      std::memcpy(&m, &ps.snorm[sl].w, 4);
      if (m >= 0 && m < (int32_t)ps.mats.size()) ctx->mat_is_light[m] = 1;
    }
  }
  ctx->ranges = ranges;
  ctx->has_scene = true;
  return BC_OK;
}

// Keeps what a later geometry-only update of this (single) scene needs.
static bc_status keep_geometry_map(bc_context* ctx, const bc_scene_desc& d, const PackedScene& ps) {
  if (ps.kids8.size() != 8 * ps.nodes.size()) return BC_OK;
  bc_status st = upload(ctx, ctx->d_kids8, ps.kids8.data(), ps.kids8.size() * sizeof(int32_t), "child map upload");
  if (st) return st;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e) return cuda_status(ctx, e, "child map upload");
  GeomInfo& g = ctx->geom;
  g.n_binary = d.n_nodes;
  g.n_lights = d.n_lights;
  g.n_materials = d.n_materials;
  g.n_node8 = (int32_t)ps.nodes.size();
  g.has_tris = false;
  for (int32_t i = 0; i < d.n_prims && !g.has_tris; i++) g.has_tris = d.prim_kind[i] == BC_PRIM_TRIANGLE;
  g.valid = true;
  return BC_OK;
}

}  // namespace bcgx

extern "C" {

bc_status bc_scene_upload(bc_context* ctx, const bc_scene_desc* scene, uint64_t scene_id, uint64_t topology_rev,
                          uint64_t geometry_rev) {
  if (!ctx || !scene) return set_error(ctx, BC_ERR_INVALID_ARG, "NULL context or scene");
  const bool same_pack = ctx->packed_merge == ctx->scene_leaf_merge;
  if (ctx->has_scene && !ctx->is_set && ctx->scene_id == scene_id && ctx->topo_rev == topology_rev &&
      ctx->geom_rev == geometry_rev && same_pack)
    return BC_OK;
  cudaSetDevice(ctx->device);
  bc_status st;
  if (ctx->has_scene && !ctx->is_set && ctx->scene_id == scene_id && ctx->topo_rev == topology_rev && same_pack) {
    // only the geometry moved: rewrite primitives and node boxes on the device
    st = update_geometry(ctx, *scene);
    if (st == BC_OK) {
      scene_extent(*scene, &ctx->ranges[0]);
      ctx->scene_gen++;  // cached photon maps of the old geometry are stale
      ctx->geom_rev = geometry_rev;
      ctx->stats[6]++;
      return BC_OK;
    }
    if (st != BC_ERR_INVALID_ARG) return st;  // a device error; the descriptor itself did not fit: full upload
  }
  PackedScene ps;
  std::string err;
  CollapseParams cp;
  cp.merge = ctx->scene_leaf_merge;
  st = pack_scene(*scene, &ps, &err, cp);
  if (st != BC_OK) return set_error(ctx, st, err);
  SceneRange r;
  r.n_lights = (int32_t)ps.lights.size();
  r.n_slots = ps.n_prims;
  scene_extent(*scene, &r);
  if ((st = install_scene(ctx, ps, std::vector<SceneRange>{r}))) return st;
  if ((st = keep_geometry_map(ctx, *scene, ps))) return st;
  ctx->packed_merge = cp.merge;
  ctx->is_set = false;
  ctx->scene_id = scene_id;
  ctx->topo_rev = topology_rev;
  ctx->geom_rev = geometry_rev;
  return BC_OK;
}

bc_status bc_scene_set_upload(bc_context* ctx, const bc_scene_desc* scenes, int32_t n_scenes, uint64_t set_id,
                              uint64_t revision) {
  if (!ctx || !scenes || n_scenes < 1) return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument or empty set");
  if (ctx->has_scene && ctx->is_set && ctx->scene_id == set_id && ctx->geom_rev == revision &&
      (int32_t)ctx->ranges.size() == n_scenes && ctx->packed_merge == ctx->scene_leaf_merge)
    return BC_OK;
  cudaSetDevice(ctx->device);
  PackedScene ps;
  std::vector<SceneRange> ranges;
  std::string err;
  CollapseParams cp;
  cp.merge = ctx->scene_leaf_merge;
  bc_status st = pack_scene_set(scenes, n_scenes, &ps, &ranges, &err, cp);
  if (st != BC_OK) return set_error(ctx, st, err);
  if ((st = install_scene(ctx, ps, ranges))) return st;
  ctx->packed_merge = cp.merge;
  ctx->is_set = true;
  ctx->scene_id = set_id;
  ctx->topo_rev = 0;
  ctx->geom_rev = revision;
  return BC_OK;
}

bc_status bc_scene_stats(const bc_context* ctx, int64_t* out, int n_out) {
  if (!ctx || !out || n_out < 0) return BC_ERR_INVALID_ARG;
  if (!ctx->has_scene) return BC_ERR_NO_SCENE;
  for (int i = 0; i < n_out && i < 7; i++) out[i] = ctx->stats[i];
  return BC_OK;
}

bc_status bc_raycast_device(bc_context* ctx, const float* d_rays, int64_t n, float* d_t_out, int32_t* d_prim_out,
                            void* stream) {
  if (!ctx) return set_error(nullptr, BC_ERR_INVALID_ARG, "NULL context");
  if (n < 0 || (n > 0 && (!d_rays || !d_t_out || !d_prim_out)))
    return set_error(ctx, BC_ERR_INVALID_ARG, "bad ray-cast arguments");
  if (((uintptr_t)d_rays & 15u) != 0) return set_error(ctx, BC_ERR_INVALID_ARG, "rays must be 16-byte aligned");
  if (!ctx->has_scene) return set_error(ctx, BC_ERR_NO_SCENE, "no scene uploaded");
  cudaSetDevice(ctx->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  void* order = nullptr;
  if (ctx->raycast_sort && n >= kMinOrderedRays && n < (int64_t(1) << 31)) {
    cudaError_t e = ctx->d_order[2].ensure(ray_order_bytes(n));
    if (e) return cuda_status(ctx, e, "ray order buffers");
    order = ctx->d_order[2].p;
  }
  void* rec = nullptr;
  if (ctx->raycast_split && ctx->raycast_exact && n > 0) {
    cudaError_t e = ctx->d_rec[2].ensure(exact_record_bytes(n));
    if (e) return cuda_status(ctx, e, "ray-cast record buffers");
    rec = ctx->d_rec[2].p;
  }
  cudaError_t e = launch_raycast_closest(ctx->ds, (const float4*)d_rays, n, d_t_out, d_prim_out,
                                         ctx->d_status_async, ctx->d_work + 2, ctx->raycast_variant, order, rec, st);
  if (e == cudaSuccess) e = raise_test_status(ctx, st);
  return cuda_status(ctx, e, "ray-cast launch");
}

// Host-buffer ray cast, pipelined: the rays go in chunks of raycast_chunk rays
// (default 2 Mi) over two streams, so the copy of chunk c+1 in, the kernel on chunk c and the copy of
// chunk c-1 out overlap (copy engines and SMs work at the same time).
bc_status bc_raycast(bc_context* ctx, const float* rays, int64_t n, float* t_out, int32_t* prim_out) {
  if (!ctx) return set_error(nullptr, BC_ERR_INVALID_ARG, "NULL context");
  if (n < 0 || (n > 0 && (!rays || !t_out || !prim_out))) return set_error(ctx, BC_ERR_INVALID_ARG, "bad ray-cast arguments");
  if (!ctx->has_scene) return set_error(ctx, BC_ERR_NO_SCENE, "no scene uploaded");
  if (n == 0) return BC_OK;
  cudaSetDevice(ctx->device);
  cudaError_t e;
  if ((e = ctx->d_rays.ensure((size_t)n * 32)) || (e = ctx->d_t.ensure((size_t)n * 4)) ||
      (e = ctx->d_prim.ensure((size_t)n * 4)))
    return cuda_status(ctx, e, "ray-cast buffers");
  if (!ctx->aux_stream) {
    e = cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_status(ctx, e, "ray-cast stream");
  }
  const int64_t chunk = ctx->raycast_chunk;
  cudaStream_t streams[2] = {ctx->stream, ctx->aux_stream};
  void* order[2] = {nullptr, nullptr};
  if (ctx->raycast_sort && n >= kMinOrderedRays)
    for (int k = 0; k < 2; k++) {
      if ((e = ctx->d_order[k].ensure(ray_order_bytes(std::min(chunk, n))))) return cuda_status(ctx, e, "ray order buffers");
      order[k] = ctx->d_order[k].p;
    }
  void* rec[2] = {nullptr, nullptr};
  if (ctx->raycast_split && ctx->raycast_exact)
    for (int k = 0; k < 2; k++) {
      if ((e = ctx->d_rec[k].ensure(exact_record_bytes(std::min(chunk, n))))) return cuda_status(ctx, e, "ray-cast record buffers");
      rec[k] = ctx->d_rec[k].p;
    }
  for (int64_t off = 0, c = 0; off < n && e == cudaSuccess; off += chunk, c++) {
    const int64_t m = std::min(chunk, n - off);
    cudaStream_t st = streams[c & 1];
    float4* dr = ctx->d_rays.as<float4>() + 2 * off;
    e = cudaMemcpyAsync(dr, rays + 8 * off, (size_t)m * 32, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
      e = launch_raycast_closest(ctx->ds, dr, m, ctx->d_t.as<float>() + off, ctx->d_prim.as<int32_t>() + off,
                                 ctx->d_status, ctx->d_work + (c & 1), ctx->raycast_variant, order[c & 1], rec[c & 1],
                                 st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(t_out + off, ctx->d_t.as<float>() + off, (size_t)m * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(prim_out + off, ctx->d_prim.as<int32_t>() + off, (size_t)m * 4, cudaMemcpyDeviceToHost, st);
  }
  cudaError_t e2 = cudaStreamSynchronize(ctx->aux_stream);
  cudaError_t e1 = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = e1 != cudaSuccess ? e1 : e2;
  if (e != cudaSuccess) return cuda_status(ctx, e, "ray cast");
  return check_kernel_status(ctx);
}

bc_status bc_occluded_device(bc_context* ctx, const float* d_rays, int64_t n, uint8_t* d_out, void* stream) {
  if (!ctx) return set_error(nullptr, BC_ERR_INVALID_ARG, "NULL context");
  if (n < 0 || (n > 0 && (!d_rays || !d_out))) return set_error(ctx, BC_ERR_INVALID_ARG, "bad any-hit arguments");
  if (((uintptr_t)d_rays & 15u) != 0) return set_error(ctx, BC_ERR_INVALID_ARG, "rays must be 16-byte aligned");
  if (!ctx->has_scene) return set_error(ctx, BC_ERR_NO_SCENE, "no scene uploaded");
  cudaSetDevice(ctx->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  void* rec = nullptr;
  void* order = nullptr;
  if (ctx->raycast_split && n > 0) {
    cudaError_t e = ctx->d_rec_any.ensure(any_record_bytes(n));
    if (e) return cuda_status(ctx, e, "any-hit record buffers");
    rec = ctx->d_rec_any.p;
    if (ctx->raycast_sort && n >= kMinOrderedRays && n < (int64_t(1) << 31)) {
      if ((e = ctx->d_order[2].ensure(ray_order_bytes(n)))) return cuda_status(ctx, e, "ray order buffers");
      order = ctx->d_order[2].p;
    }
  }
  cudaError_t e = launch_raycast_any(ctx->ds, (const float4*)d_rays, n, d_out, ctx->d_status_async,
                                     ctx->raycast_variant, ctx->d_work + 3, rec, order, st);
  if (e == cudaSuccess) e = raise_test_status(ctx, st);
  return cuda_status(ctx, e, "any-hit launch");
}

bc_status bc_sync(bc_context* ctx, void* stream) {
  if (!ctx) return set_error(nullptr, BC_ERR_INVALID_ARG, "NULL context");
  cudaSetDevice(ctx->device);
  return check_status_word(ctx, ctx->d_status_async, stream ? (cudaStream_t)stream : ctx->stream);
}

bc_status bc_occluded(bc_context* ctx, const float* rays, int64_t n, uint8_t* out) {
  if (!ctx) return set_error(nullptr, BC_ERR_INVALID_ARG, "NULL context");
  if (n < 0 || (n > 0 && (!rays || !out))) return set_error(ctx, BC_ERR_INVALID_ARG, "bad any-hit arguments");
  if (!ctx->has_scene) return set_error(ctx, BC_ERR_NO_SCENE, "no scene uploaded");
  if (n == 0) return BC_OK;
  cudaSetDevice(ctx->device);
  cudaError_t e;
  if ((e = ctx->d_rays.ensure((size_t)n * 32)) || (e = ctx->d_occ.ensure((size_t)n)))
    return cuda_status(ctx, e, "any-hit buffers");
  void* rec = nullptr;
  void* order = nullptr;
  if (ctx->raycast_split) {
    if ((e = ctx->d_rec_any.ensure(any_record_bytes(n)))) return cuda_status(ctx, e, "any-hit record buffers");
    rec = ctx->d_rec_any.p;
    if (ctx->raycast_sort && n >= kMinOrderedRays && n < (int64_t(1) << 31)) {
      if ((e = ctx->d_order[2].ensure(ray_order_bytes(n)))) return cuda_status(ctx, e, "ray order buffers");
      order = ctx->d_order[2].p;
    }
  }
  e = cudaMemcpyAsync(ctx->d_rays.p, rays, (size_t)n * 32, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = launch_raycast_any(ctx->ds, ctx->d_rays.as<float4>(), n, ctx->d_occ.as<uint8_t>(), ctx->d_status, ctx->raycast_variant,
                           ctx->d_work + 3, rec, order, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, ctx->d_occ.p, (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(ctx, e, "any hit");
  return check_kernel_status(ctx);
}

bc_status bc_set_option(bc_context* ctx, const char* name, int64_t value) {
  if (!ctx || !name) return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument");
  const std::string n(name);
  if (n == "raycast_minblocks") {
    if (value != 1 && value != 6 && value != 8)
      return set_error(ctx, BC_ERR_INVALID_ARG, "raycast_minblocks must be 1, 6 or 8");
    ctx->raycast_minblocks = (int)value;
    ctx->raycast_variant = ctx->raycast_exact ? (int)value : 0;
    return BC_OK;
  }
  if (n == "raycast_exact") {
    if (value != 0 && value != 1) return set_error(ctx, BC_ERR_INVALID_ARG, "raycast_exact must be 0 or 1");
    ctx->raycast_exact = (int)value;
    ctx->raycast_variant = value ? ctx->raycast_minblocks : 0;
    return BC_OK;
  }
  if (n == "raycast_sort") {
    if (value != 0 && value != 1) return set_error(ctx, BC_ERR_INVALID_ARG, "raycast_sort must be 0 or 1");
    ctx->raycast_sort = (int)value;
    return BC_OK;
  }
  if (n == "raycast_split") {
    if (value != 0 && value != 1) return set_error(ctx, BC_ERR_INVALID_ARG, "raycast_split must be 0 or 1");
    ctx->raycast_split = (int)value;
    return BC_OK;
  }
  if (n == "photon_grid") {
    if (value != 0 && value != 1) return set_error(ctx, BC_ERR_INVALID_ARG, "photon_grid must be 0 or 1");
    ctx->photon_grid = (int)value;
    return BC_OK;
  }
  if (n == "test_status_bits") {  // test hook: the next device-pointer call raises these status bits
    if (value < 0 || value > 0xffffffffLL) return set_error(ctx, BC_ERR_INVALID_ARG, "test_status_bits is 32 bits");
    ctx->test_status_bits = (unsigned)value;
    return BC_OK;
  }
  if (n == "raycast_chunk") {
    if (value < 65536 || value > (1LL << 28))
      return set_error(ctx, BC_ERR_INVALID_ARG, "raycast_chunk must be in [65536, 2^28]");
    ctx->raycast_chunk = (long long)value;
    return BC_OK;
  }
  if (n == "render_wave_cap") {
    if (value < 4096 || value > (1 << 27))
      return set_error(ctx, BC_ERR_INVALID_ARG, "render_wave_cap must be in [4096, 2^27]");
    ctx->render_wave_cap = (long long)value;
    return BC_OK;
  }
  if (n == "render_graph") {
    if (value != 0 && value != 1) return set_error(ctx, BC_ERR_INVALID_ARG, "render_graph must be 0 or 1");
    ctx->render_graph = (int)value;
    return BC_OK;
  }
  if (n == "render_engine") {
    if (value != 0 && value != 1) return set_error(ctx, BC_ERR_INVALID_ARG, "render_engine must be 0 or 1");
    ctx->render_engine = (int)value;
    return BC_OK;
  }
  if (n == "render_extend") {
    if (value < 0 || value > 2) return set_error(ctx, BC_ERR_INVALID_ARG, "render_extend must be 0, 1 or 2");
    ctx->render_extend = (int)value;
    return BC_OK;
  }
  if (n == "render_shade_block") {
    if (value != 128 && value != 256) return set_error(ctx, BC_ERR_INVALID_ARG, "render_shade_block must be 128 or 256");
    ctx->render_shade_block = (int)value;
    return BC_OK;
  }
  if (n == "render_timing") {
    if (value != 0 && value != 1) return set_error(ctx, BC_ERR_INVALID_ARG, "render_timing must be 0 or 1");
    ctx->render_timing = (int)value;
    return BC_OK;
  }
  if (n == "scene_leaf_merge") {
    if (value < -1 || value > 1) return set_error(ctx, BC_ERR_INVALID_ARG, "scene_leaf_merge must be -1, 0 or 1");
    ctx->scene_leaf_merge = (int)value;
    return BC_OK;
  }
  return set_error(ctx, BC_ERR_INVALID_ARG, "unknown option " + n);
}

bc_status bc_get_option(const bc_context* ctx, const char* name, int64_t* value) {
  if (!ctx || !name || !value) return BC_ERR_INVALID_ARG;
  const std::string n(name);
  if (n == "raycast_minblocks") { *value = ctx->raycast_minblocks; return BC_OK; }
  if (n == "raycast_exact") { *value = ctx->raycast_exact; return BC_OK; }
  if (n == "render_wave_cap") { *value = ctx->render_wave_cap; return BC_OK; }
  if (n == "raycast_sort") { *value = ctx->raycast_sort; return BC_OK; }
  if (n == "raycast_split") { *value = ctx->raycast_split; return BC_OK; }
  if (n == "raycast_chunk") { *value = ctx->raycast_chunk; return BC_OK; }
  if (n == "photon_grid") { *value = ctx->photon_grid; return BC_OK; }
  if (n == "render_graph") { *value = ctx->render_graph; return BC_OK; }
  if (n == "render_engine") { *value = ctx->render_engine; return BC_OK; }
  if (n == "render_extend") { *value = ctx->render_extend; return BC_OK; }
  if (n == "render_shade_block") { *value = ctx->render_shade_block; return BC_OK; }
  if (n == "render_timing") { *value = ctx->render_timing; return BC_OK; }
  if (n == "scene_leaf_merge") { *value = ctx->scene_leaf_merge; return BC_OK; }
  return BC_ERR_INVALID_ARG;
}

bc_status bc_last_timing(const bc_context* ctx, bc_timing* out) {
  if (!ctx || !out) return BC_ERR_INVALID_ARG;
  *out = ctx->last_timing;
  return BC_OK;
}

bc_status bc_cancel(bc_context* ctx) {
  if (!ctx) return BC_ERR_INVALID_ARG;
  ctx->cancel.store(1);
  if (ctx->h_cancel) *(volatile int*)ctx->h_cancel = 1;
  return BC_OK;
}

bc_status bc_reset_cancel(bc_context* ctx) {
  if (!ctx) return BC_ERR_INVALID_ARG;
  ctx->cancel.store(0);
  if (ctx->h_cancel) *(volatile int*)ctx->h_cancel = 0;
  return BC_OK;
}

}  // extern "C"

// Host-side launchers of the CUDA kernels (one declaration per kernel family).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "layout.h"

namespace bcgx {

struct DeviceScene {
  const Node8* nodes = nullptr;
  const float4* tri = nullptr;
  const double* slot64 = nullptr;
  const float4* snorm = nullptr;
  const int32_t* slot_prim = nullptr;
  const MatGPU* mats = nullptr;
  const LightGPU* lights = nullptr;
  const float* light_pdf_by_prim = nullptr;
  const BinNode* bin = nullptr;  // the caller's binary BVH of scene 0 (exact-tie replay)
  int32_t n_bin = 0;
  int32_t n_mats = 0, n_lights = 0, n_prims = 0;
  int32_t stack_need = 0;
  bool has_spheres = false;
  float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // scene bounds (ray order grid)
};

// Picks the smallest compiled stack size >= need; 0 if none fits.
int stack_variant(int need);

// Exact closest hit over n rays (8 floats each); see bc_raycast in bc_gx.h.
// `work` is an 8-byte device counter private to this launch's stream (persistent kernels).
// order_scratch (ray_order_bytes(n) bytes, or NULL): rays are traced in a
// spatially coherent order (batches of at least kMinOrderedRays rays).
// rec_scratch (exact_record_bytes(n) bytes, or NULL): the exact closest hit of
// a triangle-only scene runs as separate walk and fp64 settlement passes.
constexpr int64_t kMinOrderedRays = 65536;
size_t ray_order_bytes(int64_t n);
size_t exact_record_bytes(int64_t n);
cudaError_t launch_raycast_closest(const DeviceScene& s, const float4* rays, int64_t n, float* t_out,
                                   int32_t* prim_out, unsigned* status, unsigned long long* work, int variant,
                                   void* order_scratch, void* rec_scratch, cudaStream_t st);
// Exact any hit. rec_scratch (any_record_bytes(n) bytes) and `work` (as for the
// closest hit), or NULL: a triangle-only scene runs as walk and fp64 passes,
// in the coherent ray order when order_scratch (ray_order_bytes(n)) is given.
size_t any_record_bytes(int64_t n);
cudaError_t launch_raycast_any(const DeviceScene& s, const float4* rays, int64_t n, uint8_t* out, unsigned* status,
                               int variant, unsigned long long* work, void* rec_scratch, void* order_scratch,
                               cudaStream_t st);

}  // namespace bcgx

// Ray-cast kernels: exact closest hit and any hit over the BVH8, one thread
// per ray. Rays are 32-byte records (ox, oy, oz, tmin, dx, dy, dz, tmax) read
// with two 128-bit loads; results are written as coalesced 4-byte streams.
#include "kernels.h"
#include "trace_core.cuh"

namespace bcgx {

int stack_variant(int need) {
  if (need <= 64) return 64;
  if (need <= 128) return 128;
  if (need <= 256) return 256;
  return 0;
}

namespace {

template <int STACK, bool SPHERES, int MINB>
__global__ void __launch_bounds__(128, MINB) k_closest_exact(SceneView sv, const float4* __restrict__ rays, int64_t n,
                                                       float* __restrict__ t_out, int32_t* __restrict__ prim_out,
                                                       unsigned* status) {
  // No early return: every lane reaches the warp-converged fp64 settlement.
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = i < n;
  float4 a = make_float4(0, 0, 0, 0), b = a;
  if (active) {
    a = __ldg(rays + 2 * i);
    b = __ldg(rays + 2 * i + 1);
  }
  const Ray32 r = make_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w);
  const HitResult h = closest_hit_exact<STACK, SPHERES>(sv, r, b.w, status, active);
  if (!active) return;
  if (h.slot >= 0) {
    t_out[i] = __double2float_rn(h.t64);
    prim_out[i] = __ldg(sv.slot_prim + h.slot);
  } else {
    t_out[i] = -1.0f;
    prim_out[i] = -1;
  }
}

template <int STACK, bool SPHERES, int MINB>
__global__ void __launch_bounds__(128, MINB) k_any_exact(SceneView sv, const float4* __restrict__ rays, int64_t n,
                                                   uint8_t* __restrict__ out, unsigned* status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = __ldg(rays + 2 * i);
  const float4 b = __ldg(rays + 2 * i + 1);
  const Ray32 r = make_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w);
  out[i] = any_hit_exact<STACK, SPHERES>(sv, r, b.w, status) ? 1 : 0;
}

// Fast variant: the same walk with plain fp32 tests (no exactness contract:
// near ties and edge grazes may differ from the fp64 path).
template <int STACK, bool SPHERES>
__global__ void __launch_bounds__(128) k_closest_fast(SceneView sv, const float4* __restrict__ rays, int64_t n,
                                                      float* __restrict__ t_out, int32_t* __restrict__ prim_out,
                                                      unsigned* status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 a = __ldg(rays + 2 * i);
  const float4 b = __ldg(rays + 2 * i + 1);
  const Ray32 r = make_ray(a.x, a.y, a.z, b.x, b.y, b.z, a.w);
  const HitResult h = closest_hit_fast<STACK, SPHERES>(sv, r, b.w, status);
  t_out[i] = h.slot >= 0 ? h.t32 : -1.0f;
  prim_out[i] = h.slot >= 0 ? __ldg(sv.slot_prim + h.slot) : -1;
}

SceneView view_of(const DeviceScene& s) {
  SceneView v;
  v.nodes = s.nodes;
  v.tri = s.tri;
  v.slot64 = s.slot64;
  v.snorm = s.snorm;
  v.slot_prim = s.slot_prim;
  return v;
}

// Occupancy variants: MINB = minimum resident 128-thread blocks per SM the
// register allocation must allow (1: unconstrained, 6: <= 80 registers,
// 8: <= 64 registers). Selected per context (bc_set_option "raycast_minblocks").
template <int STACK, int MINB>
cudaError_t closest_stack(const DeviceScene& s, const float4* rays, int64_t n, float* t, int32_t* p, unsigned* status,
                          cudaStream_t st) {
  const int64_t grid = (n + 127) / 128;
  if (s.has_spheres)
    k_closest_exact<STACK, true, MINB><<<(unsigned)grid, 128, 0, st>>>(view_of(s), rays, n, t, p, status);
  else
    k_closest_exact<STACK, false, MINB><<<(unsigned)grid, 128, 0, st>>>(view_of(s), rays, n, t, p, status);
  return cudaGetLastError();
}

template <int STACK, int MINB>
cudaError_t any_stack(const DeviceScene& s, const float4* rays, int64_t n, uint8_t* out, unsigned* status,
                      cudaStream_t st) {
  const int64_t grid = (n + 127) / 128;
  if (s.has_spheres)
    k_any_exact<STACK, true, MINB><<<(unsigned)grid, 128, 0, st>>>(view_of(s), rays, n, out, status);
  else
    k_any_exact<STACK, false, MINB><<<(unsigned)grid, 128, 0, st>>>(view_of(s), rays, n, out, status);
  return cudaGetLastError();
}

template <int STACK>
cudaError_t closest_var(const DeviceScene& s, const float4* rays, int64_t n, float* t, int32_t* p, unsigned* status,
                        int variant, cudaStream_t st) {
  if (variant == 0) {  // fast, not exact
    const int64_t grid = (n + 127) / 128;
    if (s.has_spheres)
      k_closest_fast<STACK, true><<<(unsigned)grid, 128, 0, st>>>(view_of(s), rays, n, t, p, status);
    else
      k_closest_fast<STACK, false><<<(unsigned)grid, 128, 0, st>>>(view_of(s), rays, n, t, p, status);
    return cudaGetLastError();
  }
  switch (variant) {
    case 6: return closest_stack<STACK, 6>(s, rays, n, t, p, status, st);
    case 8: return closest_stack<STACK, 8>(s, rays, n, t, p, status, st);
    default: return closest_stack<STACK, 1>(s, rays, n, t, p, status, st);
  }
}

template <int STACK>
cudaError_t any_var(const DeviceScene& s, const float4* rays, int64_t n, uint8_t* out, unsigned* status, int variant,
                    cudaStream_t st) {
  switch (variant) {
    case 6: return any_stack<STACK, 6>(s, rays, n, out, status, st);
    case 8: return any_stack<STACK, 8>(s, rays, n, out, status, st);
    default: return any_stack<STACK, 1>(s, rays, n, out, status, st);
  }
}

}  // namespace

cudaError_t launch_raycast_closest(const DeviceScene& s, const float4* rays, int64_t n, float* t_out,
                                   int32_t* prim_out, unsigned* status, int variant, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  switch (stack_variant(s.stack_need)) {
    case 64: return closest_var<64>(s, rays, n, t_out, prim_out, status, variant, st);
    case 128: return closest_var<128>(s, rays, n, t_out, prim_out, status, variant, st);
    case 256: return closest_var<256>(s, rays, n, t_out, prim_out, status, variant, st);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_raycast_any(const DeviceScene& s, const float4* rays, int64_t n, uint8_t* out, unsigned* status,
                               int variant, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  switch (stack_variant(s.stack_need)) {
    case 64: return any_var<64>(s, rays, n, out, status, variant, st);
    case 128: return any_var<128>(s, rays, n, out, status, variant, st);
    case 256: return any_var<256>(s, rays, n, out, status, variant, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace bcgx

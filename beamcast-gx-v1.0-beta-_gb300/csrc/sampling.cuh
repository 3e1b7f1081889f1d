// Device-side sampling of the path integrator: the per-(pixel, sample) PCG32
// stream, the reference's samplers (renderer.go:1262-1331) and its Halton
// pixel rotation (renderer.go:1906-1915).
//
// The stream and its seeding are the oracle's (make_path_rng), so a CPU run
// and a GPU run with the same seed draw the same numbers in the same order
// (common random numbers). Rejection loops are bounded at 64 tries, far past
// any probability that matters (< 1e-40 per call), so no thread can spin.
#pragma once
#include <stdint.h>

namespace bcgx {

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Pcg32 {
  uint64_t state, inc;
  __host__ __device__ __forceinline__ uint32_t next() {
    uint64_t old = state;
    state = old * 6364136223846793005ull + inc;
    uint32_t xs = (uint32_t)(((old >> 18) ^ old) >> 27);
    uint32_t rot = (uint32_t)(old >> 59);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
  // 24-bit uniform in [0, 1): exact in fp32, identical to the oracle's value.
  __host__ __device__ __forceinline__ float uniform() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }
};

__host__ __device__ __forceinline__ Pcg32 make_path_rng(uint64_t seed, uint64_t pixel_key, uint64_t sample) {
  uint64_t key = mix64(seed + 0x9E3779B97F4A7C15ull * (pixel_key + 1)) ^
                 mix64(sample * 0xD1B54A32D192ED03ull + 0x632BE59BD9B4E019ull);
  Pcg32 r;
  r.state = 0;
  r.inc = (key << 1) | 1u;
  r.next();
  r.state += mix64(key ^ 0xA0761D6478BD642Full);
  r.next();
  return r;
}

constexpr int kMaxRejection = 64;

// rng.Intn(n) as the CPU draws it: floor(u n) of the fp64 product of the 24-bit
// uniform u = k 2^-24 and n, capped at n - 1. Below n = 2^29 the product is
// exact, so integer arithmetic gives the same index without fp64 work.
__device__ __forceinline__ int draw_index(Pcg32& r, int n) {
  const uint32_t k = r.next() >> 8;  // the draw of uniform()
  if (n < (1 << 29)) return min((int)(((uint64_t)k * (uint64_t)n) >> 24), n - 1);
  return min((int)((double)k * (1.0 / 16777216.0) * (double)n), n - 1);
}

__device__ __forceinline__ float3 rand_in_unit_sphere(Pcg32& r) {  // renderer.go:1262-1269
  float x = 0, y = 0, z = 0;
  for (int i = 0; i < kMaxRejection; i++) {
    x = r.uniform() * 2.0f - 1.0f;
    y = r.uniform() * 2.0f - 1.0f;
    z = r.uniform() * 2.0f - 1.0f;
    float l2 = x * x + y * y + z * z;
    if (l2 < 1.0f && l2 > 1e-18f) break;
  }
  return make_float3(x, y, z);
}

__device__ __forceinline__ float3 rand_unit_vector(Pcg32& r) {  // renderer.go:1273-1285
  for (int i = 0; i < kMaxRejection; i++) {
    float u = r.uniform() * 2.0f - 1.0f;
    float v = r.uniform() * 2.0f - 1.0f;
    float s = u * u + v * v;
    if (s >= 1.0f || s <= 1e-18f) continue;
    float f = 2.0f * sqrtf(1.0f - s);
    return make_float3(u * f, v * f, 1.0f - 2.0f * s);
  }
  return make_float3(0.0f, 0.0f, 1.0f);
}

// Malley's method with the branchless orthonormal basis of Duff et al. 2017
// (renderer.go:1290-1311).
__device__ __forceinline__ float3 rand_cos_hemisphere(float3 n, Pcg32& r) {
  float x = 0, y = 0, s = 0;
  for (int i = 0; i < kMaxRejection; i++) {
    x = r.uniform() * 2.0f - 1.0f;
    y = r.uniform() * 2.0f - 1.0f;
    s = x * x + y * y;
    if (s < 1.0f) break;
  }
  float z = sqrtf(fmaxf(0.0f, 1.0f - s));
  float sign = n.z < 0.0f ? -1.0f : 1.0f;
  float a = -1.0f / (sign + n.z);
  float b = n.x * n.y * a;
  float3 t = make_float3(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
  float3 bt = make_float3(b, sign + n.y * n.y * a, -n.y);
  return make_float3(t.x * x + bt.x * y + n.x * z, t.y * x + bt.y * y + n.y * z, t.z * x + bt.z * y + n.z * z);
}

// Per-pixel rotation of the sample table (renderer.go:1906-1915): the two 32-bit
// hashes whose values times 2^-32 are the rotation offsets (rx, ry) in [0, 1).
__host__ __device__ __forceinline__ void pixel_rotation_bits(int x, int y, uint32_t* h1_out, uint32_t* h2_out) {
  uint32_t h1 = ((uint32_t)x * 0x9e3779b1u) ^ ((uint32_t)y * 0x85ebca77u);
  h1 ^= h1 >> 16;
  h1 *= 0x7feb352du;
  h1 ^= h1 >> 15;
  uint32_t h2 = h1 ^ 0x68bc21ebu;
  h2 ^= h2 >> 13;
  *h1_out = h1;
  *h2_out = h2;
}

// ---- small fp32 vector helpers ---------------------------------------------
__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float3 had(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 unit3(float3 a) {  // Vec3.Unit (renderer.go:32-38)
  float l = sqrtf(dot3(a, a));
  if (l < 1e-12f) return f3(0, 0, 0);
  return a * (1.0f / l);
}
__device__ __forceinline__ float maxcomp(float3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
__device__ __forceinline__ float lum3(float3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
__device__ __forceinline__ float3 reflect3(float3 v, float3 n) { return v - n * (2.0f * dot3(v, n)); }
__device__ __forceinline__ float3 refract3(float3 uv, float3 n, float eta) {  // renderer.go:1313-1318
  float ct = fminf(dot3(uv * -1.0f, n), 1.0f);
  float3 perp = (uv + n * ct) * eta;
  float3 par = n * -sqrtf(fabsf(1.0f - dot3(perp, perp)));
  return perp + par;
}
__device__ __forceinline__ float schlick(float cosine, float ref) {  // renderer.go:1319-1326
  float r0 = (1.0f - ref) / (1.0f + ref);
  r0 *= r0;
  float x = 1.0f - cosine;
  float x2 = x * x;
  float x5 = x2 * x2 * x;
  return r0 + (1.0f - r0) * x5;
}
__device__ __forceinline__ float3 background(float3 d) {  // renderer.go:1327-1331
  float3 u = unit3(d);
  float t = 0.5f * (u.y + 1.0f);
  return f3(0.06f, 0.08f, 0.12f) * (1.0f - t) + f3(0.32f, 0.48f, 0.72f) * t;
}
__device__ __forceinline__ float power_heuristic(float a, float b) {  // renderer.go:1395-1402
  float a2 = a * a, b2 = b * b;
  if (a2 + b2 <= 1e-20f) return 0.0f;
  return a2 / (a2 + b2);
}

}  // namespace bcgx

// BVH8 traversal core shared by the ray-cast and wavefront kernels.
//
// Two precisions:
//  * EXACT (ray-cast entry points): the fp32 BVH8 walk is conservative (boxes
//    rounded outward on the host, far distances widened by 2*gamma_3 after
//    Ize, "Robust BVH Ray Traversal", JCGT 2013) and every fp32 triangle test
//    is only a filter with a forward error bound. A triangle that survives the
//    filter is re-tested in fp64 with the operation order of triHit
//    (renderer.go:684-711), using non-fusing intrinsics, so the winning
//    primitive and its fp64 distance equal the CPU path's exactly.
//  * fast (rendering): the same walk with plain fp32 tests; image parity is
//    statistical, so a 1-ulp change of a distance is immaterial there.
//
// Closest-hit tie rule: triHit accepts t <= closest (renderer.go:702), so at
// bit-identical fp64 distances the primitive the reference's traversal tests
// last wins. The EXACT walk visits the tree in its own order, so it flags a
// ray whose best fp64 distance it sees twice (HitResult.tie); the ray-cast
// passes then replay the reference's binary walk for that ray alone.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "layout.h"

namespace bcgx {

constexpr float kU = 5.9604645e-8f;  // 2^-24, fp32 unit roundoff
constexpr float kFarSlack = 8.0e-7f;  // > 2*gamma_3 + rounding of the scaling itself

// Refill policy of the persistent walks: a warp takes new queries once this many
// of its lanes are idle, or when none is busy. A refill costs the whole warp a
// ballot, a queue atomic and the new rays' loads, so taking one per finished
// lane is slower than letting a few lanes wait.
constexpr int kRefillLanes = 6;

struct Ray32 {
  float ox, oy, oz;
  float dx, dy, dz;
  float ix, iy, iz;  // 1/d, or +inf on axes with |d| < 1e-15 (the reference's zero axes)
  float dmax;        // max |d_k|
  float tmin;
};

__device__ __forceinline__ Ray32 make_ray(float ox, float oy, float oz, float dx, float dy, float dz, float tmin) {
  Ray32 r;
  r.ox = ox; r.oy = oy; r.oz = oz;
  r.dx = dx; r.dy = dy; r.dz = dz;
  r.ix = fabsf(dx) < 1e-15f ? __int_as_float(0x7f800000) : 1.0f / dx;
  r.iy = fabsf(dy) < 1e-15f ? __int_as_float(0x7f800000) : 1.0f / dy;
  r.iz = fabsf(dz) < 1e-15f ? __int_as_float(0x7f800000) : 1.0f / dz;
  r.dmax = fmaxf(fabsf(dx), fmaxf(fabsf(dy), fabsf(dz)));
  r.tmin = tmin;
  return r;
}

// Moves a far distance away from zero by the slack (conservative box test and
// culling bound). Infinities stay infinite: a slab whose far distance is -inf
// (a zero direction component with the box entirely to one side) must still
// reject the box; fma(|t|, slack, t) would turn -inf into NaN, which fminf
// ignores, and the box would be entered.
__device__ __forceinline__ float widen(float t) { return t * (t >= 0.0f ? 1.0f + kFarSlack : 1.0f - kFarSlack); }

// 1 + b 2^-15 for byte j of word (bit pattern 0x3f80bb00, exact).
__device__ __forceinline__ float byte_v(uint32_t word, int j) {
  return __uint_as_float(__byte_perm(word, 0x3f800000u, 0x7604u | ((uint32_t)j << 4)));
}

// Sorting network (Batcher odd-even merge, 19 comparators) on (near, child).
__device__ __forceinline__ void cswap(float& ka, uint32_t& va, float& kb, uint32_t& vb) {
  bool s = kb < ka;
  float tk = s ? kb : ka;
  uint32_t tv = s ? vb : va;
  kb = s ? ka : kb;
  vb = s ? va : vb;
  ka = tk;
  va = tv;
}
__device__ __forceinline__ void sort8(float k[8], uint32_t v[8]) {
  cswap(k[0], v[0], k[1], v[1]); cswap(k[2], v[2], k[3], v[3]); cswap(k[4], v[4], k[5], v[5]); cswap(k[6], v[6], k[7], v[7]);
  cswap(k[0], v[0], k[2], v[2]); cswap(k[1], v[1], k[3], v[3]); cswap(k[4], v[4], k[6], v[6]); cswap(k[5], v[5], k[7], v[7]);
  cswap(k[1], v[1], k[2], v[2]); cswap(k[5], v[5], k[6], v[6]);
  cswap(k[0], v[0], k[4], v[4]); cswap(k[1], v[1], k[5], v[5]); cswap(k[2], v[2], k[6], v[6]); cswap(k[3], v[3], k[7], v[7]);
  cswap(k[2], v[2], k[4], v[4]); cswap(k[3], v[3], k[5], v[5]);
  cswap(k[1], v[1], k[2], v[2]); cswap(k[3], v[3], k[4], v[4]); cswap(k[5], v[5], k[6], v[6]);
}

// ---- fp64 re-test with the reference's operation order -------------------
struct D3 {
  double x, y, z;
};
__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double ddot(D3 a, D3 b) { return da(da(dm(a.x, b.x), dm(a.y, b.y)), dm(a.z, b.z)); }
__device__ __forceinline__ D3 dcross(D3 a, D3 b) {
  return D3{ds(dm(a.y, b.z), dm(a.z, b.y)), ds(dm(a.z, b.x), dm(a.x, b.z)), ds(dm(a.x, b.y), dm(a.y, b.x))};
}
__device__ __forceinline__ D3 dsub3(D3 a, D3 b) { return D3{ds(a.x, b.x), ds(a.y, b.y), ds(a.z, b.z)}; }

// triHit / triAnyHit (renderer.go:684-711, 744-763): returns true and t when
// tmin <= t <= tmax.
static __device__ __noinline__ bool tri_hit64(const double* __restrict__ q, D3 o, D3 d, double tmin, double tmax,
                                          double* t_out) {
  const D3 a{__ldg(q + 0), __ldg(q + 1), __ldg(q + 2)};
  const D3 e1{__ldg(q + 3), __ldg(q + 4), __ldg(q + 5)};
  const D3 e2{__ldg(q + 6), __ldg(q + 7), __ldg(q + 8)};
  D3 h = dcross(d, e2);
  double det = ddot(e1, h);
  if (fabs(det) < 1e-10) return false;
  double f = __ddiv_rn(1.0, det);
  D3 ss = dsub3(o, a);
  double u = dm(f, ddot(ss, h));
  if (u < 0 || u > 1) return false;
  D3 qq = dcross(ss, e1);
  double v = dm(f, ddot(d, qq));
  if (v < 0 || da(u, v) > 1) return false;
  double t = dm(f, ddot(e2, qq));
  if (t < tmin || t > tmax) return false;
  *t_out = t;
  return true;
}

// sphereHitAccel / sphereAnyHitAccel (renderer.go:650-678, 724-742).
// `closest` selects the near root first, then the far root, as the reference does.
static __device__ __noinline__ bool sphere_hit64(const double* __restrict__ q, D3 o, D3 d, double tmin, double tmax,
                                             double* t_out) {
  const double dl2 = ddot(d, d);
  if (!(dl2 > 1e-18)) return false;
  const double idl2 = __ddiv_rn(1.0, dl2);
  const D3 c{__ldg(q + 0), __ldg(q + 1), __ldg(q + 2)};
  const double rad = __ldg(q + 3);
  D3 oc = dsub3(o, c);
  double hb = ddot(oc, d);
  double cc = ds(ddot(oc, oc), dm(rad, rad));
  double disc = ds(dm(hb, hb), dm(dl2, cc));
  if (disc < 0) return false;
  double sq = __dsqrt_rn(disc);
  double root = dm(ds(-hb, sq), idl2);
  if (root < tmin || root > tmax) {
    root = dm(da(-hb, sq), idl2);
    if (root < tmin || root > tmax) return false;
  }
  *t_out = root;
  return true;
}

// fp32 Moller-Trumbore with forward error bounds, classifying a triangle
// against the fp64 test of the same triangle (triHit, renderer.go:684-711):
//   kMiss  - the fp64 test certainly rejects it,
//   kHit   - the fp64 test certainly accepts it, and its fp64 distance lies in
//            [t - et, t + et],
//   kMaybe - undecided; only the fp64 test can tell.
// The bounds are first-order forward bounds of each quantity against the
// exact result on the fp64 inputs (the fp32 record holds those inputs rounded
// to nearest), with at least a factor 2 of slack; R = max|A| + max|O - A|.
constexpr int kMiss = 0, kHit = 1, kMaybe = 2;

struct TriClass {
  int state;
  float t, et;
};

__device__ __forceinline__ TriClass tri_classify(float4 A, float4 E1, float4 E2, const Ray32& r, float tmax_ray,
                                                 float tlim) {
  TriClass c;
  c.state = kMiss;
  c.t = 0.0f;
  c.et = 0.0f;
  const float hx = r.dy * E2.z - r.dz * E2.y;
  const float hy = r.dz * E2.x - r.dx * E2.z;
  const float hz = r.dx * E2.y - r.dy * E2.x;
  const float det = E1.x * hx + E1.y * hy + E1.z * hz;
  const float Mh = r.dmax * E2.w;
  const float errDet = 96.0f * kU * E1.w * Mh;
  const float adet = fabsf(det);
  if (adet + errDet < 1e-10f) return c;
  const float sx = r.ox - A.x, sy = r.oy - A.y, sz = r.oz - A.z;
  if (adet <= 2.0f * errDet || adet - errDet < 1e-10f) {  // cannot bound u, v, t
    c.state = kMaybe;
    c.et = __int_as_float(0x7f800000);
    return c;
  }
  const float R = A.w + fmaxf(fabsf(sx), fmaxf(fabsf(sy), fabsf(sz)));
  // Quick certain misses before any division, on the numerators u*det, v*det
  // and t*det: with sd = sign(det) (certain, |det| > 2 errDet), un = s.h
  // within Eun of its exact value, vn = d.q within Evn, tn = E2.q within Etn
  // (the numerator terms of eu, ev, et below), u < 0 is certain when
  // sd un + Eun < 0 and u > 1 when sd un - Eun > |det| + errDet, and so on.
  // Directed rounding keeps each comparison sound.
  const float sd = det > 0.0f ? 1.0f : -1.0f;
  const float un = sd * (sx * hx + sy * hy + sz * hz);
  const float Eun = 96.0f * kU * R * Mh;
  const float dhi = __fadd_ru(adet, errDet), dlo = __fsub_rd(adet, errDet);
  if (__fadd_ru(un, Eun) < 0.0f || __fsub_rd(un, Eun) > dhi) return c;
  const float qx = sy * E1.z - sz * E1.y;
  const float qy = sz * E1.x - sx * E1.z;
  const float qz = sx * E1.y - sy * E1.x;
  const float vn = sd * (r.dx * qx + r.dy * qy + r.dz * qz);
  const float Evn = 96.0f * kU * r.dmax * R * E1.w;
  if (__fadd_ru(vn, Evn) < 0.0f || __fsub_rd(__fsub_rd(__fadd_rd(un, vn), Eun), Evn) > dhi) return c;
  const float tn = sd * (E2.x * qx + E2.y * qy + E2.z * qz);
  const float Etn = 112.0f * kU * E2.w * R * E1.w;
  // bounds of tmin |det| and tlim |det| over |det| in [dlo, dhi] (either may be negative)
  const float tmin_det = fminf(__fmul_rd(r.tmin, dlo), __fmul_rd(r.tmin, dhi));
  const float tlim_det = fmaxf(__fmul_ru(tlim, dlo), __fmul_ru(tlim, dhi));
  if (__fadd_ru(tn, Etn) < tmin_det || __fsub_rd(tn, Etn) > tlim_det) return c;
  const float invd = 1.0f / (adet - errDet);
  const float f = 1.0f / det;
  const float u = f * (sx * hx + sy * hy + sz * hz);
  const float eu = (96.0f * kU * R * Mh + fabsf(u) * errDet) * invd + 4.0f * kU * fabsf(u);
  if (u < -eu || u > 1.0f + eu) return c;
  const float v = f * (r.dx * qx + r.dy * qy + r.dz * qz);
  const float ev = (96.0f * kU * r.dmax * R * E1.w + fabsf(v) * errDet) * invd + 4.0f * kU * fabsf(v);
  const float euv = eu + ev + 4.0f * kU * fabsf(u + v);
  if (v < -ev || u + v > 1.0f + euv) return c;
  const float t = f * (E2.x * qx + E2.y * qy + E2.z * qz);
  const float et = (112.0f * kU * E2.w * R * E1.w + fabsf(t) * errDet) * invd + 4.0f * kU * fabsf(t);
  if (t + et < r.tmin || t - et > tlim) return c;
  c.t = t;
  c.et = et;
  const bool sure = u >= eu && u <= 1.0f - eu && v >= ev && u + v <= 1.0f - euv && t - et >= r.tmin &&
                    t + et <= tmax_ray;
  c.state = sure ? kHit : kMaybe;
  return c;
}

// The fp32 tests below spell every product and sum as a round-to-nearest
// intrinsic. Left to the compiler, a*b - c*d or a dot product may contract
// into different fused forms in different kernels (the surrounding code
// steers the choice), and the wave engine's extend kernel and the one-kernel
// renderer would then round the same test differently. Spelled out, every
// kernel that inlines a test computes the same bits, at the instruction count
// contraction gives.
__device__ __forceinline__ float fdiff(float a, float b, float c, float d) {  // a b - c d
  return __fmaf_rn(a, b, -__fmul_rn(c, d));
}
__device__ __forceinline__ float fdot(float ax, float ay, float az, float bx, float by, float bz) {
  return __fmaf_rn(az, bz, __fmaf_rn(ay, by, __fmul_rn(ax, bx)));
}

// Plain fp32 triangle test for rendering (reference thresholds), with the
// barycentric and distance tests on the numerators (u det, v det, t det
// against det), so a missed triangle costs no division.
__device__ __forceinline__ bool tri_hit32(float4 A, float4 E1, float4 E2, const Ray32& r, float tmax, float* t_out) {
  const float hx = fdiff(r.dy, E2.z, r.dz, E2.y);
  const float hy = fdiff(r.dz, E2.x, r.dx, E2.z);
  const float hz = fdiff(r.dx, E2.y, r.dy, E2.x);
  const float det = fdot(E1.x, E1.y, E1.z, hx, hy, hz);
  if (fabsf(det) < 1e-10f) return false;
  const float sd = det > 0.0f ? 1.0f : -1.0f, adet = fabsf(det);
  const float sx = __fsub_rn(r.ox, A.x), sy = __fsub_rn(r.oy, A.y), sz = __fsub_rn(r.oz, A.z);
  const float un = sd * fdot(sx, sy, sz, hx, hy, hz);
  if (un < 0.0f || un > adet) return false;
  const float qx = fdiff(sy, E1.z, sz, E1.y);
  const float qy = fdiff(sz, E1.x, sx, E1.z);
  const float qz = fdiff(sx, E1.y, sy, E1.x);
  const float vn = sd * fdot(r.dx, r.dy, r.dz, qx, qy, qz);
  if (vn < 0.0f || __fadd_rn(un, vn) > adet) return false;
  const float eq = fdot(E2.x, E2.y, E2.z, qx, qy, qz);
  const float tn = sd * eq;
  if (tn < __fmul_rn(r.tmin, adet) || tn > __fmul_rn(tmax, adet)) return false;
  const float t = __fdiv_rn(eq, det);
  if (t < r.tmin || t > tmax) return false;
  *t_out = t;
  return true;
}

// Plain fp32 sphere test (sphereHitAccel in fp32) for rendering.
__device__ __forceinline__ bool sphere_hit32(float4 C, float4 S, const Ray32& r, float tmax, float* t_out) {
  const float dl2 = fdot(r.dx, r.dy, r.dz, r.dx, r.dy, r.dz);
  if (!(dl2 > 1e-18f)) return false;
  const float ocx = __fsub_rn(r.ox, C.x), ocy = __fsub_rn(r.oy, C.y), ocz = __fsub_rn(r.oz, C.z);
  const float hb = fdot(ocx, ocy, ocz, r.dx, r.dy, r.dz);
  const float cc = __fsub_rn(fdot(ocx, ocy, ocz, ocx, ocy, ocz), S.x);
  const float disc = fdiff(hb, hb, dl2, cc);
  if (disc < 0.0f) return false;
  const float sq = __fsqrt_rn(disc);
  const float idl2 = __fdiv_rn(1.0f, dl2);
  float root = __fmul_rn(__fsub_rn(-hb, sq), idl2);
  if (root < r.tmin || root > tmax) {
    root = __fmul_rn(__fadd_rn(-hb, sq), idl2);
    if (root < r.tmin || root > tmax) return false;
  }
  *t_out = root;
  return true;
}

struct SceneView {
  const Node8* __restrict__ nodes;
  const float4* __restrict__ tri;
  const double* __restrict__ slot64;
  const float4* __restrict__ snorm;
  const int32_t* __restrict__ slot_prim;
};

struct HitResult {
  int32_t slot;   // -1 on a miss
  float t32;      // fast mode distance
  double t64;     // exact mode distance
  bool tie;       // exact mode: another primitive had the same fp64 distance as a best hit
};

constexpr uint32_t kEnd = 0x7fffffffu;  // "no node": bit 31 clear and above any node index

// Per-ray constants of the fused node test.
struct RayPre {
  float ivx, ivy, ivz;  // finite 1/d (components below 1e-15 in magnitude replaced by +-1e-15)
  float nox, noy, noz;  // -o/d
  float mx, my, mz;     // 2|o/d| (rounding-bound term of the conservative test)
};

__device__ __forceinline__ RayPre ray_pre(const Ray32& r) {
  RayPre p;
  p.ivx = 1.0f / (fabsf(r.dx) < 1e-15f ? copysignf(1e-15f, r.dx) : r.dx);
  p.ivy = 1.0f / (fabsf(r.dy) < 1e-15f ? copysignf(1e-15f, r.dy) : r.dy);
  p.ivz = 1.0f / (fabsf(r.dz) < 1e-15f ? copysignf(1e-15f, r.dz) : r.dz);
  p.nox = -r.ox * p.ivx;
  p.noy = -r.oy * p.ivy;
  p.noz = -r.oz * p.ivz;
  p.mx = 2.0f * fabsf(p.nox);
  p.my = 2.0f * fabsf(p.noy);
  p.mz = 2.0f * fabsf(p.noz);
  return p;
}

// Entry distances of a node's eight children (+inf: missed or empty), decode
// and slab fused: per axis A = (p - o)/d and B = 2^e/d, a byte q enters as
// v = 1 + q 2^-15 (one byte permute) and t(q) = v B' + (A - B') with
// B' = 2^15 B; near and far bytes are picked by the sign of 1/d.
// CONS: the walk of the exact ray cast must enter every box the fp64 slab
// test of the reference enters. B' is exact (power-of-two scaling); A, A - B'
// and the final FMA add at most 4.2u (|p/d| + |o/d|) + 3.1u |B'| of absolute
// error, so near offsets are lowered and far offsets raised by
// E = 5u (|fl(p/d - o/d)| + 2|o/d| + |B'|) + 1e-30 per node and axis; the
// rounding of 1/d itself is relative and covered by the far-distance slack
// (widen). A zero direction component (|d| < 1e-15, the reference's
// origin-inside test) gets a finite 1/(+-1e-15): its E is then so large that
// the axis never rejects, which keeps the test conservative. Empty slots are
// masked by the child count. Without CONS there is no margin: fine for
// rendering.
template <bool CONS>
__device__ __forceinline__ void node_children_fused(const Node8* __restrict__ node, const RayPre& rp, float tmin,
                                                    float tlim, float near[8], uint32_t child[8]) {
  const float4* p = reinterpret_cast<const float4*>(node);
  const float4 w0 = __ldg(p + 0);
  const uint4 c0 = __ldg(reinterpret_cast<const uint4*>(p + 1));
  const uint4 c1 = __ldg(reinterpret_cast<const uint4*>(p + 2));
  const uint4 qx = __ldg(reinterpret_cast<const uint4*>(p + 3));
  const uint4 qy = __ldg(reinterpret_cast<const uint4*>(p + 4));
  const uint4 qz = __ldg(reinterpret_cast<const uint4*>(p + 5));
  const uint32_t meta = __float_as_uint(w0.w);
  const int nchild = (int)(meta >> 24);
  const float bx = __uint_as_float((meta & 0xffu) << 23) * rp.ivx * 32768.0f;
  const float by = __uint_as_float(((meta >> 8) & 0xffu) << 23) * rp.ivy * 32768.0f;
  const float bz = __uint_as_float(((meta >> 16) & 0xffu) << 23) * rp.ivz * 32768.0f;
  const float a1x = fmaf(w0.x, rp.ivx, rp.nox), a1y = fmaf(w0.y, rp.ivy, rp.noy), a1z = fmaf(w0.z, rp.ivz, rp.noz);
  float anx = a1x - bx, any = a1y - by, anz = a1z - bz;
  float afx = anx, afy = any, afz = anz;
  if (CONS) {
    const float ex = fmaf(fabsf(a1x) + fabsf(bx) + rp.mx, 5.0f * kU, 1e-30f);
    const float ey = fmaf(fabsf(a1y) + fabsf(by) + rp.my, 5.0f * kU, 1e-30f);
    const float ez = fmaf(fabsf(a1z) + fabsf(bz) + rp.mz, 5.0f * kU, 1e-30f);
    anx -= ex; any -= ey; anz -= ez;
    afx += ex; afy += ey; afz += ez;
  }
  const bool fx = rp.ivx < 0.0f, fy = rp.ivy < 0.0f, fz = rp.ivz < 0.0f;
  const uint32_t nx0 = fx ? qx.z : qx.x, nx1 = fx ? qx.w : qx.y, gx0 = fx ? qx.x : qx.z, gx1 = fx ? qx.y : qx.w;
  const uint32_t ny0 = fy ? qy.z : qy.x, ny1 = fy ? qy.w : qy.y, gy0 = fy ? qy.x : qy.z, gy1 = fy ? qy.y : qy.w;
  const uint32_t nz0 = fz ? qz.z : qz.x, nz1 = fz ? qz.w : qz.y, gz0 = fz ? qz.x : qz.z, gz1 = fz ? qz.y : qz.w;
  child[0] = c0.x; child[1] = c0.y; child[2] = c0.z; child[3] = c0.w;
  child[4] = c1.x; child[5] = c1.y; child[6] = c1.z; child[7] = c1.w;
  auto test = [&](int k) {
    const int j = k & 3;
    const float tnx = fmaf(byte_v(k < 4 ? nx0 : nx1, j), bx, anx), tfx = fmaf(byte_v(k < 4 ? gx0 : gx1, j), bx, afx);
    const float tny = fmaf(byte_v(k < 4 ? ny0 : ny1, j), by, any), tfy = fmaf(byte_v(k < 4 ? gy0 : gy1, j), by, afy);
    const float tnz = fmaf(byte_v(k < 4 ? nz0 : nz1, j), bz, anz), tfz = fmaf(byte_v(k < 4 ? gz0 : gz1, j), bz, afz);
    const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, tmin));
    const float sf = fminf(fminf(tfx, tfy), tfz);
    const float tf = fminf(CONS ? widen(sf) : sf * (1.0f + kFarSlack), tlim);
    const bool hit = CONS ? (k < nchild && tn <= tf) : tn <= tf;  // without CONS empty slots decode inverted
    near[k] = hit ? tn : __int_as_float(0x7f800000);
  };
#pragma unroll
  for (int k = 0; k < 4; k++) test(k);
  // The rendering walk tests slots 4-7 only when some lane's node has more
  // than four children (a fifth of the node visits on the Ultra-shaped scene
  // go to nodes with at most four): a warp-uniform branch, so no lane idles
  // through it alone. The exact walk tests all eight: at its 40-register
  // budget the branch costs spills (measured: ray cast 552 -> 531 Mrays/s).
  if (CONS || __any_sync(__activemask(), nchild > 4)) {
#pragma unroll
    for (int k = 4; k < 8; k++) test(k);
  } else {
#pragma unroll
    for (int k = 4; k < 8; k++) near[k] = __int_as_float(0x7f800000);
  }
}

// While-while BVH8 walk (Aila and Laine, "Understanding the Efficiency of Ray
// Traversal on GPUs", HPG 2009): a lane descends inner nodes, postponing the
// first leaf it reaches, until every active lane of the warp holds a leaf;
// then leaves are tested in their own loop. Hit children are visited
// near-first (sorting network) and culled against leaf.tlim when popped.
// `Leaf` provides `float tlim`, `bool done` and `void operator()(uint32_t leaf_ref)`.
template <int STACK, class Leaf>
__device__ __forceinline__ void walk(const SceneView& sv, const Ray32& r, Leaf& leaf, unsigned* status) {
  uint2 st[STACK];
  int sp = 0;
  uint32_t ref = 0;      // root Node8
  uint32_t pending = 0;  // postponed leaf ref, 0 = none
  const RayPre rp = ray_pre(r);
  for (;;) {
    while (ref != kEnd && !(ref & kLeafBit)) {
      float nr[8];
      uint32_t ch[8];
      node_children_fused<true>(sv.nodes + ref, rp, r.tmin, leaf.tlim, nr, ch);
      sort8(nr, ch);
      if (nr[0] == __int_as_float(0x7f800000)) {
        ref = kEnd;
        while (sp > 0) {
          const uint2 e = st[--sp];
          if (__uint_as_float(e.y) <= leaf.tlim) { ref = e.x; break; }
        }
      } else {
#pragma unroll
        for (int k = 7; k >= 1; k--) {
          if (nr[k] != __int_as_float(0x7f800000)) {
            if (sp < STACK) st[sp++] = make_uint2(ch[k], __float_as_uint(nr[k]));
            else atomicOr(status, kStatusStackOverflow);
          }
        }
        ref = ch[0];
      }
      if (ref != kEnd && (ref & kLeafBit)) {
        if (pending != 0) break;
        pending = ref;
        ref = kEnd;
        while (sp > 0) {
          const uint2 e = st[--sp];
          if (__uint_as_float(e.y) <= leaf.tlim) { ref = e.x; break; }
        }
      }
      if (__all_sync(__activemask(), pending != 0)) break;
    }
    while (pending != 0) {
      leaf(pending);
      if (leaf.done) return;
      pending = 0;
      if (ref != kEnd && (ref & kLeafBit)) {
        pending = ref;
        ref = kEnd;
        while (sp > 0) {
          const uint2 e = st[--sp];
          if (__uint_as_float(e.y) <= leaf.tlim) { ref = e.x; break; }
        }
      }
    }
    if (ref == kEnd) return;
  }
}

// A node's hit children, nearest first: the nearest becomes the next node and
// the others are pushed far-first (entry distance kept for culling at the
// pop); no hit child: the next node is popped. When no active lane of the warp
// hit more than one child, the sorting network and the pushes have nothing to
// do: the single hit child (if any) is picked with selects; when none hit more
// than four, they are ordered with five comparisons instead of the network.
template <int STACK, class W>
__device__ __forceinline__ uint32_t order_children(float nr[8], uint32_t ch[8], uint2* st, int& sp, float tlim,
                                                   unsigned* status, W& walker) {
  const float kInf = __int_as_float(0x7f800000);
  int hits = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) hits += nr[k] != kInf ? 1 : 0;
  const unsigned am = __activemask();
  if (!__any_sync(am, hits > 1)) {
    uint32_t c = kEnd;
#pragma unroll
    for (int k = 0; k < 8; k++) c = nr[k] != kInf ? ch[k] : c;
    return hits ? c : walker.pop(tlim);
  }
  if (!__any_sync(am, hits > 4)) {  // at most four: ordered with five comparisons
    float n0 = kInf, n1 = kInf, n2 = kInf, n3 = kInf;
    uint32_t c0 = kEnd, c1 = kEnd, c2 = kEnd, c3 = kEnd;
#pragma unroll
    for (int k = 7; k >= 0; k--) {  // c0..c3: the hit slots in slot order
      if (nr[k] != kInf) {
        n3 = n2;
        c3 = c2;
        n2 = n1;
        c2 = c1;
        n1 = n0;
        c1 = c0;
        n0 = nr[k];
        c0 = ch[k];
      }
    }
    if (hits == 0) return walker.pop(tlim);
    cswap(n0, c0, n1, c1);
    cswap(n2, c2, n3, c3);
    cswap(n0, c0, n2, c2);
    cswap(n1, c1, n3, c3);
    cswap(n1, c1, n2, c2);
#pragma unroll
    for (int k = 3; k >= 1; k--) {
      const float nk = k == 3 ? n3 : (k == 2 ? n2 : n1);
      const uint32_t ck = k == 3 ? c3 : (k == 2 ? c2 : c1);
      if (nk != kInf) {
        if (sp < STACK) st[sp++] = make_uint2(ck, __float_as_uint(nk));
        else atomicOr(status, kStatusStackOverflow);
      }
    }
    return c0;
  }
  sort8(nr, ch);
  if (nr[0] == kInf) return walker.pop(tlim);
#pragma unroll
  for (int k = 7; k >= 1; k--) {
    if (nr[k] != kInf) {
      if (sp < STACK) st[sp++] = make_uint2(ch[k], __float_as_uint(nr[k]));
      else atomicOr(status, kStatusStackOverflow);
    }
  }
  return ch[0];
}

// The switch of a warp's walk to its leaf phase: when at least VOTE/8 of the
// lanes still in the node loop hold a postponed leaf (8: all of them, the
// while-while rule of Aila and Laine). A lane's own sequence of node visits
// and leaf tests does not depend on it, so neither do the hits. Measured on
// one box against 8 (A/B in one call): the render walk on the Ultra-shaped
// frame 2,233 -> 2,264 / 2,373 / 2,379 / 2,292 / 2,092 Mseg/s at 6 / 4 / 3 / 2 / 1;
// the exact closest-hit ray cast 557 -> 551 / 603 / 635 / 630 Mrays/s at
// 6 / 5 / 4 / 3; the exact any hit 742 -> 496 / 523 / 626 / 723 at 7 / 6 / 4 / 3
// (a lane stops at its first hit, and any-hit walks keep 8).
constexpr int kLeafVote = 3;       // closest-hit walks of the renderer
constexpr int kExactLeafVote = 4;  // the exact closest-hit ray cast
constexpr int kAnyLeafVote = 8;    // any-hit walks
template <int VOTE>
__device__ __forceinline__ bool leaf_phase_now(uint32_t pending) {
  const unsigned am = __activemask();
  if (VOTE >= 8) return __all_sync(am, pending != 0);
  return __popc(__ballot_sync(am, pending != 0)) * 8 >= VOTE * __popc(am);
}

// The same while-while walk as a resumable per-lane state machine, for
// persistent kernels that refill a lane with a new ray as soon as its ray is
// done. step() runs one outer iteration and returns true once the walk of the
// current ray has finished (stack empty, or leaf.done).
template <int STACK, int VOTE = 8>
struct Walker {
  uint2 st[STACK];
  int sp;
  uint32_t ref;
  uint32_t pending;
  RayPre rp;
  __device__ __forceinline__ void reset(const Ray32& r, uint32_t root = 0) {  // root: Node8 index of the scene's root
    sp = 0;
    ref = root;
    pending = 0;
    rp = ray_pre(r);
  }
  __device__ __forceinline__ uint32_t pop(float tlim) {
    while (sp > 0) {
      const uint2 e = st[--sp];
      if (__uint_as_float(e.y) <= tlim) return e.x;
    }
    return kEnd;
  }
  template <class Leaf>
  __device__ __forceinline__ bool step(const SceneView& sv, const Ray32& r, Leaf& leaf, unsigned* status) {
    while (ref != kEnd && !(ref & kLeafBit)) {
      float nr[8];
      uint32_t ch[8];
      node_children_fused<true>(sv.nodes + ref, rp, r.tmin, leaf.tlim, nr, ch);
      ref = order_children<STACK>(nr, ch, st, sp, leaf.tlim, status, *this);
      if (ref != kEnd && (ref & kLeafBit)) {
        if (pending != 0) break;
        pending = ref;
        ref = pop(leaf.tlim);
      }
      if (leaf_phase_now<VOTE>(pending)) break;
    }
    while (pending != 0) {
      leaf(pending);
      if (leaf.done) return true;
      pending = 0;
      if (ref != kEnd && (ref & kLeafBit)) {
        pending = ref;
        ref = pop(leaf.tlim);
      }
    }
    return ref == kEnd;
  }
};

// ---- walk for the fast (rendering) precision -----------------------------------
// Walker with the fused node test without rounding margins (see
// node_children_fused): a box can lose a few ulps of its quantization margin,
// fine for rendering, not for the exact ray cast.
template <int STACK, int VOTE = 8>
struct FastWalker {
  uint2 st[STACK];
  int sp;
  uint32_t ref;
  uint32_t pending;
  RayPre rp;
  __device__ __forceinline__ void reset(const Ray32& r, uint32_t root = 0) {
    sp = 0;
    ref = root;
    pending = 0;
    rp = ray_pre(r);
  }
  __device__ __forceinline__ uint32_t pop(float tlim) {
    while (sp > 0) {
      const uint2 e = st[--sp];
      if (__uint_as_float(e.y) <= tlim) return e.x;
    }
    return kEnd;
  }
  template <class Leaf>
  __device__ __forceinline__ bool step(const SceneView& sv, const Ray32& r, Leaf& leaf, unsigned* status) {
    while (ref != kEnd && !(ref & kLeafBit)) {
      float nr[8];
      uint32_t ch[8];
      node_children_fused<false>(sv.nodes + ref, rp, r.tmin, leaf.tlim, nr, ch);
      ref = order_children<STACK>(nr, ch, st, sp, leaf.tlim, status, *this);
      if (ref != kEnd && (ref & kLeafBit)) {
        if (pending != 0) break;
        pending = ref;
        ref = pop(leaf.tlim);
      }
      if (leaf_phase_now<VOTE>(pending)) break;
    }
    while (pending != 0) {
      leaf(pending);
      if (leaf.done) return true;
      pending = 0;
      if (ref != kEnd && (ref & kLeafBit)) {
        pending = ref;
        ref = pop(leaf.tlim);
      }
    }
    return ref == kEnd;
  }
};

// ---- exact closest hit -------------------------------------------------------
// Candidates carry an fp32 interval [lo, hi] that holds their fp64 distance.
// `best` is the certain hit with the smallest upper bound; candidates that
// might still beat it (undecided ones, or certain ones whose interval overlaps
// best's) wait in a short per-thread list. After the walk the warp is
// re-converged and every remaining contender is settled in fp64 together, so
// the slow fp64 pipe runs with all lanes active instead of one lane at a time.
struct Contender {
  int32_t slot;
  float lo, hi;
  double t64;
  bool exact;
};

constexpr int kPending = 4;

// A pending contender keeps only what decides whether it is settled later:
// its slot and the lower end of its distance interval (settlement recomputes
// the fp64 distance).
struct PendEntry {
  int32_t slot;
  float lo;
};

template <bool SPHERES>
struct ExactClosestLeaf {
  const SceneView& sv;
  const Ray32& r;
  unsigned* status;
  float tmax_ray;
  float tlim;
  bool done;
  bool tie;  // two contenders compared equal in fp64
  Contender best;
  int npend;
  PendEntry pend[kPending];

  __device__ ExactClosestLeaf(const SceneView& s, const Ray32& ray, float tmax, unsigned* st)
      : sv(s), r(ray), status(st) {
    reset(tmax);
  }
  __device__ __forceinline__ void reset(float tmax) {
    tmax_ray = tmax;
    tlim = widen(tmax);
    done = false;
    tie = false;
    npend = 0;
    best.slot = -1;
    best.lo = tmax;
    best.hi = tmax;
    best.t64 = 0.0;
    best.exact = false;
  }
  // fp64 distance of a contender (triHit in the reference's operation order).
  __device__ __forceinline__ bool resolve(Contender& c) {
    if (c.exact) return true;
    double t;
    const D3 o{(double)r.ox, (double)r.oy, (double)r.oz}, d{(double)r.dx, (double)r.dy, (double)r.dz};
    if (!tri_hit64(sv.slot64 + 9 * (size_t)c.slot, o, d, (double)r.tmin, (double)tmax_ray, &t)) return false;
    c.t64 = t;
    c.lo = __double2float_rd(t);
    c.hi = __double2float_ru(t);
    c.exact = true;
    return true;
  }
  // c is exact and valid: compare with best now (no deferral, no recursion).
  __device__ __forceinline__ void settle_against_best(const Contender& c) {
    if (best.slot < 0 || c.hi < best.lo) {
      best = c;
    } else if (c.lo <= best.hi) {
      if (!resolve(best)) {
        atomicOr(status, kStatusBound);  // a certain hit must pass its fp64 test
        best = c;
      } else if (c.t64 < best.t64 || (c.t64 == best.t64 && c.slot > best.slot)) {
        tie = tie || c.t64 == best.t64;
        best = c;
      } else {
        tie = tie || c.t64 == best.t64;
      }
    }
    tlim = widen(best.hi);
  }
  // c may hit and may beat best: keep it for the converged settlement, or
  // settle it now when the list is full.
  __device__ __forceinline__ void defer_maybe(Contender c) {
    if (npend < kPending) {
      pend[npend++] = PendEntry{c.slot, c.lo};
      return;
    }
    if (resolve(c)) settle_against_best(c);
  }
  // c certainly hits; best keeps the smallest upper bound, an overlapping
  // loser waits in the list (or both are settled now when it is full).
  __device__ __forceinline__ void take_certain(Contender c) {
    if (best.slot < 0 || c.hi < best.lo) {
      best = c;
    } else if (c.lo > best.hi) {
      return;
    } else if (npend < kPending) {
      if (c.hi < best.hi) {
        pend[npend++] = PendEntry{best.slot, best.lo};
        best = c;
      } else {
        pend[npend++] = PendEntry{c.slot, c.lo};
      }
    } else {
      if (!resolve(c)) {
        atomicOr(status, kStatusBound);
        return;
      }
      settle_against_best(c);
      return;
    }
    tlim = widen(best.hi);
  }
  __device__ __forceinline__ void operator()(uint32_t ref) {
    const int cnt = (int)((ref >> 27) & 15u) + 1;
    const int s0 = (int)(ref & kSlotMask);
    for (int k = 0; k < cnt; k++) {
      const int s = s0 + k;
      const float4 A = __ldg(sv.tri + 3 * s);
      const float4 E1 = __ldg(sv.tri + 3 * s + 1);
      const float4 E2 = __ldg(sv.tri + 3 * s + 2);
      Contender c;
      c.slot = s;
      c.exact = false;
      c.t64 = 0.0;
      if (SPHERES && E2.w < 0.0f) {  // spheres are rare: settle in fp64 at once
        double t;
        const D3 o{(double)r.ox, (double)r.oy, (double)r.oz}, d{(double)r.dx, (double)r.dy, (double)r.dz};
        if (!sphere_hit64(sv.slot64 + 9 * (size_t)s, o, d, (double)r.tmin, (double)tmax_ray, &t)) continue;
        c.t64 = t;
        c.lo = __double2float_rd(t);
        c.hi = __double2float_ru(t);
        c.exact = true;
        take_certain(c);
        continue;
      }
      const TriClass tc = tri_classify(A, E1, E2, r, tmax_ray, tlim);
      if (tc.state == kMiss) continue;
      c.lo = __fsub_rd(tc.t, tc.et);
      c.hi = __fadd_ru(tc.t, tc.et);
      if (best.slot >= 0 && c.lo > best.hi) continue;
      if (tc.state == kHit) take_certain(c);
      else defer_maybe(c);
    }
  }
  // After the walk, warp converged: settle best and every pending contender
  // that can still win; the smallest fp64 distance wins, ties to the later slot.
  __device__ __forceinline__ void finish() {
    Contender win;
    win.slot = -1;
    win.t64 = 0.0;
    if (best.slot >= 0) {
      if (resolve(best)) win = best;
      else atomicOr(status, kStatusBound);  // a certain hit must pass its fp64 test
    }
#pragma unroll
    for (int k = 0; k < kPending; k++) {
      if (k < npend && !(best.slot >= 0 && pend[k].lo > best.hi)) {
        Contender c;
        c.slot = pend[k].slot;
        c.lo = pend[k].lo;
        c.hi = __int_as_float(0x7f800000);
        c.t64 = 0.0;
        c.exact = false;
        if (resolve(c)) {
          if (win.slot >= 0 && c.t64 == win.t64) tie = true;
          if (win.slot < 0 || c.t64 < win.t64 || (c.t64 == win.t64 && c.slot > win.slot)) win = c;
        }
      }
    }
    best = win;
  }
};

template <int STACK, bool SPHERES>
__device__ __forceinline__ HitResult closest_hit_exact(const SceneView& sv, const Ray32& r, float tmax32,
                                                       unsigned* status, bool active) {
  ExactClosestLeaf<SPHERES> leaf(sv, r, tmax32, status);
  if (active) walk<STACK>(sv, r, leaf, status);
  __syncwarp();
  if (active) leaf.finish();
  HitResult h;
  h.slot = active ? leaf.best.slot : -1;
  h.t32 = 0.0f;
  h.t64 = h.slot >= 0 ? leaf.best.t64 : -1.0;
  h.tie = h.slot >= 0 && leaf.tie;
  return h;
}

// ---- exact any hit --------------------------------------------------------------
template <bool SPHERES>
struct ExactAnyLeaf {
  const SceneView& sv;
  const Ray32& r;
  float tmax_ray;
  float tlim;
  bool done;
  __device__ ExactAnyLeaf(const SceneView& s, const Ray32& ray, float tmax)
      : sv(s), r(ray), tmax_ray(tmax), tlim(widen(tmax)), done(false) {}
  __device__ __forceinline__ void operator()(uint32_t ref) {
    const int cnt = (int)((ref >> 27) & 15u) + 1;
    const int s0 = (int)(ref & kSlotMask);
    const D3 o{(double)r.ox, (double)r.oy, (double)r.oz}, d{(double)r.dx, (double)r.dy, (double)r.dz};
    for (int k = 0; k < cnt && !done; k++) {
      const int s = s0 + k;
      const float4 A = __ldg(sv.tri + 3 * s);
      const float4 E1 = __ldg(sv.tri + 3 * s + 1);
      const float4 E2 = __ldg(sv.tri + 3 * s + 2);
      double t;
      if (SPHERES && E2.w < 0.0f) {
        done = sphere_hit64(sv.slot64 + 9 * (size_t)s, o, d, (double)r.tmin, (double)tmax_ray, &t);
        continue;
      }
      const TriClass tc = tri_classify(A, E1, E2, r, tmax_ray, tlim);
      if (tc.state == kHit) done = true;
      else if (tc.state == kMaybe)
        done = tri_hit64(sv.slot64 + 9 * (size_t)s, o, d, (double)r.tmin, (double)tmax_ray, &t);
    }
  }
};

template <int STACK, bool SPHERES>
__device__ __forceinline__ bool any_hit_exact(const SceneView& sv, const Ray32& r, float tmax32, unsigned* status) {
  ExactAnyLeaf<SPHERES> leaf(sv, r, tmax32);
  walk<STACK>(sv, r, leaf, status);
  return leaf.done;
}

// ---- fast (rendering) closest / any hit -------------------------------------------
template <bool SPHERES>
struct FastClosestLeaf {
  const SceneView& sv;
  const Ray32& r;
  float best_t;
  int32_t best_slot;
  float tlim;
  bool done;
  __device__ FastClosestLeaf(const SceneView& s, const Ray32& ray, float tmax)
      : sv(s), r(ray), best_t(tmax), best_slot(-1), tlim(widen(tmax)), done(false) {}
  __device__ __forceinline__ void reset(float tmax) {
    best_t = tmax;
    best_slot = -1;
    tlim = widen(tmax);
    done = false;
  }
  __device__ __forceinline__ void test(int s, float4 A, float4 E1, float4 E2) {
    float t;
    const bool hit = (SPHERES && E2.w < 0.0f) ? sphere_hit32(A, E1, r, best_t, &t) : tri_hit32(A, E1, E2, r, best_t, &t);
    if (hit) {
      best_t = t;
      best_slot = s;
      tlim = widen(t);
    }
  }
  // Triangles are loaded two at a time, so the second one's loads are in
  // flight while the first is tested; they are tested in slot order.
  __device__ __forceinline__ void operator()(uint32_t ref) {
    const int cnt = (int)((ref >> 27) & 15u) + 1;
    const int s0 = (int)(ref & kSlotMask);
    for (int k = 0; k < cnt; k += 2) {
      const int s = s0 + k;
      const bool two = k + 1 < cnt;
      const float4 A = __ldg(sv.tri + 3 * s);
      const float4 E1 = __ldg(sv.tri + 3 * s + 1);
      const float4 E2 = __ldg(sv.tri + 3 * s + 2);
      float4 B = A, F1 = E1, F2 = E2;
      if (two) {
        B = __ldg(sv.tri + 3 * s + 3);
        F1 = __ldg(sv.tri + 3 * s + 4);
        F2 = __ldg(sv.tri + 3 * s + 5);
      }
      test(s, A, E1, E2);
      if (two) test(s + 1, B, F1, F2);
    }
  }
};

template <bool SPHERES>
struct FastAnyLeaf {
  const SceneView& sv;
  const Ray32& r;
  float tmax;
  float tlim;
  bool done;
  __device__ FastAnyLeaf(const SceneView& s, const Ray32& ray, float tm)
      : sv(s), r(ray), tmax(tm), tlim(widen(tm)), done(false) {}
  __device__ __forceinline__ void reset(float tm) {
    tmax = tm;
    tlim = widen(tm);
    done = false;
  }
  __device__ __forceinline__ void operator()(uint32_t ref) {
    const int cnt = (int)((ref >> 27) & 15u) + 1;
    const int s0 = (int)(ref & kSlotMask);
    for (int k = 0; k < cnt && !done; k++) {
      const int s = s0 + k;
      const float4 A = __ldg(sv.tri + 3 * s);
      const float4 E1 = __ldg(sv.tri + 3 * s + 1);
      const float4 E2 = __ldg(sv.tri + 3 * s + 2);
      float t;
      done = (SPHERES && E2.w < 0.0f) ? sphere_hit32(A, E1, r, tmax, &t) : tri_hit32(A, E1, E2, r, tmax, &t);
    }
  }
};

template <int STACK, bool SPHERES>
__device__ __forceinline__ HitResult closest_hit_fast(const SceneView& sv, const Ray32& r, float tmax32,
                                                      unsigned* status) {
  FastClosestLeaf<SPHERES> leaf(sv, r, tmax32);
  walk<STACK>(sv, r, leaf, status);
  HitResult h;
  h.slot = leaf.best_slot;
  h.t32 = leaf.best_t;
  h.t64 = 0.0;
  h.tie = false;
  return h;
}

template <int STACK, bool SPHERES>
__device__ __forceinline__ bool any_hit_fast(const SceneView& sv, const Ray32& r, float tmax32, unsigned* status) {
  FastAnyLeaf<SPHERES> leaf(sv, r, tmax32);
  walk<STACK>(sv, r, leaf, status);
  return leaf.done;
}

}  // namespace bcgx

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
// bit-identical fp64 distances the later-tested primitive wins. Within a
// leaf that is the later Order slot, and the EXACT walk applies "later slot
// wins" across leaves as well.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "layout.h"

namespace bcgx {

constexpr float kU = 5.9604645e-8f;  // 2^-24, fp32 unit roundoff
constexpr float kFarSlack = 8.0e-7f;  // > 2*gamma_3 + rounding of the scaling itself

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

// Conservative limit for box culling against the current closest distance.
__device__ __forceinline__ float widen(float t) { return fmaf(fabsf(t), kFarSlack, t); }

// Slab test of one child box; returns the entry distance or +inf on a miss.
__device__ __forceinline__ float slab_near(float lox, float hix, float loy, float hiy, float loz, float hiz,
                                           const Ray32& r, float tlim) {
  float t0x = (lox - r.ox) * r.ix, t1x = (hix - r.ox) * r.ix;
  float t0y = (loy - r.oy) * r.iy, t1y = (hiy - r.oy) * r.iy;
  float t0z = (loz - r.oz) * r.iz, t1z = (hiz - r.oz) * r.iz;
  float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), r.tmin));
  float sf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z));
  float tf = fminf(widen(sf), tlim);
  return tn <= tf ? tn : __int_as_float(0x7f800000);
}

// Test all children of a node; near[k] = entry distance or +inf.
__device__ __forceinline__ void node_children(const Node8* __restrict__ node, const Ray32& r, float tlim,
                                              float near[8], uint32_t child[8]) {
  const float4* p = reinterpret_cast<const float4*>(node);
  const float4 lx0 = __ldg(p + 0), lx1 = __ldg(p + 1), hx0 = __ldg(p + 2), hx1 = __ldg(p + 3);
  const float4 ly0 = __ldg(p + 4), ly1 = __ldg(p + 5), hy0 = __ldg(p + 6), hy1 = __ldg(p + 7);
  const float4 lz0 = __ldg(p + 8), lz1 = __ldg(p + 9), hz0 = __ldg(p + 10), hz1 = __ldg(p + 11);
  const uint4 c0 = __ldg(reinterpret_cast<const uint4*>(p + 12));
  const uint4 c1 = __ldg(reinterpret_cast<const uint4*>(p + 13));
  const int nchild = __ldg(reinterpret_cast<const int*>(p + 14));
  const float lox[8] = {lx0.x, lx0.y, lx0.z, lx0.w, lx1.x, lx1.y, lx1.z, lx1.w};
  const float hix[8] = {hx0.x, hx0.y, hx0.z, hx0.w, hx1.x, hx1.y, hx1.z, hx1.w};
  const float loy[8] = {ly0.x, ly0.y, ly0.z, ly0.w, ly1.x, ly1.y, ly1.z, ly1.w};
  const float hiy[8] = {hy0.x, hy0.y, hy0.z, hy0.w, hy1.x, hy1.y, hy1.z, hy1.w};
  const float loz[8] = {lz0.x, lz0.y, lz0.z, lz0.w, lz1.x, lz1.y, lz1.z, lz1.w};
  const float hiz[8] = {hz0.x, hz0.y, hz0.z, hz0.w, hz1.x, hz1.y, hz1.z, hz1.w};
  child[0] = c0.x; child[1] = c0.y; child[2] = c0.z; child[3] = c0.w;
  child[4] = c1.x; child[5] = c1.y; child[6] = c1.z; child[7] = c1.w;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    float t = slab_near(lox[k], hix[k], loy[k], hiy[k], loz[k], hiz[k], r, tlim);
    near[k] = k < nchild ? t : __int_as_float(0x7f800000);
  }
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
__device__ __forceinline__ bool tri_hit64(const double* __restrict__ q, D3 o, D3 d, double tmin, double tmax,
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
__device__ __forceinline__ bool sphere_hit64(const double* __restrict__ q, D3 o, D3 d, double tmin, double tmax,
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

// fp32 Moller-Trumbore used as a filter: returns false only when the fp64
// test of the same triangle is certain to reject it. The error bounds are
// first-order forward bounds of each quantity against the exact result on
// the fp64 inputs (the fp32 record holds those inputs rounded to nearest),
// with at least a factor 2 of slack; R = max|A| + max|O-A|.
__device__ __forceinline__ bool tri_candidate(float4 A, float4 E1, float4 E2, const Ray32& r, float tlim) {
  const float hx = r.dy * E2.z - r.dz * E2.y;
  const float hy = r.dz * E2.x - r.dx * E2.z;
  const float hz = r.dx * E2.y - r.dy * E2.x;
  const float det = E1.x * hx + E1.y * hy + E1.z * hz;
  const float Mh = r.dmax * E2.w;
  const float errDet = 96.0f * kU * E1.w * Mh;
  const float adet = fabsf(det);
  if (adet + errDet < 1e-10f) return false;
  if (adet <= 2.0f * errDet || adet - errDet < 1e-10f) return true;  // cannot bound: re-test in fp64
  const float sx = r.ox - A.x, sy = r.oy - A.y, sz = r.oz - A.z;
  const float R = A.w + fmaxf(fabsf(sx), fmaxf(fabsf(sy), fabsf(sz)));
  const float invd = 1.0f / (adet - errDet);
  const float f = 1.0f / det;
  const float u = f * (sx * hx + sy * hy + sz * hz);
  const float eu = (96.0f * kU * R * Mh + fabsf(u) * errDet) * invd + 4.0f * kU * fabsf(u);
  if (u < -eu || u > 1.0f + eu) return false;
  const float qx = sy * E1.z - sz * E1.y;
  const float qy = sz * E1.x - sx * E1.z;
  const float qz = sx * E1.y - sy * E1.x;
  const float v = f * (r.dx * qx + r.dy * qy + r.dz * qz);
  const float ev = (96.0f * kU * r.dmax * R * E1.w + fabsf(v) * errDet) * invd + 4.0f * kU * fabsf(v);
  if (v < -ev || u + v > 1.0f + eu + ev + 4.0f * kU * fabsf(u + v)) return false;
  const float t = f * (E2.x * qx + E2.y * qy + E2.z * qz);
  const float et = (112.0f * kU * E2.w * R * E1.w + fabsf(t) * errDet) * invd + 4.0f * kU * fabsf(t);
  if (t + et < r.tmin || t - et > tlim) return false;
  return true;
}

// Plain fp32 triangle test for rendering (reference thresholds).
__device__ __forceinline__ bool tri_hit32(float4 A, float4 E1, float4 E2, const Ray32& r, float tmax, float* t_out) {
  const float hx = r.dy * E2.z - r.dz * E2.y;
  const float hy = r.dz * E2.x - r.dx * E2.z;
  const float hz = r.dx * E2.y - r.dy * E2.x;
  const float det = E1.x * hx + E1.y * hy + E1.z * hz;
  if (fabsf(det) < 1e-10f) return false;
  const float f = 1.0f / det;
  const float sx = r.ox - A.x, sy = r.oy - A.y, sz = r.oz - A.z;
  const float u = f * (sx * hx + sy * hy + sz * hz);
  if (u < 0.0f || u > 1.0f) return false;
  const float qx = sy * E1.z - sz * E1.y;
  const float qy = sz * E1.x - sx * E1.z;
  const float qz = sx * E1.y - sy * E1.x;
  const float v = f * (r.dx * qx + r.dy * qy + r.dz * qz);
  if (v < 0.0f || u + v > 1.0f) return false;
  const float t = f * (E2.x * qx + E2.y * qy + E2.z * qz);
  if (t < r.tmin || t > tmax) return false;
  *t_out = t;
  return true;
}

// Plain fp32 sphere test (sphereHitAccel in fp32) for rendering.
__device__ __forceinline__ bool sphere_hit32(float4 C, float4 S, const Ray32& r, float tmax, float* t_out) {
  const float dl2 = r.dx * r.dx + r.dy * r.dy + r.dz * r.dz;
  if (!(dl2 > 1e-18f)) return false;
  const float ocx = r.ox - C.x, ocy = r.oy - C.y, ocz = r.oz - C.z;
  const float hb = ocx * r.dx + ocy * r.dy + ocz * r.dz;
  const float cc = (ocx * ocx + ocy * ocy + ocz * ocz) - S.x;
  const float disc = hb * hb - dl2 * cc;
  if (disc < 0.0f) return false;
  const float sq = sqrtf(disc);
  const float idl2 = 1.0f / dl2;
  float root = (-hb - sq) * idl2;
  if (root < r.tmin || root > tmax) {
    root = (-hb + sq) * idl2;
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
};

// Closest hit. STACK >= the packer's stack_need; an overflow sets a status bit.
template <int STACK, bool EXACT, bool SPHERES>
__device__ __forceinline__ HitResult closest_hit(const SceneView& sv, const Ray32& r, float tmax32, double tmax64,
                                                 unsigned* status) {
  uint2 st[STACK];
  int sp = 0;
  HitResult res;
  res.slot = -1;
  res.t32 = tmax32;
  res.t64 = tmax64;
  float tlim = widen(tmax32);
  const D3 o64{(double)r.ox, (double)r.oy, (double)r.oz};
  const D3 d64{(double)r.dx, (double)r.dy, (double)r.dz};
  const double tmin64 = (double)r.tmin;
  uint32_t ref = 0;  // root Node8
  for (;;) {
    if (!(ref & kLeafBit)) {
      float nr[8];
      uint32_t ch[8];
      node_children(sv.nodes + ref, r, tlim, nr, ch);
      sort8(nr, ch);
      if (nr[0] == __int_as_float(0x7f800000)) goto pop;
#pragma unroll
      for (int k = 7; k >= 1; k--) {
        if (nr[k] != __int_as_float(0x7f800000)) {
          if (sp < STACK) {
            st[sp++] = make_uint2(ch[k], __float_as_uint(nr[k]));
          } else {
            atomicOr(status, kStatusStackOverflow);
          }
        }
      }
      ref = ch[0];
      continue;
    } else {
      const int cnt = (int)((ref >> 27) & 15u) + 1;
      const int s0 = (int)(ref & kSlotMask);
      for (int k = 0; k < cnt; k++) {
        const int s = s0 + k;
        const float4 A = __ldg(sv.tri + 3 * s);
        const float4 E1 = __ldg(sv.tri + 3 * s + 1);
        const float4 E2 = __ldg(sv.tri + 3 * s + 2);
        if (SPHERES && E2.w < 0.0f) {
          if (EXACT) {
            double t;
            if (sphere_hit64(sv.slot64 + 9 * (size_t)s, o64, d64, tmin64, res.t64, &t) &&
                (t < res.t64 || s > res.slot)) {
              res.t64 = t; res.slot = s; tlim = widen(__double2float_ru(t));
            }
          } else {
            float t;
            if (sphere_hit32(A, E1, r, res.t32, &t)) { res.t32 = t; res.slot = s; tlim = widen(t); }
          }
          continue;
        }
        if (EXACT) {
          if (!tri_candidate(A, E1, E2, r, tlim)) continue;
          double t;
          if (tri_hit64(sv.slot64 + 9 * (size_t)s, o64, d64, tmin64, res.t64, &t) && (t < res.t64 || s > res.slot)) {
            res.t64 = t; res.slot = s; tlim = widen(__double2float_ru(t));
          }
        } else {
          float t;
          if (tri_hit32(A, E1, E2, r, res.t32, &t)) { res.t32 = t; res.slot = s; tlim = widen(t); }
        }
      }
    }
  pop:
    for (;;) {
      if (sp == 0) return res;
      const uint2 e = st[--sp];
      if (__uint_as_float(e.y) <= tlim) {
        ref = e.x;
        break;
      }
    }
  }
}

// Any hit within [tmin, tmax] (Scene.Occluded semantics). Children are pushed
// unsorted; the first confirmed hit ends the walk.
template <int STACK, bool EXACT, bool SPHERES>
__device__ __forceinline__ bool any_hit(const SceneView& sv, const Ray32& r, float tmax32, double tmax64,
                                        unsigned* status) {
  uint32_t st[STACK];
  int sp = 0;
  const float tlim = widen(tmax32);
  const D3 o64{(double)r.ox, (double)r.oy, (double)r.oz};
  const D3 d64{(double)r.dx, (double)r.dy, (double)r.dz};
  const double tmin64 = (double)r.tmin;
  uint32_t ref = 0;
  for (;;) {
    if (!(ref & kLeafBit)) {
      float nr[8];
      uint32_t ch[8];
      node_children(sv.nodes + ref, r, tlim, nr, ch);
      int first = -1;
#pragma unroll
      for (int k = 0; k < 8; k++) {
        if (nr[k] != __int_as_float(0x7f800000)) {
          if (first < 0) {
            first = k;
          } else if (sp < STACK) {
            st[sp++] = ch[k];
          } else {
            atomicOr(status, kStatusStackOverflow);
          }
        }
      }
      if (first >= 0) {
        ref = ch[first];
        continue;
      }
    } else {
      const int cnt = (int)((ref >> 27) & 15u) + 1;
      const int s0 = (int)(ref & kSlotMask);
      for (int k = 0; k < cnt; k++) {
        const int s = s0 + k;
        const float4 A = __ldg(sv.tri + 3 * s);
        const float4 E1 = __ldg(sv.tri + 3 * s + 1);
        const float4 E2 = __ldg(sv.tri + 3 * s + 2);
        if (SPHERES && E2.w < 0.0f) {
          if (EXACT) {
            double t;
            if (sphere_hit64(sv.slot64 + 9 * (size_t)s, o64, d64, tmin64, tmax64, &t)) return true;
          } else {
            float t;
            if (sphere_hit32(A, E1, r, tmax32, &t)) return true;
          }
          continue;
        }
        if (EXACT) {
          double t;
          if (tri_candidate(A, E1, E2, r, tlim) && tri_hit64(sv.slot64 + 9 * (size_t)s, o64, d64, tmin64, tmax64, &t))
            return true;
        } else {
          float t;
          if (tri_hit32(A, E1, E2, r, tmax32, &t)) return true;
        }
      }
    }
    if (sp == 0) return false;
    ref = st[--sp];
  }
}

}  // namespace bcgx

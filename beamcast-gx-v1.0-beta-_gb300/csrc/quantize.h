// Quantization of a Node8's child boxes and packing of one primitive slot,
// shared by the host packer (pack.cpp, compiled by the host compiler) and the
// device geometry update (refit.cu): both paths produce the same bytes.
#pragma once
#include <math.h>
#include <algorithm>
#include <stdint.h>

#include "layout.h"

#if defined(__CUDACC__)
#define BC_HD __host__ __device__ __forceinline__
#else
#define BC_HD inline
#endif

namespace bcgx {

// Directed rounding of a double to float (toward -inf / +inf).
BC_HD float rd_f32(double x) {
  float f = (float)x;
  if ((double)f > x) f = nextafterf(f, -INFINITY);
  return f;
}
BC_HD float ru_f32(double x) {
  float f = (float)x;
  if ((double)f < x) f = nextafterf(f, INFINITY);
  return f;
}

// Quantizes nk child boxes (6 doubles each: lo xyz, hi xyz) into n's grid
// fields and child bounds; child refs and the child count are not touched.
// Per axis: p = the children's union minimum rounded down to fp32 and stepped
// one ulp further down, the grid step 2^e the smallest power of two with
// 254 * 2^e >= extent, qlo = the largest q with p + q 2^e < lo (strict), qhi =
// the smallest q with p + q 2^e > hi. The device decodes with round-down (lo)
// and round-up (hi) arithmetic or with explicit rounding margins, which keeps
// the strict inequalities, so a ray origin on a face of the fp64 box is
// strictly inside the decoded box (the reference's zero-direction axes test
// origins against closed boxes). Empty slots get qlo = 255, qhi = 0.
BC_HD void quantize_children(Node8& n, const double* boxes, int nk) {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int k = 0; k < nk; k++)
    for (int a = 0; a < 3; a++) {
      lo[a] = fmin(lo[a], boxes[6 * k + a]);
      hi[a] = fmax(hi[a], boxes[6 * k + 3 + a]);
    }
  float p[3];
  double scale[3];
  uint8_t eb[3];
  for (int a = 0; a < 3; a++) {
    p[a] = nextafterf(rd_f32(lo[a]), -INFINITY);
    const double extent = hi[a] - (double)p[a];
    // the least e in [-126, 127] with 254 * 2^e >= extent (127 if none); the
    // host starts the search at ilogb(extent) - 9, which is never above it
    int e = -126;
#ifndef __CUDA_ARCH__
    if (extent > 0) e = std::max(-126, std::min(127, ilogb(extent) - 9));
#endif
    while (e < 127 && ldexp(254.0, e) < extent) e++;
    eb[a] = (uint8_t)(e + 127);
    scale[a] = ldexp(1.0, e);
  }
  n.px = p[0];
  n.py = p[1];
  n.pz = p[2];
  n.ex = eb[0];
  n.ey = eb[1];
  n.ez = eb[2];
  uint8_t* qlo[3] = {n.qlox, n.qloy, n.qloz};
  uint8_t* qhi[3] = {n.qhix, n.qhiy, n.qhiz};
  for (int k = 0; k < 8; k++)
    for (int a = 0; a < 3; a++) {
      if (k >= nk) {
        qlo[a][k] = 255;
        qhi[a][k] = 0;
        continue;
      }
      const double bl = boxes[6 * k + a], bh = boxes[6 * k + 3 + a];
      double ql = floor((bl - (double)p[a]) / scale[a]);
      ql = fmax(0.0, fmin(255.0, ql));
      while (ql > 0 && (double)p[a] + ql * scale[a] >= bl) ql -= 1;
      double qh = ceil((bh - (double)p[a]) / scale[a]);
      qh = fmax(0.0, fmin(255.0, qh));
      while (qh < 255 && (double)p[a] + qh * scale[a] <= bh) qh += 1;
      qlo[a][k] = (uint8_t)ql;
      qhi[a][k] = (uint8_t)qh;
    }
}

// One primitive slot from the fp64 primitive (renderer.go:109-118): the fp32
// records tri[3], the fp64 record q[9] and the normal (material bits kept by
// the caller). sphere: center c, radius rad; triangle: a, e1, e2, normal nn.
BC_HD void pack_slot(bool sphere, const double* c, double rad, const double* a, const double* e1, const double* e2,
                     const double* nn, F4* r, double* q, float* normal) {
  if (sphere) {
    r[0] = F4{(float)c[0], (float)c[1], (float)c[2], (float)rad};
    r[1] = F4{(float)(rad * rad), rad > 0 ? (float)(1.0 / rad) : 0.0f, 0.0f, 0.0f};
    r[2] = F4{0.0f, 0.0f, 0.0f, -1.0f};
    q[0] = c[0]; q[1] = c[1]; q[2] = c[2]; q[3] = rad;
    for (int k = 4; k < 9; k++) q[k] = 0.0;
    normal[0] = normal[1] = normal[2] = 0.0f;
  } else {
    const double ma = fmax(fabs(a[0]), fmax(fabs(a[1]), fabs(a[2])));
    const double m1 = fmax(fabs(e1[0]), fmax(fabs(e1[1]), fabs(e1[2])));
    const double m2 = fmax(fabs(e2[0]), fmax(fabs(e2[1]), fabs(e2[2])));
    r[0] = F4{(float)a[0], (float)a[1], (float)a[2], ru_f32(ma)};
    r[1] = F4{(float)e1[0], (float)e1[1], (float)e1[2], ru_f32(m1)};
    r[2] = F4{(float)e2[0], (float)e2[1], (float)e2[2], ru_f32(m2)};
    for (int k = 0; k < 3; k++) {
      q[k] = a[k];
      q[3 + k] = e1[k];
      q[6 + k] = e2[k];
    }
    normal[0] = (float)nn[0];
    normal[1] = (float)nn[1];
    normal[2] = (float)nn[2];
  }
}

}  // namespace bcgx

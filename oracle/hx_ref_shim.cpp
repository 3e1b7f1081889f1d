// Test infrastructure only: a C entry point over the reference's own C++
// closest-hit code (beamcast::hx::PackedScene in source/src/hx.cpp, compiled
// from the reference's sources by the `ref` target of oracle/Makefile into
// oracle/_ref/). Nothing in the product links it: the ray-cast tests use it to
// cross-check the oracle's fp64 triangle test (renderer.go:684-711) against an
// independent implementation the reference ships (fp32 Moller-Trumbore,
// hx.cpp:223-231, behind its own SAH BVH, hx.cpp:237-270).
#include <cstdint>
#include <exception>
#include <vector>

#include "beamcast/hx.hpp"

extern "C" {

// verts: 9 doubles per triangle (a, b, c); rays: 8 floats (ox, oy, oz, tmin,
// dx, dy, dz, tmax). prim_out: index of the closest triangle in the caller's
// numbering (-1: miss); t_out: its fp32 distance. Triangles the reference
// rejects (zero area in fp32) are skipped and never reported. Returns 0, or -1
// if the reference threw.
int hxref_closest(int n_tris, const double* verts, int64_t n_rays, const float* rays, int32_t* prim_out,
                  float* t_out) {
  using namespace beamcast;
  try {
    hx::PackedScene scene;
    const std::uint32_t m = scene.add_lambertian(Color{0.5f, 0.5f, 0.5f});
    std::vector<int32_t> caller_index;  // hx triangle index -> caller's index
    for (int i = 0; i < n_tris; i++) {
      const double* v = verts + 9 * (size_t)i;
      try {
        scene.add_triangle(Point3{(float)v[0], (float)v[1], (float)v[2]},
                           Point3{(float)v[3], (float)v[4], (float)v[5]},
                           Point3{(float)v[6], (float)v[7], (float)v[8]}, m);
        caller_index.push_back(i);
      } catch (const std::invalid_argument&) {
      }
    }
    scene.build();
    for (int64_t k = 0; k < n_rays; k++) {
      const float* r = rays + 8 * (size_t)k;
      const Ray ray(Point3{r[0], r[1], r[2]}, Vec3{r[4], r[5], r[6]});
      hx::PackedHit h;
      if (scene.hit(ray, r[3], r[7], h) && h.primitive_type == 1) {
        prim_out[k] = caller_index[h.primitive_index];
        t_out[k] = h.t;
      } else {
        prim_out[k] = -1;
        t_out[k] = -1.0f;
      }
    }
  } catch (const std::exception&) {
    return -1;
  }
  return 0;
}

}  // extern "C"

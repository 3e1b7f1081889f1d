// Device-resident scene layout of the GB300 hot path. Shared by the host
// packer (pack.cpp) and the CUDA kernels.
//
// HBM layout (all arrays 256-byte aligned by cudaMalloc):
//   Node8  nodes[n8]      256 B each: child boxes SoA (6 x 8 fp32), 8 child refs,
//                         child count. One node = four 64-byte sectors, fetched
//                         with 128-bit loads.
//   float4 tri[3*slots]   48 B per primitive slot, slots in Scene.Order order so a
//                         leaf's primitives are contiguous:
//                           triangle: (A, max|A|) (E1, max|E1|) (E2, max|E2|)
//                           sphere:   (C, r) (r*r, 1/r, 0, 0) (0, 0, 0, -1)
//   double slot64[9*slots] the fp64 primitive (A, E1, E2 or C, r) for the
//                         exact re-test of the ray-cast entry points.
//   float4 snorm[slots]   unit normal (triangles) and material index bits in .w.
//   int32  slot_prim[slots] Scene primitive index of each slot (Scene.Order).
#pragma once
#include <stdint.h>

namespace bcgx {

// Child reference: bit 31 clear -> index of an inner Node8;
// bit 31 set -> leaf: bits 27..30 = count-1 (1..16 primitives), bits 0..26 = first slot.
// The same packing as the reference's compact node meta (gpu_opencl_windows.go:345-350).
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr uint32_t kSlotMask = 0x07ffffffu;
constexpr int32_t kMaxIndex = 1 << 27;

// Status bits written by kernels (never a trap): the host turns them into errors.
constexpr unsigned kStatusStackOverflow = 1u;
constexpr unsigned kStatusTimeout = 2u;
constexpr unsigned kStatusCapacity = 4u;
constexpr unsigned kStatusBound = 8u;  // an fp32 hit classified as certain failed its fp64 test

struct alignas(64) Node8 {
  float lox[8], hix[8], loy[8], hiy[8], loz[8], hiz[8];
  uint32_t child[8];
  int32_t nchild;
  int32_t pad[7];
};
static_assert(sizeof(Node8) == 256, "Node8 must be 256 bytes");

struct alignas(16) F4 {
  float x, y, z, w;
};

// Material record: (color, roughness) (emission, kind code)
// kind code: 0 diffuse, 1 metal, 2 glass, 3 emissive; ior in .w of the first word set.
struct alignas(16) MatGPU {
  float cr, cg, cb, rough;
  float er, eg, eb, kind;
  float ior, preview_r, preview_g, preview_b;  // ior and materialPreviewColor (renderer.go:1467)
};
static_assert(sizeof(MatGPU) == 48, "MatGPU must be 48 bytes");

// Sphere light record for next-event estimation (emissive spheres only,
// renderer.go:253-255): center, radius, emission, selection pdf, prim index.
struct alignas(16) LightGPU {
  float cx, cy, cz, r;
  float er, eg, eb, select_pdf;
  int32_t prim;
  int32_t pad;
  double cdf;  // fp64, so the CDF search takes the CPU's branch for every draw
};
static_assert(sizeof(LightGPU) == 48, "LightGPU must be 48 bytes");

}  // namespace bcgx

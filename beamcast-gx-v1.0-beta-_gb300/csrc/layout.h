// Device-resident scene layout of the GB300 hot path. Shared by the host
// packer (pack.cpp) and the CUDA kernels.
//
// HBM layout (all arrays 256-byte aligned by cudaMalloc):
//   Node8  nodes[n8]      96 B each: quantization grid (origin, 3 exponents),
//                         child count, 8 child refs, 8-bit child box bounds.
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

// Wide node with quantized child boxes (96 bytes, six 128-bit loads). Each
// axis has a power-of-two grid anchored at (px, py, pz): a child's box on that
// axis is [p + qlo * 2^(e-127), p + qhi * 2^(e-127)], decoded on the device with
// round-down / round-up FMAs. The packer picks p, e and q so that every decoded
// box strictly contains the fp64 box of the binary node it stands for.
struct alignas(16) Node8 {
  float px, py, pz;
  uint8_t ex, ey, ez;  // biased exponents of the grid step per axis
  uint8_t nchild;
  uint32_t child[8];
  uint8_t qlox[8], qhix[8], qloy[8], qhiy[8], qloz[8], qhiz[8];
};
static_assert(sizeof(Node8) == 96, "Node8 must be 96 bytes");

// The caller's binary BVH node (Scene.Nodes, renderer.go:109-118) as the
// reference traverses it: fp64 box, children (-1 for leaves), leaf range in
// Order. Only rays whose closest hit is an exact fp64 tie read these: they are
// re-walked with the reference's own traversal so the tie resolves as it does.
struct alignas(16) BinNode {
  double lo[3], hi[3];
  int32_t left, right, start, count;
};
static_assert(sizeof(BinNode) == 64, "BinNode must be 64 bytes");

// Result marker of a ray-cast pass for a ray whose closest fp64 distance is
// shared by several primitives; the tie pass replaces it by the reference's answer.
constexpr int32_t kTieMark = -2;

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
  // the largest fp32 value <= cdf: for a draw u that is an fp32 value,
  // cdf >= u exactly when cdf_dn >= u, so the search takes the CPU's fp64
  // branch for every draw without fp64 arithmetic on the device
  float cdf_dn;
  double cdf;  // the light CDF entry (fp64, as the CPU holds it)
};
static_assert(sizeof(LightGPU) == 48, "LightGPU must be 48 bytes");

}  // namespace bcgx

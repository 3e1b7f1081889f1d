// Photon map of the photon-mapping integrator on the device (PhotonMap,
// renderer.go:1623-1761) and the hit-surface helper shared by the photon
// tracer and the shading kernels.
//
// The reference keeps map[uint64][]int from photonCellKey to the indices of
// the photons in that cell, in append order. Here the photons are sorted by
// (cell key, append index), so every key's photons are one contiguous run in
// the reference's order; an open-addressing table maps a key to its run.
#pragma once
#include <stdint.h>

#include "sampling.cuh"
#include "trace_core.cuh"

namespace bcgx {

constexpr uint64_t kPhotonStream = 0xFFFFFFFFull;  // sample index of the photon emission streams
constexpr int kGatherMax = 64;                      // tracePhotonMapped gathers at most 64 photons

// Dense cell table of a photon map, written on the device with the map: for
// every cell of the box [g0, g0 + dim) the index of its key's run in the
// sorted photons, or -1; dim[0] == 0: no table (the hash lookup serves). The box
// spans the photons' cells and two more on each side, so the 27 neighbours of
// every cell within one cell of a photon's are in it.
struct PhotonGrid {
  long long g0[3];
  int dim[3];
  int pad;
};

struct PhotonView {
  const float4* pos;                // photons in (cell key, append index) order: position
  const float4* nrm;                // facing normal at the deposit
  const float4* flux;               // flux
  const unsigned long long* ukey;   // distinct cell keys
  const int2* span;                 // (first photon, count) of each distinct key
  const int* table;                 // 0: empty slot, else distinct-key index + 1; null: empty map
  int mask;                         // table size - 1
  float cell, r2, pir2;             // cell size (= radius), radius^2, pi radius^2
  const PhotonGrid* grid;           // null: no dense table
  const int* dense;
};

// photonCellKey (renderer.go:1636-1639): the int64 products wrap, as unsigned products do.
__host__ __device__ __forceinline__ unsigned long long photon_cell_key(long long x, long long y, long long z) {
  return ((unsigned long long)x * 73856093ull) ^ ((unsigned long long)y * 19349663ull) ^
         ((unsigned long long)z * 83492791ull);
}

__host__ __device__ __forceinline__ uint32_t photon_slot_hash(unsigned long long k) {
  return (uint32_t)((k * 0x9E3779B97F4A7C15ull) >> 32);
}

// Index of the distinct key `key`, or -1.
__device__ __forceinline__ int photon_cell_lookup(const PhotonView& pm, unsigned long long key) {
  uint32_t h = photon_slot_hash(key) & (uint32_t)pm.mask;
  for (int probe = 0; probe <= pm.mask; probe++) {
    const int t = __ldg(pm.table + h);
    if (t == 0) return -1;
    if (__ldg(pm.ukey + t - 1) == key) return t - 1;
    h = (h + 1) & (uint32_t)pm.mask;
  }
  return -1;
}

// The photons of run u, in append order, within the radius of p and facing n
// (renderer.go:1745-1752); true once kGatherMax photons are counted.
__device__ __forceinline__ bool gather_run(const PhotonView& pm, int u, float3 p, float3 n, float3& sum, int& count) {
  const int2 sp = __ldg(pm.span + u);
  for (int i = sp.x; i < sp.x + sp.y; i++) {
    const float4 P = __ldg(pm.pos + i);
    const float4 N = __ldg(pm.nrm + i);
    const float3 d = f3(P.x - p.x, P.y - p.y, P.z - p.z);
    const float nd = N.x * n.x + N.y * n.y + N.z * n.z;
    if (dot3(d, d) > pm.r2 || nd <= 0.05f) continue;
    const float4 F = __ldg(pm.flux + i);
    sum = sum + f3(F.x, F.y, F.z) * nd;
    if (++count >= kGatherMax) return true;
  }
  return false;
}

// PhotonMap.gather(p, n, 64) (renderer.go:1730-1761): the 27 cells around p in
// (dz, dy, dx) order, each cell's photons in append order; a key shared by two
// of the cells is visited twice, as the reference's map lookups do. With a
// dense table each cell costs one load instead of a hash probe; a point more
// than one cell outside the photons' cells has no photon within the radius
// (cells are one radius wide), so its gather is zero, as the loop would find.
__device__ __forceinline__ float3 photon_gather(const PhotonView& pm, float3 p, float3 n) {
  if (!pm.table) return f3(0.0f, 0.0f, 0.0f);
  const long long cx = (long long)floorf(p.x / pm.cell);
  const long long cy = (long long)floorf(p.y / pm.cell);
  const long long cz = (long long)floorf(p.z / pm.cell);
  float3 sum = f3(0.0f, 0.0f, 0.0f);
  int count = 0;
  bool full = false;
  const PhotonGrid* G = pm.dense ? pm.grid : nullptr;
  const int gx = G ? __ldg(&G->dim[0]) : 0;
  if (gx > 0) {
    const int gy = __ldg(&G->dim[1]), gz = __ldg(&G->dim[2]);
    const long long lx = cx - __ldg(&G->g0[0]), ly = cy - __ldg(&G->g0[1]), lz = cz - __ldg(&G->g0[2]);
    if (lx < 1 || ly < 1 || lz < 1 || lx > gx - 2 || ly > gy - 2 || lz > gz - 2) return f3(0.0f, 0.0f, 0.0f);
    for (int dz = -1; dz <= 1 && !full; dz++)
      for (int dy = -1; dy <= 1 && !full; dy++)
        for (int dx = -1; dx <= 1 && !full; dx++) {
          const int u = __ldg(pm.dense + ((lz + dz) * gy + (ly + dy)) * (long long)gx + (lx + dx));
          if (u >= 0) full = gather_run(pm, u, p, n, sum, count);
        }
  } else {
    for (int dz = -1; dz <= 1 && !full; dz++)
      for (int dy = -1; dy <= 1 && !full; dy++)
        for (int dx = -1; dx <= 1 && !full; dx++) {
          const int u = photon_cell_lookup(pm, photon_cell_key(cx + dx, cy + dy, cz + dz));
          if (u >= 0) full = gather_run(pm, u, p, n, sum, count);
        }
  }
  if (count == 0) return f3(0.0f, 0.0f, 0.0f);
  return sum * (1.0f / (pm.pir2 * (float)count));
}

// Hit point and facing normal of a closest hit at fp32 distance t: the
// sphereHitAccel normal (renderer.go:670-677) or the triangle's unit normal,
// flipped to face the ray (triHit, renderer.go:704-710). `nrm` is the slot's snorm word.
struct Surface {
  float3 p, N;
  float radius;  // sphere radius, 0 for triangles
  bool front, sphere;
};
__device__ __forceinline__ Surface hit_surface(const SceneView& sv, int slot, float4 nrm, float3 o, float3 d, float t) {
  Surface S;
  S.p = o + d * t;
  const float4 r2 = __ldg(sv.tri + 3 * slot + 2);
  S.sphere = r2.w < 0.0f;
  S.radius = 0.0f;
  if (S.sphere) {
    const float4 c = __ldg(sv.tri + 3 * slot);
    S.radius = c.w;
    const float3 outward = (S.p - f3(c.x, c.y, c.z)) * (1.0f / c.w);
    S.front = dot3(d, outward) < 0.0f;
    S.N = S.front ? outward : outward * -1.0f;
  } else {
    S.N = f3(nrm.x, nrm.y, nrm.z);
    S.front = dot3(d, S.N) < 0.0f;
    if (!S.front) S.N = S.N * -1.0f;
  }
  return S;
}

}  // namespace bcgx

// Geometry-only scene update on the device: the path of ensureSceneLocked
// that calls updateGeometryLocked (gpu_opencl_windows.go:447-468, 484-495)
// when only the geometry revision moved (an interactive drag followed by
// Scene.Refit, renderer.go:451-473). The BVH8 topology of the resident scene
// is kept; the caller's new fp64 primitives and refit binary node boxes are
// copied up and two kernels rewrite the primitive slots and re-quantize every
// Node8 from the boxes of the binary nodes its children stand for. The bytes
// equal what the host packer writes for the same primitives and boxes
// (quantize.h is shared by both).
#include <cstring>
#include <string>
#include <vector>

#include "context.h"
#include "quantize.h"

namespace bcgx {

// fp64 geometry of the caller, one array after the other (3n, 3n, 3n, 3n, 3n, n, 6m doubles).
struct GeomView {
  const double *a, *e1, *e2, *nrm, *ctr, *rad, *box;
};

__global__ void k_refit_slots(int n, const int32_t* __restrict__ slot_prim, GeomView g, float4* __restrict__ tri,
                              double* __restrict__ slot64, float4* __restrict__ snorm) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int p = slot_prim[s];
  const bool sphere = tri[3 * (size_t)s + 2].w < 0.0f;  // the kind is part of the topology
  const size_t k3 = 3 * (size_t)p;
  const double zero[3] = {0.0, 0.0, 0.0};
  F4 r[3];
  double q[9];
  float nn[3];
  pack_slot(sphere, sphere ? g.ctr + k3 : zero, sphere ? g.rad[p] : 0.0, sphere ? zero : g.a + k3,
            sphere ? zero : g.e1 + k3, sphere ? zero : g.e2 + k3, sphere ? zero : g.nrm + k3, r, q, nn);
  for (int k = 0; k < 3; k++) tri[3 * (size_t)s + k] = make_float4(r[k].x, r[k].y, r[k].z, r[k].w);
  for (int k = 0; k < 9; k++) slot64[9 * (size_t)s + k] = q[k];
  const float w = snorm[s].w;  // material bits stay
  snorm[s] = make_float4(nn[0], nn[1], nn[2], w);
}

__global__ void k_refit_nodes(int n8, const int32_t* __restrict__ kids8, const double* __restrict__ box,
                              Node8* __restrict__ nodes) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n8) return;
  Node8 nd = nodes[k];
  double boxes[48];
  const int nk = nd.nchild;
  for (int c = 0; c < nk; c++) {
    const int b = kids8[8 * (size_t)k + c];
    for (int j = 0; j < 6; j++) boxes[6 * c + j] = box[6 * (size_t)b + j];
  }
  quantize_children(nd, boxes, nk);
  nodes[k] = nd;
}

__global__ void k_refit_binary(int m, const double* __restrict__ box, BinNode* __restrict__ bin) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  for (int k = 0; k < 3; k++) {
    bin[i].lo[k] = box[6 * (size_t)i + k];
    bin[i].hi[k] = box[6 * (size_t)i + 3 + k];
  }
}

static bc_status put(bc_context* ctx, double* dst, const double* src, size_t n) {
  if (!n) return BC_OK;
  cudaError_t e = cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
  return e ? cuda_status(ctx, e, "geometry upload") : BC_OK;
}

// Returns BC_OK after updating, or BC_ERR_INVALID_ARG (without touching the
// resident scene) when the descriptor does not fit the resident topology; the
// caller then takes the full upload path.
bc_status update_geometry(bc_context* ctx, const bc_scene_desc& d) {
  GeomInfo& gi = ctx->geom;
  if (!gi.valid || d.n_prims != ctx->ds.n_prims || d.n_nodes != gi.n_binary || d.n_lights != gi.n_lights ||
      d.n_materials != gi.n_materials || !d.node_box || (gi.has_tris && (!d.prim_a || !d.prim_e1 || !d.prim_e2 ||
      !d.prim_normal)) || (ctx->ds.has_spheres && (!d.prim_center || !d.prim_radius)) ||
      (d.n_lights > 0 && (!d.light_spheres || !d.light_cdf)))
    return BC_ERR_INVALID_ARG;
  for (int32_t i = 0; i < d.n_lights; i++)  // light records index primitives: keep them in range
    if (d.light_spheres[i] < 0 || d.light_spheres[i] >= d.n_prims) return BC_ERR_INVALID_ARG;
  const size_t n = (size_t)d.n_prims, m = (size_t)d.n_nodes;
  cudaError_t e = ctx->d_geom.ensure((16 * n + 6 * m) * sizeof(double));
  if (e) return cuda_status(ctx, e, "geometry staging");
  double* base = ctx->d_geom.as<double>();
  GeomView g;
  g.a = base;
  g.e1 = base + 3 * n;
  g.e2 = base + 6 * n;
  g.nrm = base + 9 * n;
  g.ctr = base + 12 * n;
  g.rad = base + 15 * n;
  g.box = base + 16 * n;
  bc_status st;
  if (gi.has_tris && ((st = put(ctx, base, d.prim_a, 3 * n)) || (st = put(ctx, base + 3 * n, d.prim_e1, 3 * n)) ||
                      (st = put(ctx, base + 6 * n, d.prim_e2, 3 * n)) ||
                      (st = put(ctx, base + 9 * n, d.prim_normal, 3 * n))))
    return st;
  if (ctx->ds.has_spheres &&
      ((st = put(ctx, base + 12 * n, d.prim_center, 3 * n)) || (st = put(ctx, base + 15 * n, d.prim_radius, n))))
    return st;
  if ((st = put(ctx, base + 16 * n, d.node_box, 6 * m))) return st;
  k_refit_slots<<<(int)((n + 255) / 256), 256, 0, ctx->stream>>>(
      (int)n, ctx->ds.slot_prim, g, const_cast<float4*>(ctx->ds.tri), const_cast<double*>(ctx->ds.slot64),
      const_cast<float4*>(ctx->ds.snorm));
  k_refit_nodes<<<(gi.n_node8 + 127) / 128, 128, 0, ctx->stream>>>(gi.n_node8, ctx->d_kids8.as<int32_t>(), g.box,
                                                                  const_cast<Node8*>(ctx->ds.nodes));
  if (ctx->ds.n_bin == (int32_t)m)  // the binary boxes the exact-tie replay walks
    k_refit_binary<<<(int)((m + 255) / 256), 256, 0, ctx->stream>>>((int)m, g.box, const_cast<BinNode*>(ctx->ds.bin));
  if ((e = cudaGetLastError())) return cuda_status(ctx, e, "geometry update");
  // sphere lights follow their spheres (and the caller's light distribution)
  PackedScene lp;
  pack_scene_lights(d, &lp);
  if (!lp.lights.empty()) {
    e = cudaMemcpyAsync(ctx->d_lights.p, lp.lights.data(), lp.lights.size() * sizeof(LightGPU),
                        cudaMemcpyHostToDevice, ctx->stream);
    if (!e)
      e = cudaMemcpyAsync(ctx->d_lpdf.p, lp.light_pdf_by_prim.data(), lp.light_pdf_by_prim.size() * sizeof(float),
                          cudaMemcpyHostToDevice, ctx->stream);
  }
  if (!e) e = cudaStreamSynchronize(ctx->stream);  // the host arrays of lp die here
  if (e) return cuda_status(ctx, e, "geometry update");
  return BC_OK;
}

}  // namespace bcgx

// Autotuner: chooses a context's tuning options by timing the candidates on the
// caller's own work, then keeps the fastest. No counterpart in the reference,
// whose OpenCL path picks a work-group size once (gpu_opencl_windows.go:285-304).
//
//   ray cast: the exact kernels' form (raycast_split 1: walk and fp64
//             settlement passes; 0: one kernel, with register budget
//             raycast_minblocks 6, 8, 1) and the coherent ray order
//             (raycast_sort 1, 0); plain fp32 mode has the order only. CUDA events on the context's stream, best of two
//             runs after one warm-up, on the caller's rays.
//   render:   the extend kernel's variant (render_extend 0, 1, 2: register
//             budget and where the ray lives, i.e. resident blocks per SM) at
//             the current wave size, the shading kernel's block shape
//             (render_shade_block 256, 128), then paths per wave (render_wave_cap
//             2^22 .. 2^27) with the chosen variant, on the caller's batch with
//             spp scaled down so one candidate traces at most 2^27 paths.
//             Images depend on neither option, so no candidate changes a result.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "context.h"
#include "kernels.h"
#include "wave.h"

namespace bcgx {

bc_status batch_requests(bc_context* ctx, const bc_view* views, int32_t n_views, std::vector<ViewRequest>* req,
                         long long* px);  // render.cu

static bc_status time_raycast(bc_context* ctx, const float* d_rays, int64_t n, float* t, int32_t* p, float* ms) {
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaEventCreate(&a);
  if (!e) e = cudaEventCreate(&b);
  float best = 0.0f;
  for (int k = 0; k < 3 && !e; k++) {
    e = cudaEventRecord(a, ctx->stream);
    if (e) break;
    bc_status st = bc_raycast_device(ctx, d_rays, n, t, p, ctx->stream);
    if (st) {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      return st;
    }
    e = cudaEventRecord(b, ctx->stream);
    if (!e) e = cudaEventSynchronize(b);
    float m = 0.0f;
    if (!e) e = cudaEventElapsedTime(&m, a, b);
    if (k == 1 || (k == 2 && m < best)) best = m;  // run 0 warms up
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (e) return cuda_status(ctx, e, "autotune timing");
  *ms = best;
  return check_kernel_status(ctx);
}

}  // namespace bcgx

using namespace bcgx;

extern "C" {

bc_status bc_autotune_raycast(bc_context* ctx, const float* d_rays, int64_t n, bc_tune_report* out) {
  if (!ctx || !d_rays || n < 1) return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument or no rays");
  if (!ctx->has_scene) return set_error(ctx, BC_ERR_NO_SCENE, "no scene uploaded");
  cudaSetDevice(ctx->device);
  cudaError_t e = ctx->d_t.ensure((size_t)n * 4);
  if (!e) e = ctx->d_prim.ensure((size_t)n * 4);
  if (e) return cuda_status(ctx, e, "autotune buffers");
  struct Cand { int split, minblocks, sort; };
  std::vector<Cand> cands;
  if (ctx->raycast_exact) {
    for (int so : {1, 0}) cands.push_back(Cand{1, ctx->raycast_minblocks, so});
    for (int mb : {6, 8, 1})
      for (int so : {1, 0}) cands.push_back(Cand{0, mb, so});
  } else {
    cands = {Cand{ctx->raycast_split, ctx->raycast_minblocks, 1}, Cand{ctx->raycast_split, ctx->raycast_minblocks, 0}};
  }
  const int keep_mb = ctx->raycast_minblocks, keep_sort = ctx->raycast_sort, keep_split = ctx->raycast_split;
  bc_tune_report rep;
  std::memset(&rep, 0, sizeof(rep));
  int best = -1;
  for (size_t i = 0; i < cands.size(); i++) {
    ctx->raycast_split = cands[i].split;
    ctx->raycast_minblocks = cands[i].minblocks;
    ctx->raycast_variant = ctx->raycast_exact ? cands[i].minblocks : 0;
    ctx->raycast_sort = cands[i].sort;
    float ms = 0.0f;
    bc_status st = time_raycast(ctx, d_rays, n, ctx->d_t.as<float>(), ctx->d_prim.as<int32_t>(), &ms);
    if (st) {  // leave the options as they were
      ctx->raycast_split = keep_split;
      ctx->raycast_minblocks = keep_mb;
      ctx->raycast_variant = ctx->raycast_exact ? keep_mb : 0;
      ctx->raycast_sort = keep_sort;
      return st;
    }
    rep.n_timed++;
    if (cands[i].split == keep_split && cands[i].sort == keep_sort && (keep_split || cands[i].minblocks == keep_mb))
      rep.default_ms = ms;
    if (best < 0 || ms < rep.best_ms) {
      best = (int)i;
      rep.best_ms = ms;
    }
    if (ms > rep.worst_ms) rep.worst_ms = ms;
  }
  ctx->raycast_split = cands[best].split;
  ctx->raycast_minblocks = cands[best].minblocks;
  ctx->raycast_variant = ctx->raycast_exact ? cands[best].minblocks : 0;
  ctx->raycast_sort = cands[best].sort;
  rep.raycast_split = ctx->raycast_split;
  rep.raycast_minblocks = ctx->raycast_minblocks;
  rep.raycast_sort = ctx->raycast_sort;
  rep.render_wave_cap = ctx->render_wave_cap;
  rep.render_extend = ctx->render_extend;
  rep.render_shade_block = ctx->render_shade_block;
  if (out) *out = rep;
  return BC_OK;
}

bc_status bc_autotune_render(bc_context* ctx, const bc_view* views, int32_t n_views, bc_tune_report* out) {
  if (!ctx || !views || n_views < 1) return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument or no views");
  cudaSetDevice(ctx->device);
  std::vector<ViewRequest> req;
  long long px = 0;
  bc_status st = batch_requests(ctx, views, n_views, &req, &px);
  if (st) return st;
  // a bounded sample of the batch: every view keeps its size and bounces, its
  // spp scales so the sample traces at most 2^27 paths; no adaptive stop
  long long total = 0;
  for (const ViewRequest& r : req) total += (long long)r.s.width * r.s.height * effective_spp(r.s);
  const double f = std::min(1.0, (double)(1LL << 27) / (double)std::max(1LL, total));
  long long sample = 0;
  for (ViewRequest& r : req) {
    const int spp = std::max(1, (int)((double)effective_spp(r.s) * f));
    r.s.spp = spp;
    r.s.msaa = 1;
    r.s.tsaa = 0;
    r.s.adaptive_sampling = 0;
    sample += (long long)r.s.width * r.s.height * spp;
  }
  const long long keep = ctx->render_wave_cap;
  const int keep_ext = ctx->render_extend, keep_sb = ctx->render_shade_block;
  bc_tune_report rep;
  std::memset(&rep, 0, sizeof(rep));
  // one timed candidate: the second of two renders of the sample (the first
  // may allocate and capture the wave graph)
  auto time_render = [&](double* ms) -> bc_status {
    for (int k = 0; k < 2; k++) {
      const auto t0 = std::chrono::steady_clock::now();
      int64_t rays = 0;
      const bc_status s = render_views(ctx, req, (size_t)px, &rays, nullptr);
      if (s) return s;
      *ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
    rep.n_timed++;
    if (*ms > rep.worst_ms) rep.worst_ms = *ms;
    return BC_OK;
  };
  auto restore = [&]() {
    ctx->render_wave_cap = keep;
    ctx->render_extend = keep_ext;
    ctx->render_shade_block = keep_sb;
  };
  // stage 1: the extend variant at the current wave size
  int best_ext = keep_ext;
  double best_ext_ms = 0.0;
  for (int var : {1, 0, 2}) {
    ctx->render_extend = var;
    double ms = 0.0;
    if ((st = time_render(&ms))) {
      restore();
      return st;
    }
    if (var == keep_ext) rep.default_ms = ms;
    if (best_ext_ms == 0.0 || ms < best_ext_ms) {
      best_ext_ms = ms;
      best_ext = var;
    }
  }
  ctx->render_extend = best_ext;
  // stage 1b: the shading kernel's block shape, with that variant
  int best_sb = keep_sb;
  {
    const int other = keep_sb == 128 ? 256 : 128;
    ctx->render_shade_block = other;
    double ms = 0.0;
    if ((st = time_render(&ms))) {
      restore();
      return st;
    }
    if (ms < best_ext_ms) {
      best_ext_ms = ms;
      best_sb = other;
    }
    ctx->render_shade_block = best_sb;
  }
  // stage 2: the wave size with that variant
  long long best_cap = keep;
  rep.best_ms = best_ext_ms;
  std::vector<long long> caps;
  for (int lg = 22; lg <= 27; lg++) {
    const long long cap = 1LL << lg;
    if (cap > 2 * sample && lg > 22) break;  // larger waves than the work: the same launches
    if (cap != keep) caps.push_back(cap);
  }
  for (const long long cap : caps) {
    ctx->render_wave_cap = cap;
    double ms = 0.0;
    if ((st = time_render(&ms))) {
      restore();
      return st;
    }
    if (ms < rep.best_ms) {
      rep.best_ms = ms;
      best_cap = cap;
    }
  }
  ctx->render_wave_cap = best_cap;
  rep.raycast_minblocks = ctx->raycast_minblocks;
  rep.raycast_sort = ctx->raycast_sort;
  rep.render_wave_cap = best_cap;
  rep.render_extend = best_ext;
  rep.render_shade_block = best_sb;
  rep.raycast_split = ctx->raycast_split;
  if (out) *out = rep;
  return BC_OK;
}

}  // extern "C"

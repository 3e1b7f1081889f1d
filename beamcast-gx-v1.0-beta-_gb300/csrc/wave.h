// Interface of the wave engine (render.cu) for the other translation units.
#pragma once
#include <cstdint>
#include <vector>

#include "context.h"

namespace bcgx {

constexpr int kMaxGradBounces = 64;

// One view of a render: what a caller asks for, before packing.
struct ViewRequest {
  int scene;        // index into the resident scene set
  bc_camera cam;
  bc_settings s;
  int y0, rows;     // rows [y0, y0 + rows) of the frame
  long long pix_off;  // first pixel of those rows in the frame buffers
  bool want_guides;
};

// Gradient render (path replay): adjoint image and parameter map.
struct GradArgs {
  const float* dimg;         // 3 per frame pixel: dLoss / dImage
  const int32_t* mat2param;  // material -> parameter index (-1: not a parameter)
  int n_params;
  double* partial;           // [gradient_grid()][3 * n_params], accumulated over waves
};

// Renders the views; each view's mean radiance ends in render_mean(ctx) at its
// pix_off. With `grad`, also accumulates the path replay gradient into grad->partial.
bc_status render_views(bc_context* ctx, const std::vector<ViewRequest>& req, size_t frame_px, int64_t* rays,
                       const GradArgs* grad);
float* render_mean(bc_context* ctx);

// Photon maps (photon.cu). photon_map_for returns the map of resident scene
// `scene` for the seed, PhotonMapping level and bounces of `s`, from the cache
// or built on the context's stream (then *built_rays is its device ray
// counter); maps used after photon_clock() returned `pin` are not evicted.
struct PhotonView;
uint64_t photon_clock(bc_context* ctx);
bc_status photon_map_for(bc_context* ctx, int scene, const bc_settings& s, uint64_t pin, PhotonView* view,
                         const unsigned long long** built_rays);
int gradient_grid();
int effective_spp(const bc_settings& s);

}  // namespace bcgx

// Rendering entry points (wavefront path tracer and post passes).
#include "context.h"

namespace bcgx {
void destroy_render_buffers(bc_context* ctx) { (void)ctx; }
}  // namespace bcgx

using namespace bcgx;

extern "C" {

bc_status bc_render_rows(bc_context* ctx, const bc_camera* cam, const bc_settings* settings, int32_t y0,
                         int32_t rows, float* linear_out, uint32_t* guide_out, int64_t* rays_out) {
  (void)cam; (void)settings; (void)y0; (void)rows; (void)linear_out; (void)guide_out; (void)rays_out;
  return set_error(ctx, BC_ERR_INVALID_ARG, "renderer not available in this build");
}

bc_status bc_render_frame(bc_context* ctx, const bc_camera* cam, const bc_settings* settings, float* linear_out,
                          uint32_t* guide_out, uint32_t* rgba_out, int64_t* rays_out) {
  (void)cam; (void)settings; (void)linear_out; (void)guide_out; (void)rgba_out; (void)rays_out;
  return set_error(ctx, BC_ERR_INVALID_ARG, "renderer not available in this build");
}

}  // extern "C"

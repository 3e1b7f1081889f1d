// Differentiable rendering through the C ABI: the L2 image loss and its
// path-replay gradient with respect to diffuse albedos and emitter emissions.
// The forward render is the wave engine of render.cu; the backward render
// replays the same paths (same seed and per-(pixel, sample) streams) with
// vertex records on, and k_gradient (render.cu) turns the records into
// per-parameter sums.
#include <cstring>
#include <string>
#include <vector>

#include "context.h"
#include "wave.h"

struct DiffState {
  bool configured = false;
  bc_camera cam{};
  bc_settings st{};
  int n_alb = 0, n_em = 0;
  std::vector<int32_t> param_mat;  // material of each parameter, albedo parameters first
  bcgx::DevBuf d_param_mat, d_mat2param, d_params, d_target, d_dimg, d_partial, d_grad, d_loss;
  bcgx::HostBuf h_stage;
  bool has_target = false;
  bool forward_done = false;
  bool dimg_from_loss = false;  // d_dimg holds d(L2 loss)/dImage of the last forward
  uint64_t seed = 0;
};

namespace bcgx {

constexpr int kMaxParams = 1024;

void destroy_diff_state(bc_context* ctx) {
  DiffState* d = ctx->diff;
  if (!d) return;
  for (DevBuf* b : {&d->d_param_mat, &d->d_mat2param, &d->d_params, &d->d_target, &d->d_dimg, &d->d_partial,
                    &d->d_grad, &d->d_loss})
    b->release();
  d->h_stage.release();
  delete d;
  ctx->diff = nullptr;
}

// Writes the parameters into the material records, and the preview colors the
// guides derive from them (materialPreviewColor, renderer.go:1467-1475).
__global__ void k_set_params(MatGPU* __restrict__ mats, const int32_t* __restrict__ param_mat, int n_alb,
                             int n_params, const float* __restrict__ params) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_params) return;
  MatGPU& M = mats[param_mat[k]];
  const float x = params[3 * k], y = params[3 * k + 1], z = params[3 * k + 2];
  if (k < n_alb) {
    M.cr = x;
    M.cg = y;
    M.cb = z;
    const bool some = (double)x * x + (double)y * y + (double)z * z > 0.0;
    M.preview_r = some ? x : 0.8f;
    M.preview_g = some ? y : 0.8f;
    M.preview_b = some ? z : 0.8f;
  } else {
    M.er = x;
    M.eg = y;
    M.eb = z;
    M.preview_r = fminf(fmaxf(x / 8.0f, 0.0f), 1.0f);
    M.preview_g = fminf(fmaxf(y / 8.0f, 0.0f), 1.0f);
    M.preview_b = fminf(fmaxf(z / 8.0f, 0.0f), 1.0f);
  }
}

// Per-block fp64 sums of (image - target)^2 and the adjoint image
// dimg = 2 (image - target) / n3.
__global__ void __launch_bounds__(256) k_l2_loss(const float* __restrict__ img, const float* __restrict__ target,
                                                 long long n3, float* __restrict__ dimg, double* __restrict__ part) {
  __shared__ double red[256];
  double acc = 0.0;
  const float scale = (float)(2.0 / (double)n3);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3; i += (long long)gridDim.x * blockDim.x) {
    const float r = img[i] - target[i];
    acc += (double)r * (double)r;
    dimg[i] = scale * r;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// out[k] = sum over rows of partial[row][k], rows in order (deterministic).
__global__ void k_sum_rows(const double* __restrict__ partial, int rows, int cols, double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cols) return;
  double acc = 0.0;
  for (int r = 0; r < rows; r++) acc += partial[(size_t)r * cols + k];
  out[k] = acc;
}

static ViewRequest diff_view(const DiffState& d, uint64_t seed) {
  ViewRequest r;
  r.scene = 0;
  r.cam = d.cam;
  r.s = d.st;
  r.s.seed = seed;
  r.y0 = 0;
  r.rows = d.st.height;
  r.pix_off = 0;
  r.want_guides = false;
  return r;
}

}  // namespace bcgx

using namespace bcgx;

extern "C" {

bc_status bc_diff_configure(bc_context* ctx, const bc_diff_desc* desc) {
  if (!ctx || !desc) return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument");
  if (!ctx->has_scene) return set_error(ctx, BC_ERR_NO_SCENE, "no scene uploaded");
  const bc_settings& s = desc->settings;
  if (s.width < 1 || s.height < 1 || s.spp < 1 || s.bounces < 1 || (int64_t)s.width * s.height > (1 << 26))
    return set_error(ctx, BC_ERR_INVALID_ARG, "invalid render size, spp or bounces");
  if (s.bounces > kMaxGradBounces) return set_error(ctx, BC_ERR_INVALID_ARG, "gradient renders allow 64 bounces");
  if (s.firefly_clamp > 0.0)
    return set_error(ctx, BC_ERR_INVALID_ARG, "firefly clamp must be off for gradient renders");
  const int na = desc->n_albedo, ne = desc->n_emission;
  if (na < 0 || ne < 0 || na + ne < 1 || na + ne > kMaxParams || (na && !desc->albedo_materials) ||
      (ne && !desc->emission_materials))
    return set_error(ctx, BC_ERR_INVALID_ARG, "need 1..1024 parameters with their material lists");
  const int n_mats = (int)ctx->mat_kind.size();
  std::vector<int32_t> pm(na + ne);
  std::vector<int32_t> m2p(n_mats, -1);
  for (int k = 0; k < na + ne; k++) {
    const int32_t m = k < na ? desc->albedo_materials[k] : desc->emission_materials[k - na];
    if (m < 0 || m >= n_mats)
      return set_error(ctx, BC_ERR_INVALID_ARG, "parameter " + std::to_string(k) + ": material out of range");
    if (m2p[m] >= 0)
      return set_error(ctx, BC_ERR_INVALID_ARG, "material " + std::to_string(m) + " named twice");
    const int kind = ctx->mat_kind[m];
    if (k < na && kind != BC_MAT_DIFFUSE)
      return set_error(ctx, BC_ERR_INVALID_ARG, "albedo parameter on a non-diffuse material " + std::to_string(m));
    if (k >= na && kind != BC_MAT_EMISSIVE)
      return set_error(ctx, BC_ERR_INVALID_ARG, "emission parameter on a non-emissive material " + std::to_string(m));
    if (k >= na && ctx->mat_is_light[m])
      return set_error(ctx, BC_ERR_INVALID_ARG,
                       "emission parameter on a sphere-light material " + std::to_string(m) + " (fixed light records)");
    pm[k] = m;
    m2p[m] = k;
  }
  cudaSetDevice(ctx->device);
  if (!ctx->diff) ctx->diff = new DiffState();
  DiffState& d = *ctx->diff;
  d.configured = false;
  d.forward_done = false;
  d.has_target = false;
  const size_t np3 = 3 * (size_t)(na + ne);
  const size_t px3 = 3 * (size_t)s.width * s.height;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (!e) e = d.d_param_mat.ensure(pm.size() * sizeof(int32_t));
  if (!e) e = d.d_mat2param.ensure(std::max<size_t>(1, m2p.size()) * sizeof(int32_t));
  if (!e) e = d.d_params.ensure(np3 * sizeof(float));
  if (!e) e = d.d_target.ensure(px3 * sizeof(float));
  if (!e) e = d.d_dimg.ensure(px3 * sizeof(float));
  if (!e) e = d.d_partial.ensure((size_t)gradient_grid() * np3 * sizeof(double));
  if (!e) e = d.d_grad.ensure(np3 * sizeof(double));
  if (!e) e = d.d_loss.ensure((1024 + 1) * sizeof(double));
  if (!e) e = d.h_stage.ensure(std::max(px3 * sizeof(float), np3 * sizeof(double)) + 64);
  if (!e) e = cudaMemcpy(d.d_param_mat.p, pm.data(), pm.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  if (!e && !m2p.empty())
    e = cudaMemcpy(d.d_mat2param.p, m2p.data(), m2p.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
  if (e) return cuda_status(ctx, e, "gradient setup");
  d.cam = desc->camera;
  d.st = s;
  d.n_alb = na;
  d.n_em = ne;
  d.param_mat = pm;
  d.configured = true;
  return BC_OK;
}

bc_status bc_diff_set_target(bc_context* ctx, const float* target) {
  if (!ctx || !target) return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument");
  if (!ctx->diff || !ctx->diff->configured) return set_error(ctx, BC_ERR_INVALID_ARG, "bc_diff_configure first");
  cudaSetDevice(ctx->device);
  DiffState& d = *ctx->diff;
  const size_t bytes = 3 * (size_t)d.st.width * d.st.height * sizeof(float);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (!e) e = cudaMemcpy(d.d_target.p, target, bytes, cudaMemcpyHostToDevice);
  if (e) return cuda_status(ctx, e, "target upload");
  d.has_target = true;
  d.dimg_from_loss = false;
  return BC_OK;
}

bc_status bc_forward(bc_context* ctx, const float* params, uint64_t seed, float* image_out, double* loss_out) {
  if (!ctx || !params) return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument");
  if (!ctx->diff || !ctx->diff->configured) return set_error(ctx, BC_ERR_INVALID_ARG, "bc_diff_configure first");
  DiffState& d = *ctx->diff;
  if (loss_out && !d.has_target) return set_error(ctx, BC_ERR_INVALID_ARG, "loss needs a target (bc_diff_set_target)");
  cudaSetDevice(ctx->device);
  const int np = d.n_alb + d.n_em;
  d.forward_done = false;
  d.dimg_from_loss = false;
  cudaError_t e = cudaStreamSynchronize(ctx->stream);  // the staging buffer may still be in flight
  if (e) return cuda_status(ctx, e, "forward");
  std::memcpy(d.h_stage.p, params, 3 * (size_t)np * sizeof(float));
  e = cudaMemcpyAsync(d.d_params.p, d.h_stage.p, 3 * (size_t)np * sizeof(float), cudaMemcpyHostToDevice, ctx->stream);
  if (e) return cuda_status(ctx, e, "parameter upload");
  k_set_params<<<(np + 127) / 128, 128, 0, ctx->stream>>>(const_cast<MatGPU*>(ctx->ds.mats),
                                                          d.d_param_mat.as<int32_t>(), d.n_alb, np,
                                                          d.d_params.as<float>());
  if ((e = cudaGetLastError())) return cuda_status(ctx, e, "parameter update");
  const size_t px = (size_t)d.st.width * d.st.height;
  int64_t rays = 0;
  bc_status st = render_views(ctx, std::vector<ViewRequest>{diff_view(d, seed)}, px, &rays, nullptr);
  if (st) return st;
  const float* img = render_mean(ctx);
  if (d.has_target) {
    const int blocks = 1024;
    k_l2_loss<<<blocks, 256, 0, ctx->stream>>>(img, d.d_target.as<float>(), 3 * (long long)px, d.d_dimg.as<float>(),
                                               d.d_loss.as<double>());
    k_sum_rows<<<1, 32, 0, ctx->stream>>>(d.d_loss.as<double>(), blocks, 1, d.d_loss.as<double>() + blocks);
    double loss = 0.0;
    e = cudaGetLastError();
    if (!e) e = cudaMemcpyAsync(&loss, d.d_loss.as<double>() + blocks, sizeof(double), cudaMemcpyDeviceToHost,
                                ctx->stream);
    if (!e) e = cudaStreamSynchronize(ctx->stream);
    if (e) return cuda_status(ctx, e, "loss");
    if (loss_out) *loss_out = loss / (3.0 * (double)px);
    d.dimg_from_loss = true;
  }
  if (image_out) {
    e = cudaMemcpyAsync(image_out, img, 3 * px * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (!e) e = cudaStreamSynchronize(ctx->stream);
    if (e) return cuda_status(ctx, e, "image readback");
  }
  d.seed = seed;
  d.forward_done = true;
  return BC_OK;
}

bc_status bc_backward(bc_context* ctx, const float* dloss_dimage, float* grad_albedo, float* grad_emission) {
  if (!ctx) return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument");
  if (!ctx->diff || !ctx->diff->configured || !ctx->diff->forward_done)
    return set_error(ctx, BC_ERR_INVALID_ARG, "bc_backward needs a bc_forward first");
  DiffState& d = *ctx->diff;
  if (!dloss_dimage && !d.dimg_from_loss)
    return set_error(ctx, BC_ERR_INVALID_ARG, "no adjoint image: pass dloss_dimage or set a target before bc_forward");
  cudaSetDevice(ctx->device);
  const size_t px = (size_t)d.st.width * d.st.height;
  const int np = d.n_alb + d.n_em;
  const int np3 = 3 * np;
  cudaError_t e = cudaSuccess;
  if (dloss_dimage) {
    e = cudaStreamSynchronize(ctx->stream);
    if (!e) e = cudaMemcpy(d.d_dimg.p, dloss_dimage, 3 * px * sizeof(float), cudaMemcpyHostToDevice);
    if (e) return cuda_status(ctx, e, "adjoint upload");
    d.dimg_from_loss = false;
  }
  const int rows = gradient_grid();
  e = cudaMemsetAsync(d.d_partial.p, 0, (size_t)rows * np3 * sizeof(double), ctx->stream);
  if (e) return cuda_status(ctx, e, "gradient setup");
  GradArgs ga;
  ga.dimg = d.d_dimg.as<float>();
  ga.mat2param = d.d_mat2param.as<int32_t>();
  ga.n_params = np;
  ga.partial = d.d_partial.as<double>();
  int64_t rays = 0;
  bc_status st = render_views(ctx, std::vector<ViewRequest>{diff_view(d, d.seed)}, px, &rays, &ga);
  if (st) return st;
  k_sum_rows<<<(np3 + 127) / 128, 128, 0, ctx->stream>>>(d.d_partial.as<double>(), rows, np3, d.d_grad.as<double>());
  e = cudaGetLastError();
  double* h = reinterpret_cast<double*>(d.h_stage.p);
  if (!e) e = cudaMemcpyAsync(h, d.d_grad.p, np3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  if (e) return cuda_status(ctx, e, "gradient readback");
  for (int k = 0; k < np3; k++) {
    if (k < 3 * d.n_alb) {
      if (grad_albedo) grad_albedo[k] = (float)h[k];
    } else if (grad_emission) {
      grad_emission[k - 3 * d.n_alb] = (float)h[k];
    }
  }
  return BC_OK;
}

}  // extern "C"

// Post passes of RenderState.Start on the device (renderer.go:2844-2854, 2890-2895):
// guide-aware a-trous denoise (atrousDenoise, 2228-2287), bloom (applyBloom +
// boxBlur, 2490-2555) and tone mapping to RGBA8 (toneMapHDR + toRGBA, 2034-2064).
// All passes are memory-bound stencils over linear RGB (fp32, 12 B/pixel) and
// guides (float4 normal + depth, 16 B/pixel; depth < 0 marks an invalid guide).
#include <algorithm>
#include <cmath>
#include <mutex>

#include "context.h"

struct RenderBuffers;

namespace bcgx {

__device__ __forceinline__ float lumf(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

__global__ void k_atrous(int W, int H, int step, const float* __restrict__ cur, const float4* __restrict__ guide,
                         float* __restrict__ next) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const int i = y * W + x;
  const float cr = cur[3 * i], cg = cur[3 * i + 1], cb = cur[3 * i + 2];
  const float4 g0 = guide[i];
  const bool v0 = g0.w >= 0.0f;
  const float l0 = lumf(cr, cg, cb);
  float sr = 0, sg = 0, sb = 0, wsum = 0;
  for (int oy = -1; oy <= 1; oy++) {
    const int yy = y + oy * step;
    if (yy < 0 || yy >= H) continue;
    for (int ox = -1; ox <= 1; ox++) {
      const int xx = x + ox * step;
      if (xx < 0 || xx >= W) continue;
      const int j = yy * W + xx;
      const float4 g1 = guide[j];
      if (v0 != (g1.w >= 0.0f)) continue;
      const float qr = cur[3 * j], qg = cur[3 * j + 1], qb = cur[3 * j + 2];
      float wgt = 1.0f;
      if (v0) {
        const float nd = fminf(fmaxf(g0.x * g1.x + g0.y * g1.y + g0.z * g1.z, -1.0f), 1.0f);
        wgt *= expf((nd - 1.0f) * 48.0f);
        const float depthScale = fmaxf(0.15f, 0.04f * fmaxf(g0.w, 1.0f));
        wgt *= expf(-fabsf(g0.w - g1.w) / depthScale);
      }
      wgt *= expf(-fabsf(l0 - lumf(qr, qg, qb)) * 3.5f);
      if (ox == 0 && oy == 0) wgt *= 1.5f;
      sr += qr * wgt;
      sg += qg * wgt;
      sb += qb * wgt;
      wsum += wgt;
    }
  }
  if (wsum > 1e-12f) {
    const float inv = 1.0f / wsum;
    next[3 * i] = sr * inv;
    next[3 * i + 1] = sg * inv;
    next[3 * i + 2] = sb * inv;
  } else {
    next[3 * i] = cr;
    next[3 * i + 1] = cg;
    next[3 * i + 2] = cb;
  }
}

// Horizontal box blur of the bright pass (the bright pass is recomputed per tap).
__global__ void k_bloom_h(int W, int H, int radius, float threshold, const float* __restrict__ img,
                          float* __restrict__ tmp) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  float sr = 0, sg = 0, sb = 0, cnt = 0;
  for (int ox = -radius; ox <= radius; ox++) {
    const int xx = x + ox;
    if (xx < 0 || xx >= W) continue;
    const int j = y * W + xx;
    const float r = img[3 * j], g = img[3 * j + 1], b = img[3 * j + 2];
    const float l = lumf(r, g, b);
    if (l > threshold) {
      const float s = (l - threshold) / fmaxf(l, 1e-6f);
      sr += r * s;
      sg += g * s;
      sb += b * s;
    }
    cnt += 1.0f;
  }
  const float inv = 1.0f / fmaxf(cnt, 1.0f);
  const int i = y * W + x;
  tmp[3 * i] = sr * inv;
  tmp[3 * i + 1] = sg * inv;
  tmp[3 * i + 2] = sb * inv;
}

__global__ void k_bloom_v(int W, int H, int radius, float strength, const float* __restrict__ img,
                          const float* __restrict__ tmp, float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  float sr = 0, sg = 0, sb = 0, cnt = 0;
  for (int oy = -radius; oy <= radius; oy++) {
    const int yy = y + oy;
    if (yy < 0 || yy >= H) continue;
    const int j = yy * W + x;
    sr += tmp[3 * j];
    sg += tmp[3 * j + 1];
    sb += tmp[3 * j + 2];
    cnt += 1.0f;
  }
  const float inv = 1.0f / fmaxf(cnt, 1.0f);
  const int i = y * W + x;
  out[3 * i] = img[3 * i] + sr * inv * strength;
  out[3 * i + 1] = img[3 * i + 1] + sg * inv * strength;
  out[3 * i + 2] = img[3 * i + 2] + sb * inv * strength;
}

__device__ __forceinline__ float tone1(float x, int hdr) {
  switch (hdr) {
    case 0: return fminf(fmaxf(x, 0.0f), 1.0f);
    case 1: return x / (1.0f + x);
    case 3: {
      const float a = 2.51f, b = 0.03f, c = 2.43f, d = 0.59f, e = 0.14f;
      return fminf(fmaxf((x * (a * x + b)) / (x * (c * x + d) + e), 0.0f), 1.0f);
    }
    default: {
      x = fmaxf(0.0f, x - 0.004f);
      return fminf(fmaxf((x * (6.2f * x + 0.5f)) / (x * (6.2f * x + 1.7f) + 0.06f), 0.0f), 1.0f);
    }
  }
}

__global__ void k_tonemap(int n, float scale, float inv_gamma, int hdr, const float* __restrict__ img,
                          uint32_t* __restrict__ rgba) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t q[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float c = tone1(img[3 * i + k] * scale, hdr);
    c = powf(fmaxf(0.0f, c), inv_gamma);
    q[k] = (uint32_t)(fminf(fmaxf(c, 0.0f), 0.999f) * 256.0f);
  }
  rgba[i] = 0xff000000u | (q[2] << 16) | (q[1] << 8) | q[0];
}

// Runs denoise and bloom in place on `img` (ping-pong through tmp/tmp2), then tone maps.
static cudaError_t post_chain(cudaStream_t st, int W, int H, const bc_settings& s, float* img, const float4* guide,
                              float* tmp, float* tmp2, uint32_t* rgba) {
  const dim3 blk(32, 8), grd((W + 31) / 32, (H + 7) / 8);
  const size_t bytes = 3 * sizeof(float) * (size_t)W * H;
  cudaError_t e = cudaSuccess;
  if (s.denoise) {
    const int passes = 2 + std::min(3, std::max(s.taa, s.txaa));
    float* cur = img;
    float* nxt = tmp;
    for (int it = 0; it < passes; it++) {
      k_atrous<<<grd, blk, 0, st>>>(W, H, 1 << it, cur, guide, nxt);
      std::swap(cur, nxt);
    }
    if (cur != img) e = cudaMemcpyAsync(img, cur, bytes, cudaMemcpyDeviceToDevice, st);
    if (e) return e;
  }
  if (s.bloom > 0) {
    const float threshold = (float)(1.25 - 0.2 * (double)s.bloom);
    const float strength = (float)(0.08 + 0.09 * (double)s.bloom);
    k_bloom_h<<<grd, blk, 0, st>>>(W, H, 1 + s.bloom, threshold, img, tmp);
    k_bloom_v<<<grd, blk, 0, st>>>(W, H, 1 + s.bloom, strength, img, tmp, tmp2);
    e = cudaMemcpyAsync(img, tmp2, bytes, cudaMemcpyDeviceToDevice, st);
    if (e) return e;
  }
  if (rgba) {
    const float scale = (float)std::pow(2.0, s.exposure);
    const float inv_gamma = (float)(1.0 / std::max(0.1, s.gamma));
    const int n = W * H;
    k_tonemap<<<(n + 255) / 256, 256, 0, st>>>(n, scale, inv_gamma, s.hdr, img, rgba);
  }
  return cudaGetLastError();
}

}  // namespace bcgx

// Frame buffers live in render.cu; post.cu only needs these accessors.
namespace bcgx {
struct PostTargets {
  float* img;
  const float4* guide;
  float* tmp;
  float* tmp2;
  uint32_t* rgba;
};
PostTargets post_targets(bc_context* ctx);
bc_status ensure_post_scratch(bc_context* ctx, int px, PostTargets* t);

bc_status run_post(bc_context* ctx, const bc_settings& s) {
  PostTargets t = post_targets(ctx);
  cudaError_t e = post_chain(ctx->stream, s.width, s.height, s, t.img, t.guide, t.tmp, t.tmp2, t.rgba);
  return cuda_status(ctx, e, "post passes");
}
}  // namespace bcgx

using namespace bcgx;

extern "C" bc_status bc_post_process(bc_context* ctx, int32_t width, int32_t height, const float* linear_in,
                                     const float* guide_nd, const bc_settings* settings, float* linear_out,
                                     uint32_t* rgba_out) {
  if (!ctx || !linear_in || !settings || width < 1 || height < 1)
    return set_error(ctx, BC_ERR_INVALID_ARG, "bad post-process arguments");
  if (settings->denoise && !guide_nd) return set_error(ctx, BC_ERR_INVALID_ARG, "denoise needs guides");
  if ((int64_t)width * height > (1 << 26)) return set_error(ctx, BC_ERR_INVALID_ARG, "frame too large");
  cudaSetDevice(ctx->device);
  PostTargets t;
  bc_status st = ensure_post_scratch(ctx, width * height, &t);
  if (st) return st;
  const size_t n = (size_t)width * height;
  cudaError_t e = cudaMemcpyAsync(t.img, linear_in, 3 * sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream);
  if (!e && guide_nd)
    e = cudaMemcpyAsync((void*)t.guide, guide_nd, 4 * sizeof(float) * n, cudaMemcpyHostToDevice, ctx->stream);
  bc_settings s = *settings;
  s.width = width;
  s.height = height;
  if (!e) e = post_chain(ctx->stream, width, height, s, t.img, t.guide, t.tmp, t.tmp2, t.rgba);
  if (!e && linear_out)
    e = cudaMemcpyAsync(linear_out, t.img, 3 * sizeof(float) * n, cudaMemcpyDeviceToHost, ctx->stream);
  if (!e && rgba_out) e = cudaMemcpyAsync(rgba_out, t.rgba, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, ctx->stream);
  if (!e) e = cudaStreamSynchronize(ctx->stream);
  return cuda_status(ctx, e, "post process");
}

// ---- allocation-free post stack ---------------------------------------------
// For callers that cannot allocate device memory at the time they post-process
// a frame: code running inside an engine or plugin host whose GPU memory is
// owned and budgeted elsewhere, allocation-free real-time loops, and callers
// that must not synchronise the device (cudaMalloc and cudaFree can). The
// caller passes device buffers for the input, the guides and the outputs; the
// two scratch images the passes need live in this file-scope array, which
// every GPU that loads the library holds for the life of the process.
constexpr int kNoAllocMaxPixels = 1280 * 720;  // 921,600 pixels: 2 x 11,059,200 bytes of scratch
static __device__ __align__(256) float g_post_scratch[2 * 3 * kNoAllocMaxPixels];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
float* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_post_scratch for the current device, looked up once per
// device with that device current (the host-side symbol is not a device address).
cudaError_t scratch_for_current_device(float** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_post_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = static_cast<float*>(p);
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}
}  // namespace

extern "C" bc_status bc_post_process_noalloc(int32_t width, int32_t height, const float* d_linear_in,
                                             const float* d_guide_nd, const bc_settings* settings,
                                             float* d_linear_out, uint32_t* d_rgba_out, void* stream) {
  if (!d_linear_in || !d_linear_out || !settings || width < 1 || height < 1)
    return set_error(nullptr, BC_ERR_INVALID_ARG, "bad post-process arguments");
  if ((int64_t)width * height > kNoAllocMaxPixels)
    return set_error(nullptr, BC_ERR_INVALID_ARG,
                     "frame exceeds the static scratch of bc_post_process_noalloc (921600 pixels)");
  if (d_linear_in == d_linear_out)
    return set_error(nullptr, BC_ERR_INVALID_ARG, "input and output images must not alias");
  if (settings->denoise && !d_guide_nd) return set_error(nullptr, BC_ERR_INVALID_ARG, "denoise needs guides");
  float* scratch = nullptr;
  cudaError_t e = scratch_for_current_device(&scratch);
  if (e != cudaSuccess) return cuda_status(nullptr, e, "static scratch address");
  cudaStream_t st = (cudaStream_t)stream;
  const int W = width, H = height, n = W * H;
  const dim3 blk(32, 8), grd((W + 31) / 32, (H + 7) / 8);
  // Nothing in the scratch has to start at zero: every pass writes every pixel
  // it or a later pass reads.
  // No pass reads and writes the same buffer.
  float* sa = scratch;                            // denoised image when bloom follows
  float* sb = scratch + 3 * (size_t)kNoAllocMaxPixels;  // horizontal bloom blur
  const bool bloom = settings->bloom > 0;
  const float* img = d_linear_in;
  if (settings->denoise) {
    // a-trous passes ping-pong between the output and scratch A so that the
    // last pass lands in A when bloom follows, else in the output
    const int passes = 2 + std::min(3, std::max(settings->taa, settings->txaa));
    float* last = bloom ? sa : d_linear_out;
    float* other = bloom ? d_linear_out : sa;
    const float* cur = d_linear_in;
    for (int it = 0; it < passes; it++) {
      float* dst = ((passes - 1 - it) % 2 == 0) ? last : other;
      k_atrous<<<grd, blk, 0, st>>>(W, H, 1 << it, cur, reinterpret_cast<const float4*>(d_guide_nd), dst);
      cur = dst;
    }
    img = last;
  }
  if (bloom) {
    const float threshold = (float)(1.25 - 0.2 * (double)settings->bloom);
    const float strength = (float)(0.08 + 0.09 * (double)settings->bloom);
    k_bloom_h<<<grd, blk, 0, st>>>(W, H, 1 + settings->bloom, threshold, img, sb);
    k_bloom_v<<<grd, blk, 0, st>>>(W, H, 1 + settings->bloom, strength, img, sb, d_linear_out);
    img = d_linear_out;
  }
  if (img != d_linear_out) {
    e = cudaMemcpyAsync(d_linear_out, img, 3 * sizeof(float) * (size_t)n, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_status(nullptr, e, "post copy");
  }
  if (d_rgba_out) {
    const float scale = (float)std::pow(2.0, settings->exposure);
    const float inv_gamma = (float)(1.0 / std::max(0.1, settings->gamma));
    k_tonemap<<<(n + 255) / 256, 256, 0, st>>>(n, scale, inv_gamma, settings->hdr, d_linear_out, d_rgba_out);
  }
  return cuda_status(nullptr, cudaGetLastError(), "post launch");
}

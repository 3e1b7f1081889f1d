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
__device__ __forceinline__ float3 f3c(float x, float y, float z) { return make_float3(x, y, z); }

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
// The cached address belongs to the device's current primary context: after a
// cudaDeviceReset the module may load elsewhere, so a process that resets a
// device must not call bc_post_process_noalloc on it again.
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
  // The passes read their inputs through __restrict__ pointers and ping-pong
  // through the output: no written image may share a byte with any other image.
  const size_t n_px = (size_t)width * height;
  const auto lo = [](const void* p) { return reinterpret_cast<uintptr_t>(p); };
  const auto overlap = [&](const void* a, size_t abytes, const void* b, size_t bbytes) {
    return a && b && lo(a) < lo(b) + bbytes && lo(b) < lo(a) + abytes;
  };
  const size_t img_bytes = 3 * sizeof(float) * n_px, guide_bytes = 4 * sizeof(float) * n_px;
  const size_t rgba_bytes = sizeof(uint32_t) * n_px;
  if (overlap(d_linear_out, img_bytes, d_linear_in, img_bytes) ||
      overlap(d_linear_out, img_bytes, d_guide_nd, guide_bytes) ||
      overlap(d_linear_out, img_bytes, d_rgba_out, rgba_bytes) ||
      overlap(d_rgba_out, rgba_bytes, d_linear_in, img_bytes) ||
      overlap(d_rgba_out, rgba_bytes, d_guide_nd, guide_bytes))
    return set_error(nullptr, BC_ERR_INVALID_ARG, "the output buffers must not overlap each other or the inputs");
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
  // A pass count of zero or less (taa and txaa both -2 or below) denoises
  // nothing: atrousDenoise returns its input unchanged (renderer.go:2229), as
  // bc_post_process does.
  const int passes = 2 + std::min(3, std::max(settings->taa, settings->txaa));
  if (settings->denoise && passes > 0) {
    // a-trous passes ping-pong between the output and scratch A so that the
    // last pass lands in A when bloom follows, else in the output
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

// ---- the whole post stack of RenderState.Start ---------------------------------
// bc_post_stack runs Start's order (renderer.go:2838-2895) on caller buffers:
// HBAO / HBAO+ (applyHBAO, 2433-2488), a-trous denoise, temporal accumulation
// with the previous frame (temporalAccumulate + projectPoint, 2280-2364; the
// history is kept in the context as Start keeps r.history*), bloom, debug views
// (makeDebugView, 1972-2032), the basic upscaler (bicubicUpscale +
// edgeAwareSharpen, 2081-2197), FXAA (2557-2587), the TXAA resolve (2589-2595)
// and tone mapping. Guides are three float4 per pixel: (P, depth), (N, valid),
// (albedo, 0).
namespace bcgx {
namespace {

struct PostStackBufs {
  float *a, *b, *c;           // render-size images
  float *oa, *ob;             // output-size images
  float4 *gp, *gn, *ga, *gnd;  // guides; gnd = (N, depth or -1) for the a-trous kernel
  uint32_t* rgba;
  unsigned* maxbits;          // [0] max depth, [1] max luminance (positive floats as bits)
};

__global__ void k_unpack_guides(int n, const float* __restrict__ g12, float4* gp, float4* gn, float4* ga, float4* gnd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* g = g12 + 12 * (size_t)i;
  gp[i] = make_float4(g[0], g[1], g[2], g[3]);
  gn[i] = make_float4(g[4], g[5], g[6], g[7]);
  ga[i] = make_float4(g[8], g[9], g[10], 0.0f);
  gnd[i] = g[7] != 0.0f ? make_float4(g[4], g[5], g[6], g[3]) : make_float4(0.0f, 0.0f, 0.0f, -1.0f);
}

__device__ __forceinline__ float dot3f(float4 a, float4 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// applyHBAO (renderer.go:2433-2488)
__global__ void k_hbao(int W, int H, int level, int plus, const float* __restrict__ img, const float4* __restrict__ gp,
                       const float4* __restrict__ gn, float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const int i = y * W + x;
  const float4 P = gp[i], N = gn[i];
  float f = 1.0f;
  if (N.w != 0.0f) {
    int radius = 2 + level * 2;
    if (plus) radius += 2;
    float strength = 0.14f + 0.09f * (float)level;
    if (plus) strength *= 1.15f;
    const int dirs[12][2] = {{1, 0}, {-1, 0}, {0, 1}, {0, -1}, {1, 1}, {-1, 1}, {1, -1}, {-1, -1},
                             {2, 1}, {-2, 1}, {1, 2}, {-1, 2}};
    const int nd = plus ? 12 : 8;
    const int inc = max(1, radius / 3);
    float occ = 0.0f, count = 0.0f;
    const float depth = P.w;
    for (int d = 0; d < nd; d++)
      for (int step = 1; step <= radius; step += inc) {
        const int xx = x + dirs[d][0] * step, yy = y + dirs[d][1] * step;
        if (xx < 0 || xx >= W || yy < 0 || yy >= H) continue;
        const int j = yy * W + xx;
        const float4 nn = gn[j];
        if (nn.w == 0.0f) continue;
        const float nd_depth = gp[j].w;
        const float tol = 0.015f * fmaxf(depth, 1.0f) + 0.002f * (float)step;
        if (nd_depth + tol < depth) {
          const float normalTerm = fminf(fmaxf(1.0f - dot3f(N, nn), 0.0f), 1.0f);
          const float depthTerm = fminf(fmaxf((depth - nd_depth) / (0.25f * fmaxf(depth, 1.0f)), 0.0f), 1.0f);
          occ += 0.55f * depthTerm + 0.45f * normalTerm;
        }
        count += 1.0f;
      }
    if (count > 0.0f) f = fminf(fmaxf(1.0f - strength * (occ / count), 0.35f), 1.0f);
  }
  for (int k = 0; k < 3; k++) out[3 * i + k] = img[3 * i + k] * f;
}

// projectPoint's camera frame (renderer.go:2280-2314), computed in fp64 on the host
struct ProjCam {
  float px, py, pz;     // position
  float fx, fy, fz, rx, ry, rz, ux, uy, uz;
  float half_h, aspect;
  int ok;
};

// temporalAccumulate (renderer.go:2316-2364)
__global__ void k_temporal(int W, int H, float weight, ProjCam cam, const float* __restrict__ cur,
                           const float4* __restrict__ gp, const float4* __restrict__ gn,
                           const float* __restrict__ prev, const float4* __restrict__ pgp,
                           const float4* __restrict__ pgn, float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const int i = y * W + x;
  float3 o = f3c(cur[3 * i], cur[3 * i + 1], cur[3 * i + 2]);
  const float4 P = gp[i], N = gn[i];
  if (N.w != 0.0f && cam.ok) {
    const float rx = P.x - cam.px, ry = P.y - cam.py, rz = P.z - cam.pz;
    const float z = rx * cam.fx + ry * cam.fy + rz * cam.fz;
    if (z > 1e-5f) {
      const float nx = (rx * cam.rx + ry * cam.ry + rz * cam.rz) / (z * cam.half_h * cam.aspect);
      const float ny = (rx * cam.ux + ry * cam.uy + rz * cam.uz) / (z * cam.half_h);
      if (!(nx < -1.0f || nx > 1.0f || ny < -1.0f || ny > 1.0f)) {
        const int px = (int)roundf((nx * 0.5f + 0.5f) * (float)(W - 1));
        const int py = (int)roundf((0.5f - ny * 0.5f) * (float)(H - 1));
        if (px >= 0 && px < W && py >= 0 && py < H) {
          const int j = py * W + px;
          const float4 PN = pgn[j], PP = pgp[j];
          if (PN.w != 0.0f && dot3f(N, PN) >= 0.88f) {
            const float dx = P.x - PP.x, dy = P.y - PP.y, dz = P.z - PP.z;
            if (sqrtf(dx * dx + dy * dy + dz * dz) <= 0.03f * fmaxf(P.w, 1.0f)) {
              float3 lo = f3c(INFINITY, INFINITY, INFINITY), hi = f3c(-INFINITY, -INFINITY, -INFINITY);
              for (int oy = -1; oy <= 1; oy++) {
                const int yy = y + oy;
                if (yy < 0 || yy >= H) continue;
                for (int ox = -1; ox <= 1; ox++) {
                  const int xx = x + ox;
                  if (xx < 0 || xx >= W) continue;
                  const float* c = cur + 3 * (yy * W + xx);
                  lo = f3c(fminf(lo.x, c[0]), fminf(lo.y, c[1]), fminf(lo.z, c[2]));
                  hi = f3c(fmaxf(hi.x, c[0]), fmaxf(hi.y, c[1]), fmaxf(hi.z, c[2]));
                }
              }
              const float* pc = prev + 3 * j;
              const float qx = fminf(fmaxf(pc[0], lo.x), hi.x), qy = fminf(fmaxf(pc[1], lo.y), hi.y),
                          qz = fminf(fmaxf(pc[2], lo.z), hi.z);
              o = f3c(o.x * (1.0f - weight) + qx * weight, o.y * (1.0f - weight) + qy * weight,
                      o.z * (1.0f - weight) + qz * weight);
            }
          }
        }
      }
    }
  }
  out[3 * i] = o.x;
  out[3 * i + 1] = o.y;
  out[3 * i + 2] = o.z;
}

// maxima for the depth and heat views (positive floats compare as their bits)
__global__ void k_view_max(int n, const float* __restrict__ img, const float4* __restrict__ gp,
                           const float4* __restrict__ gn, unsigned* maxbits) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (gn[i].w != 0.0f && gp[i].w > 0.0f) atomicMax(&maxbits[0], __float_as_uint(gp[i].w));
  const float l = lumf(img[3 * i], img[3 * i + 1], img[3 * i + 2]);
  if (l > 0.0f) atomicMax(&maxbits[1], __float_as_uint(l));
}

// makeDebugView for the albedo (1), normal (2), depth (3) and heat (5) views
__global__ void k_debug_view(int n, int mode, const float* __restrict__ img, const float4* __restrict__ gp,
                             const float4* __restrict__ gn, const float4* __restrict__ ga,
                             const unsigned* __restrict__ maxbits, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float3 o = f3c(0.0f, 0.0f, 0.0f);
  const bool valid = gn[i].w != 0.0f;
  if (mode == 1 && valid) {
    o = f3c(ga[i].x, ga[i].y, ga[i].z);
  } else if (mode == 2 && valid) {
    o = f3c((gn[i].x + 1.0f) * 0.5f, (gn[i].y + 1.0f) * 0.5f, (gn[i].z + 1.0f) * 0.5f);
  } else if (mode == 3 && valid) {
    const float md = fmaxf(1.0f, __uint_as_float(maxbits[0]));
    const float v = 1.0f - fminf(fmaxf(gp[i].w / md, 0.0f), 1.0f);
    o = f3c(v, v, v);
  } else if (mode == 5) {
    const float ml = fmaxf(1e-6f, __uint_as_float(maxbits[1]));
    const float t = fminf(fmaxf(lumf(img[3 * i], img[3 * i + 1], img[3 * i + 2]) / ml, 0.0f), 1.0f);
    o = f3c(fminf(fmaxf(1.5f * t, 0.0f), 1.0f), fminf(fmaxf(1.2f * (1.0f - fabsf(t - 0.5f) * 2.0f), 0.0f), 1.0f),
            fminf(fmaxf(1.5f * (1.0f - t), 0.0f), 1.0f));
  }
  out[3 * i] = o.x;
  out[3 * i + 1] = o.y;
  out[3 * i + 2] = o.z;
}

__global__ void k_fill(int n3, float v, float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n3) out[i] = v;
}

__device__ __forceinline__ float cubic_hermite(float a, float b, float c, float d, float t) {
  const float ta = -0.5f * a + 1.5f * b - 1.5f * c + 0.5f * d;
  const float tb = a - 2.5f * b + 2.0f * c - 0.5f * d;
  const float tc = -0.5f * a + 0.5f * c;
  return ((ta * t + tb) * t + tc) * t + b;
}

// bicubicUpscale (renderer.go:2095-2138)
__global__ void k_bicubic(int sw, int sh, int dw, int dh, const float* __restrict__ src, float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= dw || y >= dh) return;
  const double fy = dh > 1 ? (double)y * (double)(sh - 1) / (double)(dh - 1) : 0.0;
  const double fx = dw > 1 ? (double)x * (double)(sw - 1) / (double)(dw - 1) : 0.0;
  const int yi = (int)floor(fy), xi = (int)floor(fx);
  const float ty = (float)(fy - (double)yi), tx = (float)(fx - (double)xi);
  float rows[4][3];
  for (int m = -1; m <= 2; m++) {
    const int yy = min(max(yi + m, 0), sh - 1);
    const float* r0 = src + 3 * ((size_t)yy * sw + min(max(xi - 1, 0), sw - 1));
    const float* r1 = src + 3 * ((size_t)yy * sw + min(max(xi, 0), sw - 1));
    const float* r2 = src + 3 * ((size_t)yy * sw + min(max(xi + 1, 0), sw - 1));
    const float* r3 = src + 3 * ((size_t)yy * sw + min(max(xi + 2, 0), sw - 1));
    for (int k = 0; k < 3; k++) rows[m + 1][k] = cubic_hermite(r0[k], r1[k], r2[k], r3[k], tx);
  }
  for (int k = 0; k < 3; k++)
    out[3 * ((size_t)y * dw + x) + k] = fmaxf(0.0f, cubic_hermite(rows[0][k], rows[1][k], rows[2][k], rows[3][k], ty));
}

// edgeAwareSharpen (renderer.go:2146-2183)
__global__ void k_sharpen(int W, int H, float amount, const float* __restrict__ img, float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const float* c = img + 3 * ((size_t)y * W + x);
  const float cl = lumf(c[0], c[1], c[2]);
  float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, count = 0.0f, edge = 0.0f;
  for (int oy = -1; oy <= 1; oy++) {
    const int yy = y + oy;
    if (yy < 0 || yy >= H) continue;
    for (int ox = -1; ox <= 1; ox++) {
      const int xx = x + ox;
      if (xx < 0 || xx >= W) continue;
      const float* nb = img + 3 * ((size_t)yy * W + xx);
      s0 += nb[0];
      s1 += nb[1];
      s2 += nb[2];
      count += 1.0f;
      edge += fabsf(cl - lumf(nb[0], nb[1], nb[2]));
    }
  }
  const float inv = 1.0f / fmaxf(count, 1.0f);
  const float local = amount * fminf(fmaxf(edge / 2.0f, 0.35f), 1.0f);
  float* o = out + 3 * ((size_t)y * W + x);
  o[0] = fmaxf(0.0f, c[0] + (c[0] - s0 * inv) * local);
  o[1] = fmaxf(0.0f, c[1] + (c[1] - s1 * inv) * local);
  o[2] = fmaxf(0.0f, c[2] + (c[2] - s2 * inv) * local);
}

// applyFXAA (renderer.go:2557-2587)
__global__ void k_fxaa(int W, int H, float threshold, float blend, const float* __restrict__ img,
                       float* __restrict__ out) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  const size_t i = (size_t)y * W + x;
  const float* c = img + 3 * i;
  float r0 = c[0], r1 = c[1], r2 = c[2];
  if (x >= 1 && x < W - 1 && y >= 1 && y < H - 1) {
    const float* n = img + 3 * (i - W);
    const float* s = img + 3 * (i + W);
    const float* w = img + 3 * (i - 1);
    const float* e = img + 3 * (i + 1);
    const float ln = lumf(n[0], n[1], n[2]), ls = lumf(s[0], s[1], s[2]), lw = lumf(w[0], w[1], w[2]),
                le = lumf(e[0], e[1], e[2]), lc = lumf(c[0], c[1], c[2]);
    const float lo = fminf(lc, fminf(fminf(ln, ls), fminf(lw, le)));
    const float hi = fmaxf(lc, fmaxf(fmaxf(ln, ls), fmaxf(lw, le)));
    if (!(hi - lo < threshold * fmaxf(1.0f, hi))) {
      r0 = c[0] * (1.0f - blend) + (n[0] + s[0] + w[0] + e[0]) * 0.25f * blend;
      r1 = c[1] * (1.0f - blend) + (n[1] + s[1] + w[1] + e[1]) * 0.25f * blend;
      r2 = c[2] * (1.0f - blend) + (n[2] + s[2] + w[2] + e[2]) * 0.25f * blend;
    }
  }
  out[3 * i] = r0;
  out[3 * i + 1] = r1;
  out[3 * i + 2] = r2;
}

double temporal_weight_of(int taa, int tsaa, int txaa) {  // temporalWeight (renderer.go:2419-2431)
  const int level = std::max(taa, std::max(tsaa, txaa));
  return level == 1 ? 0.48 : level == 2 ? 0.68 : level == 3 ? 0.82 : 0.0;
}

ProjCam proj_cam(const bc_camera& c) {  // projectPoint's frame in fp64 (renderer.go:2280-2292)
  auto unit = [](double v[3]) {
    const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (l < 1e-12) { v[0] = v[1] = v[2] = 0; return; }
    const double s = 1 / l;
    v[0] *= s; v[1] *= s; v[2] *= s;
  };
  double f[3] = {c.target[0] - c.position[0], c.target[1] - c.position[1], c.target[2] - c.position[2]};
  unit(f);
  double r[3] = {f[1] * c.up[2] - f[2] * c.up[1], f[2] * c.up[0] - f[0] * c.up[2], f[0] * c.up[1] - f[1] * c.up[0]};
  unit(r);
  double u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
  unit(u);
  ProjCam p;
  p.px = (float)c.position[0]; p.py = (float)c.position[1]; p.pz = (float)c.position[2];
  p.fx = (float)f[0]; p.fy = (float)f[1]; p.fz = (float)f[2];
  p.rx = (float)r[0]; p.ry = (float)r[1]; p.rz = (float)r[2];
  p.ux = (float)u[0]; p.uy = (float)u[1]; p.uz = (float)u[2];
  const double half_h = std::tan(c.fov_deg * M_PI / 360.0);
  p.half_h = (float)half_h;
  p.aspect = 1.0f;
  p.ok = half_h > 1e-8 ? 1 : 0;
  return p;
}

}  // namespace
}  // namespace bcgx

// History of the temporal pass (Start's r.historyLinear / historyGuides / historyCamera).
struct PostHistory {
  bool valid = false;
  int w = 0, h = 0;
  bc_camera cam{};
};

namespace bcgx {
void destroy_post_state(bc_context* ctx) {
  delete ctx->post_hist;
  ctx->post_hist = nullptr;
  ctx->d_post_stack.release();
  ctx->d_post_hist.release();
}
}  // namespace bcgx

extern "C" bc_status bc_post_history_reset(bc_context* ctx) {
  if (!ctx) return BC_ERR_INVALID_ARG;
  if (ctx->post_hist) ctx->post_hist->valid = false;
  return BC_OK;
}

extern "C" bc_status bc_post_stack(bc_context* ctx, const bc_post_desc* d, const float* linear_in,
                                   const float* guides_in, float* linear_out, uint32_t* rgba_out) {
  if (!ctx || !d || !linear_in) return set_error(ctx, BC_ERR_INVALID_ARG, "NULL argument");
  const int rw = d->render_width, rh = d->render_height, W = d->width, H = d->height;
  if (rw < 1 || rh < 1 || W < 1 || H < 1 || (int64_t)rw * rh > (1 << 26) || (int64_t)W * H > (1 << 26))
    return set_error(ctx, BC_ERR_INVALID_ARG, "bad post sizes");
  if (d->upscale < 0 || d->upscale > 3 || d->debug_view < 0 || d->debug_view > 5)
    return set_error(ctx, BC_ERR_INVALID_ARG, "unknown upscale mode or debug view");
  if ((rw != W || rh != H) && d->upscale == 0)
    return set_error(ctx, BC_ERR_INVALID_ARG, "output size differs from the render size without an upscaler");
  const double tw = temporal_weight_of(d->taa, d->tsaa, d->txaa);
  const bool need_guides = d->hbao > 0 || d->hbao_plus > 0 || d->denoise || tw > 0 ||
                           (d->debug_view >= 1 && d->debug_view <= 4);
  if (need_guides && !guides_in) return set_error(ctx, BC_ERR_INVALID_ARG, "these passes need guides");
  cudaSetDevice(ctx->device);
  cudaStream_t st = ctx->stream;
  const size_t n = (size_t)rw * rh, no = (size_t)W * H;
  const size_t bytes = n * (3 * 12 + 4 * 16 + 48) + no * (2 * 12 + 4) + 64 + 16 * 256;
  cudaError_t e = ctx->d_post_stack.ensure(bytes);
  if (e) return cuda_status(ctx, e, "post stack buffers");
  if (!ctx->post_hist) ctx->post_hist = new PostHistory();
  PostHistory& hist = *ctx->post_hist;
  const size_t hbytes = n * (12 + 2 * 16) + 4 * 256;
  if (ctx->d_post_hist.cap < hbytes) hist.valid = false;  // a new history buffer holds nothing
  e = ctx->d_post_hist.ensure(hbytes);
  if (e) return cuda_status(ctx, e, "post history buffers");
  char* p = (char*)ctx->d_post_stack.p;
  auto take = [&](size_t b) { char* r = p; p += ((b + 255) / 256) * 256; return (void*)r; };
  PostStackBufs B;
  B.a = (float*)take(n * 12);
  B.b = (float*)take(n * 12);
  B.c = (float*)take(n * 12);
  B.gp = (float4*)take(n * 16);
  B.gn = (float4*)take(n * 16);
  B.ga = (float4*)take(n * 16);
  B.gnd = (float4*)take(n * 16);
  float* g12 = (float*)take(n * 48);
  B.oa = (float*)take(no * 12);
  B.ob = (float*)take(no * 12);
  B.rgba = (uint32_t*)take(no * 4);
  B.maxbits = (unsigned*)take(64);
  char* hq = (char*)ctx->d_post_hist.p;
  float* h_img = (float*)hq;
  float4* h_gp = (float4*)(hq + ((n * 12 + 255) / 256) * 256);
  float4* h_gn = (float4*)((char*)h_gp + ((n * 16 + 255) / 256) * 256);

  const dim3 blk(32, 8), grd((rw + 31) / 32, (rh + 7) / 8), grdo((W + 31) / 32, (H + 7) / 8);
  const int n1 = (int)((n + 255) / 256);
  e = cudaMemcpyAsync(B.a, linear_in, n * 12, cudaMemcpyHostToDevice, st);
  if (!e && guides_in) e = cudaMemcpyAsync(g12, guides_in, n * 48, cudaMemcpyHostToDevice, st);
  if (e) return cuda_status(ctx, e, "post stack upload");
  if (guides_in) k_unpack_guides<<<n1, 256, 0, st>>>((int)n, g12, B.gp, B.gn, B.ga, B.gnd);
  float* cur = B.a;
  float* spare = B.b;
  // geometry-aware AO before temporal reconstruction and bloom
  if (d->hbao_plus > 0 || d->hbao > 0) {
    const bool plus = d->hbao_plus > 0;
    k_hbao<<<grd, blk, 0, st>>>(rw, rh, plus ? d->hbao_plus : d->hbao, plus ? 1 : 0, cur, B.gp, B.gn, spare);
    std::swap(cur, spare);
  }
  if (d->denoise) {
    const int passes = 2 + std::min(3, std::max(d->taa, d->txaa));
    for (int it = 0; it < passes; it++) {
      k_atrous<<<grd, blk, 0, st>>>(rw, rh, 1 << it, cur, B.gnd, spare);
      std::swap(cur, spare);
    }
  }
  if (tw > 0 && hist.valid && hist.w == rw && hist.h == rh) {
    ProjCam pc = proj_cam(hist.cam);
    pc.aspect = (float)((double)rw / (double)rh);
    k_temporal<<<grd, blk, 0, st>>>(rw, rh, (float)std::min(0.95, std::max(0.0, tw)), pc, cur, B.gp, B.gn, h_img,
                                    h_gp, h_gn, spare);
    std::swap(cur, spare);
  }
  if (d->bloom > 0) {
    const float threshold = (float)(1.25 - 0.2 * (double)d->bloom);
    const float strength = (float)(0.08 + 0.09 * (double)d->bloom);
    k_bloom_h<<<grd, blk, 0, st>>>(rw, rh, 1 + d->bloom, threshold, cur, B.c);
    k_bloom_v<<<grd, blk, 0, st>>>(rw, rh, 1 + d->bloom, strength, cur, B.c, spare);
    std::swap(cur, spare);
  }
  if (d->debug_view == 4) {  // AO of a white image
    const bool plus = d->hbao_plus > 0;
    const int level = plus ? d->hbao_plus : (d->hbao > 0 ? d->hbao : 2);
    k_fill<<<(int)((3 * n + 255) / 256), 256, 0, st>>>((int)(3 * n), 1.0f, B.c);
    k_hbao<<<grd, blk, 0, st>>>(rw, rh, std::max(level, 1), plus ? 1 : 0, B.c, B.gp, B.gn, spare);
    std::swap(cur, spare);
  } else if (d->debug_view != 0) {
    if (guides_in) {
      e = cudaMemsetAsync(B.maxbits, 0, 8, st);
      if (e) return cuda_status(ctx, e, "post stack");
      k_view_max<<<n1, 256, 0, st>>>((int)n, cur, B.gp, B.gn, B.maxbits);
    } else {  // heat view without guides: zero guides
      e = cudaMemsetAsync(B.gn, 0, n * 16, st);
      if (!e) e = cudaMemsetAsync(B.gp, 0, n * 16, st);
      if (!e) e = cudaMemsetAsync(B.maxbits, 0, 8, st);
      if (e) return cuda_status(ctx, e, "post stack");
      k_view_max<<<n1, 256, 0, st>>>((int)n, cur, B.gp, B.gn, B.maxbits);
    }
    k_debug_view<<<n1, 256, 0, st>>>((int)n, d->debug_view, cur, B.gp, B.gn, B.ga, B.maxbits, spare);
    std::swap(cur, spare);
  }
  // history for the next frame (only when a temporal mode consumes it)
  if (tw > 0) {
    e = cudaMemcpyAsync(h_img, cur, n * 12, cudaMemcpyDeviceToDevice, st);
    if (!e) e = cudaMemcpyAsync(h_gp, B.gp, n * 16, cudaMemcpyDeviceToDevice, st);
    if (!e) e = cudaMemcpyAsync(h_gn, B.gn, n * 16, cudaMemcpyDeviceToDevice, st);
    if (e) return cuda_status(ctx, e, "post history");
    hist.valid = true;
    hist.w = rw;
    hist.h = rh;
    hist.cam = d->camera;
  } else {
    hist.valid = false;
  }
  // output resolution: upscale, FXAA, TXAA resolve
  float* fin = cur;  // a render-size buffer; equal sizes unless upscaled
  if (d->upscale != 0 && (rw != W || rh != H)) {
    k_bicubic<<<grdo, blk, 0, st>>>(rw, rh, W, H, cur, B.oa);
    const float amount = d->upscale == 1 ? 0.10f : d->upscale == 2 ? 0.18f : 0.28f;
    k_sharpen<<<grdo, blk, 0, st>>>(W, H, amount, B.oa, B.ob);
    fin = B.ob;
  }
  auto fxaa = [&](int level) {
    static const float thresholds[4] = {0.0f, 0.16f, 0.10f, 0.065f}, blends[4] = {0.0f, 0.35f, 0.50f, 0.65f};
    const int l = std::min(level, 3);
    float* dst = fin == B.oa ? B.ob : B.oa;
    if (W >= 3 && H >= 3) {
      k_fxaa<<<grdo, blk, 0, st>>>(W, H, thresholds[l], blends[l], fin, dst);
      fin = dst;
    }
  };
  if (d->fxaa > 0) fxaa(d->fxaa);
  if (d->txaa > 0) {
    fxaa(std::min(3, d->txaa + 1));
    float* dst = fin == B.oa ? B.ob : B.oa;
    k_sharpen<<<grdo, blk, 0, st>>>(W, H, (float)(0.05 + 0.04 * (double)d->txaa), fin, dst);
    fin = dst;
  }
  if (rgba_out) {
    const float scale = (float)std::pow(2.0, d->exposure);
    const float inv_gamma = (float)(1.0 / std::max(0.1, d->gamma));
    k_tonemap<<<(int)((no + 255) / 256), 256, 0, st>>>((int)no, scale, inv_gamma, d->hdr, fin, B.rgba);
  }
  e = cudaGetLastError();
  if (!e && linear_out) e = cudaMemcpyAsync(linear_out, fin, no * 12, cudaMemcpyDeviceToHost, st);
  if (!e && rgba_out) e = cudaMemcpyAsync(rgba_out, B.rgba, no * 4, cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  return cuda_status(ctx, e, "post stack");
}

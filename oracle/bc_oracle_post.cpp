// Test infrastructure only: fp64 restatement of the rest of RenderState.Start's
// post stack (renderer.go:2838-2895): HBAO / HBAO+, temporal accumulation,
// debug views, the basic upscaler, FXAA and the TXAA resolve, and their order.
// Each function follows the Go code expression by expression.
#include <algorithm>
#include <cmath>

#include "bc_oracle.h"

namespace orc {

// applyHBAO (renderer.go:2433-2488)
std::vector<V3> apply_hbao(const std::vector<V3>& img, const std::vector<Guide>& g, int w, int h, int level,
                           bool plus) {
  if (level <= 0 || (int)img.size() != w * h || (int)g.size() != w * h) return img;
  std::vector<V3> out(img.size());
  int radius = 2 + level * 2;
  if (plus) radius += 2;
  double strength = 0.14 + 0.09 * (double)level;
  if (plus) strength *= 1.15;
  std::vector<std::pair<int, int>> dirs = {{1, 0}, {-1, 0}, {0, 1}, {0, -1}, {1, 1}, {-1, 1}, {1, -1}, {-1, -1}};
  if (plus) {
    dirs.push_back({2, 1});
    dirs.push_back({-2, 1});
    dirs.push_back({1, 2});
    dirs.push_back({-1, 2});
  }
  const int step_inc = std::max(1, radius / 3);
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      const int i = y * w + x;
      const Guide& gc = g[i];
      if (!gc.valid) {
        out[i] = img[i];
        continue;
      }
      double occ = 0.0, count = 0.0;
      for (const auto& d : dirs)
        for (int step = 1; step <= radius; step += step_inc) {
          const int xx = x + d.first * step, yy = y + d.second * step;
          if (xx < 0 || xx >= w || yy < 0 || yy >= h) continue;
          const Guide& ng = g[yy * w + xx];
          if (!ng.valid) continue;
          const double depthTol = 0.015 * gmax(gc.depth, 1.0) + 0.002 * (double)step;
          if (ng.depth + depthTol < gc.depth) {
            const double normalTerm = clampd(1.0 - dot(gc.n, ng.n), 0, 1);
            const double depthTerm = clampd((gc.depth - ng.depth) / (0.25 * gmax(gc.depth, 1.0)), 0, 1);
            occ += 0.55 * depthTerm + 0.45 * normalTerm;
          }
          count++;
        }
      double factor = 1.0;
      if (count > 0) factor = clampd(1.0 - strength * (occ / count), 0.35, 1.0);
      out[i] = mul(img[i], factor);
    }
  return out;
}

// projectPoint (renderer.go:2280-2314)
bool project_point(const Camera& cam, V3 p, int w, int h, int* ox, int* oy) {
  const V3 f = unit(sub(cam.target, cam.position));
  const V3 r = unit(cross(f, cam.up));
  const V3 u = unit(cross(r, f));
  const V3 rel = sub(p, cam.position);
  const double z = dot(rel, f);
  if (z <= 1e-5) return false;
  const double halfH = std::tan(cam.fov * M_PI / 360.0);
  if (halfH <= 1e-8) return false;
  const double aspect = (double)w / (double)h;
  const double nx = dot(rel, r) / (z * halfH * aspect);
  const double ny = dot(rel, u) / (z * halfH);
  if (nx < -1 || nx > 1 || ny < -1 || ny > 1) return false;
  const int x = (int)std::round((nx * 0.5 + 0.5) * (double)(w - 1));
  const int y = (int)std::round((0.5 - ny * 0.5) * (double)(h - 1));
  if (x < 0 || x >= w || y < 0 || y >= h) return false;
  *ox = x;
  *oy = y;
  return true;
}

// temporalAccumulate (renderer.go:2316-2364)
std::vector<V3> temporal_accumulate(const std::vector<V3>& cur, const std::vector<Guide>& g, int w, int h,
                                    const std::vector<V3>& prev, const std::vector<Guide>& pg_all,
                                    const Camera& prev_cam, double weight) {
  if ((int)cur.size() != w * h || (int)g.size() != w * h || (int)prev.size() != w * h ||
      (int)pg_all.size() != w * h)
    return cur;
  weight = clampd(weight, 0, 0.95);
  std::vector<V3> out = cur;
  for (int i = 0; i < w * h; i++) {
    const Guide& gi = g[i];
    if (!gi.valid) continue;
    int x, y;
    if (!project_point(prev_cam, gi.p, w, h, &x, &y)) continue;
    const int j = y * w + x;
    const Guide& pg = pg_all[j];
    if (!pg.valid) continue;
    if (dot(gi.n, pg.n) < 0.88) continue;
    const double posTol = 0.03 * gmax(gi.depth, 1.0);
    if (len(sub(gi.p, pg.p)) > posTol) continue;
    V3 lo = v3(INFINITY, INFINITY, INFINITY), hi = v3(-INFINITY, -INFINITY, -INFINITY);
    const int cx = i % w, cy = i / w;
    for (int oy = -1; oy <= 1; oy++) {
      const int yy = cy + oy;
      if (yy < 0 || yy >= h) continue;
      for (int ox = -1; ox <= 1; ox++) {
        const int xx = cx + ox;
        if (xx < 0 || xx >= w) continue;
        const V3 c = cur[yy * w + xx];
        lo = v3(gmin(lo.x, c.x), gmin(lo.y, c.y), gmin(lo.z, c.z));
        hi = v3(gmax(hi.x, c.x), gmax(hi.y, c.y), gmax(hi.z, c.z));
      }
    }
    V3 pc = prev[j];
    pc = v3(clampd(pc.x, lo.x, hi.x), clampd(pc.y, lo.y, hi.y), clampd(pc.z, lo.z, hi.z));
    out[i] = add(mul(cur[i], 1 - weight), mul(pc, weight));
  }
  return out;
}

// temporalWeight (renderer.go:2419-2431)
double temporal_weight(int taa, int tsaa, int txaa) {
  const int level = std::max(taa, std::max(tsaa, txaa));
  switch (level) {
    case 1: return 0.48;
    case 2: return 0.68;
    case 3: return 0.82;
    default: return 0;
  }
}

// makeDebugView (renderer.go:1972-2032): 0 beauty, 1 albedo, 2 normal, 3 depth, 4 AO, 5 heat
std::vector<V3> make_debug_view(const std::vector<V3>& lin, const std::vector<Guide>& g, int w, int h, int mode,
                                int hbao, int hbao_plus) {
  if (mode == 0) return lin;
  std::vector<V3> out(lin.size(), v3(0, 0, 0));
  switch (mode) {
    case 1:
      for (size_t i = 0; i < g.size(); i++)
        if (g[i].valid) out[i] = g[i].albedo;
      break;
    case 2:
      for (size_t i = 0; i < g.size(); i++)
        if (g[i].valid) out[i] = mul(add(g[i].n, v3(1, 1, 1)), 0.5);
      break;
    case 3: {
      double maxDepth = 1.0;
      for (const Guide& gg : g)
        if (gg.valid && gg.depth > maxDepth) maxDepth = gg.depth;
      for (size_t i = 0; i < g.size(); i++)
        if (g[i].valid) {
          const double v = 1 - clampd(g[i].depth / maxDepth, 0, 1);
          out[i] = v3(v, v, v);
        }
      break;
    }
    case 4: {
      std::vector<V3> base(lin.size(), v3(1, 1, 1));
      int level = 2;
      bool plus = false;
      if (hbao_plus > 0) {
        level = hbao_plus;
        plus = true;
      } else if (hbao > 0) {
        level = hbao;
      }
      out = apply_hbao(base, g, w, h, std::max(level, 1), plus);
      break;
    }
    case 5: {
      double maxLum = 1e-6;
      for (const V3& c : lin) {
        const double l = luminance(c);
        if (l > maxLum) maxLum = l;
      }
      for (size_t i = 0; i < lin.size(); i++) {
        const double t = clampd(luminance(lin[i]) / maxLum, 0, 1);
        out[i] = v3(clampd(1.5 * t, 0, 1), clampd(1.2 * (1 - std::fabs(t - 0.5) * 2), 0, 1), clampd(1.5 * (1 - t), 0, 1));
      }
      break;
    }
    default:
      out = lin;
  }
  return out;
}

// cubicHermite, sampleClamped, bicubicUpscale (renderer.go:2081-2138)
static double cubic_hermite(double a, double b, double c, double d, double t) {
  const double ta = -0.5 * a + 1.5 * b - 1.5 * c + 0.5 * d;
  const double tb = a - 2.5 * b + 2 * c - 0.5 * d;
  const double tc = -0.5 * a + 0.5 * c;
  const double td = b;
  return ((ta * t + tb) * t + tc) * t + td;
}
static V3 sample_clamped(const std::vector<V3>& src, int w, int h, int x, int y) {
  x = std::min(std::max(x, 0), w - 1);
  y = std::min(std::max(y, 0), h - 1);
  return src[y * w + x];
}
std::vector<V3> bicubic_upscale(const std::vector<V3>& src, int sw, int sh, int dw, int dh) {
  if (sw == dw && sh == dh) return src;
  std::vector<V3> out((size_t)dw * dh, v3(0, 0, 0));
  if (sw <= 0 || sh <= 0 || dw <= 0 || dh <= 0) return out;
  for (int y = 0; y < dh; y++) {
    double fy = 0.0;
    if (dh > 1) fy = (double)y * (double)(sh - 1) / (double)(dh - 1);
    const int yi = (int)std::floor(fy);
    const double ty = fy - (double)yi;
    for (int x = 0; x < dw; x++) {
      double fx = 0.0;
      if (dw > 1) fx = (double)x * (double)(sw - 1) / (double)(dw - 1);
      const int xi = (int)std::floor(fx);
      const double tx = fx - (double)xi;
      V3 rows[4];
      for (int m = -1; m <= 2; m++) {
        const V3 p0 = sample_clamped(src, sw, sh, xi - 1, yi + m), p1 = sample_clamped(src, sw, sh, xi, yi + m);
        const V3 p2 = sample_clamped(src, sw, sh, xi + 1, yi + m), p3 = sample_clamped(src, sw, sh, xi + 2, yi + m);
        rows[m + 1] = v3(cubic_hermite(p0.x, p1.x, p2.x, p3.x, tx), cubic_hermite(p0.y, p1.y, p2.y, p3.y, tx),
                         cubic_hermite(p0.z, p1.z, p2.z, p3.z, tx));
      }
      const V3 c = v3(cubic_hermite(rows[0].x, rows[1].x, rows[2].x, rows[3].x, ty),
                      cubic_hermite(rows[0].y, rows[1].y, rows[2].y, rows[3].y, ty),
                      cubic_hermite(rows[0].z, rows[1].z, rows[2].z, rows[3].z, ty));
      out[(size_t)y * dw + x] = v3(gmax(0, c.x), gmax(0, c.y), gmax(0, c.z));
    }
  }
  return out;
}

// edgeAwareSharpen (renderer.go:2146-2183)
std::vector<V3> edge_aware_sharpen(const std::vector<V3>& img, int w, int h, double amount) {
  if (amount <= 0 || w <= 0 || h <= 0) return img;
  std::vector<V3> out(img.size());
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      V3 sum = v3(0, 0, 0);
      double count = 0.0;
      const V3 center = img[y * w + x];
      const double centerLum = luminance(center);
      double edgeWeight = 0.0;
      for (int oy = -1; oy <= 1; oy++) {
        const int yy = y + oy;
        if (yy < 0 || yy >= h) continue;
        for (int ox = -1; ox <= 1; ox++) {
          const int xx = x + ox;
          if (xx < 0 || xx >= w) continue;
          const V3 nb = img[yy * w + xx];
          sum = add(sum, nb);
          count++;
          edgeWeight += std::fabs(centerLum - luminance(nb));
        }
      }
      const V3 blur = mul(sum, 1 / gmax(count, 1));
      const double local = amount * clampd(edgeWeight / 2.0, 0.35, 1.0);
      const V3 c = add(center, mul(sub(center, blur), local));
      out[y * w + x] = v3(gmax(0, c.x), gmax(0, c.y), gmax(0, c.z));
    }
  return out;
}

// upscaleDLSSBasic (renderer.go:2185-2197): mode 0 off, 1 ultra quality, 2 balanced, 3 performance
std::vector<V3> upscale_basic(const std::vector<V3>& src, int sw, int sh, int dw, int dh, int mode) {
  std::vector<V3> out = bicubic_upscale(src, sw, sh, dw, dh);
  switch (mode) {
    case 1: return edge_aware_sharpen(out, dw, dh, 0.10);
    case 2: return edge_aware_sharpen(out, dw, dh, 0.18);
    case 3: return edge_aware_sharpen(out, dw, dh, 0.28);
    default: return out;
  }
}

// internalSize (renderer.go:2066-2079)
void internal_size(int width, int height, int mode, int* rw, int* rh) {
  double scale = 1.0;
  if (mode == 1) scale = 0.77;
  else if (mode == 2) scale = 0.67;
  else if (mode == 3) scale = 0.50;
  *rw = std::max(16, (int)std::round((double)width * scale));
  *rh = std::max(16, (int)std::round((double)height * scale));
}

// applyFXAA (renderer.go:2557-2587)
std::vector<V3> apply_fxaa(const std::vector<V3>& img, int w, int h, int level) {
  if (level <= 0 || (int)img.size() != w * h || w < 3 || h < 3) return img;
  std::vector<V3> out = img;
  static const double thresholds[4] = {0, 0.16, 0.10, 0.065}, blends[4] = {0, 0.35, 0.50, 0.65};
  const double threshold = thresholds[std::min(level, 3)], blend = blends[std::min(level, 3)];
  for (int y = 1; y < h - 1; y++)
    for (int x = 1; x < w - 1; x++) {
      const int i = y * w + x;
      const V3 c = img[i];
      const double ln = luminance(img[(y - 1) * w + x]), ls = luminance(img[(y + 1) * w + x]);
      const double lw = luminance(img[y * w + x - 1]), le = luminance(img[y * w + x + 1]);
      const double lc = luminance(c);
      const double lo = gmin(lc, gmin(gmin(ln, ls), gmin(lw, le)));
      const double hi = gmax(lc, gmax(gmax(ln, ls), gmax(lw, le)));
      if (hi - lo < threshold * gmax(1.0, hi)) continue;
      const V3 avg = mul(add(add(add(img[(y - 1) * w + x], img[(y + 1) * w + x]), img[y * w + x - 1]), img[y * w + x + 1]), 0.25);
      out[i] = add(mul(c, 1 - blend), mul(avg, blend));
    }
  return out;
}

// applyTXAAResolve (renderer.go:2589-2595)
std::vector<V3> apply_txaa_resolve(const std::vector<V3>& img, int w, int h, int level) {
  if (level <= 0) return img;
  std::vector<V3> resolved = apply_fxaa(img, w, h, std::min(3, level + 1));
  const double amount = 0.05 + 0.04 * (double)level;
  return edge_aware_sharpen(resolved, w, h, amount);
}

}  // namespace orc

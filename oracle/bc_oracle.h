// Test infrastructure only: the CPU oracle for the Beamcast GX path-tracing
// hot path. It restates the portable Go renderer (windows_portable/renderer.go)
// in C++17 fp64 with floating-point contraction disabled, so that each
// expression rounds exactly like the Go code compiled for amd64.
//
// Only tests, the smoke check and the CPU-baseline leg of the benchmark use
// this library; the product path never links or calls it.
//
// Parity pins: structural results (BVH node sets, escape tables, light PMF,
// Halton tables, presets, AABB slab test, stack/stackless/any-hit agreement)
// are checked against the reference's own unit tests (renderer_test.go).
// Rendered radiance has no golden image in the reference, and its RNG is
// time-seeded (renderer.go:2741), so image parity is statistical.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>
#include <string>
#include <atomic>
#include <unordered_map>

namespace orc {

struct V3 {
  double x, y, z;
};
// renderer.go:23-39. Every helper keeps Go's left-to-right evaluation order.
inline V3 v3(double x, double y, double z) { return V3{x, y, z}; }
inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 mul(V3 a, double s) { return v3(a.x * s, a.y * s, a.z * s); }
inline V3 had(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
double len(V3 a);
V3 unit(V3 a);
inline double gmax(double a, double b) { return a > b ? a : (b > a ? b : (a == 0 && b == 0 ? (std::signbit(a) ? b : a) : a)); }
inline double gmin(double a, double b) { return a < b ? a : (b < a ? b : (a == 0 && b == 0 ? (std::signbit(a) ? a : b) : a)); }
inline double maxcomp(V3 a) { return gmax(a.x, gmax(a.y, a.z)); }
inline double clampd(double x, double a, double b) { return x < a ? a : (x > b ? b : x); }
inline double luminance(V3 c) { return 0.2126 * c.x + 0.7152 * c.y + 0.0722 * c.z; }  // renderer.go:2142

struct Ray { V3 o, d; };
struct RayAccel {  // renderer.go:52-81
  Ray ray;
  V3 inv{0, 0, 0};
  double dirLen2 = 0, invDirLen2 = 0;
  bool zx = false, zy = false, zz = false;
};
RayAccel prepare_ray(const Ray& r);

struct AABB { V3 mn, mx; };
AABB empty_aabb();
AABB expand_point(AABB b, V3 p);
AABB expand_box(AABB b, const AABB& c);
double surface_area(const AABB& b);
bool aabb_hit(const AABB& b, const RayAccel& r, double tmin, double tmax, double* near_out);

enum MatKind { MatDiffuse = 0, MatMetal = 1, MatGlass = 2, MatEmissive = 3 };
struct Material {
  int kind = MatDiffuse;
  V3 color{0, 0, 0};
  double roughness = 0, ior = 0;
  V3 emission{0, 0, 0};
};
enum PrimKind { PrimSphere = 0, PrimTriangle = 1 };
struct Primitive {
  int kind = PrimTriangle;
  int material = 0;
  V3 center{0, 0, 0};
  double radius = 0;
  V3 a{0, 0, 0}, b{0, 0, 0}, c{0, 0, 0}, e1{0, 0, 0}, e2{0, 0, 0}, normal{0, 0, 0};
  AABB box;
  V3 centroid{0, 0, 0};
};
struct Node { AABB box; int left = -1, right = -1, start = 0, count = 0; };
struct Hit { double t = 0; V3 n{0, 0, 0}; int material = 0; int primitive = -1; bool front = false; };

// Traversal counters feed the algorithmic-bytes model of the benchmark:
// boxes = AABB.HitAccel calls, tris = triHit calls, spheres = sphere tests.
struct Counters { int64_t boxes = 0, tris = 0, spheres = 0; };

struct Scene {
  std::vector<Material> materials;
  std::vector<Primitive> prims;
  std::vector<Node> nodes;
  std::vector<int> order;
  std::vector<int> light_spheres;
  std::vector<double> light_cdf;
  std::vector<double> light_pdf_by_prim;
  std::string bvh_mode = "SAH";
  int bvh_bins = 16, bvh_leaf = 4;
  uint64_t topo_rev = 0, geom_rev = 0;

  int add_material(const Material& m);
  void add_sphere(V3 c, double r, int mat);
  void add_triangle(V3 a, V3 b, V3 c, int mat);
  void rebuild_light_distribution();
  void build();
  void refit();
  int build_sah(int start, int end);
  int build_median(int start, int end);
  void node_bounds(int start, int end, AABB* box, AABB* cb) const;

  bool hit(const Ray& r, double tmin, double tmax, Hit* out, Counters* c) const;
  bool occluded(const Ray& r, double tmin, double tmax, Counters* c) const;
  bool hit_threaded(const Ray& r, double tmin, double tmax, const std::vector<int32_t>& esc, Hit* out) const;
  bool hit_recursive(int ni, const RayAccel& ar, double tmin, double tmax, Hit* out, Counters* c) const;
  bool occluded_recursive(int ni, const RayAccel& ar, double tmin, double tmax, Counters* c) const;
};

std::vector<int32_t> threaded_escapes(const std::vector<Node>& nodes);
bool prim_hit(const Primitive& p, const RayAccel& ar, double tmin, double tmax, Hit* h);
bool prim_any_hit(const Primitive& p, const RayAccel& ar, double tmin, double tmax);

struct Camera { V3 position, target, up; double fov; };
void camera_basis(const Camera& c, double aspect, V3* origin, V3* lower, V3* horiz, V3* vert);

enum Sampler { SamplerRandom = 0, SamplerHalton = 1, SamplerR2 = 2 };
struct Settings {
  int width = 320, height = 240, spp = 16, bounces = 5;
  int msaa = 1, tsaa = 0;
  int sampler = SamplerHalton;
  bool mis = true, power_light = true;
  double firefly_clamp = 0;
  int rr_depth = 4;
  bool adaptive = false;
  double adaptive_threshold = 0.0006;
  bool denoise = false;
  int taa = 0, txaa = 0, bloom = 0, hdr = 2;
  double exposure = 0, gamma = 2.2;
  int tile = 8;
  int integrator = 0;      // IntegratorMode (renderer.go:1002-1006): 0 path, 1 recursive, 2 photon
  int photon_mapping = 0;  // RenderSettings.PhotonMapping level (photon budget and radius)
  int64_t photon_seed = -1;  // seed of the photon map's emission streams; < 0: the render seed
  // pixel window [win_x, win_x + win_w) x [win_y, win_y + win_h) of the frame;
  // win_w == 0 renders the whole frame. Pixels keep their frame coordinates
  // (camera ray, sample rotation, RNG stream), so a window equals that part of
  // the whole frame.
  int win_x = 0, win_y = 0, win_w = 0, win_h = 0;
};
enum Integrator { IntegratorPath = 0, IntegratorRecursive = 1, IntegratorPhoton = 2 };
int effective_spp(const Settings& s);  // renderer.go:2395

// PCG32 stream; the GPU kernels draw from the same generator so that a
// common-random-number run can replay a path decision by decision.
struct Rng {
  uint64_t state = 0, inc = 1;
  uint32_t next_u32();
  double float64();  // 24-bit uniform in [0,1)
  int intn(int n);
};
Rng make_path_rng(uint64_t seed, uint64_t pixel_key, uint64_t sample);

V3 rand_in_unit_sphere(Rng& r);
V3 rand_unit_vector(Rng& r);
V3 rand_cos_hemisphere(V3 n, Rng& r);
V3 reflect(V3 v, V3 n);
V3 refract(V3 uv, V3 n, double eta);
double schlick(double c, double ref);
V3 background(V3 d);
double power_heuristic(double a, double b);
double light_selection_pdf(const Scene& s, int prim, bool power);
double light_directional_pdf(const Scene& s, int prim, V3 from, V3 lp, V3 ln, bool power);
double radical_inverse(uint64_t n, uint64_t base);
double fractd(double x);
void pixel_sample_rotation(int x, int y, double* rx, double* ry);
void build_sample_sequence(const Settings& s, std::vector<double>* X, std::vector<double>* Y);
V3 clamp_firefly(V3 c, double limit);
std::vector<int> make_tile_order(int tx, int ty, const std::string& mode);

struct Guide { V3 p{0, 0, 0}, n{0, 0, 0}, albedo{0, 0, 0}; double depth = 0; bool valid = false; };
struct TraceStats { int64_t segments = 0, shadow = 0; Counters c; };

V3 trace(const Scene& s, Ray ray, const Settings& st, Rng& rng, TraceStats* stats, Guide* guide);
V3 direct_light(const Scene& s, const Hit& h, V3 hitP, const Material& mat, Rng& rng, const Settings& st,
                TraceStats* stats);
V3 material_preview_color(const Material& m);

// bc_oracle_integrators.cpp: the recursive and photon-mapping integrators
// (renderer.go:1565-1831). Photon emission k draws from its own stream,
// make_path_rng(seed, k, kPhotonStream), where the reference draws every
// emission from one time-seeded generator (renderer.go:1651).
constexpr uint64_t kPhotonStream = 0xFFFFFFFFull;
struct Photon { V3 p, n, flux; int emission = 0; };
struct PhotonMap {
  std::vector<Photon> photons;                          // append order
  std::unordered_map<uint64_t, std::vector<int>> grid;  // cell key -> photon indices in append order
  double cell = 0, radius = 0;
};
AABB scene_bounds(const Scene& s);              // renderer.go:1137-1146
int photon_budget(int level);                   // renderer.go:1148-1161
double photon_radius(const Scene& s, int level);  // renderer.go:1163-1182
uint64_t photon_cell_key(int64_t x, int64_t y, int64_t z);  // renderer.go:1636-1639
PhotonMap build_photon_map(const Scene& s, const Settings& st, uint64_t seed, int64_t* rays);
V3 photon_gather(const PhotonMap& pm, V3 p, V3 n, int max_photons);
V3 trace_recursive(const Scene& s, Ray ray, const Settings& st, Rng& rng, TraceStats* stats, Guide* guide);
V3 trace_photon(const Scene& s, Ray ray, const Settings& st, Rng& rng, TraceStats* stats, Guide* guide,
                const PhotonMap& pm);
// pixelRadiance (renderer.go:1833-1842)
V3 pixel_radiance(const Scene& s, Ray ray, const Settings& st, Rng& rng, TraceStats* stats, Guide* guide,
                  const PhotonMap* pm);

struct RenderOut {
  std::vector<V3> linear;   // mean radiance per pixel
  std::vector<V3> sumsq;    // per-channel mean of squared sample radiance
  std::vector<Guide> guides;
  int64_t segments = 0, shadow = 0;
  int64_t photon_rays = 0;  // rays of the photon map build (RenderState.Start adds them to Rays)
  Counters c;
};
// Tile-parallel render shaped like RenderState.Start's CPU path
// (renderer.go:2692-2826): center-first tiles, one-tile atomic claims. With a
// window (Settings::win_w > 0) the outputs hold the window's pixels, row-major.
void render(const Scene& s, const Camera& cam, const Settings& st, uint64_t seed, int threads,
            RenderOut* out, const std::atomic<bool>* cancel);

std::vector<V3> atrous_denoise(const std::vector<V3>& img, const std::vector<Guide>& g, int w, int h, int iters);
std::vector<V3> box_blur(const std::vector<V3>& img, int w, int h, int radius);
std::vector<V3> apply_bloom(const std::vector<V3>& img, int w, int h, int level);
V3 tone_map_hdr(V3 c, int hdr);
uint32_t to_rgba(V3 c, double exposure, double gamma, int hdr);

// bc_oracle_post.cpp: the rest of RenderState.Start's post stack
std::vector<V3> apply_hbao(const std::vector<V3>& img, const std::vector<Guide>& g, int w, int h, int level, bool plus);
bool project_point(const Camera& cam, V3 p, int w, int h, int* ox, int* oy);
std::vector<V3> temporal_accumulate(const std::vector<V3>& cur, const std::vector<Guide>& g, int w, int h,
                                    const std::vector<V3>& prev, const std::vector<Guide>& pg, const Camera& prev_cam,
                                    double weight);
double temporal_weight(int taa, int tsaa, int txaa);
std::vector<V3> make_debug_view(const std::vector<V3>& lin, const std::vector<Guide>& g, int w, int h, int mode,
                                int hbao, int hbao_plus);
std::vector<V3> bicubic_upscale(const std::vector<V3>& src, int sw, int sh, int dw, int dh);
std::vector<V3> edge_aware_sharpen(const std::vector<V3>& img, int w, int h, double amount);
std::vector<V3> upscale_basic(const std::vector<V3>& src, int sw, int sh, int dw, int dh, int mode);
void internal_size(int width, int height, int mode, int* rw, int* rh);
std::vector<V3> apply_fxaa(const std::vector<V3>& img, int w, int h, int level);
std::vector<V3> apply_txaa_resolve(const std::vector<V3>& img, int w, int h, int level);

}  // namespace orc

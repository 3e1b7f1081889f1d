/*
 * bc_gx.h - C ABI of the GB300-native Beamcast GX path-tracing hot path.
 *
 * This library replaces the explicit-GPU OpenCL slot of the portable Go
 * renderer (windows_portable/gpu_opencl_windows.go, stub gpu_opencl_stub.go).
 * Every entry point takes plain pointers and sizes, returns a bc_status, and
 * never aborts or traps: a failure is reported through the status and
 * bc_last_error(). There is no CPU fallback: without a usable GPU the calls
 * fail with BC_ERR_NO_DEVICE.
 *
 * Threading: a bc_context is not thread-safe (the Go glue holds a mutex, as
 * persistentCL.mu does at gpu_opencl_windows.go:94-131). bc_cancel() alone may
 * be called from any thread.
 *
 * Memory: host buffers are caller-owned and are not retained after a call
 * returns; device memory and pinned staging are owned by the context and
 * released by bc_destroy().
 */
#ifndef BC_GX_H
#define BC_GX_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bc_status {
  BC_OK = 0,
  BC_ERR_NO_DEVICE = 1,     /* no CUDA device / driver, or not sm_103 */
  BC_ERR_OOM = 2,           /* device or pinned allocation failed */
  BC_ERR_BAD_SCENE = 3,     /* scene encoding rejected (gpu_opencl_windows.go:470-482) */
  BC_ERR_CANCELLED = 4,     /* bc_cancel() observed ("render cancelled", gpu_opencl_windows.go:645) */
  BC_ERR_TIMEOUT = 5,       /* a bounded device-side wait gave up */
  BC_ERR_DEVICE = 6,        /* any other CUDA error; the context may need bc_destroy() */
  BC_ERR_INVALID_ARG = 7,   /* null pointer, bad size, bad setting */
  BC_ERR_NO_SCENE = 8,      /* render or ray cast before bc_scene_upload() */
  BC_ERR_CAPACITY = 9       /* a queue or buffer limit of the context was exceeded */
} bc_status;

typedef struct bc_context bc_context;

/* Material kinds (renderer.go:85-92) and primitive kinds (renderer.go:102-107). */
enum { BC_MAT_DIFFUSE = 0, BC_MAT_METAL = 1, BC_MAT_GLASS = 2, BC_MAT_EMISSIVE = 3 };
enum { BC_PRIM_SPHERE = 0, BC_PRIM_TRIANGLE = 1 };
/* Samplers (renderer.go:1019-1025). */
enum { BC_SAMPLER_RANDOM = 0, BC_SAMPLER_HALTON = 1, BC_SAMPLER_R2 = 2 };

/*
 * Scene hand-off. Mirrors the fields of Go's Scene (renderer.go:225-240) after
 * Scene.Build(): primitives as the reference stores them (fp64), the binary
 * BVH produced by the reference's own builder (Nodes + Order), and the light
 * distribution (LightSpheres, LightCDF, LightPDFByPrim). The library copies
 * what it needs; nothing is retained after bc_scene_upload() returns.
 * Arrays marked 3n/6n are row-major (x, y, z) triples / (min xyz, max xyz).
 */
typedef struct bc_scene_desc {
  int32_t n_materials;
  const int32_t* mat_kind;        /* n_materials */
  const double* mat_color;        /* 3n */
  const double* mat_roughness;    /* n */
  const double* mat_ior;          /* n */
  const double* mat_emission;     /* 3n */

  int32_t n_prims;
  const int32_t* prim_kind;       /* BC_PRIM_* */
  const int32_t* prim_material;
  const double* prim_center;      /* 3n, spheres */
  const double* prim_radius;      /* n, spheres */
  const double* prim_a;           /* 3n, triangle vertex A */
  const double* prim_e1;          /* 3n, B - A */
  const double* prim_e2;          /* 3n, C - A */
  const double* prim_normal;      /* 3n, unit(E1 x E2) */

  int32_t n_nodes;
  const double* node_box;         /* 6n */
  const int32_t* node_left;       /* -1 for leaves */
  const int32_t* node_right;
  const int32_t* node_start;      /* leaves: first index into order */
  const int32_t* node_count;      /* leaves: 1..16 primitives; 0 for internal nodes */
  const int32_t* order;           /* n_prims permutation (Scene.Order) */

  int32_t n_lights;
  const int32_t* light_spheres;   /* prim indices of emissive spheres */
  const double* light_cdf;        /* n_lights */
  const double* light_pdf_by_prim;/* n_prims */
} bc_scene_desc;

/* Pinhole camera (renderer.go:941-960). */
typedef struct bc_camera {
  double position[3], target[3], up[3];
  double fov_deg;
} bc_camera;

/* IntegratorMode (renderer.go:1002-1006); pixelRadiance (1833-1842) dispatches on it. */
#define BC_INTEGRATOR_PATH 0      /* trace (1484-1563) */
#define BC_INTEGRATOR_RECURSIVE 1 /* traceRecursive (1565-1621) */
#define BC_INTEGRATOR_PHOTON 2    /* tracePhotonMapped (1763-1831) over buildPhotonMap (1642-1728) */

/*
 * The subset of RenderSettings (renderer.go:1027-1062) that the hot path reads.
 */
typedef struct bc_settings {
  int32_t width, height, spp, bounces;
  int32_t msaa, tsaa;             /* effectiveSPP factors (renderer.go:2395-2417) */
  int32_t sampler;                /* BC_SAMPLER_* */
  int32_t mis, power_light_sampling;
  double firefly_clamp;           /* <= 0: off */
  int32_t rr_depth;               /* < 1 means 4 (renderer.go:1550-1553) */
  int32_t adaptive_sampling;
  double adaptive_threshold;
  int32_t denoise, taa, txaa;     /* a-trous passes = 2 + min(3, max(taa, txaa)) (renderer.go:2845) */
  int32_t bloom, hdr;             /* bloom level, tone-map curve (renderer.go:2034-2053) */
  double exposure, gamma;
  uint64_t seed;                  /* path RNG seed: equal seeds give equal images */
  int32_t integrator;             /* BC_INTEGRATOR_* */
  int32_t photon_mapping;         /* PhotonMapping level 1-4 (budget 512..16384 photons); others: no photons */
} bc_settings;

/* ---- context ------------------------------------------------------------ */

/* Availability probe; replaces openCLGPUAvailable() (gpu_opencl_windows.go:172,
 * stub gpu_opencl_stub.go:10). Returns 1 if a usable device exists, else 0,
 * and writes a one-line reason into reason[reason_len] either way. */
int bc_gpu_available(char* reason, size_t reason_len);

/* Create a context on a CUDA device ordinal (persistentCL initLocked,
 * gpu_opencl_windows.go:224). */
bc_status bc_create(int device_ordinal, bc_context** out);
void bc_destroy(bc_context* ctx);
/* Copies the last error message of this context (thread-local message when ctx is NULL). */
bc_status bc_last_error(const bc_context* ctx, char* buf, size_t len);
bc_status bc_device_name(const bc_context* ctx, char* buf, size_t len);

/* ---- scene -------------------------------------------------------------- */

/*
 * Upload or update a scene; replaces ensureSceneLocked (gpu_opencl_windows.go:484-495)
 * with uploadFullSceneLocked (379) and updateGeometryLocked (447). scene_id
 * identifies the caller's scene object (Go: the *Scene pointer value). When
 * scene_id and topology_rev match the resident scene and only geometry_rev
 * changed, the primitives and the caller's refit node boxes replace the
 * resident ones on the device (same primitive and node counts required, else
 * a full upload); when all three match, the call is a no-op.
 * Leaves with more than 16 primitives or more than 2^27 nodes/primitives are
 * rejected with BC_ERR_BAD_SCENE, as validateGPUSceneEncoding (470-482) does.
 */
bc_status bc_scene_upload(bc_context* ctx, const bc_scene_desc* scene, uint64_t scene_id, uint64_t topology_rev,
                          uint64_t geometry_rev);

/*
 * Upload a resident scene set for batched rendering (bc_render_batch): scenes[k]
 * becomes scene k of the set, with its own BVH root, materials and lights in one
 * set of device arrays. No reference counterpart (the reference keeps one scene
 * resident, gpu_opencl_windows.go:94-131); this is the batching entry point's
 * scene side. set_id names the caller's set: an upload with the set_id, count
 * and revision of the resident set is a no-op. A set replaces the resident
 * scene; the single-view calls (bc_raycast, bc_render_frame, ...) use scene 0.
 */
bc_status bc_scene_set_upload(bc_context* ctx, const bc_scene_desc* scenes, int32_t n_scenes, uint64_t set_id,
                              uint64_t revision);

/*
 * Binned SAH build on the device with the result of Scene.Build's SAH mode
 * (buildNodeSAH, renderer.go:526-633): the same nodes in the same pre-order
 * numbering and the same Scene.Order, bit for bit. prim_box: 6 doubles per
 * primitive (the padded Primitive.Box: min xyz, max xyz); centroid: 3 doubles
 * per primitive; bins and leaf_size are clamped as Scene.Build clamps them.
 * Outputs (host arrays): node arrays of capacity 2 * n_prims - 1, filled up to
 * *n_nodes_out; node_box 6 doubles per node; left/right -1 for leaves; start
 * and count 0 for inner nodes; order_out n_prims. No reference counterpart on
 * the GPU (the reference builds on the host).
 */
bc_status bc_build_sah(bc_context* ctx, int32_t n_prims, const double* prim_box, const double* centroid, int32_t bins,
                       int32_t leaf_size, int32_t* n_nodes_out, double* node_box, int32_t* node_left,
                       int32_t* node_right, int32_t* node_start, int32_t* node_count, int32_t* order_out);

/* Statistics of the resident scene: out[0] BVH8 nodes, out[1] primitive slots,
 * out[2] binary nodes, out[3] BVH8 depth, out[4] traversal stack entries needed,
 * out[5] device bytes held by the scene, out[6] geometry-only updates applied
 * by this context (the device path of bc_scene_upload when only geometry_rev
 * moved: new primitives and refit node boxes are copied up, slots rewritten and
 * every BVH8 node re-quantized on the GPU, the BVH8 topology kept). */
bc_status bc_scene_stats(const bc_context* ctx, int64_t* out, int n_out);

/* ---- ray casting (closest hit / any hit) -------------------------------- */

/*
 * Closest hit for n rays, each 8 floats: (ox, oy, oz, tmin, dx, dy, dz, tmax).
 * Semantics are those of Scene.Hit (renderer.go:777-849) evaluated in fp64 on
 * the fp32 ray: prim_out[i] is the Scene primitive index of the nearest hit
 * (-1 on a miss) and t_out[i] = float32(t_fp64) (-1 on a miss). Exact: the hit
 * index equals the fp64 CPU path's, exact ties included: a ray whose nearest
 * fp64 distance several primitives share is walked again over the caller's
 * binary BVH as Scene.Hit walks it, so it gets the primitive the reference
 * keeps (the last one tested at that distance, renderer.go:702, 800-808).
 * Host pointers; copies in and out are part of the call.
 */
bc_status bc_raycast(bc_context* ctx, const float* rays, int64_t n, float* t_out, int32_t* prim_out);
/* Same on device pointers, enqueued on `stream` (a cudaStream_t; NULL = the
 * context's own stream) on the context's device; asynchronous. The returned
 * status covers the arguments and the launch; what the kernels find while they
 * run (a traversal stack or record limit) goes to a status word of the
 * device-pointer calls that bc_sync() returns. The context's scratch (ray
 * order, per-ray records of the split passes, work counter) is shared by its
 * calls: calls of one context must not overlap on different streams. */
bc_status bc_raycast_device(bc_context* ctx, const float* d_rays, int64_t n, float* d_t_out, int32_t* d_prim_out,
                            void* stream);
/* Any hit (Scene.Occluded, renderer.go:851-895): occluded_out[i] = 1 if any primitive
 * is hit within [tmin, tmax], fp64-exact like bc_raycast. */
bc_status bc_occluded(bc_context* ctx, const float* rays, int64_t n, uint8_t* occluded_out);
bc_status bc_occluded_device(bc_context* ctx, const float* d_rays, int64_t n, uint8_t* d_occluded_out, void* stream);
/* Waits for `stream` (NULL = the context's own stream) and returns the kernel
 * status of the bc_raycast_device / bc_occluded_device calls enqueued since the
 * last bc_sync (BC_OK, or the error a kernel flagged: BC_ERR_CAPACITY for a
 * traversal stack or queue limit, BC_ERR_TIMEOUT, BC_ERR_DEVICE), then clears
 * it. That status never surfaces through another call. Replaces the blocking
 * read after each OpenCL enqueue (gpu_opencl_windows.go:671-690), whose error
 * becomes the render's (clErr, 180-185). */
bc_status bc_sync(bc_context* ctx, void* stream);

/* ---- rendering ---------------------------------------------------------- */

/*
 * Render rows [y0, y0 + rows) of the frame; replaces one chunk iteration of
 * renderOpenCL (gpu_opencl_windows.go:643-720). linear_out receives rows*width
 * RGB float triples (the linear HDR mean per pixel, Start's jobLinear).
 * guide_out (may be NULL) receives rows*width*3 uint32 in the reference's
 * compact guide encoding (gpu_opencl_windows.go:519-521, 791-797): depth float
 * bits; valid<<31 | material<<20 | octN.y<<10 | octN.x; jitter v<<16 | u.
 * rays_out (may be NULL) receives the number of extension rays traced (the
 * reference's Rays, renderer.go:1491), plus the photon map's rays in the call
 * that builds it (renderer.go:2809).
 *
 * settings->integrator picks pixelRadiance's integrator (renderer.go:1833-1842).
 * The photon integrator builds its photon map (buildPhotonMap) once per scene,
 * seed, PhotonMapping level and bounce count and keeps it for the next chunks
 * and frames; emission k of the map draws from its own stream keyed by
 * (seed, k). The recursive integrator runs in the wave engine only
 * (render_engine 1 rejects it).
 */
bc_status bc_render_rows(bc_context* ctx, const bc_camera* cam, const bc_settings* settings, int32_t y0,
                         int32_t rows, float* linear_out, uint32_t* guide_out, int64_t* rays_out);

/*
 * Whole frame with the post stack of RenderState.Start on the device
 * (renderer.go:2844-2854, 2890-2895): a-trous denoise when settings->denoise,
 * bloom when settings->bloom > 0, then tone map to RGBA8. Any output pointer may be NULL.
 * linear_out: width*height RGB floats after denoise and bloom; rgba_out: packed
 * 0xff<<24 | b<<16 | g<<8 | r (toRGBA, renderer.go:2055-2064).
 */
bc_status bc_render_frame(bc_context* ctx, const bc_camera* cam, const bc_settings* settings, float* linear_out,
                          uint32_t* guide_out, uint32_t* rgba_out, int64_t* rays_out);

/*
 * Convergence statistics of a frame without post: mean_out and meansq_out each
 * receive width*height RGB floats, the per-pixel mean of the (firefly-clamped)
 * sample radiance and the mean of its square. The per-pixel Monte Carlo
 * standard error is sqrt((meansq - mean^2) / (spp - 1)). Same samples as
 * bc_render_frame with the same settings.
 */
bc_status bc_render_moments(bc_context* ctx, const bc_camera* cam, const bc_settings* settings, float* mean_out,
                            float* meansq_out, int64_t* rays_out);

/*
 * One view of a batch: a camera and settings over scene `scene` of the resident
 * set. The settings fields read are those bc_render_frame reads for the linear
 * image (no post stack, no guides).
 */
typedef struct bc_view {
  int32_t scene;
  int32_t reserved;  /* 0 */
  bc_camera camera;
  bc_settings settings;
} bc_view;

/*
 * Render n_views views in one pass of the wave engine: every view's (sample,
 * pixel) paths are scheduled in one index space, so small views share waves
 * and the device stays full; one wave is a captured CUDA graph replayed until
 * the batch is done. linear_out[v] (array and entries may be NULL) receives
 * views[v]'s width*height RGB floats, the same mean radiance bc_render_frame
 * returns for that view with post off. rays_out: extension rays over all views.
 * No reference counterpart: the reference renders one view per call
 * (renderOpenCL, gpu_opencl_windows.go:565).
 */
bc_status bc_render_batch(bc_context* ctx, const bc_view* views, int32_t n_views, float* const* linear_out,
                          int64_t* rays_out);

/*
 * The photon map of the photon integrator (buildPhotonMap, renderer.go:1642-1728)
 * for scene `scene` of the resident set (0 after bc_scene_upload) and the seed,
 * bounces and photon_mapping level of *settings: the same map the renders use.
 * photons_out receives min(n, capacity) photons of 10 floats (position,
 * normal, flux, emission index) in the reference's append order; *n_out the
 * photon count n (0 without sphere lights or for levels outside 1-4);
 * *rays_out the rays traced by the emissions that ran. Outputs may be NULL
 * when capacity is 0.
 */
bc_status bc_photon_map(bc_context* ctx, int32_t scene, const bc_settings* settings, int32_t capacity,
                        float* photons_out, int32_t* n_out, int64_t* rays_out);

/* ---- differentiable rendering ------------------------------------------ */

/*
 * Gradient of an image loss with respect to material parameters by path
 * replay: bc_backward re-traces the paths of the last bc_forward (same seed,
 * same random streams) and, once each path's radiance is known, adds for every
 * diffuse vertex on an albedo parameter d * (L_path - L_before) / albedo and
 * for every emitter hit on an emission parameter d * throughput * MIS weight,
 * d being dLoss/dImage of the path's pixel over spp. Russian roulette
 * probabilities are held fixed (set rr_depth >= bounces for the exact
 * derivative of the sample estimator). No reference counterpart: the
 * reference renders forward only (renderer.go:1484-1563).
 *
 * Parameters, in order: n_albedo albedo RGB triples (diffuse materials
 * albedo_materials[i]), then n_emission emission RGB triples (emissive
 * materials emission_materials[i], not used by sphere lights). At most 1024.
 * The view renders scene 0 of the resident set; settings->firefly_clamp must
 * be 0 and settings->bounces at most 64.
 */
typedef struct bc_diff_desc {
  bc_camera camera;
  bc_settings settings;
  int32_t n_albedo;
  const int32_t* albedo_materials;
  int32_t n_emission;
  const int32_t* emission_materials;
} bc_diff_desc;

bc_status bc_diff_configure(bc_context* ctx, const bc_diff_desc* desc);
/* Target image of the L2 loss, width*height RGB floats:
 * loss = sum over pixels and channels of (image - target)^2 / (3 * width * height). */
bc_status bc_diff_set_target(bc_context* ctx, const float* target);
/*
 * Writes `params` (3 * (n_albedo + n_emission) floats) into the resident
 * materials and renders the configured view with path seed `seed`.
 * image_out (may be NULL): width*height RGB mean radiance. loss_out (may be
 * NULL; needs a target): the L2 loss.
 */
bc_status bc_forward(bc_context* ctx, const float* params, uint64_t seed, float* image_out, double* loss_out);
/*
 * Gradient of the loss at the last bc_forward. dloss_dimage: width*height RGB
 * floats, or NULL for the L2 loss against the target. grad_albedo:
 * 3 * n_albedo floats, grad_emission: 3 * n_emission floats (either may be NULL).
 */
bc_status bc_backward(bc_context* ctx, const float* dloss_dimage, float* grad_albedo, float* grad_emission);

/*
 * The whole post stack of RenderState.Start (renderer.go:2838-2895) on caller
 * buffers, in Start's order: HBAO+ (hbao_plus > 0) or HBAO (applyHBAO,
 * 2433-2488), a-trous denoise (2 + min(3, max(taa, txaa)) passes), temporal
 * accumulation with the previous call's frame (temporalAccumulate, 2316-2364;
 * weight from max(taa, tsaa, txaa), 2419-2431; the history is kept by the
 * context when a temporal mode is on and dropped when none is), bloom, a debug
 * view (makeDebugView, 1972-2032), the basic upscaler to width x height
 * (bicubicUpscale + edgeAwareSharpen, 2081-2197; internalSize gives the render
 * size, 2066-2079), FXAA (2557-2587), the TXAA resolve (2589-2595) and tone
 * mapping to RGBA8. linear_in: render_width x render_height RGB floats;
 * guides_in: 12 floats per pixel (P xyz, depth, N xyz, valid 0/1, albedo xyz,
 * 0), required when HBAO, denoise, a temporal mode or a guide-based debug view
 * is on. linear_out (width x height RGB floats) and rgba_out may be NULL.
 */
typedef struct bc_post_desc {
  int32_t width, height;                /* output (RenderSettings.Width, Height) */
  int32_t render_width, render_height;  /* size of linear_in and guides_in */
  int32_t hbao, hbao_plus;
  int32_t denoise, taa, tsaa, txaa;
  int32_t bloom, fxaa;
  int32_t upscale;     /* 0 off, 1 ultra quality, 2 balanced, 3 performance */
  int32_t debug_view;  /* 0 beauty, 1 albedo, 2 normal, 3 depth, 4 AO, 5 heat */
  int32_t hdr, reserved;
  double exposure, gamma;
  bc_camera camera;    /* this frame's camera (the next call reprojects into it) */
} bc_post_desc;

bc_status bc_post_stack(bc_context* ctx, const bc_post_desc* desc, const float* linear_in, const float* guides_in,
                        float* linear_out, uint32_t* rgba_out);
/* Drops the temporal history (Start sets historyValid = false, e.g. on a new scene). */
bc_status bc_post_history_reset(bc_context* ctx);

/*
 * The post stack alone, on caller buffers (the part of RenderState.Start that
 * follows the render call, renderer.go:2844-2854 and 2890-2895): a-trous denoise
 * with `2 + min(3, max(taa, txaa))` passes when settings->denoise, bloom when
 * settings->bloom > 0, tone map to RGBA8. linear_in: width*height RGB floats;
 * guide_nd: width*height (nx, ny, nz, depth) floats with depth < 0 for pixels
 * without a first hit (may be NULL when denoise is off). Outputs may be NULL.
 */
bc_status bc_post_process(bc_context* ctx, int32_t width, int32_t height, const float* linear_in,
                          const float* guide_nd, const bc_settings* settings, float* linear_out, uint32_t* rgba_out);

/*
 * Allocation-free variant of bc_post_process. It has no counterpart in the
 * reference. It is for callers that cannot allocate device memory when they
 * post-process a frame: an engine or plugin host that owns the GPU memory
 * budget, an allocation-free real-time loop, or code that must not synchronise
 * the device (cudaMalloc and cudaFree can). It needs no context, takes device
 * pointers for every image (width*height RGB floats in and out, width*height
 * (nx, ny, nz, depth) guides, width*height RGBA8 words or NULL), enqueues on
 * `stream` (a cudaStream_t, NULL = legacy default) and returns once the work is
 * enqueued. It calls no cudaMalloc, cudaFree or allocating library routine.
 * Its scratch is a static device array of two images of at most 921,600 pixels
 * (22 MB), which every GPU that loads the library holds until the process
 * exits; larger frames are rejected with BC_ERR_INVALID_ARG, and so are
 * output buffers (linear or RGBA) that share any byte with each other or with
 * an input. Every call shares that array: calls that overlap on the
 * GPU (different streams, or devices sharing it across threads without
 * ordering) race on it. The first call on each device looks up the array's
 * device address (cudaGetSymbolAddress) with that device current; make that
 * first call before any stream capture. The address is kept for the life of
 * the process: do not call this entry point on a device after cudaDeviceReset
 * on it.
 */
bc_status bc_post_process_noalloc(int32_t width, int32_t height, const float* d_linear_in, const float* d_guide_nd,
                                  const bc_settings* settings, float* d_linear_out, uint32_t* d_rgba_out,
                                  void* stream);

/*
 * Tuning options of a context (no counterpart in the reference, whose OpenCL
 * path picks a work-group size once, gpu_opencl_windows.go:285-304):
 *   "raycast_split"      1 (default): the exact closest hit of a triangle-only
 *                        scene runs as passes: a walk with fp32 classification only
 *                        (twelve 128-thread blocks per SM), an fp64 settlement pass,
 *                        and a re-trace of the rays whose contender list overflowed;
 *                        it holds 52 bytes of device scratch per ray of a call (per
 *                        chunk for bc_raycast). The exact any hit likewise: a walk,
 *                        then fp64 tests of the undecided triangles of the rays
 *                        the walk could not decide (28 bytes per ray). 0: one
 *                        kernel walks and settles. Both give the same results.
 *   "raycast_minblocks"  1, 6 or 8: register budget of the one-kernel ray-cast
 *                        kernels (resident 128-thread blocks per SM the allocation
 *                        must allow).
 *   "raycast_exact"      1 (default): bc_raycast is exact as documented there;
 *                        0: plain fp32 closest hit, t = the fp32 distance, with no
 *                        exactness contract near edges and ties.
 *   "raycast_sort"       1 (default): batches of at least 65,536 rays are traced
 *                        in a spatially coherent order (origin Morton code on a
 *                        64^3 grid over the scene bounds, then direction octant);
 *                        results are returned in the caller's order either way.
 *   "photon_grid"        1 (default): photon gathers find a cell's photons in a
 *                        dense cell table built with the map; 0: by hash lookup.
 *                        Both give the same photons in the same order.
 *   "raycast_chunk"      rays per chunk of bc_raycast (host buffers),
 *                        65,536 .. 2^28 (default 2^21): chunks alternate
 *                        between two streams, so one chunk's copies overlap
 *                        another's kernel.
 *   "render_wave_cap"    paths in flight per wave of the renderer, 4096 .. 2^27
 *                        (default 2^27: ~160 bytes of device memory per path,
 *                        allocated up to what a render needs); images do not
 *                        depend on it. Each wave ends in a latency-bound tail of
 *                        long paths, so larger waves render faster.
 *   "render_graph"       1 (default): a render of several waves replays one
 *                        captured CUDA graph per wave, and a single-wave render
 *                        is captured when the same launches repeat (from the
 *                        second identical call on); 0: plain stream launches.
 *   "render_extend"      variant of the wave engine's closest-hit kernel; all
 *                        give the same hits. 0: ray in registers, no register
 *                        budget (nine 128-thread blocks per SM); 1 (default):
 *                        ray in registers, 48 registers (ten blocks); 2: ray
 *                        in shared memory, 40 registers (twelve blocks).
 *   "render_shade_block" 256 (default) or 128: threads per block of the wave
 *                        engine's shading kernel (four or eight blocks per SM, 64 registers).
 *   "render_timing"      0 (default); 1: the renders record an event before every
 *                        kernel launch (no captured graph) for bc_last_timing's
 *                        per-kernel times; images are the same.
 *   "scene_leaf_merge"   -1 (default): scenes of at most 1,024 primitives are
 *                        packed with merged BVH8 leaves (inner binary subtrees of
 *                        up to 8 primitives in one contiguous slot range become
 *                        one leaf where a surface-area cost with a triangle test
 *                        at 0.2 node visits favours it); 1: every scene; 0: the
 *                        BVH8 leaves are the binary tree's leaves. Applies to the
 *                        next scene upload; hits are the same either way.
 *   "render_engine"      0 (default): the wave engine; 1: one kernel launch per
 *                        view, one thread per pixel looping over samples and
 *                        bounces (the reference OpenCL kernel's shape, kept as the
 *                        measured baseline; gradient renders always use the wave engine).
 * Unknown names or values return BC_ERR_INVALID_ARG.
 */
bc_status bc_set_option(bc_context* ctx, const char* name, int64_t value);
bc_status bc_get_option(const bc_context* ctx, const char* name, int64_t* value);

/*
 * Autotuner: times the candidate values of the tuning options on the caller's
 * own work and keeps the fastest in the context (no counterpart in the
 * reference). Results never depend on the options: every candidate returns the
 * same hits and images.
 *
 * bc_autotune_raycast: device rays as for bc_raycast_device; candidates are
 * raycast_split 1 with raycast_sort 1 and 0, then raycast_split 0 with
 * raycast_minblocks 6, 8, 1 and raycast_sort 1 and 0 (exact mode; plain fp32
 * mode: raycast_sort only). Best of two timed runs each (CUDA events).
 * bc_autotune_render: the views as for bc_render_batch; first render_extend
 * 1, 0, 2 at the current wave size, then the other render_shade_block, then
 * render_wave_cap 2^22 .. 2^27 (up to twice the sample's paths) with the
 * chosen variants. Each view's spp is scaled
 * down so that a candidate traces at most 2^27 paths; the adaptive stop is off
 * while timing. The second of two runs is timed.
 */
typedef struct bc_tune_report {
  int32_t raycast_minblocks, raycast_sort;  /* options in force after the call */
  int64_t render_wave_cap;
  int32_t n_timed;                          /* candidates timed */
  int32_t render_extend;                    /* option in force after the call */
  double best_ms, default_ms, worst_ms;     /* chosen, the options before the call, slowest */
  int32_t raycast_split, render_shade_block; /* options in force after the call */
} bc_tune_report;
bc_status bc_autotune_raycast(bc_context* ctx, const float* d_rays, int64_t n, bc_tune_report* out);
bc_status bc_autotune_render(bc_context* ctx, const bc_view* views, int32_t n_views, bc_tune_report* out);

/*
 * Device time of the last render call of the context (bc_render_rows,
 * bc_render_frame, bc_render_moments, bc_render_batch, bc_forward,
 * bc_backward): CUDA events recorded on the context's stream before its first
 * and after its last device work (render, and the post stack for
 * bc_render_frame). With the option "render_timing" 1 the wave engine launches
 * without its captured graph and records an event before every kernel, and the
 * per-class fields give the device time between consecutive events, charged to
 * the kernel launched at the first of them. A photon-map build that a render
 * starts runs before its first event and is not counted. No reference counterpart (the
 * reference times whole renders on the host, benchmark.go:103-135).
 */
typedef struct bc_timing {
  double device_ms;         /* whole call */
  int64_t launches;         /* kernels the call launched */
  int64_t extend_launches;  /* of which closest-hit launches of the wave engine */
  int32_t kernel_timing;    /* 1: the per-class times below were measured */
  int32_t reserved;
  double generate_ms, extend_ms, shade_ms, connect_ms, accumulate_ms, post_ms, other_ms;
} bc_timing;
bc_status bc_last_timing(const bc_context* ctx, bc_timing* out);

/* Request cancellation of the running or next render of ctx; safe from any thread. */
bc_status bc_cancel(bc_context* ctx);
/* Clear a pending cancellation. */
bc_status bc_reset_cancel(bc_context* ctx);

#ifdef __cplusplus
}
#endif
#endif /* BC_GX_H */

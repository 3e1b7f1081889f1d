/*
 * bc_host_scene.h - host-side scene builder of the Beamcast GX hot path.
 *
 * The Go renderer builds its scene and BVH itself (Scene.AddSphere,
 * Scene.AddTriangle, Scene.Build; renderer.go:246-269, 409-449) and hands the
 * result to bc_scene_upload(). Callers without the Go renderer (C, C++,
 * Python) use this builder instead: it produces the same primitives, the same
 * binned-SAH (or median) tree with the same node numbering and the same
 * Scene.Order permutation, and the same light distribution, in fp64.
 * All functions are host-only and need no GPU.
 */
#ifndef BC_HOST_SCENE_H
#define BC_HOST_SCENE_H

#include <stdint.h>

#include "bc_gx.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bc_hscene bc_hscene;

bc_hscene* bc_hscene_create(void);
void bc_hscene_destroy(bc_hscene* s);

/* Scene.AddMaterial (renderer.go:242-245); returns the material index. */
int32_t bc_hscene_add_material(bc_hscene* s, int32_t kind, const double color[3], double roughness, double ior,
                               const double emission[3]);
/* Scene.AddSphere (renderer.go:246-256): ignored when r <= 0; emissive spheres become lights. */
void bc_hscene_add_sphere(bc_hscene* s, const double center[3], double radius, int32_t material);
/* Scene.AddTriangle (renderer.go:257-269) for n triangles: verts holds 9 doubles per
 * triangle (A, B, C); degenerate triangles (|E1 x E2|^2 < 1e-18) are dropped. */
void bc_hscene_add_triangles(bc_hscene* s, int64_t n, const double* verts, const int32_t* materials);
/* translatePrimitive (renderer.go:310-330) on primitive `index`. */
bc_status bc_hscene_translate_prim(bc_hscene* s, int32_t index, const double delta[3]);

/* BVHMode ("SAH" or "Median"), BVHBins and BVHLeafSize; clamped by Build as the reference does. */
void bc_hscene_set_bvh(bc_hscene* s, const char* mode, int32_t bins, int32_t leaf_size);
/* Scene.Build (renderer.go:409-449): light distribution, then the BVH. Bumps both revisions. */
bc_status bc_hscene_build(bc_hscene* s);
/* Scene.Build with the BVH built on the device (bc_build_sah): the same result as
 * bc_hscene_build in SAH mode; the Median mode is built on the host. */
bc_status bc_hscene_build_device(bc_hscene* s, bc_context* ctx);
/* Scene.Refit (renderer.go:451-473): bottom-up box refit; bumps the geometry revision. */
bc_status bc_hscene_refit(bc_hscene* s);

/* out: [0] primitives, [1] nodes, [2] lights, [3] materials, [4] topology rev, [5] geometry rev. */
void bc_hscene_counts(const bc_hscene* s, int64_t out[6]);
/* Fill a descriptor that points into the builder's arrays; valid until the next mutation. */
bc_status bc_hscene_describe(const bc_hscene* s, bc_scene_desc* out);

#ifdef __cplusplus
}
#endif
#endif /* BC_HOST_SCENE_H */

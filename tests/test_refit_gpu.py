"""Geometry-only scene updates (bc_scene_upload with the same scene id and
topology revision and a new geometry revision: primitives moved, node boxes
refit by Scene.Refit, renderer.go:451-473, as updateGeometryLocked expects,
gpu_opencl_windows.go:447-468).

The device rewrites the primitive slots and re-quantizes every BVH8 node from
the refit boxes, keeping the BVH8 topology. Checked: the exact ray cast after
the update equals the fp64 oracle on the same moved-and-refit scene (hit index
and t bit for bit); it equals a full upload of the moved scene; images equal a
full upload's (apart from fp32 distance ties, which the BVH8 shape may order
differently); sphere lights follow their spheres; a descriptor whose counts do
not match falls back to a full upload.
"""
import numpy as np
import pytest

from bcgx import scenes

pytestmark = pytest.mark.gpu


def _move(scene, orc_scene, idx, rng, scale):
    for i in idx:
        d = rng.normal(0.0, scale, 3)
        scene.translate_primitive(int(i), d)
        if orc_scene is not None:
            orc_scene.translate(int(i), d)
    scene.refit()
    if orc_scene is not None:
        orc_scene.refit()


def test_refit_update_is_exact(gpu_ctx, orc):
    spec = scenes.random_triangles(60_000, seed=0xBEAC0101)
    s = scenes.to_scene(spec)
    ref = orc.OracleScene.from_spec(spec)
    gpu_ctx.upload(s)
    before = gpu_ctx.scene_stats()["geometry_updates"]
    rng = np.random.default_rng(11)
    _move(s, ref, rng.choice(60_000, 600, replace=False), rng, 0.02)
    topo0, geom0 = s.revisions()
    gpu_ctx.upload(s)
    assert gpu_ctx.scene_stats()["geometry_updates"] == before + 1, "the device geometry path was not taken"
    rays = scenes.random_rays(65_536, seed=0xBEAC0102)
    t, p = gpu_ctx.raycast(rays)
    t_ref, p_ref, _ = ref.hit_f32(rays)
    assert np.array_equal(p, p_ref)
    hit = p >= 0
    assert np.array_equal(t[hit], t_ref[hit].astype(np.float32))
    # a full upload of the same moved scene (new scene id) gives the same answers
    gpu_ctx.upload(s, scene_id=0xF011)
    t2, p2 = gpu_ctx.raycast(rays)
    assert np.array_equal(p2, p) and np.array_equal(t2, t)
    assert gpu_ctx.scene_stats()["geometry_updates"] == before + 1


def test_refit_update_moves_lights_and_renders(gpu_ctx):
    spec, cam = scenes.cornell_reference_scene()
    s = scenes.to_scene(spec)
    gpu_ctx.upload(s)
    before = gpu_ctx.scene_stats()["geometry_updates"]
    n = s.counts()["prims"]
    rng = np.random.default_rng(3)
    _move(s, None, range(n), rng, 0.01)  # every primitive, sphere lights included
    gpu_ctx.upload(s)
    assert gpu_ctx.scene_stats()["geometry_updates"] == before + 1
    from bcgx import quality
    st = quality("Draft")
    st.width, st.height, st.spp, st.bounces = 96, 64, 8, 5
    st.denoise, st.bloom, st.adaptive_sampling = False, 0, False
    st.seed = 9
    a = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)
    gpu_ctx.upload(s, scene_id=0xF012)  # full upload of the moved scene
    b = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)
    same = np.all(a["linear"] == b["linear"], axis=-1).mean()
    assert same >= 0.999, same
    assert abs(a["rays"] - b["rays"]) <= 1e-3 * b["rays"]


def test_mismatched_descriptor_takes_the_full_path(gpu_ctx):
    spec = scenes.random_triangles(5000, seed=0xBEAC0103)
    s = scenes.to_scene(spec)
    gpu_ctx.upload(s, scene_id=77, topology_rev=1, geometry_rev=1)
    before = gpu_ctx.scene_stats()["geometry_updates"]
    other = scenes.to_scene(scenes.random_triangles(5001, seed=0xBEAC0104))
    # same id and topology revision but different counts: must not be applied in place
    gpu_ctx.upload(other, scene_id=77, topology_rev=1, geometry_rev=2)
    assert gpu_ctx.scene_stats()["geometry_updates"] == before
    assert gpu_ctx.scene_stats()["slots"] == 5001
    rays = scenes.random_rays(4096, seed=5)
    t, p = gpu_ctx.raycast(rays)
    assert (p < 5001).all()

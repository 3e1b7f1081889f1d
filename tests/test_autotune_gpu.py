"""The autotuner (bc_autotune_raycast, bc_autotune_render) on the GPU: it times
candidate option values on the caller's own work and keeps the fastest; no
candidate changes a result, so hits and images are the same before and after."""
import numpy as np
import pytest

import bcgx
from bcgx import scenes

pytestmark = pytest.mark.gpu


def test_autotune_raycast_keeps_results(gpu_ctx):
    import torch
    spec = scenes.random_triangles(100_000, seed=0xBEAC0201)
    gpu_ctx.upload(scenes.to_scene(spec))
    rays = scenes.random_rays(262_144, seed=0xBEAC0202)
    dev = torch.device("cuda", 0)
    r = torch.from_numpy(np.ascontiguousarray(rays)).to(dev)
    t0 = torch.empty(len(rays), dtype=torch.float32, device=dev)
    p0 = torch.empty(len(rays), dtype=torch.int32, device=dev)
    gpu_ctx.raycast_device(r.data_ptr(), len(rays), t0.data_ptr(), p0.data_ptr())
    torch.cuda.synchronize()
    try:
        rep = gpu_ctx.autotune_raycast(r.data_ptr(), len(rays))
        assert rep["n_timed"] == 8
        assert rep["raycast_minblocks"] in (1, 6, 8) and rep["raycast_sort"] in (0, 1)
        assert rep["raycast_split"] in (0, 1) and gpu_ctx.get_option("raycast_split") == rep["raycast_split"]
        assert 0 < rep["best_ms"] <= rep["default_ms"] <= rep["worst_ms"]
        assert gpu_ctx.get_option("raycast_minblocks") == rep["raycast_minblocks"]
        assert gpu_ctx.get_option("raycast_sort") == rep["raycast_sort"]
        t1 = torch.empty_like(t0)
        p1 = torch.empty_like(p0)
        gpu_ctx.raycast_device(r.data_ptr(), len(rays), t1.data_ptr(), p1.data_ptr())
        torch.cuda.synchronize()
        assert torch.equal(p0, p1) and torch.equal(t0, t1)
    finally:
        gpu_ctx.set_option("raycast_minblocks", 6)
        gpu_ctx.set_option("raycast_sort", 1)
        gpu_ctx.set_option("raycast_split", 1)


def test_autotune_render_keeps_images(gpu_ctx):
    spec, cam = scenes.cornell_reference_scene()
    gpu_ctx.upload_set([scenes.to_scene(spec)])
    st = bcgx.quality("Draft")
    st.width, st.height, st.spp, st.bounces, st.adaptive_sampling = 160, 120, 16, 5, False
    st2 = st.copy()
    st2.width, st2.height, st2.spp = 96, 64, 8
    views = [(0, cam, st), (0, cam, st2)]
    before, _ = gpu_ctx.render_batch(views)
    try:
        rep = gpu_ctx.autotune_render(views)
        assert rep["n_timed"] >= 4 and rep["render_wave_cap"] >= 1 << 22
        assert rep["render_extend"] in (0, 1, 2) and rep["render_shade_block"] in (128, 256)
        assert gpu_ctx.get_option("render_shade_block") == rep["render_shade_block"]
        assert 0 < rep["best_ms"] <= rep["worst_ms"] and rep["default_ms"] > 0
        assert gpu_ctx.get_option("render_wave_cap") == rep["render_wave_cap"]
        assert gpu_ctx.get_option("render_extend") == rep["render_extend"]
        after, _ = gpu_ctx.render_batch(views)
        assert all(np.array_equal(a, b) for a, b in zip(before, after))
    finally:
        gpu_ctx.set_option("render_wave_cap", 1 << 26)
        gpu_ctx.set_option("render_extend", 1)
        gpu_ctx.set_option("render_shade_block", 256)


@pytest.mark.parametrize("which", ["showcase", "batch_tris"])
def test_extend_variants_same_images(gpu_ctx, which):
    """The three closest-hit variants of the wave engine (register budget, ray in
    registers or shared memory) and the two block shapes of its shading kernel
    give bit-identical images and ray counts. Sphere scene and triangle-only scene."""
    if which == "showcase":
        spec, cam = scenes.showcase_scene()
        st = bcgx.quality("Draft")
        st.width, st.height, st.spp, st.bounces, st.adaptive_sampling = 128, 80, 6, 6, False
        gpu_ctx.upload_set([scenes.to_scene(spec)])
        views = [(0, cam, st)]
    else:
        specs, views = scenes.batch_views(n_views=4, sizes=(4000, 9000), max_side=(160, 90), spp_range=(2, 4))
        gpu_ctx.upload_set([scenes.to_scene(s) for s in specs])
    out = {}
    try:
        for var in (0, 1, 2):
            gpu_ctx.set_option("render_extend", var)
            assert gpu_ctx.get_option("render_extend") == var
            out[var] = gpu_ctx.render_batch(views)
        gpu_ctx.set_option("render_shade_block", 128)
        out["sb128"] = gpu_ctx.render_batch(views)
    finally:
        gpu_ctx.set_option("render_extend", 1)
        gpu_ctx.set_option("render_shade_block", 256)
    for var in (0, 2, "sb128"):
        imgs, rays = out[var]
        assert rays == out[1][1]
        assert all(np.array_equal(a, b) for a, b in zip(imgs, out[1][0]))
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):
        gpu_ctx.set_option("render_extend", 3)
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):
        gpu_ctx.set_option("render_shade_block", 64)


def test_autotune_argument_errors(gpu_ctx):
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):
        gpu_ctx.autotune_raycast(0, 16)
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):
        gpu_ctx.autotune_render([])

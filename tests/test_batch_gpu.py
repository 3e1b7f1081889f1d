"""Batched multi-view rendering (bc_scene_set_upload + bc_render_batch).

Every (pixel, sample) path draws from its own seeded stream and each pixel
adds its samples in sample order, so a view rendered inside a batch must be
bit-identical to the same view rendered alone, whatever the other views, the
wave capacity or the launch form (captured graph or plain stream launches).
The single-view renderer is checked against the fp64 oracle in
test_render_gpu.py; these tests tie the batch engine to it exactly.
"""
import numpy as np
import pytest

import bcgx
from bcgx import scenes

pytestmark = pytest.mark.gpu


def _settings(W, H, spp, bounces, seed, sampler="Halton", power=True, clamp=0.0):
    st = bcgx.quality("Draft")
    st.width, st.height, st.spp, st.bounces = W, H, spp, bounces
    st.msaa, st.tsaa = 1, 0
    st.sampler, st.mis, st.power_light_sampling = sampler, True, power
    st.firefly_clamp, st.rr_depth, st.adaptive_sampling = clamp, 3, False
    st.denoise, st.bloom = False, 0
    st.seed = seed
    return st


def _scene_mix():
    """Three scenes with different material tables and lights: sphere lights
    (NEE, power-weighted light choice) in two of them, so light, material and
    primitive offsets of the set are all exercised."""
    a, cam_a = scenes.cornell_reference_scene()
    b, cam_b, _ = scenes.cornell_box()
    c, cam_c = scenes.showcase_scene()
    return [a, b, c], [cam_a, cam_b, cam_c]


def _alone(ctx, spec, cam, st):
    ctx.upload(scenes.to_scene(spec))
    return ctx.render_frame(cam, st, want_guides=False, want_rgba=False)


def test_batch_equals_single_views(gpu_ctx):
    specs, cams = _scene_mix()
    built = [scenes.to_scene(s) for s in specs]
    views = [
        (0, cams[0], _settings(96, 64, 8, 6, 11)),
        (1, cams[1], _settings(80, 60, 12, 5, 12, sampler="R2")),
        (2, cams[2], _settings(120, 72, 5, 7, 13, sampler="Random", power=False, clamp=9.0)),
        (0, cams[0], _settings(33, 17, 3, 2, 14)),
        (2, cams[2], _settings(64, 64, 16, 4, 15)),
    ]
    alone = []
    for k, cam, st in views:
        gpu_ctx.upload(built[k])
        r = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)
        alone.append((r["linear"], r["rays"]))
    gpu_ctx.upload_set(built)
    outs, rays = gpu_ctx.render_batch(views)
    for v, (o, (ref, _)) in enumerate(zip(outs, alone)):
        assert o.shape == ref.shape
        assert np.array_equal(o, ref), f"view {v}: batch differs from the view rendered alone"
    assert rays == sum(r for _, r in alone)


@pytest.mark.parametrize("cap,graph", [(4096, 1), (4096, 0), (50_000, 1)])
def test_batch_independent_of_wave_split(gpu_ctx, cap, graph):
    specs, cams = _scene_mix()
    built = [scenes.to_scene(s) for s in specs]
    views = [(k % 3, cams[k % 3], _settings(40 + 8 * k, 30 + 4 * k, 4 + k, 5, 100 + k)) for k in range(7)]
    gpu_ctx.upload_set(built)
    ref, rays_ref = gpu_ctx.render_batch(views)
    old_cap, old_graph = gpu_ctx.get_option("render_wave_cap"), gpu_ctx.get_option("render_graph")
    try:
        gpu_ctx.set_option("render_wave_cap", cap)
        gpu_ctx.set_option("render_graph", graph)
        outs, rays = gpu_ctx.render_batch(views)
    finally:
        gpu_ctx.set_option("render_wave_cap", old_cap)
        gpu_ctx.set_option("render_graph", old_graph)
    assert rays == rays_ref
    for v in range(len(views)):
        assert np.array_equal(outs[v], ref[v]), f"view {v} depends on the wave split"


def test_wave_graph_reuse_across_batch_shapes(gpu_ctx):
    """A captured wave is replayed by later calls: calls that differ in view
    count, sample-table size and frame size must still match plain launches."""
    specs, cams = _scene_mix()
    gpu_ctx.upload_set([scenes.to_scene(s) for s in specs])
    calls = [
        [(k % 3, cams[k % 3], _settings(48 + 4 * k, 40, 6 + 2 * k, 5, 300 + k)) for k in range(6)],
        [(1, cams[1], _settings(90, 70, 9, 5, 400))],
        [(2, cams[2], _settings(64, 48, 17, 5, 401)), (0, cams[0], _settings(30, 20, 2, 5, 402))],
        [(0, cams[0], _settings(100, 80, 5, 5, 403, sampler="Random"))],
    ]
    old_cap, old_graph = gpu_ctx.get_option("render_wave_cap"), gpu_ctx.get_option("render_graph")
    try:
        gpu_ctx.set_option("render_wave_cap", 4096)
        got = []
        gpu_ctx.set_option("render_graph", 1)
        for views in calls:
            got.append(gpu_ctx.render_batch(views))
        gpu_ctx.set_option("render_graph", 0)
        for c, views in enumerate(calls):
            ref, rays = gpu_ctx.render_batch(views)
            assert got[c][1] == rays, f"call {c}: ray count differs under graph replay"
            for v in range(len(views)):
                assert np.array_equal(got[c][0][v], ref[v]), f"call {c} view {v} differs under graph replay"
    finally:
        gpu_ctx.set_option("render_wave_cap", old_cap)
        gpu_ctx.set_option("render_graph", old_graph)


def test_single_frame_independent_of_wave_split(gpu_ctx):
    spec, cam, st = scenes.cornell_box()
    st = st.copy()
    st.width, st.height, st.spp = 160, 120, 24
    st.denoise, st.bloom = False, 0
    gpu_ctx.upload(scenes.to_scene(spec))
    ref = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)
    old = gpu_ctx.get_option("render_wave_cap")
    try:
        gpu_ctx.set_option("render_wave_cap", 7000)  # not a multiple of the frame: waves split samples
        out = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)
    finally:
        gpu_ctx.set_option("render_wave_cap", old)
    assert np.array_equal(out["linear"], ref["linear"])
    assert out["rays"] == ref["rays"]


def test_batch_small_workload_matches_single(gpu_ctx):
    """A scaled-down batching workload (4 scenes, 8 views) through both forms."""
    specs, views = scenes.batch_views(n_views=8, sizes=(2000, 4000, 8000, 16000), max_side=(192, 108),
                                      spp_range=(2, 6))
    built = [scenes.to_scene(s) for s in specs]
    gpu_ctx.upload_set(built)
    batch, rays_b = gpu_ctx.render_batch(views)
    plain_rays = 0
    for v, view in enumerate(views):
        out, r = gpu_ctx.render_batch([view])
        plain_rays += r
        assert np.array_equal(out[0], batch[v])
    assert plain_rays == rays_b
    for o in batch:
        assert np.isfinite(o).all() and o.mean() > 0


def test_batch_argument_errors(gpu_ctx):
    specs, cams = _scene_mix()
    gpu_ctx.upload_set([scenes.to_scene(s) for s in specs[:2]])
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):
        gpu_ctx.render_batch([(2, cams[0], _settings(16, 16, 1, 1, 1))])
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):
        gpu_ctx.render_batch([(0, cams[0], _settings(0, 16, 1, 1, 1))])
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):
        gpu_ctx.set_option("render_wave_cap", 100)
    # single-view calls see scene 0 of the set
    st = _settings(48, 32, 4, 3, 5)
    a = gpu_ctx.render_frame(cams[0], st, want_guides=False, want_rgba=False)["linear"]
    b, _ = gpu_ctx.render_batch([(0, cams[0], st)])
    assert np.array_equal(a, b[0])

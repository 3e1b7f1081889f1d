"""The recursive and photon-mapping integrators (renderer.go:1565-1831) on the
GPU against the fp64 oracle's restatement.

* Photon map (buildPhotonMap): emission k draws from stream (seed, k) on both
  sides, so the GPU's photon list, in append order, replays the oracle's
  emission by emission; an emission's path can split only at an fp32-vs-fp64
  boundary decision. Checked: the photon counts, the per-emission deposits and
  the photons themselves (position, normal, flux) for the emissions that match.
* Images: z-tests of 2x2 pixel blocks at 256 spp against the oracle (zstats.py), and common random
  numbers (same seed): the recursive integrator draws its light samples after
  the subtree below each vertex, as the reference's recursion does, and the
  GPU defers them in the same order, so CRN replays hold for it too.
"""
import numpy as np
import pytest

import bcgx
from bcgx import scenes
from zstats import assert_parity

pytestmark = pytest.mark.gpu

RECURSIVE, PHOTON = bcgx.INTEGRATOR_RECURSIVE, bcgx.INTEGRATOR_PHOTON


def _settings(integrator, w=96, h=64, spp=8, bounces=5, level=1, sampler="Halton", seed=42):
    st = bcgx.quality("Draft")
    st.width, st.height, st.spp, st.bounces = w, h, spp, bounces
    st.sampler, st.mis, st.power_light_sampling = sampler, True, True
    st.firefly_clamp, st.rr_depth, st.adaptive_sampling = 0.0, 3, False
    st.integrator, st.photon_mapping, st.seed = integrator, level, seed
    return st


@pytest.fixture(scope="module")
def cornell(orc):
    spec, cam = scenes.cornell_reference_scene()
    return spec, cam, orc.OracleScene.from_spec(spec)


@pytest.mark.parametrize("level", [1, 2])
def test_photon_map_replays_the_oracle(gpu_ctx, cornell, level):
    spec, cam, ref = cornell
    gpu_ctx.upload(scenes.to_scene(spec))
    st = _settings(PHOTON, level=level, bounces=6, seed=9)
    g = gpu_ctx.photon_map(st)
    c = ref.photon_map(st, seed=9)
    budget = {1: 512, 2: 2048}[level]
    pg, pc = g["photons"].astype(np.float64), c["photons"]
    assert len(pc) >= budget and len(pc) < budget + max(2, st.bounces)
    assert abs(len(pg) - len(pc)) <= max(2, st.bounces)
    assert abs(g["rays"] - c["rays"]) <= 0.02 * c["rays"]
    # group by emission: equal deposit counts for nearly every emission
    eg = pg[:, 9].astype(np.int64)
    ec = pc[:, 9].astype(np.int64)
    k = min(eg.max(), ec.max())
    cg = np.bincount(eg, minlength=k + 1)[:k + 1]
    cc = np.bincount(ec, minlength=k + 1)[:k + 1]
    same = cg == cc
    assert same.mean() > 0.98, f"{same.mean():.4f} of emissions deposit alike"
    # the photons of the first deposit of every emission that deposits alike
    first_g = np.searchsorted(eg, np.arange(k + 1))
    first_c = np.searchsorted(ec, np.arange(k + 1))
    sel = np.nonzero(same & (cc > 0))[0]
    a, b = pg[first_g[sel]], pc[first_c[sel]]
    scale = np.abs(pc[:, 0:3]).max()
    pos_ok = np.all(np.abs(a[:, 0:3] - b[:, 0:3]) <= 1e-4 * scale, axis=1)
    nrm_ok = np.all(np.abs(a[:, 3:6] - b[:, 3:6]) <= 1e-4, axis=1)
    flux_ok = np.all(np.abs(a[:, 6:9] - b[:, 6:9]) <= 1e-4 * (1 + np.abs(b[:, 6:9])), axis=1)
    assert pos_ok.mean() > 0.99 and nrm_ok.mean() > 0.99 and flux_ok.mean() > 0.99


def test_photon_map_empty_cases(gpu_ctx, cornell):
    spec, cam, ref = cornell
    gpu_ctx.upload(scenes.to_scene(spec))
    for level in (0, 5, -1):  # photonBudget is 0 outside levels 1-4
        g = gpu_ctx.photon_map(_settings(PHOTON, level=level))
        assert len(g["photons"]) == 0 and g["rays"] == 0
    # a scene without sphere lights has no photon map (the c1 Cornell box lights with a quad)
    spec1, _, _ = scenes.cornell_box()
    gpu_ctx.upload(scenes.to_scene(spec1))
    g = gpu_ctx.photon_map(_settings(PHOTON, level=2))
    assert len(g["photons"]) == 0


@pytest.mark.parametrize("integrator", [RECURSIVE, PHOTON])
def test_common_random_numbers(gpu_ctx, cornell, integrator):
    spec, cam, ref = cornell
    gpu_ctx.upload(scenes.to_scene(spec))
    st = _settings(integrator, spp=8, bounces=6, seed=42)
    m_g, _, rays = gpu_ctx.render_moments(cam, st)
    out = ref.render(cam, st, seed=42, threads=0)
    m_c = out["linear"]
    close = np.all(np.abs(m_g - m_c) <= 2e-3 * (1 + np.abs(m_c)), axis=2)
    assert close.mean() > 0.95, f"only {close.mean():.4f} of pixels replay the CPU paths"
    segs = out["stats"]["segments"] + out["stats"]["photon_rays"]
    assert abs(rays - segs) <= 0.01 * segs


@pytest.mark.parametrize("integrator,which", [(RECURSIVE, "cornell_ref"), (RECURSIVE, "showcase"),
                                              (PHOTON, "cornell_ref"), (PHOTON, "showcase")])
def test_statistical_parity(gpu_ctx, orc, integrator, which):
    spec, cam = {"cornell_ref": scenes.cornell_reference_scene, "showcase": scenes.showcase_scene}[which]()
    gpu_ctx.upload(scenes.to_scene(spec))
    st = _settings(integrator, w=128, h=80, spp=256, bounces=6, level=2, seed=5)
    m_g, q_g, _ = gpu_ctx.render_moments(cam, st)
    # independent pixel samples (seed 6) over the same photon map (emission seed 5):
    # a photon map is one draw for the whole frame, so the pixels' sample
    # variance does not cover a difference of maps
    out = orc.OracleScene.from_spec(spec).render(cam, st, seed=6, threads=0, photon_seed=5)
    assert_parity(f"{integrator} {which}", m_g, q_g, st.spp, out["linear"], out["sumsq"], st.spp)


def test_research_integrators_smoke(gpu_ctx):
    """TestResearchIntegrators (renderer_test.go:236-268): Cornell, Draft 32x24,
    1 spp, 3 bounces, each integrator renders a full frame."""
    spec, cam = scenes.cornell_reference_scene()
    gpu_ctx.upload(scenes.to_scene(spec))
    for integ in (bcgx.INTEGRATOR_PATH, RECURSIVE, PHOTON):
        st = bcgx.quality("Draft")
        st.width, st.height, st.spp, st.bounces, st.denoise = 32, 24, 1, 3, False
        st.integrator = integ
        if integ == PHOTON:
            st.photon_mapping = 1
        r = gpu_ctx.render_frame(cam, st)
        lin, rgba, rays = r["linear"], r["rgba"], r["rays"]
        assert lin.shape == (24, 32, 3) and rgba.shape == (24, 32)
        assert np.all(np.isfinite(lin)) and lin.min() >= 0 and lin.max() > 0 and rays > 0


def test_chunks_batches_and_engines(gpu_ctx):
    """Row chunks share the frame's photon map; a view inside a batch equals the
    view alone; the one-kernel form renders the photon integrator and rejects
    the recursive one; the recursive integrator's wave capacity changes nothing."""
    spec, cam = scenes.cornell_reference_scene()
    gpu_ctx.upload(scenes.to_scene(spec))
    st_p = _settings(PHOTON, w=80, h=48, spp=4, bounces=5, level=2, seed=3)
    st_r = _settings(RECURSIVE, w=64, h=40, spp=4, bounces=5, seed=4)
    full_p = gpu_ctx.render_frame(cam, st_p, want_guides=False, want_rgba=False)["linear"]
    rows = [gpu_ctx.render_rows(cam, st_p, y0, 16)[0] for y0 in (0, 16, 32)]
    assert np.array_equal(np.concatenate(rows, axis=0), full_p)
    full_r = gpu_ctx.render_frame(cam, st_r, want_guides=False, want_rgba=False)["linear"]
    st_path = _settings(bcgx.INTEGRATOR_PATH, w=48, h=32, spp=4, bounces=5, seed=7)
    full_path = gpu_ctx.render_frame(cam, st_path, want_guides=False, want_rgba=False)["linear"]
    outs, _ = gpu_ctx.render_batch([(0, cam, st_r), (0, cam, st_path), (0, cam, st_p)])
    assert np.array_equal(outs[0], full_r) and np.array_equal(outs[1], full_path) and np.array_equal(outs[2], full_p)
    for cap in (4096, 50_000):
        gpu_ctx.set_option("render_wave_cap", cap)
        try:
            small = gpu_ctx.render_frame(cam, st_r, want_guides=False, want_rgba=False)["linear"]
        finally:
            gpu_ctx.set_option("render_wave_cap", 1 << 26)
        assert np.array_equal(small, full_r)
    gpu_ctx.set_option("render_engine", 1)
    try:
        plain_p = gpu_ctx.render_frame(cam, st_p, want_guides=False, want_rgba=False)["linear"]
        with pytest.raises(bcgx.BCError, match="INVALID_ARG"):
            gpu_ctx.render_frame(cam, st_r)
    finally:
        gpu_ctx.set_option("render_engine", 0)
    # the one-kernel form draws the same numbers; fp32 contraction may differ per kernel
    close = np.all(np.abs(plain_p - full_p) <= 2e-3 * (1 + np.abs(full_p)), axis=2)
    assert close.mean() > 0.97


def test_integrator_argument_errors(gpu_ctx):
    spec, cam = scenes.cornell_reference_scene()
    gpu_ctx.upload(scenes.to_scene(spec))
    st = _settings(bcgx.INTEGRATOR_PATH)
    sc = st.c()
    sc.integrator = 7
    import ctypes as C
    out = np.zeros((st.height, st.width, 3), np.float32)
    rc = bcgx.lib().bc_render_rows(gpu_ctx.handle, C.byref(cam.c()), C.byref(sc), 0, st.height,
                                   out.ctypes.data_as(C.POINTER(C.c_float)), None, None)
    assert rc == 7  # BC_ERR_INVALID_ARG
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):
        gpu_ctx.photon_map(st, scene=3)


def test_batch_with_more_photon_maps_than_the_cache_holds(gpu_ctx):
    """20 photon views with 20 seeds need 20 maps in one call (the cache keeps 16
    between calls): the maps of the call are never evicted under it, and every
    view equals the same view rendered alone."""
    spec, cam = scenes.cornell_reference_scene()
    gpu_ctx.upload(scenes.to_scene(spec))
    views = [(0, cam, _settings(PHOTON, w=32, h=24, spp=2, bounces=4, level=1, seed=500 + k)) for k in range(20)]
    outs, _ = gpu_ctx.render_batch(views)
    outs2, _ = gpu_ctx.render_batch(views[::-1])  # the same maps again, in another order
    for k, (_, c, st) in enumerate(views):
        alone = gpu_ctx.render_frame(c, st, want_guides=False, want_rgba=False)["linear"]
        assert np.array_equal(outs[k], alone), k
        assert np.array_equal(outs2[19 - k], alone), k


def test_photon_maps_of_a_scene_set(gpu_ctx):
    """Views of two resident scenes at two photon levels in one batch: each view
    uses its own scene's map (radius from its own bounds) and equals the view alone."""
    a, cam_a = scenes.cornell_reference_scene()
    b, cam_b = scenes.showcase_scene()
    gpu_ctx.upload_set([scenes.to_scene(a), scenes.to_scene(b)])
    va = (0, cam_a, _settings(PHOTON, w=48, h=32, spp=2, bounces=4, level=1, seed=61))
    vb = (1, cam_b, _settings(PHOTON, w=40, h=30, spp=2, bounces=4, level=2, seed=62))
    outs, _ = gpu_ctx.render_batch([va, vb])
    (oa,), _ = gpu_ctx.render_batch([va])
    (ob,), _ = gpu_ctx.render_batch([vb])
    assert np.array_equal(outs[0], oa) and np.array_equal(outs[1], ob)
    ma = gpu_ctx.photon_map(va[2], scene=0)["photons"]
    mb = gpu_ctx.photon_map(vb[2], scene=1)["photons"]
    assert 512 <= len(ma) < 512 + 4 and 2048 <= len(mb) < 2048 + 4


def test_photon_map_follows_a_geometry_update(gpu_ctx):
    """A geometry-only update (moved primitives, refit boxes) drops the cached
    photon map: the next photon frame equals a fresh upload of the moved scene."""
    spec, cam = scenes.cornell_reference_scene()
    s = scenes.to_scene(spec)
    gpu_ctx.upload(s)
    st = _settings(PHOTON, w=64, h=48, spp=4, bounces=5, level=2, seed=71)
    before = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)["linear"]
    map_before = gpu_ctx.photon_map(st)["photons"]
    updates = gpu_ctx.scene_stats()["geometry_updates"]
    rng = np.random.default_rng(4)
    for i in range(s.counts()["prims"]):
        s.translate_primitive(int(i), tuple(rng.uniform(-0.05, 0.05, 3)))
    s.refit()
    gpu_ctx.upload(s)
    assert gpu_ctx.scene_stats()["geometry_updates"] == updates + 1
    moved = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)["linear"]
    map_moved = gpu_ctx.photon_map(st)["photons"]
    gpu_ctx.upload(s, scene_id=0xF0F0)  # full upload of the moved scene
    fresh = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)["linear"]
    map_fresh = gpu_ctx.photon_map(st)["photons"]
    assert not np.array_equal(map_before[:, 0:3], map_moved[:, 0:3][:len(map_before)])
    # emission by emission, the rebuilt map equals the fresh upload's (a re-quantized
    # node box may turn an fp32 traversal decision and split one emission's path)
    assert abs(len(map_moved) - len(map_fresh)) < max(2, st.bounces)
    em, ef = map_moved[:, 9].astype(np.int64), map_fresh[:, 9].astype(np.int64)
    k = int(min(em.max(), ef.max()))
    same = 0
    for e in range(k + 1):
        a_, b_ = map_moved[em == e], map_fresh[ef == e]
        same += int(a_.shape == b_.shape and (a_.size == 0 or np.abs(a_ - b_).max() <= 1e-5))
    assert same >= 0.98 * (k + 1), same / (k + 1)
    assert np.all(moved == fresh, axis=-1).mean() >= 0.99
    assert not np.array_equal(before, moved)


def test_recursive_with_adaptive_stop(gpu_ctx, cornell):
    """adaptivePixel's early stop (renderer.go:1957-1968) over recursive samples:
    CRN against the oracle with the stop on."""
    spec, cam, ref = cornell
    gpu_ctx.upload(scenes.to_scene(spec))
    st = _settings(RECURSIVE, spp=32, bounces=5, seed=81)
    st.adaptive_sampling, st.adaptive_threshold = True, 0.002
    m_g, _, _ = gpu_ctx.render_moments(cam, st)
    m_c = ref.render(cam, st, seed=81, threads=0)["linear"]
    close = np.all(np.abs(m_g - m_c) <= 2e-3 * (1 + np.abs(m_c)), axis=2)
    assert close.mean() > 0.95, f"only {close.mean():.4f} of pixels replay the CPU paths"


def test_dense_photon_table_equals_hash_lookups(gpu_ctx):
    """Gathers through the dense cell table and through the hash table visit the
    same photons in the same order: bit-identical photon renders at every level."""
    spec, cam = scenes.cornell_reference_scene()
    gpu_ctx.upload(scenes.to_scene(spec))
    for level in (1, 2, 3, 4):
        st = _settings(PHOTON, w=64, h=48, spp=4, bounces=5, level=level, seed=90 + level)
        dense = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)["linear"]
        gpu_ctx.set_option("photon_grid", 0)
        try:
            hashed = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)["linear"]
        finally:
            gpu_ctx.set_option("photon_grid", 1)
        assert np.array_equal(dense, hashed), level

"""Adaptive sampling on the GPU (adaptivePixel's early stop, renderer.go:1928-1970).

A pixel stops after sample n (n even, n >= min(8, spp)) once the population
variance of its sample luminance falls below max(1e-8, AdaptiveThreshold); its
value is then the mean of the n samples taken.

* With a threshold no pixel can miss, every pixel stops at min(8, spp), and the
  image must equal, bit for bit, the non-adaptive render at 8 spp (same
  streams, same summation order), for both render forms.
* Against the fp64 oracle with the same seed (common random numbers), an
  adaptive render agrees on most pixels; stop decisions taken on fp32 vs fp64
  luminance can differ on borderline pixels only.
"""
import numpy as np
import pytest

import bcgx
from bcgx import scenes

pytestmark = pytest.mark.gpu


def _settings(spp, adaptive, thr, seed=31):
    spec, cam, st = scenes.cornell_box()
    st = st.copy()
    st.width, st.height, st.spp = 96, 72, spp
    st.adaptive_sampling, st.adaptive_threshold = adaptive, thr
    st.denoise, st.bloom = False, 0
    st.seed = seed
    return spec, cam, st


@pytest.mark.parametrize("engine", [0, 1])
def test_everything_stops_at_min_samples(gpu_ctx, engine):
    spec, cam, st = _settings(32, True, 1e9)
    gpu_ctx.upload(scenes.to_scene(spec))
    ref_st = st.copy()
    ref_st.spp, ref_st.adaptive_sampling = 8, False
    old = gpu_ctx.get_option("render_engine")
    try:
        gpu_ctx.set_option("render_engine", engine)
        a = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)
        b = gpu_ctx.render_frame(cam, ref_st, want_guides=False, want_rgba=False)
    finally:
        gpu_ctx.set_option("render_engine", old)
    assert np.array_equal(a["linear"], b["linear"])
    if engine == 1:  # the one-kernel form traces only the samples it takes
        assert a["rays"] == b["rays"]


def test_adaptive_matches_oracle_with_common_random_numbers(gpu_ctx, orc):
    spec, cam, st = _settings(64, True, 2e-3, seed=77)
    gpu_ctx.upload(scenes.to_scene(spec))
    g = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)["linear"].astype(np.float64)
    out = orc.OracleScene.from_spec(spec).render(cam, st, seed=77, threads=0)
    c = out["linear"]
    close = np.all(np.abs(g - c) <= 2e-3 * np.maximum(np.abs(c), 1e-3) + 1e-4, axis=-1)
    assert close.mean() > 0.95, f"{close.mean():.4f} of pixels agree"
    assert abs(g.mean() - c.mean()) <= 0.01 * c.mean()
    # the stop saves work: fewer segments than the full 64 spp
    full = st.copy()
    full.adaptive_sampling = False
    old = gpu_ctx.get_option("render_engine")
    try:
        gpu_ctx.set_option("render_engine", 1)
        r_adapt = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)["rays"]
        r_full = gpu_ctx.render_frame(cam, full, want_guides=False, want_rgba=False)["rays"]
    finally:
        gpu_ctx.set_option("render_engine", old)
    assert r_adapt < r_full
    assert abs(r_adapt - out["stats"]["segments"]) <= 0.02 * out["stats"]["segments"]


def test_adaptive_forms_agree(gpu_ctx):
    spec, cam, st = _settings(48, True, 5e-3, seed=5)
    gpu_ctx.upload(scenes.to_scene(spec))
    old = gpu_ctx.get_option("render_engine")
    try:
        imgs = []
        for eng in (0, 1):
            gpu_ctx.set_option("render_engine", eng)
            imgs.append(gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)["linear"])
    finally:
        gpu_ctx.set_option("render_engine", old)
    same = np.all(imgs[0] == imgs[1], axis=-1).mean()
    assert same >= 0.9, same
    assert abs(float(imgs[0].mean()) - float(imgs[1].mean())) <= 5e-3 * float(imgs[1].mean())

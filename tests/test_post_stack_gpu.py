"""The whole post stack of RenderState.Start on the GPU (bc_post_stack) against
the fp64 oracle's restatement of the same passes in the same order
(renderer.go:2838-2895): HBAO / HBAO+, a-trous denoise, temporal
accumulation with the previous frame, bloom, debug views, the basic upscaler,
FXAA, TXAA resolve. Inputs: an oracle render of the reference's Cornell scene
and its first-hit guides (P, N, albedo, depth, valid).

The GPU runs in fp32. Passes with thresholds (FXAA's contrast test, HBAO's depth
tolerance, the temporal pass's reprojection rounding and acceptance tests) may
decide differently on a pixel sitting on a threshold, so the bound is: at most
0.5% of pixels off by more than 1e-3 relative, and a small mean error.
"""
import numpy as np
import pytest

import bcgx
from bcgx import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def frames(orc):
    spec, cam = scenes.cornell_reference_scene()
    ref = orc.OracleScene.from_spec(spec)
    st = bcgx.quality("Draft")
    st.width, st.height, st.spp, st.bounces = 96, 64, 4, 4
    st.sampler, st.adaptive_sampling, st.firefly_clamp = "Halton", False, 0.0
    out = []
    cams = [cam, bcgx.Camera(tuple(np.add(cam.position, (0.03, 0.0, 0.01))), cam.target, cam.up, cam.fov)]
    for c in cams:
        r = ref.render(c, st, seed=3, threads=0)
        out.append((r["linear"], r["guides"], c))
    return out


def _g12(g11):
    g = np.zeros(g11.shape[:2] + (12,), np.float32)
    g[..., 0:3] = g11[..., 0:3]
    g[..., 3] = g11[..., 9]
    g[..., 4:7] = g11[..., 3:6]
    g[..., 7] = g11[..., 10]
    g[..., 8:11] = g11[..., 6:9]
    return g


def _close(gpu, cpu, frac=5e-3, mean=2e-4):
    gpu = gpu.astype(np.float64)
    assert gpu.shape == cpu.shape
    off = np.abs(gpu - cpu) > 1e-3 * (1.0 + np.abs(cpu))
    bad = np.any(off, axis=-1).mean()
    err = np.abs(gpu - cpu).mean() / max(1e-6, np.abs(cpu).mean())
    assert bad <= frac and err <= mean, f"{bad:.4%} of pixels off, mean relative error {err:.2e}"


CASES = [
    dict(hbao=2), dict(hbao_plus=1), dict(hbao=3, hbao_plus=2),
    dict(fxaa=1), dict(fxaa=2), dict(fxaa=3), dict(txaa=1), dict(txaa=2),
    dict(denoise=1, taa=1), dict(bloom=1), dict(bloom=2),
    dict(debug_view=1), dict(debug_view=2), dict(debug_view=3), dict(debug_view=4, hbao=2), dict(debug_view=5),
]


@pytest.mark.parametrize("lv", CASES, ids=lambda d: ",".join(f"{k}={v}" for k, v in d.items()))
def test_single_frame_passes(gpu_ctx, orc, frames, lv):
    lin, g11, cam = frames[0]
    H, W = lin.shape[:2]
    cpu, _ = orc.post_stack(lin, g11, W, H, None, cam, **lv)
    gpu_ctx.post_history_reset()  # an independent frame: no history
    gpu, rgba = gpu_ctx.post_stack(lin, _g12(g11), cam, W, H, **lv)
    _close(gpu, cpu)
    assert rgba is not None and rgba.shape == (H, W)


@pytest.mark.parametrize("mode", [1, 2, 3])
def test_upscale(gpu_ctx, orc, frames, mode):
    lin, g11, cam = frames[0]
    H, W = 70, 97  # output size; the render size comes from internalSize
    rw, rh = orc.internal_size(W, H, mode)
    src = lin[:rh, :rw] if lin.shape[0] >= rh and lin.shape[1] >= rw else None
    if src is None:
        pytest.skip("frame smaller than the render size")
    src = np.ascontiguousarray(src)
    gs = np.ascontiguousarray(g11[:rh, :rw])
    cpu, _ = orc.post_stack(src, gs, W, H, None, cam, upscale=mode, fxaa=1)
    gpu_ctx.post_history_reset()
    gpu, _ = gpu_ctx.post_stack(src, _g12(gs), cam, W, H, upscale=mode, fxaa=1)
    _close(gpu, cpu)


def test_temporal_two_frames(gpu_ctx, orc, frames):
    (lin0, g0, cam0), (lin1, g1, cam1) = frames
    H, W = lin0.shape[:2]
    lv = dict(taa=2, denoise=1, bloom=1)
    # frame 0 has no history; frame 1 reprojects into frame 0
    cpu0, hist = orc.post_stack(lin0, g0, W, H, None, cam0, **lv)
    gpu_ctx.post_history_reset()
    gpu0, _ = gpu_ctx.post_stack(lin0, _g12(g0), cam0, W, H, **lv)
    _close(gpu0, cpu0)
    cpu1, _ = orc.post_stack(lin1, g1, W, H, hist, cam1, **lv)
    gpu1, _ = gpu_ctx.post_stack(lin1, _g12(g1), cam1, W, H, **lv)
    _close(gpu1, cpu1, frac=1e-2)
    # the history changed the frame (some pixels were blended)
    plain, _ = orc.post_stack(lin1, g1, W, H, None, cam1, **lv)
    assert np.abs(cpu1 - plain).max() > 1e-6


def test_full_stack(gpu_ctx, orc, frames):
    lin, g11, cam = frames[0]
    H, W = lin.shape[:2]
    lv = dict(hbao_plus=2, denoise=1, txaa=1, bloom=1, fxaa=1)
    cpu, _ = orc.post_stack(lin, g11, W, H, None, cam, **lv)
    gpu_ctx.post_history_reset()
    gpu, rgba = gpu_ctx.post_stack(lin, _g12(g11), cam, W, H, **lv)
    _close(gpu, cpu, frac=1e-2)
    ref_rgba = np.asarray(orc.to_rgba(cpu, 0.0, 2.2, 2), dtype=np.uint32).reshape(H, W)
    diff = np.abs(rgba.view(np.uint8).astype(np.int32) - ref_rgba.view(np.uint8).astype(np.int32))
    assert np.mean(diff.reshape(H, W, 4).max(axis=-1) > 1) < 0.01


def test_post_stack_argument_errors(gpu_ctx, frames):
    lin, g11, cam = frames[0]
    H, W = lin.shape[:2]
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):  # HBAO without guides
        gpu_ctx.post_stack(lin, None, cam, W, H, hbao=1)
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):  # size change without an upscaler
        gpu_ctx.post_stack(lin, _g12(g11), cam, W + 1, H)

"""Wavefront renderer parity on the GPU through the C-ABI.

* Statistical: means of 2x2 pixel blocks within 3 sigma of the combined Monte
  Carlo standard error of the fp64 CPU integrator and the GPU at equal spp, on
  the same BVH, at 256 spp so that block means are close to Gaussian: at most
  0.27% of (block, channel) pairs beyond 3 sigma plus four binomial standard
  deviations (zstats.py), and a global z-test on the image mean.
* Common random numbers: with the same seed the GPU and the oracle draw the
  same PCG32 numbers in the same order, so almost every pixel matches closely;
  only fp32-vs-fp64 boundary decisions can split a path.
"""

import numpy as np
import pytest

import bcgx
from bcgx import scenes
from zstats import assert_parity

pytestmark = pytest.mark.gpu


def _render_both(ctx, orc, spec, cam, st, seed_gpu, seed_cpu):
    s = scenes.to_scene(spec)
    ctx.upload(s)
    st = st.copy()
    st.seed = seed_gpu
    m_g, q_g, rays = ctx.render_moments(cam, st)
    ref = orc.OracleScene.from_spec(spec)
    out = ref.render(cam, st, seed=seed_cpu, threads=0)
    return m_g.astype(np.float64), q_g.astype(np.float64), out, rays


def test_c1_cornell_box_statistical_parity(gpu_ctx, orc):
    """The Cornell-box configuration (320x240, 5 bounces, RR from bounce 3,
    Halton, MIS, power lights) at 256 spp instead of 16, so that the block
    means the z-test compares are near-Gaussian."""
    spec, cam, st = scenes.cornell_box()
    assert (st.width, st.height, st.spp, st.bounces, st.rr_depth) == (320, 240, 16, 5, 3)
    st = st.copy()
    st.spp = 256
    m_g, q_g, out, rays = _render_both(gpu_ctx, orc, spec, cam, st, 101, 202)
    assert_parity("cornell box", m_g, q_g, st.spp, out["linear"], out["sumsq"], st.spp)
    # extension-ray counts agree statistically (same integrator, same RR)
    assert abs(rays - out["stats"]["segments"]) / out["stats"]["segments"] < 0.002


@pytest.mark.parametrize("which", ["cornell_ref", "showcase"])
def test_sphere_lights_nee_mis_parity(gpu_ctx, orc, which):
    """Scenes with emissive spheres exercise NEE, power-weighted light choice,
    MIS on emitter hits, glass and metal."""
    spec, cam = {"cornell_ref": scenes.cornell_reference_scene, "showcase": scenes.showcase_scene}[which]()
    st = bcgx.quality("Draft")
    st.width, st.height, st.spp, st.bounces = 160, 96, 256, 6
    st.sampler, st.mis, st.power_light_sampling = "Halton", True, True
    st.firefly_clamp, st.rr_depth, st.adaptive_sampling = 0.0, 4, False
    m_g, q_g, out, _ = _render_both(gpu_ctx, orc, spec, cam, st, 7, 8)
    assert out["stats"]["shadow"] > 0
    assert_parity(which, m_g, q_g, st.spp, out["linear"], out["sumsq"], st.spp)


@pytest.mark.parametrize("sampler,clamp,power", [("Halton", 0.0, True), ("Random", 12.0, False), ("R2", 0.0, True)])
def test_common_random_numbers(gpu_ctx, orc, sampler, clamp, power):
    """Same seed on both sides: path-by-path replay of the CPU integrator."""
    spec, cam = scenes.cornell_reference_scene()
    st = bcgx.quality("Draft")
    st.width, st.height, st.spp, st.bounces = 96, 64, 8, 6
    st.sampler, st.mis, st.power_light_sampling = sampler, True, power
    st.firefly_clamp, st.rr_depth, st.adaptive_sampling = clamp, 3, False
    m_g, _, out, rays = _render_both(gpu_ctx, orc, spec, cam, st, 42, 42)
    m_c = out["linear"]
    close = np.all(np.abs(m_g - m_c) <= 2e-3 * (1 + np.abs(m_c)), axis=2)
    assert close.mean() > 0.97, f"only {close.mean():.4f} of pixels replay the CPU paths"
    assert abs(rays - out["stats"]["segments"]) <= 0.01 * out["stats"]["segments"]


def _decode_oct(qx, qy):  # decodeOctNormal (gpu_opencl_windows.go:549-559)
    x = qx / 1023.0 * 2 - 1
    y = qy / 1023.0 * 2 - 1
    z = 1 - np.abs(x) - np.abs(y)
    neg = z < 0
    ox, oy = x.copy(), y.copy()
    x = np.where(neg, (1 - np.abs(oy)) * np.copysign(1, ox), x)
    y = np.where(neg, (1 - np.abs(ox)) * np.copysign(1, oy), y)
    v = np.stack([x, y, z], -1)
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def test_compact_guides_and_chunks(gpu_ctx, orc):
    """renderOpenCL's chunk loop and compact guide encoding, checked against the
    oracle's sample-0 first-hit guide; chunked rows equal a whole-frame render."""
    spec, cam = scenes.cornell_reference_scene()
    st = bcgx.quality("Draft")
    st.width, st.height, st.spp, st.bounces = 128, 96, 4, 4
    st.denoise, st.progressive_updates, st.publish_hz = True, True, 60  # 32-row chunks
    st.sampler, st.adaptive_sampling, st.firefly_clamp = "Halton", False, 0.0
    s = scenes.to_scene(spec)
    chunks = []
    lin, g, rays, name = bcgx.render_cuda(s, cam, st, on_chunk=lambda y0, r, d, p: chunks.append((y0, r, p)))
    assert [c[0] for c in chunks] == [0, 32, 64] and chunks[-1][2] == 1.0
    assert "GB300" in name or name
    ctx = bcgx.persistent_context()
    plain = st.copy()
    plain.denoise, plain.bloom = False, 0
    full = ctx.render_frame(cam, plain, want_guides=True, want_rgba=False)
    assert np.array_equal(full["linear"], lin)
    ref = orc.OracleScene.from_spec(spec).render(cam, st, seed=st.seed)
    gr = ref["guides"]
    valid_ref = gr[..., 10] > 0
    valid_gpu = (g[..., 1] & 0x80000000) != 0
    assert (valid_ref == valid_gpu).mean() > 0.995
    both = valid_ref & valid_gpu
    n_gpu = _decode_oct(g[..., 1] & 1023, (g[..., 1] >> 10) & 1023)
    cosang = (n_gpu[both] * gr[..., 3:6][both]).sum(-1)
    assert np.mean(cosang > 0.99) > 0.99
    depth_gpu = g[..., 0].view(np.float32)
    # the compact depth is Euclidean (the Go decoder walks a unit direction)
    o, lower, horiz, vert = orc.camera_basis(cam, st.width / st.height)
    ys, xs = np.nonzero(both)
    jit = g[..., 2][both]
    u = (xs + (jit & 0xFFFF) / 65535.0) / (st.width - 1)
    v = (st.height - 1 - ys + (jit >> 16) / 65535.0) / (st.height - 1)
    dirs = lower + u[:, None] * horiz + v[:, None] * vert - o
    eu = gr[..., 9][both] * np.linalg.norm(dirs, axis=1)
    rel = np.abs(depth_gpu[both] - eu) / eu
    assert np.mean(rel < 1e-3) > 0.99
    mats = (g[..., 1] >> 20) & 2047
    assert mats[both].max() < len(spec.materials)


def test_post_stack_parity(gpu_ctx, orc):
    """Denoise (3 passes), bloom and ACES tone map on identical inputs (the
    reference's TestParallelPostDeterminism image, renderer_test.go:720)."""
    w, h = 96, 64
    img = np.zeros((h, w, 3))
    guides = np.zeros((h, w, 11))
    for y in range(h):
        for x in range(w):
            v = ((x * 13 + y * 7) % 97) / 97.0
            img[y, x] = (0.1 + 2 * v, 0.2 + v, 0.3 + 0.5 * v)
            guides[y, x, 0:3] = (x * 0.01, y * 0.01, -2 - v)
            guides[y, x, 3:6] = (0, 0, 1)
            guides[y, x, 9] = 2 + v
            guides[y, x, 10] = 1
    guides[5:9, 10:20, 10] = 0  # a patch without first hits
    img32 = img.astype(np.float32)
    img_in = img32.astype(np.float64)
    st = bcgx.ultra_realism_settings("CPU")  # denoise 3 passes, bloom 1, ACES
    g4 = np.concatenate([guides[..., 3:6], np.where(guides[..., 10:11] > 0, guides[..., 9:10], -1.0)], -1)
    out, rgba = gpu_ctx.post_process(img32, g4.astype(np.float32), st)
    ref = orc.bloom(orc.atrous(img_in, guides, 2 + min(3, max(st.taa, st.txaa))), st.bloom)
    rel = np.abs(out - ref) / np.maximum(np.abs(ref), 1e-3)
    assert rel.max() < 2e-4, rel.max()
    rgba_ref = orc.to_rgba(ref, st.exposure, st.gamma, st.hdr)
    ch_g = np.stack([(rgba >> s) & 255 for s in (0, 8, 16)], -1).astype(int)
    ch_r = np.stack([(rgba_ref >> s) & 255 for s in (0, 8, 16)], -1).astype(int)
    assert np.abs(ch_g - ch_r).max() <= 1
    assert np.mean(ch_g == ch_r) > 0.995
    # the other tone curves
    for hdr in (0, 1, 2):
        st2 = st.copy()
        st2.hdr, st2.denoise, st2.bloom, st2.exposure = hdr, False, 0, 0.5
        _, rg = gpu_ctx.post_process(img32, None, st2)
        rr = orc.to_rgba(img_in, 0.5, st.gamma, hdr)
        d = np.abs(np.stack([(rg >> s) & 255 for s in (0, 8, 16)], -1).astype(int) -
                   np.stack([(rr >> s) & 255 for s in (0, 8, 16)], -1).astype(int))
        assert d.max() <= 1 and np.mean(d == 0) > 0.995


def test_determinism_and_cancel(gpu_ctx):
    spec, cam, st = scenes.cornell_box()
    st = st.copy()
    st.width, st.height, st.spp = 64, 48, 4
    gpu_ctx.upload(scenes.to_scene(spec))
    a = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)
    b = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)
    assert np.array_equal(a["linear"], b["linear"]) and a["rays"] == b["rays"]
    st2 = st.copy()
    st2.seed += 1
    c = gpu_ctx.render_frame(cam, st2, want_guides=False, want_rgba=False)
    assert not np.array_equal(a["linear"], c["linear"])
    gpu_ctx.cancel()
    with pytest.raises(bcgx.BCError) as e:
        gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)
    assert e.value.status == 4
    gpu_ctx.reset_cancel()
    d = gpu_ctx.render_frame(cam, st, want_guides=False, want_rgba=False)
    assert np.array_equal(a["linear"], d["linear"])


def test_render_argument_errors(gpu_ctx):
    spec, cam, st = scenes.cornell_box()
    gpu_ctx.upload(scenes.to_scene(spec))
    bad = st.copy()
    bad.spp = 0
    with pytest.raises(bcgx.BCError) as e:
        gpu_ctx.render_frame(cam, bad)
    assert e.value.status == 7
    with pytest.raises(bcgx.BCError):
        gpu_ctx.render_rows(cam, st, st.height - 1, 4)

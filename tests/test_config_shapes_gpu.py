"""Oracle parity at the shapes of the Ultra-shaped frame, the 64-view batch and
the differentiation configurations, through the C-ABI.

* Ultra shape: displaced geodesic icospheres on a ground quad under emissive
  quads, half the spheres rough metal (Roughness U[0.05, 1]: MatMetal's fuzz,
  renderer.go:1520-1527), 16 bounces, Russian roulette from bounce 6
  (renderer.go:1550-1560), Halton, MIS, power lights, no clamp. An 8 x 8 grid
  of spheres keeps the oracle's share of the test short; the materials, light
  model, path length and sampler are the full configuration's. z-test of 2x2
  pixel blocks at 256 spp (zstats.py) and a common-random-number replay.
* Batch shape: views over two random-mesh scenes of the batching workload
  (the ray-cast triangle generator plus one emissive quad, 8 bounces),
  rendered inside one batch; each batched view equals its single-view render
  bit for bit, and that render passes the z-test against the oracle.
* Differentiation shape: 256 albedo slots, 8 emissive quads, 8 bounces, no
  Russian roulette; the adjoint against central finite differences of the fp64
  oracle's forward with common random numbers, within 2% (plus 0.5% of the RMS
  gradient), at 256 spp.
"""
import numpy as np
import pytest

from bcgx import scenes
from zstats import assert_parity

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ultra_small(orc):
    spec, cam, st = scenes.icosphere_grid(n=8, n_lights=8)
    st = st.copy()
    st.denoise, st.bloom = False, 0
    st.width, st.height = 128, 72
    assert (st.bounces, st.rr_depth, st.sampler, st.firefly_clamp) == (16, 6, "Halton", 0.0)
    assert st.mis and st.power_light_sampling and not st.adaptive_sampling
    return spec, cam, st, orc.OracleScene.from_spec(spec)


def test_ultra_shape_materials(ultra_small):
    """The scene holds what the configuration asks for: rough metal with
    roughness spread over [0.05, 1], diffuse spheres and emitters."""
    spec = ultra_small[0]
    metal = [m for m in spec.materials if m.kind == scenes.MAT_METAL]
    assert len(metal) >= 16 and min(m.roughness for m in metal) < 0.2 and max(m.roughness for m in metal) > 0.8
    assert any(m.kind == scenes.MAT_DIFFUSE for m in spec.materials)
    assert sum(m.kind == scenes.MAT_EMISSIVE for m in spec.materials) == 8


def test_ultra_shape_statistical_parity(gpu_ctx, ultra_small):
    spec, cam, st, ref = ultra_small
    gpu_ctx.upload(scenes.to_scene(spec))
    st = st.copy()
    st.spp, st.seed = 256, 31
    m_g, q_g, rays = gpu_ctx.render_moments(cam, st)
    out = ref.render(cam, st, seed=32, threads=0)
    assert out["stats"]["segments"] > 2 * st.width * st.height * st.spp  # multi-bounce paths
    assert_parity("ultra shape", m_g, q_g, st.spp, out["linear"], out["sumsq"], st.spp)
    assert abs(rays - out["stats"]["segments"]) / out["stats"]["segments"] < 0.005


def test_ultra_shape_common_random_numbers(gpu_ctx, ultra_small):
    """Same seed on both sides: the GPU replays the oracle's paths through metal
    fuzz, 16 bounces and the roulette, up to fp32-vs-fp64 boundary decisions."""
    spec, cam, st, ref = ultra_small
    gpu_ctx.upload(scenes.to_scene(spec))
    st = st.copy()
    st.spp, st.seed = 8, 77
    m_g, _, rays = gpu_ctx.render_moments(cam, st)
    out = ref.render(cam, st, seed=77, threads=0)
    m_c = out["linear"]
    close = np.all(np.abs(m_g - m_c) <= 2e-3 * (1 + np.abs(m_c)), axis=2)
    assert close.mean() > 0.95, f"only {close.mean():.4f} of pixels replay the CPU paths"
    assert abs(rays - out["stats"]["segments"]) <= 0.01 * out["stats"]["segments"]


def test_batch_shape_views_against_oracle(gpu_ctx, orc):
    specs = [scenes.batch_scene(10_000, scenes.SEED_BATCH + 1), scenes.batch_scene(50_000, scenes.SEED_BATCH + 2)]
    _, views = scenes.batch_views(n_views=4, sizes=(10_000, 50_000))
    built = [scenes.to_scene(s) for s in specs]
    picked = []
    for k, (scene_k, cam, st) in enumerate(views[:2]):
        st = st.copy()
        st.width, st.height = (96, 72) if k == 0 else (80, 64)
        st.spp = 256
        assert st.bounces == 8 and scene_k == k
        picked.append((scene_k, cam, st))
    extra = views[2][0], views[2][1], views[2][2].copy()  # a third view of another size in the batch
    extra[2].width, extra[2].height, extra[2].spp = 64, 40, 16
    gpu_ctx.upload_set(built, set_id=0xBA7C4, revision=1)
    imgs, _ = gpu_ctx.render_batch(picked + [extra])
    for k, (scene_k, cam, st) in enumerate(picked):
        gpu_ctx.upload(built[scene_k])
        m_g, q_g, rays = gpu_ctx.render_moments(cam, st)
        assert np.array_equal(imgs[k], m_g), f"batched view {k} differs from its single-view render"
        out = orc.OracleScene.from_spec(specs[scene_k]).render(cam, st, seed=1000 + k, threads=0)
        assert_parity(f"batch view {k}", m_g, q_g, st.spp, out["linear"], out["sumsq"], st.spp)
        assert abs(rays - out["stats"]["segments"]) / out["stats"]["segments"] < 0.005


def test_diff_shape_adjoint_against_oracle_fd(gpu_ctx, orc):
    """C5's parameter layout (256 albedo slots, 8 emitters) and path length (8
    bounces, no roulette) on a 20k-triangle scene at 48x32, 256 spp. The target
    is the true parameters' image at 4096 spp; the adjoint of the GPU forward is
    compared with central differences (h = 1e-3) of the oracle's forward loss
    against the same target, same seed (common random numbers)."""
    pb = scenes.diff_scene(n_tris=20_000, width=48, height=32, spp=256, bounces=8)
    assert len(pb.albedo_materials) == 256 and len(pb.emission_materials) == 8
    assert pb.settings.rr_depth >= pb.settings.bounces
    seed = 0xBEAC0005
    gpu_ctx.upload(scenes.to_scene(pb.spec))
    st_t = pb.settings.copy()
    st_t.spp = 4096
    gpu_ctx.diff_configure(pb.cam, st_t, pb.albedo_materials, pb.emission_materials)
    target, _ = gpu_ctx.forward(pb.true_params, seed + 1)
    gpu_ctx.diff_configure(pb.cam, pb.settings, pb.albedo_materials, pb.emission_materials)
    gpu_ctx.diff_set_target(target)
    params = pb.init_params
    gpu_ctx.forward(params, seed, want_image=False)
    ga, ge = gpu_ctx.backward()
    adj = np.concatenate([ga, ge]).reshape(-1).astype(np.float64)
    ref = orc.OracleScene.from_spec(pb.spec)
    mats = np.concatenate([pb.albedo_materials, pb.emission_materials])
    n_alb = len(pb.albedo_materials)
    tgt = target.astype(np.float64)

    def oracle_loss(q):
        for k, m in enumerate(mats):
            if k < n_alb:
                ref.set_material(int(m), color=q[k].astype(np.float64))
            else:
                ref.set_material(int(m), emission=q[k].astype(np.float64))
        img = ref.render(pb.cam, pb.settings, seed=seed, threads=0)["linear"]
        return float(np.mean((img - tgt) ** 2))

    rng = np.random.default_rng(seed)
    picks = np.sort(np.concatenate([rng.choice(3 * n_alb, 24, replace=False),
                                    3 * n_alb + rng.choice(3 * len(pb.emission_materials), 8, replace=False)]))
    fd = []
    for k in picks:
        p, m = params.copy(), params.copy()
        p.flat[k] += 1e-3
        m.flat[k] -= 1e-3
        fd.append((oracle_loss(p) - oracle_loss(m)) / (float(p.flat[k]) - float(m.flat[k])))
    fd = np.array(fd)
    scale = np.sqrt(np.mean(fd ** 2))
    assert scale > 0
    err = np.abs(adj[picks] - fd)
    rel = err / np.maximum(np.abs(fd), 1e-30)
    live = np.abs(fd) > 1e-3 * scale
    assert live.sum() >= 24, "most picked parameters must move the loss"
    print(f"DIFFSTAT {live.sum()} of {len(fd)} live: max rel {rel[live].max():.5f}, median rel "
          f"{np.median(rel[live]):.5f}, max err/rms {err.max() / scale:.5f}")
    bad = err > 2e-2 * np.abs(fd) + 5e-3 * scale
    assert not bad.any(), (f"{bad.sum()} of {len(fd)} gradients beyond 2% (+0.5% of rms {scale:.3e}): "
                           f"adjoint {adj[picks][bad]}, fd {fd[bad]}")

"""Path-replay gradients (bc_diff_configure / bc_forward / bc_backward).

The adjoint is checked against central finite differences, h = 1e-3, on 32
seeded parameters, with common random numbers (the same seed, so the same
paths on both sides of the difference), on two forwards:

* the GPU forward itself: the adjoint is the derivative of the same fp32
  estimator, so the two agree closely;
* the fp64 oracle forward (same PCG32 streams, so nearly the same paths):
  agreement within the fp32-vs-fp64 path splits.

Russian roulette is off (rr_depth = bounces): its decisions are not smooth in
the parameters, and the adjoint holds their probabilities fixed.
"""
import numpy as np
import pytest

import bcgx
from bcgx import scenes

pytestmark = pytest.mark.gpu

H_FD = 1e-3
N_CHECK = 32
SEED = 0xBEAC0005


@pytest.fixture(scope="module")
def problem():
    return scenes.diff_scene(n_tris=20_000, width=64, height=48, spp=16, bounces=6)


@pytest.fixture(scope="module")
def target(gpu_ctx, problem):
    """The image of the true parameters at 16x the samples (same seed)."""
    gpu_ctx.upload(scenes.to_scene(problem.spec))
    st = problem.settings.copy()
    st.spp = problem.settings.spp * 16
    gpu_ctx.diff_configure(problem.cam, st, problem.albedo_materials, problem.emission_materials)
    img, _ = gpu_ctx.forward(problem.true_params, SEED)
    return img


@pytest.fixture()
def ctx(gpu_ctx, problem, target):
    gpu_ctx.upload(scenes.to_scene(problem.spec))
    gpu_ctx.diff_configure(problem.cam, problem.settings, problem.albedo_materials, problem.emission_materials)
    gpu_ctx.diff_set_target(target)
    return gpu_ctx


def _picks(n_params):
    rng = np.random.default_rng(SEED)
    return np.sort(rng.choice(3 * n_params, N_CHECK, replace=False))


def _adjoint(ctx, params):
    ctx.forward(params, SEED, want_image=False)
    ga, ge = ctx.backward()
    return np.concatenate([ga, ge]).reshape(-1).astype(np.float64)


def _fd(loss_fn, params, k):
    p, m = params.copy(), params.copy()
    p.flat[k] += H_FD
    m.flat[k] -= H_FD
    step = float(p.flat[k]) - float(m.flat[k])  # the float32 step actually taken
    return (loss_fn(p) - loss_fn(m)) / step


def _check(adj, fd, rel, floor_frac):
    scale = np.sqrt(np.mean(fd ** 2))
    assert scale > 0, "all picked gradients are zero: the check has no signal"
    err = np.abs(adj - fd)
    bad = err > rel * np.abs(fd) + floor_frac * scale
    assert not bad.any(), (f"{bad.sum()} of {len(fd)} gradients off: adjoint {adj[bad]}, fd {fd[bad]}, "
                           f"rms {scale:.3e}")


def test_adjoint_matches_gpu_finite_differences(ctx, problem):
    params = problem.init_params
    adj = _adjoint(ctx, params)
    picks = _picks(len(params))
    fd = np.array([_fd(lambda q: ctx.forward(q, SEED, want_image=False)[1], params, k) for k in picks])
    _check(adj[picks], fd, rel=1e-2, floor_frac=1e-2)
    # the pick covers both kinds of parameter once the emission block is hit
    assert np.count_nonzero(adj) > len(adj) // 2


def test_adjoint_matches_oracle_finite_differences(ctx, problem, target, orc):
    params = problem.init_params
    adj = _adjoint(ctx, params)
    ref = orc.OracleScene.from_spec(problem.spec)
    mats = np.concatenate([problem.albedo_materials, problem.emission_materials])
    n_alb = len(problem.albedo_materials)
    tgt = target.astype(np.float64)

    def oracle_loss(q):
        for k, m in enumerate(mats):
            if k < n_alb:
                ref.set_material(int(m), color=q[k].astype(np.float64))
            else:
                ref.set_material(int(m), emission=q[k].astype(np.float64))
        img = ref.render(problem.cam, problem.settings, seed=SEED, threads=0)["linear"]
        return float(np.mean((img - tgt) ** 2))

    picks = _picks(len(params))
    fd = np.array([_fd(oracle_loss, params, k) for k in picks])
    _check(adj[picks], fd, rel=5e-2, floor_frac=3e-2)


def test_custom_adjoint_image(ctx, problem):
    """bc_backward with a caller dLoss/dImage: the gradient of sum(W * image)."""
    params = problem.init_params
    H, W = problem.settings.height, problem.settings.width
    w = np.random.default_rng(7).uniform(-1, 1, (H, W, 3)).astype(np.float32)
    ctx.forward(params, SEED, want_image=False)
    ga, ge = ctx.backward(w)
    adj = np.concatenate([ga, ge]).reshape(-1).astype(np.float64)

    def weighted(q):
        img, _ = ctx.forward(q, SEED)
        return float(np.sum(w.astype(np.float64) * img))

    picks = _picks(len(params))[:12]
    fd = np.array([_fd(weighted, params, k) for k in picks])
    _check(adj[picks], fd, rel=1e-2, floor_frac=1e-2)


def test_gradient_descent_reduces_loss(gpu_ctx, problem):
    """With the target rendered from the true parameters at the same seed and
    spp, common random numbers make the loss a deterministic function of the
    parameters (zero at the truth) and the adjoint its exact gradient: a
    backtracking descent along it must bring the loss well down."""
    ctx = gpu_ctx
    ctx.upload(scenes.to_scene(problem.spec))
    ctx.diff_configure(problem.cam, problem.settings, problem.albedo_materials, problem.emission_materials)
    tgt, _ = ctx.forward(problem.true_params, SEED)
    ctx.diff_set_target(tgt)
    assert ctx.forward(problem.true_params, SEED, want_image=False)[1] == 0.0
    params = problem.init_params.copy()
    na = len(problem.albedo_materials)

    def clip(q):
        q = q.copy()
        q[:na] = np.clip(q[:na], 0.01, 0.99)
        q[na:] = np.maximum(q[na:], 0.0)
        return q

    loss = l_init = ctx.forward(params, SEED, want_image=False)[1]
    assert l_init > 0
    alpha = None
    for it in range(10):
        ctx.forward(params, SEED, want_image=False)
        ga, ge = ctx.backward()
        g = np.concatenate([ga, ge])
        assert np.isfinite(g).all()
        if alpha is None:
            alpha = 0.05 / float(np.abs(g).max())
        for _ in range(8):
            cand = clip(params - alpha * g)
            lc = ctx.forward(cand, SEED, want_image=False)[1]
            if lc < loss:
                params, loss = cand, lc
                alpha *= 1.5
                break
            alpha *= 0.5
    assert loss < 0.5 * l_init, (l_init, loss)


def test_backward_is_repeatable(ctx, problem):
    a = _adjoint(ctx, problem.init_params)
    b = _adjoint(ctx, problem.init_params)
    np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-12)


def test_diff_argument_errors(gpu_ctx, problem):
    gpu_ctx.upload(scenes.to_scene(problem.spec))
    st = problem.settings
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):  # albedo on an emissive material
        gpu_ctx.diff_configure(problem.cam, st, problem.emission_materials[:1], [])
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):  # emission on a diffuse material
        gpu_ctx.diff_configure(problem.cam, st, [], problem.albedo_materials[:1])
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):  # a material named twice
        gpu_ctx.diff_configure(problem.cam, st, [0, 0], [])
    bad = st.copy()
    bad.firefly_clamp = 4.0
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):
        gpu_ctx.diff_configure(problem.cam, bad, problem.albedo_materials, [])
    gpu_ctx.diff_configure(problem.cam, st, problem.albedo_materials, problem.emission_materials)
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):  # no forward yet
        gpu_ctx.backward()
    gpu_ctx.forward(problem.init_params, SEED, want_image=False)
    with pytest.raises(bcgx.BCError, match="INVALID_ARG"):  # no target, no adjoint image
        gpu_ctx.backward()

"""Device SAH build (bc_build_sah / Scene.build_device) against the host
builder, which restates buildNodeSAH (renderer.go:526-633) and is pinned
against the reference's tests: node boxes, children, leaf ranges and
Scene.Order must be identical, bit for bit, node for node."""
import numpy as np
import pytest

from bcgx import scenes

pytestmark = pytest.mark.gpu


def _arrays(scene):
    a = scene.arrays()
    return a.node_box, a.node_left, a.node_right, a.node_start, a.node_count, a.order


def _same_tree(spec, gpu_ctx, bins=32, leaf=4):
    host = scenes.to_scene(spec, build=False)
    dev = scenes.to_scene(spec, build=False)
    for s in (host, dev):
        s.bvh_mode, s.bvh_bins, s.bvh_leaf = "SAH", bins, leaf
    host.build()
    dev.build_device(gpu_ctx)
    h, d = _arrays(host), _arrays(dev)
    names = ("node_box", "node_left", "node_right", "node_start", "node_count", "order")
    for name, x, y in zip(names, h, d):
        assert x.shape == y.shape, f"{name}: {x.shape} vs {y.shape}"
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8)), f"{name} differs"
    return len(h[1])


@pytest.mark.parametrize("n,bins,leaf", [(100_000, 32, 4), (30_000, 16, 2), (5_000, 8, 16), (2_000, 32, 1)])
def test_random_triangles(gpu_ctx, n, bins, leaf):
    _same_tree(scenes.random_triangles(n, seed=0xBEAC0201 + n), gpu_ctx, bins, leaf)


@pytest.mark.parametrize("which", ["stress", "showcase", "cornell_ref", "cornell_box", "icospheres"])
def test_reference_and_workload_scenes(gpu_ctx, which):
    spec = {"stress": lambda: scenes.stress_scene()[0], "showcase": lambda: scenes.showcase_scene()[0],
            "cornell_ref": lambda: scenes.cornell_reference_scene()[0], "cornell_box": lambda: scenes.cornell_box()[0],
            "icospheres": lambda: scenes.icosphere_grid(n=6, n_lights=4)[0]}[which]()
    _same_tree(spec, gpu_ctx)


def test_degenerate_and_tiny(gpu_ctx):
    rng = np.random.default_rng(5)
    # many triangles sharing a centroid plane (zero extent on two axes), duplicates, and a cluster
    base = scenes.random_triangle_verts(3000, seed=7)
    dup = np.repeat(base[:50], 20, axis=0)
    flat = base.copy()
    flat[:, 1::3] = 0.25
    spec = scenes.SceneSpec(name="degenerate", bvh_mode="SAH", bvh_bins=32, bvh_leaf=4)
    m = spec.material(scenes.Material(0, (0.5, 0.5, 0.5)))
    spec.triangles(np.concatenate([dup, flat, base * 1e-9 + 0.5]), m)
    _same_tree(spec, gpu_ctx)
    for n in (1, 2, 5, 17):
        _same_tree(scenes.random_triangles(n, seed=100 + n), gpu_ctx)


def test_device_built_scene_renders_and_casts(gpu_ctx, orc):
    spec = scenes.random_triangles(50_000, seed=0xBEAC0202)
    dev = scenes.to_scene(spec, build=False)
    dev.bvh_mode, dev.bvh_bins, dev.bvh_leaf = "SAH", 32, 4
    dev.build_device(gpu_ctx)
    gpu_ctx.upload(dev)
    rays = scenes.random_rays(32_768, seed=3)
    t, p = gpu_ctx.raycast(rays)
    t_ref, p_ref, _ = orc.OracleScene.from_spec(spec).hit_f32(rays)
    assert np.array_equal(p, p_ref)
    assert np.array_equal(t[p >= 0], t_ref[p >= 0].astype(np.float32))

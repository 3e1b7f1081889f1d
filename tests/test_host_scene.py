"""The native host builder (product) against the oracle's restatement of
Scene.Build: identical primitives, node sets, numbering, Order and lights."""
import numpy as np
import pytest

from bcgx import scenes


def _compare(spec, orc, mode=None, bins=None, leaf=None):
    if mode:
        spec.bvh_mode, spec.bvh_bins, spec.bvh_leaf = mode, bins, leaf
    prod = scenes.to_scene(spec).arrays()
    ref = orc.OracleScene.from_spec(spec)
    o = ref.arrays()
    for f in ("prim_kind", "prim_material", "prim_center", "prim_radius", "prim_a", "prim_e1", "prim_e2",
              "prim_normal", "node_box", "node_left", "node_right", "node_start", "node_count", "order",
              "light_spheres", "light_cdf", "light_pdf_by_prim", "mat_kind", "mat_color", "mat_emission"):
        a, b = getattr(prod, f), getattr(o, f)
        assert a.shape == b.shape, f
        assert np.array_equal(a, b), f  # bit-identical fp64 and integers
    return prod


@pytest.mark.parametrize("maker", ["stress", "showcase", "cornell_ref", "c1"])
def test_builder_matches_oracle_builtin(native_lib, orc, maker):
    spec = {"stress": lambda: scenes.stress_scene()[0], "showcase": lambda: scenes.showcase_scene()[0],
            "cornell_ref": lambda: scenes.cornell_reference_scene()[0], "c1": lambda: scenes.cornell_box()[0]}[maker]()
    _compare(spec, orc)


@pytest.mark.parametrize("bins,leaf", [(32, 4), (16, 4), (8, 1), (4, 16)])
def test_builder_matches_oracle_random_tris(native_lib, orc, bins, leaf):
    spec = scenes.random_triangles(20000, seed=7)
    _compare(spec, orc, "SAH", bins, leaf)


def test_builder_median_matches_oracle(native_lib, orc):
    spec = scenes.random_triangles(5000, seed=11)
    _compare(spec, orc, "Median", 16, 4)


def test_refit_and_revisions(native_lib, orc):  # TestGPURevisionTracking, renderer_test.go:692
    spec, _ = scenes.stress_scene()
    s = scenes.to_scene(spec)
    t0, g0 = s.revisions()
    assert t0 >= 1 and g0 >= 1
    s.translate_primitive(3, [0.75, 0.1, -0.25])
    s.refit()
    t1, g1 = s.revisions()
    assert t1 == t0 and g1 > g0
    ref = orc.OracleScene.from_spec(spec)
    ref.translate(3, [0.75, 0.1, -0.25])
    ref.refit()
    a, b = s.arrays(), ref.arrays()
    assert np.array_equal(a.node_box, b.node_box)
    assert np.array_equal(a.prim_center, b.prim_center)
    s.build()
    assert s.revisions()[0] > t1


def test_degenerate_triangles_dropped(native_lib, orc):
    spec = scenes.SceneSpec()
    m = spec.material(scenes.Material(scenes.MAT_DIFFUSE, (0.5, 0.5, 0.5)))
    v = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0], [0, 0, 0, 1, 0, 0, 2, 0, 0], [0, 0, 0, 1e-10, 0, 0, 0, 1e-10, 0]],
                 dtype=np.float64)
    spec.triangles(v, m)
    p = _compare(spec, orc)
    assert len(p.prim_kind) == 1


def test_single_leaf_and_empty(native_lib):
    spec = scenes.SceneSpec()
    m = spec.material(scenes.Material(scenes.MAT_DIFFUSE, (0.5, 0.5, 0.5)))
    spec.sphere((0, 0, 0), 1, m)
    s = scenes.to_scene(spec).arrays()
    assert len(s.node_left) == 1 and s.node_count[0] == 1
    e = scenes.to_scene(scenes.SceneSpec()).counts()
    assert e["prims"] == 0 and e["nodes"] == 0

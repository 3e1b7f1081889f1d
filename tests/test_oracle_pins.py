"""The oracle against the reference's own unit-test pins (renderer_test.go).

The reference's ray sets come from Go math/rand seeds; equivalent rays are
drawn here from numpy with the same construction formulas.
"""
import math
import os
import struct

import numpy as np
import pytest

from bcgx import scenes
from conftest import ROOT


def bits(x):
    return struct.pack("<d", x).hex()


def test_effective_spp(orc, pins):  # TestSamplingLevels, renderer_test.go:198
    for c in pins["effective_spp"]:
        got = orc.effective_spp(c["spp"], c["msaa"], c["tsaa"])
        if c["want"] == 4096:
            assert got <= 4096
        assert got == c["want"]


def test_power_heuristic_and_light_pmf(orc, pins):  # TestPowerWeightedLightPDF, renderer_test.go:310
    spec, _ = scenes.showcase_scene()
    s = orc.OracleScene.from_spec(spec)
    sp, cdf, pdf = s.lights()
    assert len(sp) == pins["showcase_scene"]["lights"]
    total = 0.0
    for pi in sp:
        p = s.light_selection_pdf(pi, True)
        assert p > 0
        total += p
    assert abs(total - 1) <= 1e-9
    h = orc.power_heuristic(0.5, 0.5)
    assert pins["power_heuristic_half"]["lo"] <= h <= pins["power_heuristic_half"]["hi"]
    assert abs(cdf[-1] - 1) <= 1e-12  # TestCachedLightDistribution, renderer_test.go:563
    assert abs(pdf[sp].sum() - 1) <= 1e-9


def test_light_pmf_many_lights(orc):
    """Power-weighted PMF over several emissive spheres sums to 1 and is proportional to power."""
    spec, _ = scenes.showcase_scene()
    for k, (em, r) in enumerate([((4, 4, 4), 0.3), ((30, 10, 1), 0.5), ((1, 2, 3), 1.2)]):
        m = spec.material(scenes.Material(scenes.MAT_EMISSIVE, emission=em))
        spec.sphere((k, 6, -4), r, m)
    s = orc.OracleScene.from_spec(spec)
    sp, cdf, pdf = s.lights()
    assert len(sp) == 4
    assert abs(pdf[sp].sum() - 1) <= 1e-9
    assert np.all(np.diff(cdf) > 0) and cdf[-1] == 1


def test_fast_aabb_matches_inline_reference(orc, pins):  # renderer_test.go:361
    for c in pins["aabb_cases"]:
        box6 = c["box"][0] + c["box"][1]
        ray6 = c["ray"][0] + c["ray"][1]
        ok, _ = orc.aabb_hit(box6, ray6, 1e-4, 1e30)
        assert ok == c["hit"], c


def test_tile_order(orc, pins):  # TestCenterTileOrderIsPermutation, renderer_test.go:542
    t = pins["tile_order"]
    for mode in ("Center", "Scanline"):
        o = orc.tile_order(t["tx"], t["ty"], mode)
        assert sorted(o.tolist()) == list(range(t["tx"] * t["ty"]))
    first = orc.tile_order(t["tx"], t["ty"], "Center")[0]
    assert [first % t["tx"], first // t["tx"]] == t["first_xy"]


def test_radical_inverse_and_rotation_bits(orc, pins):
    for base in (2, 3):
        want = pins["radical_inverse"][str(base)]
        for n in range(1, 257):
            assert bits(orc.radical_inverse(n, base)) == want[n - 1]
    for c in pins["pixel_rotation"]:
        rx, ry = orc.pixel_sample_rotation(c["x"], c["y"])
        assert [bits(rx), bits(ry)] == c["r"]


def test_sample_sequences_in_unit_square(orc):  # TestPreparedSampleSequenceBounds, renderer_test.go:610
    for sampler in (1, 2):
        X, Y = orc.sample_sequence(sampler, 64, 1, 0)
        assert len(X) == 64
        rx, ry = orc.pixel_sample_rotation(17, 29)
        x = np.mod(X + rx, 1.0)
        y = np.mod(Y + ry, 1.0)
        assert np.all((x >= 0) & (x < 1) & (y >= 0) & (y < 1))


def test_cosine_sampler(orc):  # TestCosineSamplerDistribution, renderer_test.go:673
    n = np.array([0.2, 0.9, 0.38])
    n = n / math.sqrt((n * n).sum())
    d = orc.cos_hemisphere(n, 123456789, 20000)
    assert np.all(np.abs((d * d).sum(axis=1) - 1) <= 2e-12)
    assert np.all(d @ n >= -1e-12)
    assert d.mean(axis=0) @ n > 0


def test_firefly_clamp(orc):  # TestSpecialistSamplingAndClamp, renderer_test.go:291
    c = orc.clamp_firefly([100, 50, 25], 10)
    assert c.max() <= 10.000001


def _stress_rays(cam, n, seed, sx, sy, sz):
    rng = np.random.default_rng(seed)
    r = rng.random((n, 3))
    tgt = np.asarray(cam.target) + (r - 0.5) * np.array([sx, sy, sz])
    return np.broadcast_to(np.asarray(cam.position, dtype=np.float64), (n, 3)).copy(), tgt - np.asarray(cam.position)


def test_sah_and_median_agree(orc):  # TestSAHAndMedianAgree, renderer_test.go:415
    spec, cam = scenes.stress_scene()
    o, d = _stress_rays(cam, 400, 42, 14, 5, 14)
    med = orc.OracleScene.from_spec(spec, mode="Median", bins=16, leaf=4)
    sah = orc.OracleScene.from_spec(spec, mode="SAH", bins=16, leaf=4)
    tm, pm, _ = med.hit(o, d)
    ts, ps, _ = sah.hit(o, d)
    assert np.array_equal(pm >= 0, ps >= 0)
    hit = ps >= 0
    assert hit.sum() > 100
    assert np.all(np.abs(tm[hit] - ts[hit]) <= 1e-7)


def test_refit_matches_rebuild(orc):  # TestBVHRefitMatchesRebuild, renderer_test.go:464
    spec, cam = scenes.stress_scene()
    s = orc.OracleScene.from_spec(spec, mode="SAH", bins=16, leaf=4)
    s.translate(3, [0.75, 0.1, -0.25])
    s.refit()
    pos, tgt = np.asarray(cam.position, float), np.asarray(cam.target, float)
    dirs = np.stack([tgt - pos, tgt + [3, 1, -2] - pos, tgt + [-4, 0.5, 3] - pos])
    orig = np.broadcast_to(pos, (3, 3)).copy()
    t1, p1, _ = s.hit(orig, dirs)
    s.build()
    t2, p2, _ = s.hit(orig, dirs)
    assert np.array_equal(p1 >= 0, p2 >= 0)
    assert np.all(np.abs(t1 - t2)[p1 >= 0] <= 1e-7)


def test_occluded_matches_closest_hit(orc):  # TestOccludedMatchesClosestHit, renderer_test.go:658
    spec, cam = scenes.stress_scene()
    s = orc.OracleScene.from_spec(spec)
    rng = np.random.default_rng(424242)
    n = 3000
    tgt = np.asarray(cam.target) + (rng.random((n, 3)) - 0.5) * np.array([24, 8, 24])
    d = tgt - np.asarray(cam.position)
    tmax = 0.25 + rng.random(n) * 30
    o = np.broadcast_to(np.asarray(cam.position, float), (n, 3)).copy()
    for i in range(0, n, 500):
        sl = slice(i, i + 500)
        for j in range(i, min(n, i + 500)):
            t, p, _ = s.hit(o[j:j + 1], d[j:j + 1], 1e-4, float(tmax[j]))
            occ = s.occluded(o[j:j + 1], d[j:j + 1], float(tmax[j]))
            assert bool(occ[0]) == bool(p[0] >= 0), j
        del sl


def test_threaded_escapes(orc):  # TestThreadedBVHEscapeTraversal, renderer_test.go:772
    spec, _ = scenes.stress_scene()
    s = orc.OracleScene.from_spec(spec)
    esc = s.escapes()
    _, left, right, _, count = s.nodes()
    assert len(esc) == len(left) and esc[0] == -1
    stack = [(0, -1)]
    while stack:
        idx, want = stack.pop()
        assert esc[idx] == want
        if count[idx] == 0:
            stack.append((left[idx], right[idx]))
            stack.append((right[idx], want))


def test_threaded_closest_hit_equivalence(orc):  # renderer_test.go:797
    spec, cam = scenes.stress_scene()
    s = orc.OracleScene.from_spec(spec)
    dirs = []
    for y in range(31):
        for x in range(47):
            v = np.array([(x - 23) * 0.065, (y - 15) * 0.055, -1.0])
            dirs.append(v / math.sqrt((v * v).sum()))
    dirs = np.array(dirs)
    o = np.broadcast_to(np.asarray(cam.position, float), dirs.shape).copy()
    ta, pa, _ = s.hit(o, dirs)
    tb, pb, _ = s.hit(o, dirs, threaded=True)
    assert np.array_equal(pa >= 0, pb >= 0)
    assert np.all(np.abs(ta - tb)[pa >= 0] <= 1e-9)


def test_ultra_realism_preset(pins):  # TestUltraRealismPreset, renderer_test.go:846
    import bcgx
    want = pins["ultra_realism_cpu"]
    q = bcgx.ultra_realism_settings("CPU")
    assert q.quality == want["quality"] and q.width == want["width"] and q.height == want["height"]
    assert q.spp >= want["spp_min"] and q.bounces >= want["bounces_min"]
    assert q.mis and q.power_light_sampling and q.sampler == want["sampler"]
    assert q.hbao == 0 and q.hbao_plus == 0 and q.fxaa == 0 and q.firefly_clamp == 0
    assert q.rr_depth == want["rr_depth"] and q.bvh_bins == want["bvh_bins"] and q.tile_size == want["tile_size"]
    g = bcgx.ultra_realism_settings("OpenCL GPU")
    assert g.spp >= 256 and g.bounces >= 16 and g.denoise and not g.adaptive_sampling
    assert g.mis and g.power_light_sampling and g.sampler == "Halton"  # the CUDA path keeps the CPU transport


def test_stress_scene_counts(orc, pins):
    spec, _ = scenes.stress_scene()
    s = orc.OracleScene.from_spec(spec)
    c = s.counts()
    assert c["prims"] == pins["stress_scene"]["spheres"] and c["lights"] == pins["stress_scene"]["lights"]


def test_photon_functions(orc, pins):
    """photonBudget, photonCellKey and photonRadius of NewCornellScene
    (renderer.go:1148-1182, 1636-1639) against the pure-Python restatement."""
    import struct
    from bcgx import scenes
    for lv, want in pins["photon_budget"].items():
        assert orc.lib().orc_photon_budget(int(lv)) == want
    for case in pins["photon_cell_key"]:
        assert format(orc.lib().orc_photon_cell_key(*case["c"]), "016x") == case["key"]
    spec, _ = scenes.cornell_reference_scene()
    ref = orc.OracleScene.from_spec(spec)
    for lv, bits in pins["photon_radius_cornell"].items():
        assert struct.pack("<d", ref.photon_radius(int(lv))).hex() == bits, lv


def test_photon_map_properties(orc):
    """buildPhotonMap on the Cornell-like room: the stop rule (the budget is
    checked before each emission, so the last one may overshoot by fewer than
    max(2, bounces) photons), append order by emission, every photon on a
    diffuse surface facing its normal, flux along a path never growing before
    Russian roulette rescales it; empty maps for levels outside 1-4."""
    import numpy as np
    import bcgx
    from bcgx import scenes
    spec, _ = scenes.cornell_reference_scene()
    ref = orc.OracleScene.from_spec(spec)
    st = bcgx.quality("Draft")
    st.bounces = 5
    for lv, budget in ((1, 512), (2, 2048)):
        st.photon_mapping = lv
        m = ref.photon_map(st, seed=3)
        ph = m["photons"]
        assert budget <= len(ph) < budget + max(2, st.bounces)
        em = ph[:, 9]
        assert np.all(np.diff(em) >= 0)
        # all but the last emission ran before the budget was reached
        last = em[-1]
        assert np.sum(em < last) < budget
        assert np.allclose(np.linalg.norm(ph[:, 3:6], axis=1), 1.0, atol=1e-9)
        assert np.all(ph[:, 6:9] >= 0) and np.all(ph[:, 6:9].max(axis=1) > 0)
        assert m["rays"] >= len(ph)
        assert m["radius"] > 0
    for lv in (0, 5):
        st.photon_mapping = lv
        assert len(ref.photon_map(st, seed=3)["photons"]) == 0


def test_window_render_equals_frame(orc):
    """A pixel window of the oracle's render (used for converged crops) holds the
    whole frame's pixels bit for bit, and a window outside the frame is refused."""
    spec, cam, st = scenes.cornell_box()
    st.width, st.height, st.spp = 64, 48, 4
    s = orc.OracleScene.from_spec(spec)
    full = s.render(cam, st, seed=3, threads=4)
    win = s.render(cam, st, seed=3, threads=4, window=(10, 7, 21, 13))
    assert win["linear"].shape == (13, 21, 3)
    assert np.array_equal(full["linear"][7:20, 10:31], win["linear"])
    assert np.array_equal(full["sumsq"][7:20, 10:31], win["sumsq"])
    with pytest.raises(ValueError):
        s.render(cam, st, window=(60, 0, 10, 4))


def test_triangle_closest_hit_against_the_reference_cpp(orc):
    """The oracle's Scene.Hit restatement (fp64 triHit, renderer.go:684-711,
    over the 32-bin SAH tree) against the closest hit of the reference's own C++
    engine (beamcast::hx::PackedScene::hit, source/src/hx.cpp:237-270: fp32
    Moller-Trumbore at hx.cpp:223-231 over its own BVH), on seeded random
    triangles and rays. The fixture holds the reference's answers
    (tests/golden/make_hx_golden.py); where the reference library is built here
    (oracle/_ref) it is run as well and must reproduce the fixture. The two tests
    differ only in precision (fp32 against fp64) and in their det threshold and
    t-range ends, which random rays do not meet: every ray has the same hit
    index, and t agrees to fp32 rounding of an ill-conditioned test."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "hx_closest.npz"))
    verts = scenes.random_triangle_verts(int(g["n_tris"]), int(g["tri_seed"]))
    rays = scenes.random_rays(int(g["n_rays"]), seed=int(g["ray_seed"]))
    live = orc.hx_reference_closest(verts, rays)
    if live is not None:
        assert np.array_equal(live[1], g["prim"]) and np.array_equal(live[0], g["t"])
    spec = scenes.random_triangles(int(g["n_tris"]), int(g["tri_seed"]))
    t_o, p_o, _ = orc.OracleScene.from_spec(spec).hit_f32(rays)
    assert np.array_equal(p_o, g["prim"])
    hit = p_o >= 0
    assert hit.sum() > 5000
    rel = np.abs(t_o[hit] - g["t"][hit]) / np.abs(t_o[hit])
    assert rel.max() < 2e-4 and np.percentile(rel, 99.9) < 2e-5

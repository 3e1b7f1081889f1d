"""Writes tests/golden/reference_pins.json.

Golden values pinned by the reference's own unit tests
(windows_portable/renderer_test.go) and by the deterministic functions of
renderer.go, computed here in pure Python independently of the C++ oracle:

* TestSamplingLevels (renderer_test.go:198-212): effectiveSPP = 24 for
  SPP 2 / MSAA 4 / TSAA 2; 4096 cap.
* TestPowerWeightedLightPDF (310-329): powerHeuristic(.5, .5) in [0.49, 0.51].
* TestFastAABBMatchesReference (361-413): the test's inline slab test,
  restated below, evaluated on the test's 3 boxes x 5 rays.
* TestCenterTileOrderIsPermutation (542-561): 7x5 tiles, first = (3, 2).
* TestUltraRealismPreset (846-864): preset fields.
* radicalInverse (renderer.go:1844-1858) for n = 1..256, bases 2 and 3, and
  pixelSampleRotation (1906-1915) on a grid of pixels: both are integer or
  fixed-order fp64 arithmetic, so Python floats reproduce them bit for bit.
* photonBudget (renderer.go:1148-1161) for levels -1..6, photonCellKey
  (1636-1639) on integer cells (int64 products wrapping, then XOR), and
  photonRadius (1163-1182) of NewCornellScene (2960-2979): Scene.Bounds
  (1137-1146) over AddTriangle's padded boxes (257-269) and AddSphere's (246-256).

Run: python tests/golden/make_golden.py
"""
import json
import os
import struct

HERE = os.path.dirname(os.path.abspath(__file__))


def f64_bits(x: float) -> str:
    return struct.pack("<d", x).hex()


def inline_slab(box, ray):
    """The inline reference of TestFastAABBMatchesReference (renderer_test.go:380-405)."""
    tmin, tmax = 1e-4, 1e30
    o, d = ray
    mn, mx = box
    for i in range(3):
        if abs(d[i]) < 1e-15:
            if o[i] < mn[i] or o[i] > mx[i]:
                return False
            continue
        inv = 1 / d[i]
        t0, t1 = (mn[i] - o[i]) * inv, (mx[i] - o[i]) * inv
        if inv < 0:
            t0, t1 = t1, t0
        if t0 > tmin:
            tmin = t0
        if t1 < tmax:
            tmax = t1
        if tmax <= tmin:
            return False
    return True


def radical_inverse(n: int, base: int) -> float:
    if base == 2:
        r = int(format(n, "064b")[::-1], 2)
        return float(r) * 5.421010862427522e-20
    inv_base = 1.0 / float(base)
    inv = inv_base
    result = 0.0
    while n > 0:
        digit = n % base
        result += float(digit) * inv
        n //= base
        inv *= inv_base
    return result


def pixel_sample_rotation(x: int, y: int):
    M = 0xFFFFFFFF
    h1 = ((x * 0x9E3779B1) & M) ^ ((y * 0x85EBCA77) & M)
    h1 ^= h1 >> 16
    h1 = (h1 * 0x7FEB352D) & M
    h1 ^= h1 >> 15
    h2 = h1 ^ 0x68BC21EB
    h2 ^= h2 >> 13
    inv = 1.0 / 4294967296.0
    return float(h1) * inv, float(h2) * inv


def photon_budget(level: int) -> int:
    return {1: 512, 2: 2048, 3: 8192, 4: 16384}.get(level, 0)


def photon_cell_key(x: int, y: int, z: int) -> int:
    m = (1 << 64) - 1
    return ((x * 73856093) & m) ^ ((y * 19349663) & m) ^ ((z * 83492791) & m)


def cornell_bounds():
    tris = [((-3, -2, -8), (3, -2, -8), (3, -2, -2)), ((-3, -2, -8), (3, -2, -2), (-3, -2, -2)),
            ((-3, -2, -8), (-3, -2, -2), (-3, 4, -2)), ((-3, -2, -8), (-3, 4, -2), (-3, 4, -8)),
            ((3, -2, -2), (3, -2, -8), (3, 4, -8)), ((3, -2, -2), (3, 4, -8), (3, 4, -2))]
    spheres = [((-.9, -1, -5.2), 1), ((1.1, -1.2, -4.2), .8), ((0, 3.2, -5), .65)]
    lo, hi = [float("inf")] * 3, [float("-inf")] * 3
    for t in tris:
        for k in range(3):
            lo[k] = min(lo[k], min(float(v[k]) for v in t) - 1e-6)
            hi[k] = max(hi[k], max(float(v[k]) for v in t) + 1e-6)
    for c, r in spheres:
        for k in range(3):
            lo[k] = min(lo[k], c[k] - r)
            hi[k] = max(hi[k], c[k] + r)
    return lo, hi


def photon_radius(lo, hi, level: int) -> float:
    e = [hi[k] - lo[k] for k in range(3)]
    diag = (e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) ** 0.5
    if diag < 1e-3:
        diag = 10.0
    base = diag * 0.03
    return {1: base * 1.8, 2: base * 1.2, 3: base * 0.85, 4: base * 0.6}.get(level, base)


def main():
    boxes = [((-1, -1, -1), (1, 1, 1)), ((2, -3, -4), (6, 5, 2)), ((-10, 0, -2), (-2, 0.1, 8))]
    rays = [((0, 0, 5), (0, 0, -1)), ((0, 0, 0), (1, 0, 0)), ((4, 10, 0), (0, -1, 0)), ((20, 20, 20), (1, 1, 1)),
            ((-5, 0.05, 10), (0, 0, -1))]
    aabb = [{"box": [list(b[0]), list(b[1])], "ray": [list(r[0]), list(r[1])], "hit": inline_slab(b, r)}
            for b in boxes for r in rays]
    pins = {
        "effective_spp": [{"spp": 2, "msaa": 4, "tsaa": 2, "want": 24}, {"spp": 200, "msaa": 8, "tsaa": 3, "want": 4096}],
        "power_heuristic_half": {"lo": 0.49, "hi": 0.51},
        "aabb_cases": aabb,
        "tile_order": {"tx": 7, "ty": 5, "first_xy": [3, 2]},
        "ultra_realism_cpu": {"quality": "Ultra Realism", "width": 2560, "height": 1440, "spp_min": 256,
                              "bounces_min": 16, "mis": True, "power_light_sampling": True, "sampler": "Halton",
                              "hbao": 0, "hbao_plus": 0, "fxaa": 0, "firefly_clamp": 0, "rr_depth": 6,
                              "bvh_bins": 32, "bvh_leaf_size": 4, "tile_size": 8},
        "radical_inverse": {str(b): [f64_bits(radical_inverse(n, b)) for n in range(1, 257)] for b in (2, 3)},
        "pixel_rotation": [{"x": x, "y": y, "r": [f64_bits(v) for v in pixel_sample_rotation(x, y)]}
                           for x in (0, 1, 17, 319, 2559) for y in (0, 1, 29, 239, 1439)],
        "stress_scene": {"spheres": 1 + 20 * 41 + 1, "lights": 1},
        "showcase_scene": {"spheres": 5, "lights": 1},
        "photon_budget": {str(lv): photon_budget(lv) for lv in range(-1, 7)},
        "photon_cell_key": [{"c": list(c), "key": format(photon_cell_key(*c), "016x")}
                            for c in ((0, 0, 0), (1, 2, 3), (-1, -1, -1), (-7, 12, -3), (100000, -250000, 3),
                                      (-(1 << 40), 1 << 41, -(1 << 42)), (2147483647, -2147483648, 1))],
        "photon_radius_cornell": {str(lv): f64_bits(photon_radius(*cornell_bounds(), lv)) for lv in range(0, 6)},
    }
    with open(os.path.join(HERE, "reference_pins.json"), "w") as f:
        json.dump(pins, f, indent=1, sort_keys=True)
    print("wrote", os.path.join(HERE, "reference_pins.json"))


if __name__ == "__main__":
    main()

"""Seeded synthetic workloads and the reference's built-in scenes.

A SceneSpec is builder-neutral (materials, spheres, triangles in insertion
order), so the same spec feeds the native builder (`to_scene`) and any
checker. Seeds and shapes:

  cornell_box      seed 0xBEAC0001: 5 walls (10 tris), 2 axis-aligned cubes
                   (24 tris, half-size U[0.15, 0.35]), one emissive quad (2 tris,
                   0.5 x 0.5, emission (17, 12, 4)), Lambertian albedo U[0.2, 0.8]^3.
  random_triangles seed 0xBEAC0002: centroids U[0,1]^3, two edges with lengths
                   LogNormal(-5, 0.5) along uniform directions.
  random_rays      origins U[0,1]^3, directions uniform on the sphere.
  icosphere_grid   seed 0xBEAC0003: 64 x 64 displaced frequency-5 icospheres
                   (500 tris each), ground quad, 64 emissive quads.
  batch_views      seed 0xBEAC0004: 4 random-triangle scenes (10k / 50k / 200k /
                   500k tris, one emissive quad each) and 64 views with
                   log-uniform sizes 128x128 .. 1920x1080, spp U{4..64},
                   8 bounces, cameras orbiting the unit cube.
  diff_scene       seed 0xBEAC0005: random triangles with 256 diffuse material
                   slots (true albedo U[0.2, 0.8]^3, start = true +- U[-0.1, 0.1])
                   and 8 emissive quads (true emission U[2, 10]^3); 512^2,
                   64 spp, 8 bounces, Russian roulette off.
The reference's own scenes (renderer.go:2944-2994) are test inputs only.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .scene import MAT_DIFFUSE, MAT_EMISSIVE, MAT_GLASS, MAT_METAL, Material, Scene
from .settings import Camera, RenderSettings, quality

SEED_CORNELL, SEED_TRIS, SEED_ULTRA, SEED_BATCH, SEED_DIFF = 0xBEAC0001, 0xBEAC0002, 0xBEAC0003, 0xBEAC0004, 0xBEAC0005
SEED_RAYS = 0xBEAC0003  # the ray-cast workload's rays


@dataclass
class SceneSpec:
    name: str = ""
    materials: list = field(default_factory=list)
    # primitives in insertion order: ("s", center, radius, mat) or ("t", start, count) runs
    spheres: list = field(default_factory=list)
    tri_verts: list = field(default_factory=list)   # list of (n, 9) arrays
    tri_mats: list = field(default_factory=list)    # list of (n,) arrays
    ops: list = field(default_factory=list)          # insertion order: ("s", idx) / ("t", idx)
    bvh_mode: str = "SAH"
    bvh_bins: int = 16
    bvh_leaf: int = 4

    def material(self, m: Material) -> int:
        self.materials.append(m)
        return len(self.materials) - 1

    def sphere(self, c, r, mat):
        self.spheres.append((tuple(float(v) for v in c), float(r), int(mat)))
        self.ops.append(("s", len(self.spheres) - 1))

    def triangles(self, verts, mats):
        v = np.ascontiguousarray(np.asarray(verts, dtype=np.float64).reshape(-1, 9))
        m = np.asarray(mats, dtype=np.int32)
        if m.ndim == 0:
            m = np.full(len(v), int(m), dtype=np.int32)
        self.tri_verts.append(v)
        self.tri_mats.append(np.ascontiguousarray(m))
        self.ops.append(("t", len(self.tri_verts) - 1))

    def n_triangles(self) -> int:
        return int(sum(len(v) for v in self.tri_verts))


def to_scene(spec: SceneSpec, build: bool = True) -> Scene:
    s = Scene(spec.name)
    for m in spec.materials:
        s.add_material(m)
    for kind, i in spec.ops:
        if kind == "s":
            c, r, m = spec.spheres[i]
            s.add_sphere(c, r, m)
        else:
            s.add_triangles(spec.tri_verts[i], spec.tri_mats[i])
    s.bvh_mode, s.bvh_bins, s.bvh_leaf = spec.bvh_mode, spec.bvh_bins, spec.bvh_leaf
    if build:
        s.build()
    return s


def quad(p0, p1, p2, p3):
    """Two triangles (p0, p1, p2), (p0, p2, p3)."""
    p0, p1, p2, p3 = (np.asarray(p, dtype=np.float64) for p in (p0, p1, p2, p3))
    return np.stack([np.concatenate([p0, p1, p2]), np.concatenate([p0, p2, p3])])


def box_tris(center, half):
    """12 triangles of an axis-aligned cube (face order of the reference's preset cube)."""
    c = np.asarray(center, dtype=np.float64)
    h = np.asarray(half, dtype=np.float64) * np.ones(3)
    v = [c + np.array(s) * h for s in ((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1),
                                       (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1))]
    faces = [(0, 1, 2), (0, 2, 3), (4, 6, 5), (4, 7, 6), (0, 4, 5), (0, 5, 1), (3, 2, 6), (3, 6, 7), (0, 3, 7),
             (0, 7, 4), (1, 5, 6), (1, 6, 2)]
    return np.stack([np.concatenate([v[a], v[b], v[c2]]) for a, b, c2 in faces])


# ---------------------------------------------------------------------------
# Workload 1: Cornell-style box, CPU-runnable.
def cornell_box(seed: int = SEED_CORNELL) -> tuple[SceneSpec, Camera, RenderSettings]:
    rng = np.random.default_rng(seed)
    sp = SceneSpec(name="cornell-box-c1", bvh_mode="SAH", bvh_bins=32, bvh_leaf=4)

    def albedo():
        return tuple(rng.uniform(0.2, 0.8, 3))

    walls = {
        "floor": quad((-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1)),
        "ceiling": quad((-1, 1, -1), (-1, 1, 1), (1, 1, 1), (1, 1, -1)),
        "back": quad((-1, -1, -1), (-1, 1, -1), (1, 1, -1), (1, -1, -1)),
        "left": quad((-1, -1, -1), (-1, -1, 1), (-1, 1, 1), (-1, 1, -1)),
        "right": quad((1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1)),
    }
    for _, tris in walls.items():
        m = sp.material(Material(MAT_DIFFUSE, albedo()))
        sp.triangles(tris, m)
    for k in range(2):
        h = rng.uniform(0.15, 0.35)
        x = rng.uniform(-0.6, -0.2) if k == 0 else rng.uniform(0.2, 0.6)
        z = rng.uniform(-0.5, 0.3)
        m = sp.material(Material(MAT_DIFFUSE, albedo()))
        sp.triangles(box_tris((x, -1 + h, z), h), m)
    light = sp.material(Material(MAT_EMISSIVE, emission=(17.0, 12.0, 4.0)))
    y = 0.999
    sp.triangles(quad((-0.25, y, -0.25), (0.25, y, -0.25), (0.25, y, 0.25), (-0.25, y, 0.25)), light)
    cam = Camera((0.0, 0.0, 3.4), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0)
    st = quality("Draft")
    st.width, st.height, st.spp, st.bounces = 320, 240, 16, 5
    st.msaa, st.tsaa = 1, 0
    st.sampler, st.mis, st.power_light_sampling = "Halton", True, True
    st.firefly_clamp, st.rr_depth = 0.0, 3
    st.adaptive_sampling = False
    st.denoise, st.bloom, st.taa, st.txaa, st.fxaa = False, 0, 0, 0, 0
    st.bvh_mode, st.bvh_bins, st.bvh_leaf_size = "SAH", 32, 4
    st.progressive_updates = False
    return sp, cam, st


# ---------------------------------------------------------------------------
# Workload 2: ray-cast microbenchmark.
def _unit_vectors(rng, n):
    v = rng.normal(size=(n, 3))
    l = np.linalg.norm(v, axis=1)
    bad = l < 1e-12
    while bad.any():
        v[bad] = rng.normal(size=(int(bad.sum()), 3))
        l = np.linalg.norm(v, axis=1)
        bad = l < 1e-12
    return v / l[:, None]


def random_triangle_verts(n: int, seed: int = SEED_TRIS, lo=0.0, hi=1.0) -> np.ndarray:
    """(n, 9) fp64 triangles; regenerates those AddTriangle would drop (|E1 x E2|^2 < 1e-18)."""
    rng = np.random.default_rng(seed)
    out = np.empty((n, 9), dtype=np.float64)
    filled = 0
    while filled < n:
        m = n - filled
        c = rng.uniform(lo, hi, size=(m, 3))
        l1 = rng.lognormal(-5.0, 0.5, size=m)
        l2 = rng.lognormal(-5.0, 0.5, size=m)
        e1 = _unit_vectors(rng, m) * l1[:, None]
        e2 = _unit_vectors(rng, m) * l2[:, None]
        a = c - (e1 + e2) / 3.0
        b = a + e1
        cc = a + e2
        # the same test as AddTriangle, on the vertices as stored
        ee1, ee2 = b - a, cc - a
        nn = np.cross(ee1, ee2)
        ok = (nn * nn).sum(axis=1) >= 1e-18
        k = int(ok.sum())
        out[filled:filled + k] = np.concatenate([a[ok], b[ok], cc[ok]], axis=1)
        filled += k
    return out


def random_triangles(n: int = 1_000_000, seed: int = SEED_TRIS) -> SceneSpec:
    sp = SceneSpec(name=f"random-tris-{n}", bvh_mode="SAH", bvh_bins=32, bvh_leaf=4)
    m = sp.material(Material(MAT_DIFFUSE, (0.7, 0.7, 0.7)))
    sp.triangles(random_triangle_verts(n, seed), m)
    return sp


def random_rays(n: int = 4_194_304, seed: int = SEED_RAYS, tmin: float = 1e-4, tmax: float = 1e30) -> np.ndarray:
    """(n, 8) float32 ray records (ox, oy, oz, tmin, dx, dy, dz, tmax)."""
    rng = np.random.default_rng(seed)
    r = np.empty((n, 8), dtype=np.float32)
    r[:, 0:3] = rng.uniform(0.0, 1.0, size=(n, 3))
    r[:, 3] = tmin
    r[:, 4:7] = _unit_vectors(rng, n)
    r[:, 7] = tmax
    return r


# ---------------------------------------------------------------------------
# The reference's built-in scenes (renderer.go:2944-2994), for structural tests.
def showcase_scene() -> tuple[SceneSpec, Camera]:
    sp = SceneSpec(name="Material Showcase")
    ground = sp.material(Material(MAT_DIFFUSE, (.55, .57, .6)))
    red = sp.material(Material(MAT_DIFFUSE, (.72, .12, .10)))
    gold = sp.material(Material(MAT_METAL, (.93, .72, .28), roughness=.08))
    glass = sp.material(Material(MAT_GLASS, (.98, .99, 1), ior=1.5))
    light = sp.material(Material(MAT_EMISSIVE, emission=(18, 15, 11)))
    sp.sphere((0, -1001, -4), 1000, ground)
    sp.sphere((-1.8, 0, -4.2), 1, red)
    sp.sphere((.25, 0, -3.2), 1, glass)
    sp.sphere((2.2, 0, -4.4), 1, gold)
    sp.sphere((0, 5, -4), .8, light)
    return sp, Camera((6, 3.2, 5.5), (0, 0, -4), (0, 1, 0), 40)


def cornell_reference_scene() -> tuple[SceneSpec, Camera]:
    sp = SceneSpec(name="Cornell-like Room")
    white = sp.material(Material(MAT_DIFFUSE, (.72, .72, .72)))
    red = sp.material(Material(MAT_DIFFUSE, (.70, .08, .06)))
    green = sp.material(Material(MAT_DIFFUSE, (.08, .55, .12)))
    glass = sp.material(Material(MAT_GLASS, (.98, .99, 1), ior=1.5))
    light = sp.material(Material(MAT_EMISSIVE, emission=(22, 20, 16)))
    T = [((-3, -2, -8), (3, -2, -8), (3, -2, -2), white), ((-3, -2, -8), (3, -2, -2), (-3, -2, -2), white),
         ((-3, -2, -8), (-3, -2, -2), (-3, 4, -2), red), ((-3, -2, -8), (-3, 4, -2), (-3, 4, -8), red),
         ((3, -2, -2), (3, -2, -8), (3, 4, -8), green), ((3, -2, -2), (3, 4, -8), (3, 4, -2), green)]
    for a, b, c, m in T:
        sp.triangles(np.concatenate([a, b, c]).reshape(1, 9), m)
    sp.sphere((-.9, -1, -5.2), 1, glass)
    sp.sphere((1.1, -1.2, -4.2), .8, white)
    sp.sphere((0, 3.2, -5), .65, light)
    return sp, Camera((0, .5, 5), (0, 0, -5), (0, 1, 0), 38)


def stress_scene() -> tuple[SceneSpec, Camera]:
    sp = SceneSpec(name="Stress Grid")
    ground = sp.material(Material(MAT_DIFFUSE, (.45, .48, .52)))
    blue = sp.material(Material(MAT_METAL, (.25, .52, .92), roughness=.12))
    light = sp.material(Material(MAT_EMISSIVE, emission=(25, 22, 18)))
    sp.sphere((0, -1001, -10), 1000, ground)
    for z in range(20):
        for x in range(-20, 21):
            sp.sphere((float(x) * .58, -.65, -3 - float(z) * .58), .22, blue)
    sp.sphere((0, 8, -8), 1.2, light)
    return sp, Camera((9, 5, 8), (0, -.5, -8), (0, 1, 0), 42)


# ---------------------------------------------------------------------------
# Workload 3: Ultra-Realism-shaped frame.
def _icosahedron():
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2],
                  [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5],
                  [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    return v / np.linalg.norm(v, axis=1, keepdims=True), f


def geodesic_sphere(freq: int = 5) -> np.ndarray:
    """Unit geodesic sphere: each icosahedron face split into freq^2 triangles, (20 freq^2, 3, 3)."""
    v, f = _icosahedron()
    tris = []
    for a, b, c in f:
        A, B, C = v[a], v[b], v[c]

        def P(i, j):  # barycentric grid point i along AB, j along AC
            p = A + (B - A) * (i / freq) + (C - A) * (j / freq)
            return p / np.linalg.norm(p)
        for i in range(freq):
            for j in range(freq - i):
                tris.append([P(i, j), P(i + 1, j), P(i, j + 1)])
                if i + j < freq - 1:
                    tris.append([P(i + 1, j), P(i + 1, j + 1), P(i, j + 1)])
    return np.array(tris)


def _value_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """Seeded trilinear value noise in [-1, 1] on an integer lattice (period 64)."""
    rng = np.random.default_rng(seed)
    lat = rng.uniform(-1, 1, size=(64, 64, 64))
    q = np.floor(p).astype(np.int64)
    f = p - q
    s = f * f * (3 - 2 * f)
    out = np.zeros(len(p))
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                w = ((s[:, 0] if dx else 1 - s[:, 0]) * (s[:, 1] if dy else 1 - s[:, 1]) *
                     (s[:, 2] if dz else 1 - s[:, 2]))
                out += w * lat[(q[:, 0] + dx) % 64, (q[:, 1] + dy) % 64, (q[:, 2] + dz) % 64]
    return out


def icosphere_grid(seed: int = SEED_ULTRA, n: int = 64, freq: int = 5, spacing: float = 1.0, radius: float = 0.4,
                   amplitude: float = 0.05, n_lights: int = 64) -> tuple[SceneSpec, Camera, RenderSettings]:
    """n x n displaced icospheres (20 freq^2 triangles each), a ground quad and n_lights
    emissive quads with LogNormal(1, 1) luminance; spheres are 50% diffuse
    (albedo U[0.2, 0.8]^3) and 50% rough metal (roughness U[0.05, 1]: the
    reference has no GGX material, its metal fuzz stands in)."""
    rng = np.random.default_rng(seed)
    sp = SceneSpec(name=f"icosphere-grid-{n}x{n}", bvh_mode="SAH", bvh_bins=32, bvh_leaf=4)
    base = geodesic_sphere(freq)                       # (T, 3, 3) on the unit sphere
    uniq, inv = np.unique(np.round(base.reshape(-1, 3), 12), axis=0, return_inverse=True)
    inv = inv.reshape(-1)
    ground = sp.material(Material(MAT_DIFFUSE, (0.45, 0.45, 0.45)))
    ext = n * spacing
    sp.triangles(quad((-1, 0, -1), (-1, 0, ext + 1), (ext + 1, 0, ext + 1), (ext + 1, 0, -1)), ground)
    mats = []
    for k in range(n * n):
        if rng.random() < 0.5:
            mats.append(sp.material(Material(MAT_DIFFUSE, tuple(rng.uniform(0.2, 0.8, 3)))))
        else:
            mats.append(sp.material(Material(MAT_METAL, tuple(rng.uniform(0.5, 0.95, 3)),
                                             roughness=float(rng.uniform(0.05, 1.0)))))
    verts = np.empty((n * n, len(base), 9))
    for k in range(n * n):
        cx, cz = (k % n + 0.5) * spacing, (k // n + 0.5) * spacing
        center = np.array([cx, radius + amplitude, cz])
        disp = _value_noise(uniq * 3.0 + np.array([k % 61, k // 61, 7.0]), seed) * amplitude
        pts = center + uniq * (radius + disp)[:, None]
        verts[k] = pts[inv].reshape(-1, 9)
    sp.triangles(verts.reshape(-1, 9), np.repeat(np.array(mats, dtype=np.int32), len(base)))
    for k in range(n_lights):
        lum = rng.lognormal(1.0, 1.0)
        tint = rng.uniform(0.6, 1.0, 3)
        em = tuple(tint / (0.2126 * tint[0] + 0.7152 * tint[1] + 0.0722 * tint[2]) * lum)
        m = sp.material(Material(MAT_EMISSIVE, emission=em))
        x, z = rng.uniform(0, ext, 2)
        s, y = rng.uniform(0.5, 1.5), rng.uniform(2.5, 4.0)
        sp.triangles(quad((x, y, z), (x + s, y, z), (x + s, y, z + s), (x, y, z + s)), m)
    cam = Camera((ext * 0.5, ext * 0.35, -ext * 0.25), (ext * 0.5, 0.0, ext * 0.45), (0, 1, 0), 50.0)
    st = quality("Ultra Realism")
    st.adaptive_sampling = False  # equal spp, as the reference's own benchmark recipe (benchmark.go:82)
    st.progressive_updates = False
    return sp, cam, st


# ---------------------------------------------------------------------------
# Workload 4: many views over a resident scene set.
def batch_scene(n_tris: int, seed: int) -> SceneSpec:
    """The random-triangle generator in the unit cube, plus one emissive quad above it."""
    sp = SceneSpec(name=f"batch-tris-{n_tris}", bvh_mode="SAH", bvh_bins=32, bvh_leaf=4)
    m = sp.material(Material(MAT_DIFFUSE, (0.7, 0.7, 0.7)))
    sp.triangles(random_triangle_verts(n_tris, seed), m)
    e = sp.material(Material(MAT_EMISSIVE, emission=(8.0, 7.0, 6.0)))
    sp.triangles(quad((0.25, 1.3, 0.25), (0.75, 1.3, 0.25), (0.75, 1.3, 0.75), (0.25, 1.3, 0.75)), e)
    return sp


def batch_views(seed: int = SEED_BATCH, n_views: int = 64, sizes=(10_000, 50_000, 200_000, 500_000),
                max_side: tuple[int, int] = (1920, 1080), spp_range: tuple[int, int] = (4, 64), bounces: int = 8):
    """Scenes and views of the batching workload: view v renders scene v mod len(sizes)
    at W = round(128 * r_w^t), H = round(128 * r_h^t), t ~ U[0, 1] (log-uniform from
    128 x 128 up to max_side), spp ~ U{spp_range}, from a seeded orbit camera."""
    rng = np.random.default_rng(seed)
    specs = [batch_scene(n, seed + 1 + k) for k, n in enumerate(sizes)]
    rw, rh = max_side[0] / 128.0, max_side[1] / 128.0
    views = []
    for v in range(n_views):
        t = rng.uniform()
        W, H = int(round(128 * rw ** t)), int(round(128 * rh ** t))
        spp = int(rng.integers(spp_range[0], spp_range[1] + 1))
        az, el = rng.uniform(0, 2 * np.pi), rng.uniform(0.1, 0.6)
        dist = rng.uniform(1.8, 2.6)
        c = np.array([0.5, 0.5, 0.5])
        pos = c + dist * np.array([np.cos(el) * np.cos(az), np.sin(el), np.cos(el) * np.sin(az)])
        cam = Camera(tuple(pos), tuple(c), (0, 1, 0), 45.0)
        st = quality("Draft")
        st.width, st.height, st.spp, st.bounces = W, H, spp, bounces
        st.msaa, st.tsaa = 1, 0
        st.sampler, st.mis, st.power_light_sampling = "Halton", True, True
        st.firefly_clamp, st.rr_depth, st.adaptive_sampling = 0.0, 4, False
        st.denoise, st.bloom = False, 0
        st.seed = seed + 0x100 + v
        views.append((v % len(sizes), cam, st))
    return specs, views


# ---------------------------------------------------------------------------
# Workload 5: inverse rendering of material parameters.
@dataclass
class DiffProblem:
    spec: SceneSpec
    cam: Camera
    settings: RenderSettings
    albedo_materials: np.ndarray   # (n_slots,) material indices
    emission_materials: np.ndarray  # (n_lights,)
    true_params: np.ndarray         # (n_slots + n_lights, 3) float32
    init_params: np.ndarray         # (n_slots + n_lights, 3) float32


def diff_scene(seed: int = SEED_DIFF, n_tris: int = 200_000, n_slots: int = 256, n_lights: int = 8,
               width: int = 512, height: int = 512, spp: int = 64, bounces: int = 8) -> DiffProblem:
    """Random triangles in the unit cube, each on one of n_slots diffuse
    materials, lit by n_lights emissive quads above the cube and the sky."""
    rng = np.random.default_rng(seed)
    sp = SceneSpec(name=f"diff-tris-{n_tris}", bvh_mode="SAH", bvh_bins=32, bvh_leaf=4)
    true_alb = rng.uniform(0.2, 0.8, (n_slots, 3))
    init_alb = np.clip(true_alb + rng.uniform(-0.1, 0.1, (n_slots, 3)), 0.02, 0.98)
    alb_mats = np.array([sp.material(Material(MAT_DIFFUSE, tuple(c))) for c in init_alb], dtype=np.int32)
    true_em = rng.uniform(2.0, 10.0, (n_lights, 3))
    init_em = true_em + rng.uniform(-1.0, 1.0, (n_lights, 3))
    em_mats = np.array([sp.material(Material(MAT_EMISSIVE, emission=tuple(e))) for e in init_em], dtype=np.int32)
    verts = random_triangle_verts(n_tris, seed + 1)
    sp.triangles(verts, alb_mats[rng.integers(0, n_slots, n_tris)])
    for k in range(n_lights):
        x, z = 0.125 + 0.25 * (k % 4), 0.25 + 0.5 * (k // 4) if n_lights > 4 else 0.5
        s = 0.09
        sp.triangles(quad((x - s, 1.25, z - s), (x + s, 1.25, z - s), (x + s, 1.25, z + s), (x - s, 1.25, z + s)),
                     em_mats[k])
    cam = Camera((0.5, 1.1, -1.1), (0.5, 0.45, 0.5), (0, 1, 0), 45.0)
    st = quality("Draft")
    st.width, st.height, st.spp, st.bounces = width, height, spp, bounces
    st.msaa, st.tsaa = 1, 0
    st.sampler, st.mis, st.power_light_sampling = "Halton", True, True
    st.firefly_clamp, st.rr_depth, st.adaptive_sampling = 0.0, bounces, False
    st.denoise, st.bloom = False, 0
    st.seed = seed
    true_p = np.concatenate([true_alb, true_em]).astype(np.float32)
    init_p = np.concatenate([init_alb, init_em]).astype(np.float32)
    return DiffProblem(sp, cam, st, alb_mats, em_mats, true_p, init_p)

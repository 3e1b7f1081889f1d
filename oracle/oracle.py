"""Test infrastructure only: ctypes wrapper of the fp64 CPU oracle.

The oracle restates windows_portable/renderer.go (see bc_oracle.h). It is
imported by tests, by the smoke check and by the CPU-baseline leg of the
benchmark, never by the product path. Builds with `make -C oracle`.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libbcoracle.so")
P = C.POINTER
f64p, i32p, i64p, u8p, u32p, f32p = P(C.c_double), P(C.c_int32), P(C.c_int64), P(C.c_uint8), P(C.c_uint32), P(C.c_float)


class OrcSettings(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("bounces", C.c_int32),
                ("msaa", C.c_int32), ("tsaa", C.c_int32), ("sampler", C.c_int32), ("mis", C.c_int32),
                ("power_light", C.c_int32), ("firefly_clamp", C.c_double), ("rr_depth", C.c_int32),
                ("adaptive", C.c_int32), ("adaptive_threshold", C.c_double), ("tile", C.c_int32),
                ("integrator", C.c_int32), ("photon_mapping", C.c_int32), ("photon_seed", C.c_int64)]

_INTEGRATOR_CODE = {"Path Tracing": 0, "Recursive Ray Tracing": 1, "Photon Mapping": 2}


def _orc_settings(st, tile=8, photon_seed=None):
    return OrcSettings(width=st.width, height=st.height, spp=st.spp, bounces=st.bounces, msaa=st.msaa,
                       tsaa=st.tsaa, sampler={"Random": 0, "Halton": 1, "R2": 2}[st.sampler], mis=int(st.mis),
                       power_light=int(st.power_light_sampling), firefly_clamp=float(st.firefly_clamp),
                       rr_depth=st.rr_depth, adaptive=int(st.adaptive_sampling),
                       adaptive_threshold=float(st.adaptive_threshold), tile=tile,
                       integrator=_INTEGRATOR_CODE[getattr(st, "integrator", "Path Tracing")],
                       photon_mapping=int(getattr(st, "photon_mapping", 0)),
                       photon_seed=-1 if photon_seed is None else int(photon_seed))


_SIG = [
    ("orc_scene_new", C.c_void_p, []), ("orc_scene_free", None, [C.c_void_p]),
    ("orc_scene_set_bvh", None, [C.c_void_p, C.c_char_p, C.c_int, C.c_int]),
    ("orc_add_material", C.c_int, [C.c_void_p, C.c_int, f64p, C.c_double, C.c_double, f64p]),
    ("orc_set_material", C.c_int, [C.c_void_p, C.c_int, f64p, f64p]),
    ("orc_hbao", None, [f64p, f64p, C.c_int, C.c_int, C.c_int, C.c_int, f64p]),
    ("orc_temporal", None, [f64p, f64p, C.c_int, C.c_int, f64p, f64p, f64p, C.c_double, f64p]),
    ("orc_temporal_weight", C.c_double, [C.c_int, C.c_int, C.c_int]),
    ("orc_debug_view", None, [f64p, f64p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, f64p]),
    ("orc_upscale", None, [f64p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, f64p]),
    ("orc_sharpen", None, [f64p, C.c_int, C.c_int, C.c_double, f64p]),
    ("orc_fxaa", None, [f64p, C.c_int, C.c_int, C.c_int, f64p]),
    ("orc_txaa", None, [f64p, C.c_int, C.c_int, C.c_int, f64p]),
    ("orc_internal_size", None, [C.c_int, C.c_int, C.c_int, P(C.c_int)]),
    ("orc_project_point", C.c_int, [f64p, f64p, C.c_int, C.c_int, P(C.c_int)]),
    ("orc_add_sphere", None, [C.c_void_p, f64p, C.c_double, C.c_int]),
    ("orc_add_triangles", None, [C.c_void_p, C.c_int64, f64p, i32p]),
    ("orc_build", None, [C.c_void_p]), ("orc_refit", None, [C.c_void_p]),
    ("orc_translate_prim", None, [C.c_void_p, C.c_int, f64p]),
    ("orc_counts", None, [C.c_void_p, i64p]),
    ("orc_get_nodes", None, [C.c_void_p, f64p, i32p, i32p, i32p, i32p]),
    ("orc_get_order", None, [C.c_void_p, i32p]), ("orc_get_escapes", None, [C.c_void_p, i32p]),
    ("orc_get_lights", None, [C.c_void_p, i32p, f64p, f64p]),
    ("orc_get_prims", None, [C.c_void_p, i32p, i32p, f64p, f64p, f64p, f64p, f64p, f64p, f64p]),
    ("orc_get_materials", None, [C.c_void_p, i32p, f64p, f64p, f64p, f64p]),
    ("orc_aabb_hit", C.c_int, [f64p, f64p, C.c_double, C.c_double, f64p]),
    ("orc_hit_batch", None, [C.c_void_p, C.c_int64, f64p, C.c_double, C.c_double, C.c_int, f64p, i32p, i64p, C.c_int]),
    ("orc_hit_batch_f32", None, [C.c_void_p, C.c_int64, f32p, f64p, i32p, i64p, C.c_int]),
    ("orc_occluded_batch_f32", None, [C.c_void_p, C.c_int64, f32p, u8p, i64p, C.c_int]),
    ("orc_tie_sets_f32", None, [C.c_void_p, C.c_int64, f32p, C.c_int, i32p, i32p]),
    ("orc_occluded_batch", None, [C.c_void_p, C.c_int64, f64p, f64p, C.c_double, u8p, C.c_int]),
    ("orc_radical_inverse", C.c_double, [C.c_uint64, C.c_uint64]),
    ("orc_pixel_sample_rotation", None, [C.c_int, C.c_int, f64p]),
    ("orc_effective_spp", C.c_int, [C.c_int, C.c_int, C.c_int]),
    ("orc_build_sample_sequence", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, f64p, f64p]),
    ("orc_cos_hemisphere", None, [f64p, C.c_uint64, C.c_int64, f64p]),
    ("orc_unit_vectors", None, [C.c_uint64, C.c_int64, f64p]),
    ("orc_rng_floats", None, [C.c_uint64, C.c_uint64, C.c_uint64, C.c_int64, f64p]),
    ("orc_make_tile_order", None, [C.c_int, C.c_int, C.c_char_p, i32p]),
    ("orc_power_heuristic", C.c_double, [C.c_double, C.c_double]),
    ("orc_light_selection_pdf", C.c_double, [C.c_void_p, C.c_int, C.c_int]),
    ("orc_clamp_firefly", None, [f64p, C.c_double, f64p]),
    ("orc_camera_basis", None, [f64p, C.c_double, f64p]),
    ("orc_render", C.c_int, [C.c_void_p, f64p, P(OrcSettings), C.c_uint64, C.c_int, f64p, f64p, f64p, i64p]),
    ("orc_render_window", C.c_int, [C.c_void_p, f64p, P(OrcSettings), C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_uint64, C.c_int, f64p, f64p, f64p, i64p]),
    ("orc_photon_budget", C.c_int, [C.c_int]),
    ("orc_photon_cell_key", C.c_uint64, [C.c_int64, C.c_int64, C.c_int64]),
    ("orc_photon_radius", C.c_double, [C.c_void_p, C.c_int]),
    ("orc_photon_map", C.c_int64, [C.c_void_p, P(OrcSettings), C.c_uint64, C.c_int64, f64p, f64p]),
    ("orc_photon_gather", None, [C.c_void_p, P(OrcSettings), C.c_uint64, C.c_int64, f64p, f64p]),
    ("orc_atrous", None, [f64p, f64p, C.c_int, C.c_int, C.c_int, f64p]),
    ("orc_bloom", None, [f64p, C.c_int, C.c_int, C.c_int, f64p]),
    ("orc_tone_map", None, [f64p, C.c_int64, C.c_int, f64p]),
    ("orc_to_rgba", None, [f64p, C.c_int64, C.c_double, C.c_double, C.c_int, u32p]),
]

_lib = None


REF_TREE = "/root/reference"  # the reference's sources, where this repository is built from them
HX_LIB = os.path.join(HERE, "_ref", "libhxref.so")


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if os.path.isdir(os.path.join(REF_TREE, "source", "src")):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_TREE}"], check=True)


def hx_reference_closest(verts9, rays8):
    """Closest hit of the reference's own C++ code (beamcast::hx::PackedScene,
    built by `make -C oracle ref` into _ref/), or None when it was not built.
    verts9: (n, 9) triangle vertices; rays8: (m, 8) float32 rays. Returns
    (t float32, prim int32) in the triangles' numbering."""
    if not os.path.exists(HX_LIB):
        return None
    L = C.CDLL(HX_LIB)
    f = L.hxref_closest
    f.restype = C.c_int
    f.argtypes = [C.c_int, C.POINTER(C.c_double), C.c_int64, C.POINTER(C.c_float), C.POINTER(C.c_int32),
                  C.POINTER(C.c_float)]
    v = np.ascontiguousarray(verts9, dtype=np.float64).reshape(-1, 9)
    r = np.ascontiguousarray(rays8, dtype=np.float32).reshape(-1, 8)
    prim = np.empty(len(r), np.int32)
    t = np.empty(len(r), np.float32)
    if f(len(v), _p(v, C.c_double), len(r), _p(r, C.c_float), _p(prim, C.c_int32), _p(t, C.c_float)) != 0:
        raise RuntimeError("the reference's closest hit threw")
    return t, prim


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        for name, res, args in _SIG:
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        _lib = L
    return _lib


def _p(a, ct):
    return None if a is None else a.ctypes.data_as(P(ct))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class OracleScene:
    """The Go Scene restated in fp64 (renderer.go:225-939)."""

    def __init__(self):
        self.h = lib().orc_scene_new()

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_scene_free(self.h)
            self.h = None

    @classmethod
    def from_spec(cls, spec, build=True, mode=None, bins=None, leaf=None):
        s = cls()
        for m in spec.materials:
            s.add_material(m.kind, m.color, m.roughness, m.ior, m.emission)
        for kind, i in spec.ops:
            if kind == "s":
                c, r, m = spec.spheres[i]
                s.add_sphere(c, r, m)
            else:
                s.add_triangles(spec.tri_verts[i], spec.tri_mats[i])
        s.set_bvh(mode or spec.bvh_mode, bins or spec.bvh_bins, leaf or spec.bvh_leaf)
        if build:
            s.build()
        return s

    def set_bvh(self, mode, bins, leaf):
        lib().orc_scene_set_bvh(self.h, mode.encode(), int(bins), int(leaf))

    def add_material(self, kind, color, rough, ior, emission):
        return lib().orc_add_material(self.h, int(kind), _p(_f64(color), C.c_double), float(rough), float(ior),
                                      _p(_f64(emission), C.c_double))

    def set_material(self, idx, color=None, emission=None):
        """In-place color / emission change (the light CDF of build() is kept)."""
        c = _f64(color) if color is not None else None
        e = _f64(emission) if emission is not None else None
        rc = lib().orc_set_material(self.h, int(idx), _p(c, C.c_double), _p(e, C.c_double))
        if rc != 0:
            raise IndexError(f"material {idx} out of range")

    def add_sphere(self, c, r, mat):
        lib().orc_add_sphere(self.h, _p(_f64(c), C.c_double), float(r), int(mat))

    def add_triangles(self, verts, mats):
        v = _f64(np.asarray(verts).reshape(-1, 9))
        m = np.ascontiguousarray(np.broadcast_to(np.asarray(mats, dtype=np.int32), (len(v),)))
        lib().orc_add_triangles(self.h, len(v), _p(v, C.c_double), _p(m, C.c_int32))

    def build(self):
        lib().orc_build(self.h)

    def refit(self):
        lib().orc_refit(self.h)

    def translate(self, idx, d):
        lib().orc_translate_prim(self.h, int(idx), _p(_f64(d), C.c_double))

    def counts(self):
        o = np.zeros(6, dtype=np.int64)
        lib().orc_counts(self.h, _p(o, C.c_int64))
        return dict(zip(("prims", "nodes", "lights", "materials", "topology_rev", "geometry_rev"), o.tolist()))

    def nodes(self):
        n = self.counts()["nodes"]
        box = np.zeros((n, 6)); l = np.zeros(n, np.int32); r = np.zeros(n, np.int32)
        s = np.zeros(n, np.int32); c = np.zeros(n, np.int32)
        lib().orc_get_nodes(self.h, _p(box, C.c_double), _p(l, C.c_int32), _p(r, C.c_int32), _p(s, C.c_int32),
                            _p(c, C.c_int32))
        return box, l, r, s, c

    def order(self):
        o = np.zeros(self.counts()["prims"], np.int32)
        lib().orc_get_order(self.h, _p(o, C.c_int32))
        return o

    def escapes(self):
        e = np.zeros(self.counts()["nodes"], np.int32)
        lib().orc_get_escapes(self.h, _p(e, C.c_int32))
        return e

    def lights(self):
        c = self.counts()
        sp = np.zeros(c["lights"], np.int32); cdf = np.zeros(c["lights"]); pdf = np.zeros(c["prims"])
        lib().orc_get_lights(self.h, _p(sp, C.c_int32), _p(cdf, C.c_double), _p(pdf, C.c_double))
        return sp, cdf, pdf

    def arrays(self):
        """The built scene as the hand-off arrays of bc_scene_desc (a Go caller's view)."""
        import importlib
        bcgx = importlib.import_module("bcgx")
        c = self.counts()
        n, nm = c["prims"], c["materials"]
        kind = np.zeros(n, np.int32); mat = np.zeros(n, np.int32); cen = np.zeros((n, 3)); rad = np.zeros(n)
        a = np.zeros((n, 3)); e1 = np.zeros((n, 3)); e2 = np.zeros((n, 3)); nn = np.zeros((n, 3)); pb = np.zeros((n, 6))
        lib().orc_get_prims(self.h, _p(kind, C.c_int32), _p(mat, C.c_int32), _p(cen, C.c_double), _p(rad, C.c_double),
                            _p(a, C.c_double), _p(e1, C.c_double), _p(e2, C.c_double), _p(nn, C.c_double),
                            _p(pb, C.c_double))
        mk = np.zeros(nm, np.int32); mc = np.zeros((nm, 3)); mr = np.zeros(nm); mi = np.zeros(nm); me = np.zeros((nm, 3))
        lib().orc_get_materials(self.h, _p(mk, C.c_int32), _p(mc, C.c_double), _p(mr, C.c_double),
                                _p(mi, C.c_double), _p(me, C.c_double))
        box, l, r, s, cn = self.nodes()
        ls, cdf, pdf = self.lights()
        return bcgx.SceneArrays(mat_kind=mk, mat_color=mc, mat_roughness=mr, mat_ior=mi, mat_emission=me,
                                prim_kind=kind, prim_material=mat, prim_center=cen, prim_radius=rad, prim_a=a,
                                prim_e1=e1, prim_e2=e2, prim_normal=nn, node_box=box, node_left=l, node_right=r,
                                node_start=s, node_count=cn, order=self.order(), light_spheres=ls, light_cdf=cdf,
                                light_pdf_by_prim=pdf)

    # -- queries --
    def hit(self, origins, dirs, tmin=1e-4, tmax=1e30, threaded=False, threads=0):
        o = _f64(origins).reshape(-1, 3); d = _f64(dirs).reshape(-1, 3)
        rays = np.ascontiguousarray(np.concatenate([o, d], axis=1))
        n = len(rays)
        t = np.zeros(n); p = np.zeros(n, np.int32); cnt = np.zeros(3, np.int64)
        lib().orc_hit_batch(self.h, n, _p(rays, C.c_double), tmin, tmax, 1 if threaded else 0, _p(t, C.c_double),
                            _p(p, C.c_int32), _p(cnt, C.c_int64), threads)
        return t, p, cnt

    def hit_f32(self, rays8, threads=0):
        r = np.ascontiguousarray(rays8, dtype=np.float32).reshape(-1, 8)
        n = len(r)
        t = np.zeros(n); p = np.zeros(n, np.int32); cnt = np.zeros(3, np.int64)
        lib().orc_hit_batch_f32(self.h, n, _p(r, C.c_float), _p(t, C.c_double), _p(p, C.c_int32), _p(cnt, C.c_int64),
                                threads)
        return t, p, cnt

    def tie_sets_f32(self, rays8, k=8):
        """(count, members) of primitives at exactly the minimal fp64 distance (brute force)."""
        r = np.ascontiguousarray(rays8, dtype=np.float32).reshape(-1, 8)
        cnt = np.zeros(len(r), np.int32)
        mem = np.full((len(r), k), -1, np.int32)
        lib().orc_tie_sets_f32(self.h, len(r), _p(r, C.c_float), k, _p(cnt, C.c_int32), _p(mem, C.c_int32))
        return cnt, mem

    def occluded_f32(self, rays8, threads=0):
        r = np.ascontiguousarray(rays8, dtype=np.float32).reshape(-1, 8)
        out = np.zeros(len(r), np.uint8); cnt = np.zeros(3, np.int64)
        lib().orc_occluded_batch_f32(self.h, len(r), _p(r, C.c_float), _p(out, C.c_uint8), _p(cnt, C.c_int64), threads)
        return out.astype(bool), cnt

    def occluded(self, origins, dirs, tmax, tmin=1e-4, threads=0):
        o = _f64(origins).reshape(-1, 3); d = _f64(dirs).reshape(-1, 3)
        rays = np.ascontiguousarray(np.concatenate([o, d], axis=1))
        tm = _f64(np.broadcast_to(np.asarray(tmax, dtype=np.float64), (len(rays),)))
        out = np.zeros(len(rays), np.uint8)
        lib().orc_occluded_batch(self.h, len(rays), _p(rays, C.c_double), _p(tm, C.c_double), tmin,
                                 _p(out, C.c_uint8), threads)
        return out.astype(bool)

    def light_selection_pdf(self, prim, power=True):
        return lib().orc_light_selection_pdf(self.h, int(prim), 1 if power else 0)

    def render(self, cam, st, seed=1, threads=0, tile=8, photon_seed=None, window=None):
        """Returns dict(linear, sumsq, guides (H,W,11), stats). photon_seed: seed of
        the photon map's emission streams (default: `seed`). window = (x0, y0, w, h)
        renders only those pixels of the frame (arrays of shape (h, w, ...)), each
        equal to the whole frame's pixel."""
        cs = _orc_settings(st, tile, photon_seed)
        cam10 = _f64(list(cam.position) + list(cam.target) + list(cam.up) + [cam.fov])
        W, H = (st.width, st.height) if window is None else (int(window[2]), int(window[3]))
        lin = np.zeros((H, W, 3)); sq = np.zeros((H, W, 3)); g = np.zeros((H, W, 11)); stats = np.zeros(6, np.int64)
        if window is None:
            lib().orc_render(self.h, _p(cam10, C.c_double), C.byref(cs), int(seed), int(threads),
                             _p(lin, C.c_double), _p(sq, C.c_double), _p(g, C.c_double), _p(stats, C.c_int64))
        else:
            x0, y0 = int(window[0]), int(window[1])
            if lib().orc_render_window(self.h, _p(cam10, C.c_double), C.byref(cs), x0, y0, W, H, int(seed),
                                       int(threads), _p(lin, C.c_double), _p(sq, C.c_double), _p(g, C.c_double),
                                       _p(stats, C.c_int64)) != 0:
                raise ValueError(f"window {tuple(window)} outside the {st.width}x{st.height} frame")
        return {"linear": lin, "sumsq": sq, "guides": g,
                "stats": dict(zip(("segments", "shadow", "boxes", "tris", "spheres", "photon_rays"),
                                  stats.tolist()))}

    def photon_radius(self, level):
        return lib().orc_photon_radius(self.h, int(level))

    def photon_map(self, st, seed=1):
        """buildPhotonMap: dict(photons (n, 10): P, N, flux, emission index, in append
        order; radius; rays)."""
        cs = _orc_settings(st)
        cap = 16384 + max(2, st.bounces) + 16
        out = np.zeros((cap, 10)); o3 = np.zeros(3)
        n = lib().orc_photon_map(self.h, C.byref(cs), int(seed), cap, _p(out, C.c_double), _p(o3, C.c_double))
        return {"photons": out[:min(n, cap)].copy(), "radius": float(o3[0]), "rays": int(o3[1])}

    def photon_gather(self, st, points, normals, seed=1):
        """PhotonMap.gather(p, n, 64) at each point over the map of (st, seed)."""
        pn = np.ascontiguousarray(np.concatenate([np.asarray(points, np.float64),
                                                  np.asarray(normals, np.float64)], axis=1))
        out = np.zeros((len(pn), 3))
        lib().orc_photon_gather(self.h, C.byref(_orc_settings(st)), int(seed), len(pn), _p(pn, C.c_double),
                                _p(out, C.c_double))
        return out


def aabb_hit(box6, ray6, tmin=1e-4, tmax=1e30):
    near = C.c_double(0)
    ok = lib().orc_aabb_hit(_p(_f64(box6), C.c_double), _p(_f64(ray6), C.c_double), tmin, tmax, C.byref(near))
    return bool(ok), near.value


def radical_inverse(n, base):
    return lib().orc_radical_inverse(int(n), int(base))


def pixel_sample_rotation(x, y):
    o = np.zeros(2)
    lib().orc_pixel_sample_rotation(int(x), int(y), _p(o, C.c_double))
    return float(o[0]), float(o[1])


def effective_spp(spp, msaa, tsaa):
    return lib().orc_effective_spp(int(spp), int(msaa), int(tsaa))


def sample_sequence(sampler, spp, msaa=1, tsaa=0):
    n = effective_spp(spp, msaa, tsaa)
    X = np.zeros(n); Y = np.zeros(n)
    k = lib().orc_build_sample_sequence(int(sampler), int(spp), int(msaa), int(tsaa), _p(X, C.c_double), _p(Y, C.c_double))
    return X[:k], Y[:k]


def cos_hemisphere(n3, seed, count):
    out = np.zeros((count, 3))
    lib().orc_cos_hemisphere(_p(_f64(n3), C.c_double), int(seed), int(count), _p(out, C.c_double))
    return out


def rng_floats(seed, pixel, sample, count):
    out = np.zeros(count)
    lib().orc_rng_floats(int(seed), int(pixel), int(sample), int(count), _p(out, C.c_double))
    return out


def tile_order(tx, ty, mode="Center"):
    o = np.zeros(tx * ty, np.int32)
    lib().orc_make_tile_order(tx, ty, mode.encode(), _p(o, C.c_int32))
    return o


def power_heuristic(a, b):
    return lib().orc_power_heuristic(float(a), float(b))


def clamp_firefly(c, limit):
    o = np.zeros(3)
    lib().orc_clamp_firefly(_p(_f64(c), C.c_double), float(limit), _p(o, C.c_double))
    return o


def camera_basis(cam, aspect):
    cam10 = _f64(list(cam.position) + list(cam.target) + list(cam.up) + [cam.fov])
    o = np.zeros(12)
    lib().orc_camera_basis(_p(cam10, C.c_double), float(aspect), _p(o, C.c_double))
    return o.reshape(4, 3)


def atrous(img, guides11, iters):
    H, W = img.shape[:2]
    out = np.zeros((H, W, 3))
    lib().orc_atrous(_p(_f64(img), C.c_double), _p(_f64(guides11), C.c_double), W, H, int(iters), _p(out, C.c_double))
    return out


def bloom(img, level):
    H, W = img.shape[:2]
    out = np.zeros((H, W, 3))
    lib().orc_bloom(_p(_f64(img), C.c_double), W, H, int(level), _p(out, C.c_double))
    return out


def tone_map(img, hdr):
    a = _f64(img).reshape(-1, 3)
    out = np.zeros_like(a)
    lib().orc_tone_map(_p(a, C.c_double), len(a), int(hdr), _p(out, C.c_double))
    return out.reshape(np.shape(img))


def to_rgba(img, exposure, gamma, hdr):
    a = _f64(img).reshape(-1, 3)
    out = np.zeros(len(a), np.uint32)
    lib().orc_to_rgba(_p(a, C.c_double), len(a), float(exposure), float(gamma), int(hdr), _p(out, C.c_uint32))
    return out.reshape(np.shape(img)[:-1])


# ---- the rest of RenderState.Start's post stack (bc_oracle_post.cpp) ----------------
def _img_out(h, w):
    return np.zeros((h, w, 3))


def hbao(img, guides11, level, plus):
    H, W = img.shape[:2]
    out = _img_out(H, W)
    lib().orc_hbao(_p(_f64(img), C.c_double), _p(_f64(guides11), C.c_double), W, H, int(level), int(plus),
                   _p(out, C.c_double))
    return out


def cam10(cam):
    return _f64(list(cam.position) + list(cam.target) + list(cam.up) + [cam.fov])


def temporal(cur, guides11, prev, prev_guides11, prev_cam, weight):
    H, W = cur.shape[:2]
    out = _img_out(H, W)
    lib().orc_temporal(_p(_f64(cur), C.c_double), _p(_f64(guides11), C.c_double), W, H, _p(_f64(prev), C.c_double),
                       _p(_f64(prev_guides11), C.c_double), _p(cam10(prev_cam), C.c_double), float(weight),
                       _p(out, C.c_double))
    return out


def temporal_weight(taa, tsaa, txaa):
    return lib().orc_temporal_weight(int(taa), int(tsaa), int(txaa))


def debug_view(lin, guides11, mode, hbao_level=0, hbao_plus=0):
    H, W = lin.shape[:2]
    out = _img_out(H, W)
    lib().orc_debug_view(_p(_f64(lin), C.c_double), _p(_f64(guides11), C.c_double), W, H, int(mode), int(hbao_level),
                         int(hbao_plus), _p(out, C.c_double))
    return out


def upscale(src, dw, dh, mode):
    sh, sw = src.shape[:2]
    out = _img_out(dh, dw)
    lib().orc_upscale(_p(_f64(src), C.c_double), sw, sh, int(dw), int(dh), int(mode), _p(out, C.c_double))
    return out


def sharpen(img, amount):
    H, W = img.shape[:2]
    out = _img_out(H, W)
    lib().orc_sharpen(_p(_f64(img), C.c_double), W, H, float(amount), _p(out, C.c_double))
    return out


def fxaa(img, level):
    H, W = img.shape[:2]
    out = _img_out(H, W)
    lib().orc_fxaa(_p(_f64(img), C.c_double), W, H, int(level), _p(out, C.c_double))
    return out


def txaa(img, level):
    H, W = img.shape[:2]
    out = _img_out(H, W)
    lib().orc_txaa(_p(_f64(img), C.c_double), W, H, int(level), _p(out, C.c_double))
    return out


def internal_size(w, h, mode):
    out = (C.c_int * 2)()
    lib().orc_internal_size(int(w), int(h), int(mode), out)
    return out[0], out[1]


def post_stack(lin, guides11, width, height, history=None, cam=None, **lv):
    """RenderState.Start's post order (renderer.go:2838-2895) composed from the
    passes above. history: None or (prev_lin, prev_guides11, prev_cam). Returns
    (final linear, new history or None)."""
    g = lambda k: int(lv.get(k, 0))
    rh, rw = lin.shape[:2]
    job = _f64(lin)
    if g("hbao_plus") > 0:
        job = hbao(job, guides11, g("hbao_plus"), True)
    elif g("hbao") > 0:
        job = hbao(job, guides11, g("hbao"), False)
    if g("denoise"):
        job = atrous(job, guides11, 2 + min(3, max(g("taa"), g("txaa"))))
    tw = temporal_weight(g("taa"), g("tsaa"), g("txaa"))
    if tw > 0 and history is not None and history[0].shape[:2] == (rh, rw):
        job = temporal(job, guides11, history[0], history[1], history[2], tw)
    if g("bloom") > 0:
        job = bloom(job, g("bloom"))
    job = debug_view(job, guides11, g("debug_view"), g("hbao"), g("hbao_plus"))
    new_hist = (job.copy(), _f64(guides11).copy(), cam) if tw > 0 else None
    final = job
    if g("upscale") != 0 and (rw != width or rh != height):
        final = upscale(job, width, height, g("upscale"))
    if g("fxaa") > 0:
        final = fxaa(final, g("fxaa"))
    if g("txaa") > 0:
        final = txaa(final, g("txaa"))
    return final, new_hist

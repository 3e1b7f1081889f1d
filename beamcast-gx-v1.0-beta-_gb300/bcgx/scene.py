"""Host scene: Python face of the native builder (include/bc_host_scene.h).

Method names follow the Go Scene of the reference renderer
(windows_portable/renderer.go:225-473): add_material, add_sphere,
add_triangle(s), build, refit, translate_primitive. The BVH is built by
native code with the reference's binned-SAH rules, so the tree handed to the
GPU is the one the Go renderer would build.
"""
from __future__ import annotations

import ctypes as C
import itertools
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import check, lib, ptr

MAT_DIFFUSE, MAT_METAL, MAT_GLASS, MAT_EMISSIVE = 0, 1, 2, 3
PRIM_SPHERE, PRIM_TRIANGLE = 0, 1

_ids = itertools.count(1)


@dataclass
class Material:
    kind: int = MAT_DIFFUSE
    color: tuple = (0.0, 0.0, 0.0)
    roughness: float = 0.0
    ior: float = 0.0
    emission: tuple = (0.0, 0.0, 0.0)


class Scene:
    """Scene model plus BVH; `scene_id` identifies it to the GPU scene cache."""

    def __init__(self, name: str = ""):
        self._h = lib().bc_hscene_create()
        if not self._h:
            raise MemoryError("bc_hscene_create failed")
        self.name = name
        self.scene_id = next(_ids)
        self.bvh_mode, self.bvh_bins, self.bvh_leaf = "SAH", 16, 4
        self.materials: list[Material] = []

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().bc_hscene_destroy(h)
            self._h = None

    # -- construction (renderer.go:242-269) --
    def add_material(self, m: Material) -> int:
        col = np.asarray(m.color, dtype=np.float64)
        em = np.asarray(m.emission, dtype=np.float64)
        self.materials.append(m)
        return lib().bc_hscene_add_material(self._h, int(m.kind), ptr(col, C.c_double), float(m.roughness),
                                            float(m.ior), ptr(em, C.c_double))

    def add_sphere(self, center, radius: float, mat: int):
        c = np.asarray(center, dtype=np.float64)
        lib().bc_hscene_add_sphere(self._h, ptr(c, C.c_double), float(radius), int(mat))

    def add_triangle(self, a, b, c, mat: int):
        self.add_triangles(np.asarray([a, b, c], dtype=np.float64).reshape(1, 9), np.asarray([mat], dtype=np.int32))

    def add_triangles(self, verts, mats):
        """verts: (n, 9) or (n, 3, 3) fp64 (A, B, C); mats: (n,) int32 or a scalar."""
        v = np.ascontiguousarray(np.asarray(verts, dtype=np.float64).reshape(-1, 9))
        m = np.asarray(mats, dtype=np.int32)
        if m.ndim == 0:
            m = np.full(len(v), int(m), dtype=np.int32)
        m = np.ascontiguousarray(m)
        lib().bc_hscene_add_triangles(self._h, len(v), ptr(v, C.c_double), ptr(m, C.c_int32))

    def translate_primitive(self, index: int, delta):
        d = np.asarray(delta, dtype=np.float64)
        check(lib().bc_hscene_translate_prim(self._h, int(index), ptr(d, C.c_double)))

    # -- BVH (renderer.go:409-473) --
    def build(self):
        lib().bc_hscene_set_bvh(self._h, self.bvh_mode.encode(), int(self.bvh_bins), int(self.bvh_leaf))
        check(lib().bc_hscene_build(self._h))

    def build_device(self, ctx):
        """Scene.Build with the SAH tree built on the GPU of `ctx` (same result as build())."""
        lib().bc_hscene_set_bvh(self._h, self.bvh_mode.encode(), int(self.bvh_bins), int(self.bvh_leaf))
        check(lib().bc_hscene_build_device(self._h, ctx.handle), ctx.handle)

    def refit(self):
        check(lib().bc_hscene_refit(self._h))

    def counts(self) -> dict:
        out = (C.c_int64 * 6)()
        lib().bc_hscene_counts(self._h, out)
        keys = ("prims", "nodes", "lights", "materials", "topology_rev", "geometry_rev")
        return dict(zip(keys, list(out)))

    def desc(self) -> _lib.SceneDesc:
        d = _lib.SceneDesc()
        check(lib().bc_hscene_describe(self._h, C.byref(d)))
        return d

    def arrays(self) -> "SceneArrays":
        """Copies the built scene out as numpy arrays (Scene fields)."""
        d = self.desc()
        n, nn, nl, nm = d.n_prims, d.n_nodes, d.n_lights, d.n_materials

        def a(p, count, dtype):
            if count == 0 or not p:
                return np.zeros(0, dtype=dtype)
            return np.ctypeslib.as_array(p, shape=(count,)).astype(dtype, copy=True)

        return SceneArrays(
            mat_kind=a(d.mat_kind, nm, np.int32), mat_color=a(d.mat_color, 3 * nm, np.float64).reshape(-1, 3),
            mat_roughness=a(d.mat_roughness, nm, np.float64), mat_ior=a(d.mat_ior, nm, np.float64),
            mat_emission=a(d.mat_emission, 3 * nm, np.float64).reshape(-1, 3),
            prim_kind=a(d.prim_kind, n, np.int32), prim_material=a(d.prim_material, n, np.int32),
            prim_center=a(d.prim_center, 3 * n, np.float64).reshape(-1, 3), prim_radius=a(d.prim_radius, n, np.float64),
            prim_a=a(d.prim_a, 3 * n, np.float64).reshape(-1, 3), prim_e1=a(d.prim_e1, 3 * n, np.float64).reshape(-1, 3),
            prim_e2=a(d.prim_e2, 3 * n, np.float64).reshape(-1, 3),
            prim_normal=a(d.prim_normal, 3 * n, np.float64).reshape(-1, 3),
            node_box=a(d.node_box, 6 * nn, np.float64).reshape(-1, 6), node_left=a(d.node_left, nn, np.int32),
            node_right=a(d.node_right, nn, np.int32), node_start=a(d.node_start, nn, np.int32),
            node_count=a(d.node_count, nn, np.int32), order=a(d.order, n, np.int32),
            light_spheres=a(d.light_spheres, nl, np.int32), light_cdf=a(d.light_cdf, nl, np.float64),
            light_pdf_by_prim=a(d.light_pdf_by_prim, n, np.float64))

    def revisions(self):
        c = self.counts()
        return c["topology_rev"], c["geometry_rev"]


@dataclass
class SceneArrays:
    """A built scene as plain arrays: the hand-off a Go caller makes with its own Scene."""
    mat_kind: np.ndarray
    mat_color: np.ndarray
    mat_roughness: np.ndarray
    mat_ior: np.ndarray
    mat_emission: np.ndarray
    prim_kind: np.ndarray
    prim_material: np.ndarray
    prim_center: np.ndarray
    prim_radius: np.ndarray
    prim_a: np.ndarray
    prim_e1: np.ndarray
    prim_e2: np.ndarray
    prim_normal: np.ndarray
    node_box: np.ndarray
    node_left: np.ndarray
    node_right: np.ndarray
    node_start: np.ndarray
    node_count: np.ndarray
    order: np.ndarray
    light_spheres: np.ndarray
    light_cdf: np.ndarray
    light_pdf_by_prim: np.ndarray
    _keep: list = field(default_factory=list, repr=False)

    def desc(self) -> _lib.SceneDesc:
        d = _lib.SceneDesc()
        keep = self._keep
        keep.clear()

        def p(a, dtype, ctype):
            a = np.ascontiguousarray(a, dtype=dtype)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(ctype)) if a.size else None

        d.n_materials = len(self.mat_kind)
        d.mat_kind = p(self.mat_kind, np.int32, C.c_int32)
        d.mat_color = p(self.mat_color, np.float64, C.c_double)
        d.mat_roughness = p(self.mat_roughness, np.float64, C.c_double)
        d.mat_ior = p(self.mat_ior, np.float64, C.c_double)
        d.mat_emission = p(self.mat_emission, np.float64, C.c_double)
        d.n_prims = len(self.prim_kind)
        d.prim_kind = p(self.prim_kind, np.int32, C.c_int32)
        d.prim_material = p(self.prim_material, np.int32, C.c_int32)
        d.prim_center = p(self.prim_center, np.float64, C.c_double)
        d.prim_radius = p(self.prim_radius, np.float64, C.c_double)
        d.prim_a = p(self.prim_a, np.float64, C.c_double)
        d.prim_e1 = p(self.prim_e1, np.float64, C.c_double)
        d.prim_e2 = p(self.prim_e2, np.float64, C.c_double)
        d.prim_normal = p(self.prim_normal, np.float64, C.c_double)
        d.n_nodes = len(self.node_left)
        d.node_box = p(self.node_box, np.float64, C.c_double)
        d.node_left = p(self.node_left, np.int32, C.c_int32)
        d.node_right = p(self.node_right, np.int32, C.c_int32)
        d.node_start = p(self.node_start, np.int32, C.c_int32)
        d.node_count = p(self.node_count, np.int32, C.c_int32)
        d.order = p(self.order, np.int32, C.c_int32)
        d.n_lights = len(self.light_spheres)
        d.light_spheres = p(self.light_spheres, np.int32, C.c_int32)
        d.light_cdf = p(self.light_cdf, np.float64, C.c_double)
        d.light_pdf_by_prim = p(self.light_pdf_by_prim, np.float64, C.c_double)
        return d

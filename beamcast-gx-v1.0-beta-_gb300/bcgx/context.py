"""GPU context: the Python face of the C-ABI in include/bc_gx.h.

`render_cuda` mirrors renderOpenCL (windows_portable/gpu_opencl_windows.go:565):
scene, camera and settings in; linear HDR rows, compact guides, the extension
ray count and the device name out, with the same chunked row loop and
`on_chunk(y0, rows, data, progress)` callback. A GPU error raises; there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import DiffDescC, PostDescC, SceneDesc, TimingC, TuneReportC, ViewC, check, lib, ptr
from .scene import Scene, SceneArrays
from .settings import Camera, RenderSettings


def gpu_available() -> tuple[bool, str]:
    """openCLGPUAvailable (gpu_opencl_windows.go:172) for the CUDA backend."""
    buf = C.create_string_buffer(512)
    ok = lib().bc_gpu_available(buf, len(buf))
    return bool(ok), buf.value.decode(errors="replace")


class Context:
    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().bc_create(int(device), C.byref(h)))
        self._h = h
        self._desc_keep = None

    def close(self):
        if getattr(self, "_h", None):
            lib().bc_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def device_name(self) -> str:
        buf = C.create_string_buffer(256)
        check(lib().bc_device_name(self._h, buf, len(buf)), self._h)
        return buf.value.decode()

    # -- scene --
    def upload(self, scene, scene_id: int | None = None, topology_rev: int | None = None,
               geometry_rev: int | None = None):
        """ensureSceneLocked (gpu_opencl_windows.go:484-495) by revision."""
        if isinstance(scene, Scene):
            d = scene.desc()
            t, g = scene.revisions()
            sid = scene.scene_id
        elif isinstance(scene, SceneArrays):
            d = scene.desc()
            sid, t, g = id(scene), 1, 1
        else:
            raise TypeError("scene must be a Scene or SceneArrays")
        sid = sid if scene_id is None else scene_id
        t = t if topology_rev is None else topology_rev
        g = g if geometry_rev is None else geometry_rev
        check(lib().bc_scene_upload(self._h, C.byref(d), sid, t, g), self._h)
        self._desc_keep = scene

    def upload_set(self, scenes, set_id: int | None = None, revision: int = 1):
        """Resident scene set for render_batch: scenes[k] is scene k of the set."""
        descs = []
        for sc in scenes:
            if not isinstance(sc, (Scene, SceneArrays)):
                raise TypeError("scenes must be Scene or SceneArrays objects")
            descs.append(sc.desc())
        arr = (SceneDesc * len(descs))(*descs)
        sid = id(scenes) if set_id is None else set_id
        check(lib().bc_scene_set_upload(self._h, arr, len(descs), sid, revision), self._h)
        self._desc_keep = list(scenes)

    def scene_stats(self) -> dict:
        out = (C.c_int64 * 7)()
        check(lib().bc_scene_stats(self._h, out, 7), self._h)
        keys = ("nodes8", "slots", "binary_nodes", "depth8", "stack_need", "device_bytes", "geometry_updates")
        return dict(zip(keys, list(out)))

    # -- ray casting --
    def raycast(self, rays: np.ndarray, t_out: np.ndarray | None = None, prim_out: np.ndarray | None = None):
        """rays: (n, 8) float32 (ox, oy, oz, tmin, dx, dy, dz, tmax) -> (t float32, prim int32).
        Optional output arrays (e.g. in pinned host memory) are filled in place."""
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = len(r)
        t = np.empty(n, dtype=np.float32) if t_out is None else t_out
        p = np.empty(n, dtype=np.int32) if prim_out is None else prim_out
        assert t.dtype == np.float32 and p.dtype == np.int32 and len(t) == n and len(p) == n
        check(lib().bc_raycast(self._h, ptr(r, C.c_float), n, ptr(t, C.c_float), ptr(p, C.c_int32)), self._h)
        return t, p

    def occluded(self, rays: np.ndarray) -> np.ndarray:
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        out = np.empty(len(r), dtype=np.uint8)
        check(lib().bc_occluded(self._h, ptr(r, C.c_float), len(r), ptr(out, C.c_uint8)), self._h)
        return out.astype(bool)

    def raycast_device(self, d_rays: int, n: int, d_t: int, d_prim: int, stream: int = 0):
        """Device-pointer variant (asynchronous on `stream`)."""
        check(lib().bc_raycast_device(self._h, C.c_void_p(d_rays), int(n), C.c_void_p(d_t), C.c_void_p(d_prim),
                                      C.c_void_p(stream) if stream else None), self._h)

    def occluded_device(self, d_rays: int, n: int, d_out: int, stream: int = 0):
        check(lib().bc_occluded_device(self._h, C.c_void_p(d_rays), int(n), C.c_void_p(d_out),
                                       C.c_void_p(stream) if stream else None), self._h)

    def last_timing(self) -> dict:
        """Device time of the last render call (bc_last_timing): CUDA events on
        the context's stream; per-kernel classes when render_timing is 1."""
        t = TimingC()
        check(lib().bc_last_timing(self._h, C.byref(t)), self._h)
        return {name: getattr(t, name) for name, _ in TimingC._fields_ if name != "reserved"}

    def sync(self, stream: int = 0):
        """Waits for `stream` and raises the kernel status of the device-pointer
        calls enqueued since the last sync (bc_sync)."""
        check(lib().bc_sync(self._h, C.c_void_p(stream) if stream else None), self._h)

    # -- rendering --
    def render_rows(self, cam: Camera, settings: RenderSettings, y0: int, rows: int, guides: bool = False):
        W = settings.width
        lin = np.empty((rows, W, 3), dtype=np.float32)
        g = np.empty((rows, W, 3), dtype=np.uint32) if guides else None
        rays = C.c_int64(0)
        cc, sc = cam.c(), settings.c()
        check(lib().bc_render_rows(self._h, C.byref(cc), C.byref(sc), int(y0), int(rows), ptr(lin, C.c_float),
                                   ptr(g, C.c_uint32), C.byref(rays)), self._h)
        return lin, g, rays.value

    def render_frame(self, cam: Camera, settings: RenderSettings, want_guides: bool = True, want_rgba: bool = True):
        W, H = settings.width, settings.height
        lin = np.empty((H, W, 3), dtype=np.float32)
        g = np.empty((H, W, 3), dtype=np.uint32) if want_guides else None
        rgba = np.empty((H, W), dtype=np.uint32) if want_rgba else None
        rays = C.c_int64(0)
        cc, sc = cam.c(), settings.c()
        check(lib().bc_render_frame(self._h, C.byref(cc), C.byref(sc), ptr(lin, C.c_float), ptr(g, C.c_uint32),
                                    ptr(rgba, C.c_uint32), C.byref(rays)), self._h)
        return {"linear": lin, "guides": g, "rgba": rgba, "rays": rays.value}

    def render_moments(self, cam: Camera, settings: RenderSettings):
        """Per-pixel mean and mean of squares of the sample radiance (no post)."""
        W, H = settings.width, settings.height
        mean = np.empty((H, W, 3), dtype=np.float32)
        msq = np.empty((H, W, 3), dtype=np.float32)
        rays = C.c_int64(0)
        cc, sc = cam.c(), settings.c()
        check(lib().bc_render_moments(self._h, C.byref(cc), C.byref(sc), ptr(mean, C.c_float), ptr(msq, C.c_float),
                                      C.byref(rays)), self._h)
        return mean, msq, rays.value

    def render_batch(self, views, readback: bool = True):
        """views: list of (scene_index, Camera, RenderSettings) over the resident set.
        Returns ([linear (H, W, 3)] or None per view, extension rays)."""
        n = len(views)
        vc = (ViewC * n)()
        outs = []
        ptrs = (C.POINTER(C.c_float) * n)()
        for i, (k, cam, st) in enumerate(views):
            vc[i].scene = int(k)
            vc[i].reserved = 0
            vc[i].camera = cam.c()
            vc[i].settings = st.c()
            o = np.empty((st.height, st.width, 3), dtype=np.float32) if readback else None
            outs.append(o)
            ptrs[i] = ptr(o, C.c_float)
        rays = C.c_int64(0)
        check(lib().bc_render_batch(self._h, vc, n, ptrs if readback else None, C.byref(rays)), self._h)
        return outs, rays.value

    def photon_map(self, settings: RenderSettings, scene: int = 0):
        """buildPhotonMap for (scene, settings): dict(photons (n, 10): position, normal,
        flux, emission index in append order; rays)."""
        sc = settings.c()
        n = C.c_int32(0)
        rays = C.c_int64(0)
        check(lib().bc_photon_map(self._h, int(scene), C.byref(sc), 0, None, C.byref(n), C.byref(rays)), self._h)
        out = np.zeros((max(n.value, 1), 10), dtype=np.float32)
        check(lib().bc_photon_map(self._h, int(scene), C.byref(sc), n.value, ptr(out, C.c_float), C.byref(n),
                                  C.byref(rays)), self._h)
        return {"photons": out[:n.value], "rays": rays.value}

    # -- autotuner --
    @staticmethod
    def _report(r) -> dict:
        return {k: getattr(r, k) for k, _ in r._fields_ if k != "reserved"}

    def autotune_raycast(self, d_rays: int, n: int) -> dict:
        """Times the ray-cast variants on these device rays and keeps the fastest."""
        r = TuneReportC()
        check(lib().bc_autotune_raycast(self._h, C.c_void_p(d_rays), int(n), C.byref(r)), self._h)
        return self._report(r)

    def autotune_render(self, views) -> dict:
        """views as for render_batch: times the extend-kernel variants, then the wave
        sizes, on a sample of the batch, and keeps the fastest."""
        n = len(views)
        vc = (ViewC * n)()
        for i, (k, cam, st) in enumerate(views):
            vc[i].scene, vc[i].reserved, vc[i].camera, vc[i].settings = int(k), 0, cam.c(), st.c()
        r = TuneReportC()
        check(lib().bc_autotune_render(self._h, vc, n, C.byref(r)), self._h)
        return self._report(r)

    # -- differentiable rendering --
    def diff_configure(self, cam: Camera, settings: RenderSettings, albedo_materials, emission_materials=()):
        """Parameters: albedo RGB of each diffuse material in albedo_materials, then
        emission RGB of each emissive material in emission_materials."""
        a = np.ascontiguousarray(albedo_materials, dtype=np.int32)
        e = np.ascontiguousarray(emission_materials, dtype=np.int32)
        d = DiffDescC()
        d.camera = cam.c()
        d.settings = settings.c()
        d.n_albedo, d.albedo_materials = len(a), ptr(a, C.c_int32) if len(a) else None
        d.n_emission, d.emission_materials = len(e), ptr(e, C.c_int32) if len(e) else None
        check(lib().bc_diff_configure(self._h, C.byref(d)), self._h)
        self._diff_shape = (settings.height, settings.width, len(a), len(e))
        self._diff_has_target = False

    def diff_set_target(self, target: np.ndarray):
        H, W, _, _ = self._diff_shape
        t = np.ascontiguousarray(target, dtype=np.float32)
        assert t.shape == (H, W, 3)
        check(lib().bc_diff_set_target(self._h, ptr(t, C.c_float)), self._h)
        self._diff_has_target = True

    def forward(self, params: np.ndarray, seed: int, want_image: bool = True, want_loss: bool | None = None):
        """params: (n_albedo + n_emission, 3) float32. Returns (image or None, loss or None);
        the loss is computed when a target is set."""
        H, W, na, ne = self._diff_shape
        if want_loss is None:
            want_loss = self._diff_has_target
        p = np.ascontiguousarray(params, dtype=np.float32).reshape(-1)
        assert p.size == 3 * (na + ne)
        img = np.empty((H, W, 3), np.float32) if want_image else None
        loss = C.c_double(0)
        check(lib().bc_forward(self._h, ptr(p, C.c_float), int(seed), ptr(img, C.c_float),
                               C.byref(loss) if want_loss else None), self._h)
        return img, (loss.value if want_loss else None)

    def backward(self, dloss_dimage: np.ndarray | None = None):
        """Gradient at the last forward: (grad_albedo (n_albedo, 3), grad_emission (n_emission, 3))."""
        H, W, na, ne = self._diff_shape
        dd = None if dloss_dimage is None else np.ascontiguousarray(dloss_dimage, dtype=np.float32)
        ga = np.zeros((na, 3), np.float32)
        ge = np.zeros((ne, 3), np.float32)
        check(lib().bc_backward(self._h, ptr(dd, C.c_float), ptr(ga, C.c_float) if na else None,
                                ptr(ge, C.c_float) if ne else None), self._h)
        return ga, ge

    def post_stack(self, linear: np.ndarray, guides12: np.ndarray | None, cam: Camera, width: int, height: int,
                   want_rgba: bool = True, **levels):
        """RenderState.Start's whole post stack on caller buffers. linear: (rh, rw, 3);
        guides12: (rh, rw, 12) = P xyz, depth, N xyz, valid, albedo xyz, 0. levels: hbao,
        hbao_plus, denoise, taa, tsaa, txaa, bloom, fxaa, upscale (0-3), debug_view (0-5),
        hdr, exposure, gamma. Returns (linear (height, width, 3), rgba or None)."""
        lin = np.ascontiguousarray(linear, dtype=np.float32)
        rh, rw = lin.shape[:2]
        g = None if guides12 is None else np.ascontiguousarray(guides12, dtype=np.float32)
        d = PostDescC()
        d.width, d.height, d.render_width, d.render_height = int(width), int(height), rw, rh
        for k in ("hbao", "hbao_plus", "denoise", "taa", "tsaa", "txaa", "bloom", "fxaa", "upscale", "debug_view"):
            setattr(d, k, int(levels.get(k, 0)))
        d.hdr = int(levels.get("hdr", 2))
        d.exposure = float(levels.get("exposure", 0.0))
        d.gamma = float(levels.get("gamma", 2.2))
        d.camera = cam.c()
        out = np.empty((height, width, 3), np.float32)
        rgba = np.empty((height, width), np.uint32) if want_rgba else None
        check(lib().bc_post_stack(self._h, C.byref(d), ptr(lin, C.c_float), ptr(g, C.c_float), ptr(out, C.c_float),
                                  ptr(rgba, C.c_uint32)), self._h)
        return out, rgba

    def post_history_reset(self):
        check(lib().bc_post_history_reset(self._h), self._h)

    def post_process(self, linear: np.ndarray, guide_nd: np.ndarray | None, settings: RenderSettings,
                     want_rgba: bool = True):
        """Denoise / bloom / tone map on caller buffers: linear (H, W, 3), guide_nd (H, W, 4)."""
        H, W = linear.shape[:2]
        lin = np.ascontiguousarray(linear, dtype=np.float32)
        g = None if guide_nd is None else np.ascontiguousarray(guide_nd, dtype=np.float32)
        out = np.empty((H, W, 3), dtype=np.float32)
        rgba = np.empty((H, W), dtype=np.uint32) if want_rgba else None
        sc = settings.c()
        check(lib().bc_post_process(self._h, W, H, ptr(lin, C.c_float), ptr(g, C.c_float), C.byref(sc),
                                    ptr(out, C.c_float), ptr(rgba, C.c_uint32)), self._h)
        return out, rgba

    def set_option(self, name: str, value: int):
        check(lib().bc_set_option(self._h, name.encode(), int(value)), self._h)

    def get_option(self, name: str) -> int:
        v = C.c_int64(0)
        check(lib().bc_get_option(self._h, name.encode(), C.byref(v)), self._h)
        return v.value

    def cancel(self):
        lib().bc_cancel(self._h)

    def reset_cancel(self):
        lib().bc_reset_cancel(self._h)


_persistent: Context | None = None


def persistent_context() -> Context:
    """One context per process, like persistentCL (gpu_opencl_windows.go:132)."""
    global _persistent
    if _persistent is None:
        _persistent = Context(0)
    return _persistent


def internal_size(settings: RenderSettings):
    return settings.width, settings.height


def render_cuda(scene: Scene, cam: Camera, settings: RenderSettings, cancel=None, on_chunk=None):
    """renderOpenCL's contract on the CUDA backend.

    Returns (linear (H, W, 3) float32, compact guides (H, W, 3) uint32 or None,
    extension rays, device name). Raises on any GPU error.
    """
    if scene is None or scene.counts()["prims"] == 0 or scene.counts()["nodes"] == 0:
        raise ValueError("CUDA backend requires a non-empty built scene")
    ctx = persistent_context()
    ctx.upload(scene)
    w, h = internal_size(settings)
    need_guides = (settings.denoise or settings.hbao > 0 or settings.hbao_plus > 0 or settings.taa > 0
                   or settings.tsaa > 0 or settings.txaa > 0)
    chunk = 64
    if not settings.progressive_updates:
        chunk = h
    elif settings.publish_hz <= 15:
        chunk = 128
    elif settings.publish_hz >= 60:
        chunk = 32
    linear = np.empty((h, w, 3), dtype=np.float32)
    guides = np.empty((h, w, 3), dtype=np.uint32) if need_guides else None
    rays = 0
    for y0 in range(0, h, chunk):
        if cancel is not None and cancel():
            raise RuntimeError("render cancelled")
        rows = min(chunk, h - y0)
        lin, g, r = ctx.render_rows(cam, settings, y0, rows, guides=need_guides)
        linear[y0:y0 + rows] = lin
        if need_guides:
            guides[y0:y0 + rows] = g
        rays += r
        if on_chunk is not None:
            on_chunk(y0, rows, lin, (y0 + rows) / h)
    return linear, guides, rays, ctx.device_name()

"""ctypes binding of libbcgx.so (include/bc_gx.h, include/bc_host_scene.h).

The library is built in-tree by ../build.py. Loading fails loudly when it is
missing: there is no CPU fallback anywhere on the product path.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "_build", "libbcgx.so")

BC_OK = 0
STATUS_NAMES = {
    0: "BC_OK", 1: "BC_ERR_NO_DEVICE", 2: "BC_ERR_OOM", 3: "BC_ERR_BAD_SCENE", 4: "BC_ERR_CANCELLED",
    5: "BC_ERR_TIMEOUT", 6: "BC_ERR_DEVICE", 7: "BC_ERR_INVALID_ARG", 8: "BC_ERR_NO_SCENE", 9: "BC_ERR_CAPACITY",
}

P = C.POINTER
i32p, f64p, f32p, u32p, u8p, i64p = P(C.c_int32), P(C.c_double), P(C.c_float), P(C.c_uint32), P(C.c_uint8), P(C.c_int64)


class SceneDesc(C.Structure):
    _fields_ = [
        ("n_materials", C.c_int32), ("mat_kind", i32p), ("mat_color", f64p), ("mat_roughness", f64p),
        ("mat_ior", f64p), ("mat_emission", f64p),
        ("n_prims", C.c_int32), ("prim_kind", i32p), ("prim_material", i32p), ("prim_center", f64p),
        ("prim_radius", f64p), ("prim_a", f64p), ("prim_e1", f64p), ("prim_e2", f64p), ("prim_normal", f64p),
        ("n_nodes", C.c_int32), ("node_box", f64p), ("node_left", i32p), ("node_right", i32p),
        ("node_start", i32p), ("node_count", i32p), ("order", i32p),
        ("n_lights", C.c_int32), ("light_spheres", i32p), ("light_cdf", f64p), ("light_pdf_by_prim", f64p),
    ]


class CameraC(C.Structure):
    _fields_ = [("position", C.c_double * 3), ("target", C.c_double * 3), ("up", C.c_double * 3),
                ("fov_deg", C.c_double)]


class SettingsC(C.Structure):
    _fields_ = [
        ("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("bounces", C.c_int32),
        ("msaa", C.c_int32), ("tsaa", C.c_int32), ("sampler", C.c_int32), ("mis", C.c_int32),
        ("power_light_sampling", C.c_int32), ("firefly_clamp", C.c_double), ("rr_depth", C.c_int32),
        ("adaptive_sampling", C.c_int32), ("adaptive_threshold", C.c_double), ("denoise", C.c_int32),
        ("taa", C.c_int32), ("txaa", C.c_int32), ("bloom", C.c_int32), ("hdr", C.c_int32),
        ("exposure", C.c_double), ("gamma", C.c_double), ("seed", C.c_uint64),
        ("integrator", C.c_int32), ("photon_mapping", C.c_int32),
    ]


class ViewC(C.Structure):
    _fields_ = [("scene", C.c_int32), ("reserved", C.c_int32), ("camera", CameraC), ("settings", SettingsC)]


class DiffDescC(C.Structure):
    _fields_ = [("camera", CameraC), ("settings", SettingsC), ("n_albedo", C.c_int32),
                ("albedo_materials", P(C.c_int32)), ("n_emission", C.c_int32),
                ("emission_materials", P(C.c_int32))]


class TuneReportC(C.Structure):
    _fields_ = [("raycast_minblocks", C.c_int32), ("raycast_sort", C.c_int32), ("render_wave_cap", C.c_int64),
                ("n_timed", C.c_int32), ("render_extend", C.c_int32), ("best_ms", C.c_double), ("default_ms", C.c_double),
                ("worst_ms", C.c_double), ("raycast_split", C.c_int32), ("render_shade_block", C.c_int32)]


class TimingC(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("launches", C.c_int64), ("extend_launches", C.c_int64),
                ("kernel_timing", C.c_int32), ("reserved", C.c_int32), ("generate_ms", C.c_double),
                ("extend_ms", C.c_double), ("shade_ms", C.c_double), ("connect_ms", C.c_double),
                ("accumulate_ms", C.c_double), ("post_ms", C.c_double), ("other_ms", C.c_double)]


class PostDescC(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("render_width", C.c_int32),
                ("render_height", C.c_int32), ("hbao", C.c_int32), ("hbao_plus", C.c_int32),
                ("denoise", C.c_int32), ("taa", C.c_int32), ("tsaa", C.c_int32), ("txaa", C.c_int32),
                ("bloom", C.c_int32), ("fxaa", C.c_int32), ("upscale", C.c_int32), ("debug_view", C.c_int32),
                ("hdr", C.c_int32), ("reserved", C.c_int32), ("exposure", C.c_double), ("gamma", C.c_double),
                ("camera", CameraC)]


# (name, restype, argtypes) for every exported symbol of the two headers.
SIGNATURES = [
    ("bc_gpu_available", C.c_int, [C.c_char_p, C.c_size_t]),
    ("bc_create", C.c_int, [C.c_int, P(C.c_void_p)]),
    ("bc_destroy", None, [C.c_void_p]),
    ("bc_last_error", C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    ("bc_device_name", C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    ("bc_scene_upload", C.c_int, [C.c_void_p, P(SceneDesc), C.c_uint64, C.c_uint64, C.c_uint64]),
    ("bc_scene_set_upload", C.c_int, [C.c_void_p, P(SceneDesc), C.c_int32, C.c_uint64, C.c_uint64]),
    ("bc_build_sah", C.c_int, [C.c_void_p, C.c_int32, f64p, f64p, C.c_int32, C.c_int32, i32p, f64p, i32p, i32p,
                               i32p, i32p, i32p]),
    ("bc_scene_stats", C.c_int, [C.c_void_p, i64p, C.c_int]),
    ("bc_raycast", C.c_int, [C.c_void_p, f32p, C.c_int64, f32p, i32p]),
    ("bc_raycast_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("bc_occluded", C.c_int, [C.c_void_p, f32p, C.c_int64, u8p]),
    ("bc_occluded_device", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    ("bc_sync", C.c_int, [C.c_void_p, C.c_void_p]),
    ("bc_render_rows", C.c_int, [C.c_void_p, P(CameraC), P(SettingsC), C.c_int32, C.c_int32, f32p, u32p, i64p]),
    ("bc_render_frame", C.c_int, [C.c_void_p, P(CameraC), P(SettingsC), f32p, u32p, u32p, i64p]),
    ("bc_render_moments", C.c_int, [C.c_void_p, P(CameraC), P(SettingsC), f32p, f32p, i64p]),
    ("bc_render_batch", C.c_int, [C.c_void_p, P(ViewC), C.c_int32, P(f32p), i64p]),
    ("bc_autotune_raycast", C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, P(TuneReportC)]),
    ("bc_autotune_render", C.c_int, [C.c_void_p, P(ViewC), C.c_int32, P(TuneReportC)]),
    ("bc_photon_map", C.c_int, [C.c_void_p, C.c_int32, P(SettingsC), C.c_int32, f32p, P(C.c_int32), i64p]),
    ("bc_diff_configure", C.c_int, [C.c_void_p, P(DiffDescC)]),
    ("bc_diff_set_target", C.c_int, [C.c_void_p, f32p]),
    ("bc_forward", C.c_int, [C.c_void_p, f32p, C.c_uint64, f32p, f64p]),
    ("bc_backward", C.c_int, [C.c_void_p, f32p, f32p, f32p]),
    ("bc_post_stack", C.c_int, [C.c_void_p, P(PostDescC), f32p, f32p, f32p, u32p]),
    ("bc_post_history_reset", C.c_int, [C.c_void_p]),
    ("bc_post_process", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, f32p, f32p, P(SettingsC), f32p, u32p]),
    ("bc_post_process_noalloc", C.c_int, [C.c_int32, C.c_int32, C.c_void_p, C.c_void_p, P(SettingsC), C.c_void_p,
                                          C.c_void_p, C.c_void_p]),
    ("bc_set_option", C.c_int, [C.c_void_p, C.c_char_p, C.c_int64]),
    ("bc_get_option", C.c_int, [C.c_void_p, C.c_char_p, i64p]),
    ("bc_last_timing", C.c_int, [C.c_void_p, C.POINTER(TimingC)]),
    ("bc_cancel", C.c_int, [C.c_void_p]),
    ("bc_reset_cancel", C.c_int, [C.c_void_p]),
    ("bc_hscene_create", C.c_void_p, []),
    ("bc_hscene_destroy", None, [C.c_void_p]),
    ("bc_hscene_add_material", C.c_int32, [C.c_void_p, C.c_int32, f64p, C.c_double, C.c_double, f64p]),
    ("bc_hscene_add_sphere", None, [C.c_void_p, f64p, C.c_double, C.c_int32]),
    ("bc_hscene_add_triangles", None, [C.c_void_p, C.c_int64, f64p, i32p]),
    ("bc_hscene_translate_prim", C.c_int, [C.c_void_p, C.c_int32, f64p]),
    ("bc_hscene_set_bvh", None, [C.c_void_p, C.c_char_p, C.c_int32, C.c_int32]),
    ("bc_hscene_build", C.c_int, [C.c_void_p]),
    ("bc_hscene_build_device", C.c_int, [C.c_void_p, C.c_void_p]),
    ("bc_hscene_refit", C.c_int, [C.c_void_p]),
    ("bc_hscene_counts", None, [C.c_void_p, i64p]),
    ("bc_hscene_describe", C.c_int, [C.c_void_p, P(SceneDesc)]),
]

_lib = None


def lib():
    """Loads libbcgx.so once; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libbcgx.so not built ({LIB_PATH}); run build.py or __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def declared_symbols(include_dir: str) -> list[str]:
    """Function names declared in the public headers (for the export check)."""
    import re
    names = []
    for h in ("bc_gx.h", "bc_host_scene.h"):
        with open(os.path.join(include_dir, h)) as f:
            text = f.read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(bc_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


class BCError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def check(status: int, ctx=None):
    if status != BC_OK:
        buf = C.create_string_buffer(1024)
        lib().bc_last_error(ctx, buf, len(buf))
        raise BCError(status, buf.value.decode(errors="replace"))


def ptr(a, ctype):
    """ctypes pointer to a contiguous numpy array (None for None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(P(ctype))

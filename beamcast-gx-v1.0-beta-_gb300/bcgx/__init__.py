"""Beamcast GX on GB300: Python host side of the CUDA path-tracing hot path.

The compute path is libbcgx.so (hand-written CUDA for sm_103a behind the
C-ABI in include/bc_gx.h); this package only builds scenes, marshals
arguments and mirrors the reference renderer's interface.
"""
from ._lib import BCError, LIB_PATH, lib
from .context import Context, gpu_available, persistent_context, render_cuda
from .scene import (MAT_DIFFUSE, MAT_EMISSIVE, MAT_GLASS, MAT_METAL, PRIM_SPHERE, PRIM_TRIANGLE, Material, Scene,
                    SceneArrays)
from .settings import (INTEGRATOR_PATH, INTEGRATOR_PHOTON, INTEGRATOR_RECURSIVE, Camera, RenderSettings, default_camera,
                       effective_spp, quality, ultra_realism_settings)

__all__ = [
    "BCError", "LIB_PATH", "lib", "Context", "gpu_available", "persistent_context", "render_cuda",
    "MAT_DIFFUSE", "MAT_EMISSIVE", "MAT_GLASS", "MAT_METAL", "PRIM_SPHERE", "PRIM_TRIANGLE", "Material", "Scene",
    "SceneArrays", "Camera", "RenderSettings", "default_camera", "effective_spp", "quality",
    "ultra_realism_settings", "INTEGRATOR_PATH", "INTEGRATOR_RECURSIVE", "INTEGRATOR_PHOTON",
]

"""Render settings and quality presets of the portable renderer.

RenderSettings mirrors renderer.go:1027-1062 (the fields the path-tracing
hot path reads, plus the post fields that choose denoise/bloom/tone map);
quality() mirrors Quality (renderer.go:1064-1117) and
ultra_realism_settings() mirrors UltraRealismSettings (renderer.go:1119-1135).
"""
from __future__ import annotations

import copy
from dataclasses import dataclass

from . import _lib

SAMPLER_RANDOM, SAMPLER_HALTON, SAMPLER_R2 = "Random", "Halton", "R2"
_SAMPLER_CODE = {SAMPLER_RANDOM: 0, SAMPLER_HALTON: 1, SAMPLER_R2: 2}
BACKEND_AUTO, BACKEND_CPU, BACKEND_GPU = "Auto", "CPU", "OpenCL GPU"
# IntegratorMode (renderer.go:1002-1006)
INTEGRATOR_PATH, INTEGRATOR_RECURSIVE, INTEGRATOR_PHOTON = "Path Tracing", "Recursive Ray Tracing", "Photon Mapping"
_INTEGRATOR_CODE = {INTEGRATOR_PATH: 0, INTEGRATOR_RECURSIVE: 1, INTEGRATOR_PHOTON: 2}


@dataclass
class Camera:
    position: tuple
    target: tuple
    up: tuple = (0.0, 1.0, 0.0)
    fov: float = 40.0

    def c(self) -> _lib.CameraC:
        cc = _lib.CameraC()
        cc.position[:] = [float(v) for v in self.position]
        cc.target[:] = [float(v) for v in self.target]
        cc.up[:] = [float(v) for v in self.up]
        cc.fov_deg = float(self.fov)
        return cc


def default_camera() -> Camera:  # renderer.go:946
    return Camera((6, 3.2, 5.5), (0, 0, -4), (0, 1, 0), 40)


@dataclass
class RenderSettings:
    width: int = 960
    height: int = 540
    spp: int = 8
    bounces: int = 6
    denoise: bool = True
    quality: str = "Preview"
    backend: str = BACKEND_AUTO
    exposure: float = 0.0
    gamma: float = 2.2
    fxaa: int = 1
    taa: int = 1
    tsaa: int = 0
    txaa: int = 0
    hbao: int = 0
    hbao_plus: int = 0
    bloom: int = 1
    hdr: int = 2
    msaa: int = 1
    tile_size: int = 24
    adaptive_sampling: bool = True
    adaptive_threshold: float = 0.0006
    sampler: str = SAMPLER_HALTON
    mis: bool = True
    power_light_sampling: bool = True
    firefly_clamp: float = 24.0
    rr_depth: int = 4
    progressive_updates: bool = True
    publish_hz: int = 30
    bvh_mode: str = "SAH"
    bvh_bins: int = 16
    bvh_leaf_size: int = 4
    integrator: str = INTEGRATOR_PATH
    photon_mapping: int = 0
    seed: int = 0x5EED

    def c(self) -> _lib.SettingsC:
        s = _lib.SettingsC()
        s.width, s.height, s.spp, s.bounces = self.width, self.height, self.spp, self.bounces
        s.msaa, s.tsaa = self.msaa, self.tsaa
        s.sampler = _SAMPLER_CODE[self.sampler]
        s.mis, s.power_light_sampling = int(self.mis), int(self.power_light_sampling)
        s.firefly_clamp = float(self.firefly_clamp)
        s.rr_depth = self.rr_depth
        s.adaptive_sampling, s.adaptive_threshold = int(self.adaptive_sampling), float(self.adaptive_threshold)
        s.denoise, s.taa, s.txaa = int(self.denoise), self.taa, self.txaa
        s.bloom, s.hdr = self.bloom, self.hdr
        s.exposure, s.gamma = float(self.exposure), float(self.gamma)
        s.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        s.integrator = _INTEGRATOR_CODE[self.integrator]
        s.photon_mapping = int(self.photon_mapping)
        return s

    def copy(self) -> "RenderSettings":
        return copy.copy(self)


def effective_spp(s: RenderSettings) -> int:
    """effectiveSPP (renderer.go:2395-2417)."""
    msaa = s.msaa if s.msaa in (2, 4, 8) else 1
    tsaa = {1: 2, 2: 3, 3: 4}.get(s.tsaa, 1)
    v = s.spp * msaa * tsaa
    return 1 if v < 1 else min(v, 4096)


def quality(name: str) -> RenderSettings:
    """Quality presets (renderer.go:1064-1117)."""
    b = RenderSettings(backend=BACKEND_AUTO, exposure=0.0, gamma=2.2, fxaa=1, taa=1, tsaa=0, txaa=0, hbao=0,
                       hbao_plus=0, bloom=1, hdr=2, msaa=1, tile_size=16, adaptive_sampling=True,
                       adaptive_threshold=0.0006, sampler=SAMPLER_HALTON, mis=True, power_light_sampling=True,
                       firefly_clamp=24, rr_depth=4, progressive_updates=True, publish_hz=30, bvh_mode="SAH",
                       bvh_bins=16, bvh_leaf_size=4)
    if name == "Draft":
        b.width, b.height, b.spp, b.bounces, b.denoise, b.quality = 640, 360, 2, 4, False, name
        b.fxaa, b.taa, b.bloom, b.hdr = 1, 0, 0, 1
        b.tile_size, b.adaptive_threshold, b.firefly_clamp = 32, 0.002, 12
    elif name == "Balanced":
        b.width, b.height, b.spp, b.bounces, b.denoise, b.quality = 1280, 720, 16, 8, True, name
        b.fxaa, b.taa, b.hbao, b.bloom, b.hdr, b.msaa = 2, 2, 1, 1, 2, 1
        b.photon_mapping = 1
        b.adaptive_threshold = 0.0008
    elif name == "High":
        b.width, b.height, b.spp, b.bounces, b.denoise, b.quality = 1600, 900, 48, 10, True, name
        b.fxaa, b.taa, b.tsaa, b.hbao_plus, b.bloom, b.hdr, b.msaa = 2, 2, 1, 2, 2, 3, 2
        b.photon_mapping = 2
        b.adaptive_threshold, b.firefly_clamp = 0.00035, 32
    elif name == "Ultra":
        b.width, b.height, b.spp, b.bounces, b.denoise, b.quality = 1920, 1080, 96, 12, True, name
        b.fxaa, b.taa, b.tsaa, b.txaa, b.hbao_plus, b.bloom, b.hdr, b.msaa = 3, 3, 2, 1, 3, 3, 3, 2
        b.photon_mapping = 3
        b.adaptive_threshold, b.firefly_clamp = 0.00018, 48
    elif name == "Ultra Realism":
        b.width, b.height, b.spp, b.bounces, b.denoise, b.quality = 2560, 1440, 256, 16, True, name
        b.fxaa, b.taa, b.tsaa, b.txaa, b.msaa = 0, 1, 0, 0, 1
        b.hbao, b.hbao_plus = 0, 0
        b.bloom, b.hdr = 1, 3
        b.sampler, b.mis, b.power_light_sampling = SAMPLER_HALTON, True, True
        b.firefly_clamp, b.rr_depth = 0, 6
        b.adaptive_sampling, b.adaptive_threshold = True, 0.00008
        b.tile_size, b.progressive_updates = 8, False
        b.bvh_mode, b.bvh_bins, b.bvh_leaf_size = "SAH", 32, 4
    else:
        b.width, b.height, b.spp, b.bounces, b.denoise, b.quality = 960, 540, 8, 6, True, "Preview"
        b.fxaa, b.taa, b.hdr, b.tile_size = 1, 1, 2, 24
    return b


def ultra_realism_settings(backend: str) -> RenderSettings:
    """UltraRealismSettings (renderer.go:1119-1135). The CUDA path implements the
    full CPU transport stack (Halton, MIS, power-weighted lights), so unlike the
    OpenCL path it keeps the CPU preset's transport settings for the GPU backend."""
    return quality("Ultra Realism") if backend != BACKEND_GPU else _gpu_ultra()


def _gpu_ultra() -> RenderSettings:
    q = quality("Ultra Realism")
    q.backend = BACKEND_GPU
    q.adaptive_sampling = False
    q.progressive_updates = False
    return q

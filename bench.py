"""Benchmark of the GB300 hot path (one JSON line on rank 0).

Default workload, the configuration the metric is quoted on: the
Ultra-Realism-shaped frame. 2,048,130 seeded triangles (64x64 displaced
geodesic icospheres, a ground quad, 64 emissive quads with LogNormal(1, 1)
luminance; spheres 50% diffuse, 50% rough metal with roughness U[0.05, 1]),
32-bin SAH BVH collapsed to BVH8, 2560x1440, 256 spp, 16 bounces, Russian
roulette from bounce 6, Halton, MIS, power-weighted lights, no clamp, denoise
(3 a-trous passes), bloom 1, ACES; the adaptive stop is off (equal spp, as the
reference's own benchmark recipe sets it, benchmark.go:82). A step is one frame
through bc_render_frame (render and post stack) with the scene resident in
HBM and the output left on the device. A path segment is one extension ray,
the unit the reference counts as Rays (renderer.go:1491).

  value   : Mpath-segments/s of the wave engine: extension rays / device time
            of the frame (CUDA events the library records on its launching
            stream before the frame's first and after its last device work,
            read with bc_last_timing). The path state (128 Mi paths x 100 B)
            and the scene (~300 MB) exceed L2, so no flush is needed.
  plain   : the same frames (same seeds, same samples, so equal RMSE) by the
            one-kernel form: one launch per view, a thread per pixel looping
            over samples and bounces, the reference OpenCL kernel's shape;
            wave_over_plain = value / plain.
  e2e     : bc_render_frame with the linear HDR image and RGBA8 read back into
            pinned host buffers, wall clock around the call.
  roofline: the closest-hit kernel k_extend (the dominant kernel): algorithmic
            bytes per extension query from the oracle's binary-BVH traversal
            counters on the CPU-baseline sample (32 B per box test, 40 per
            triangle test, 32 per sphere, 24 ray in + 8 hit out) times the
            queries of one frame, over k_extend's device time in that frame
            (events before every launch: option render_timing 1).
  rmse    : linear radiance on a 128x72 window at the frame centre against a
            16,384-spp image of that window rendered by the GPU wave engine
            (whose per-pixel means the oracle parity tests check): the wave
            engine, the one-kernel form and the oracle at 256 spp.
  cpu_baseline: the oracle (fp64 restatement of the reference integrator) on
            the machine's host cores, the full frame at 32 spp.
  configs : the other configurations measured in the same run: ray cast
            (Mrays/s), Cornell box, 64-view batch, adjoint s/iter.

Multi-GPU: replicas only (pixels, samples and views are independent): every
rank renders its own frames (its own seeds), value = all ranks' segments over
the slowest rank's time. `--impl reference` times the CPU restatement of the
reference renderer (the oracle port) on the host cores instead.
`--workload raycast|cornell|batch|diff|refit|build|integrators|calibration`
prints the line of one other configuration.
"""
from __future__ import annotations

import argparse
import copy
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "beamcast-gx-v1.0-beta-_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

N_TRIS = 1_000_000
N_RAYS = 4_194_304
METRIC = "Mpath-segments/s"
RAY_METRIC = "Mrays/s"
WORKLOAD = "raycast: 1M random tris (32-bin SAH -> BVH8), 4M random rays, exact closest hit"
DATA = "synthetic, seeded (tris seed 0xBEAC0002, rays seed 0xBEAC0003)"
ULTRA_WORKLOAD = ("ultra-realism shape: 2,048,130 tris (64x64 displaced icospheres + ground + 64 emissive quads), "
                  "2560x1440, 256 spp, 16 bounces, RR from bounce 6, Halton, MIS, power lights, denoise x3, "
                  "bloom 1, ACES; adaptive stop off (equal spp)")
ULTRA_DATA = "synthetic, seeded (scene seed 0xBEAC0003)"
CPU_SPP_ULTRA = 32   # oracle sample of the frame for cpu_baseline (about 13 s on 16 cores)
REF_SPP_ULTRA = 2    # oracle sample per step of the reference arm
CONVERGED_SPP = 16384


def _dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _make_workload():
    from bcgx import scenes
    spec = scenes.random_triangles(N_TRIS, seed=scenes.SEED_TRIS)
    rays = scenes.random_rays(N_RAYS, seed=scenes.SEED_RAYS)
    return spec, rays


def rank_rays(rank: int, n: int | None = None):
    """The rays one rank casts: the workload's seeded rays on rank 0, the next
    seeds on the other ranks (weak scaling: every rank casts its own rays over
    the replicated scene, with no collective on the data path)."""
    from bcgx import scenes
    return scenes.random_rays(N_RAYS if n is None else n, seed=scenes.SEED_RAYS + rank)


def max_over_ranks(dist, values, device):
    """Element-wise maximum of per-rank values over the process group (a job's
    time is its slowest rank's); without a group, the values themselves."""
    import torch
    t = torch.tensor([float(v) for v in values], device=device, dtype=torch.float64)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t]


def cpu_baseline(spec, rays, seconds_target=15.0, threads=0):
    """The oracle (fp64 restatement of Scene.Hit) on a bounded sample of rays.
    Returns (Mrays/s, cores, sample description, algorithmic bytes per ray)."""
    import numpy as np
    import oracle
    ref = oracle.OracleScene.from_spec(spec)
    cores = threads or os.cpu_count() or 1
    n = 65_536
    t0 = time.perf_counter()
    _, _, cnt = ref.hit_f32(rays[:n], threads=cores)
    dt = time.perf_counter() - t0
    # grow the sample to roughly seconds_target of CPU work
    m = int(min(len(rays), max(n, n * seconds_target / max(dt, 1e-3))))
    rng = np.random.default_rng(1234)
    idx = np.sort(rng.choice(len(rays), m, replace=False))
    sample = np.ascontiguousarray(rays[idx])
    t0 = time.perf_counter()
    _, _, cnt = ref.hit_f32(sample, threads=cores)
    dt = time.perf_counter() - t0
    boxes, tris, sph = (int(x) for x in cnt)
    bytes_per_ray = (32 * boxes + 40 * tris + 32 * sph) / m + 24 + 8
    return m / dt / 1e6, cores, f"{m} of {len(rays)} rays (seeded subset), {dt:.1f} s", bytes_per_ray, \
        {"box_tests_per_ray": boxes / m, "tri_tests_per_ray": tris / m}


def run_reference_raycast(args):
    ws, rank, _ = _dist_env()
    if rank != 0:
        return 0
    spec, rays = _make_workload()
    import numpy as np
    import oracle
    ref = oracle.OracleScene.from_spec(spec)
    cores = os.cpu_count() or 1
    per_step = 262_144
    rng = np.random.default_rng(99)
    for _ in range(args.warmup):
        idx = rng.choice(len(rays), per_step, replace=False)
        ref.hit_f32(np.ascontiguousarray(rays[np.sort(idx)]), threads=cores)
    times = []
    for _ in range(args.steps):
        idx = rng.choice(len(rays), per_step, replace=False)
        sample = np.ascontiguousarray(rays[np.sort(idx)])
        t0 = time.perf_counter()
        ref.hit_f32(sample, threads=cores)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = per_step * args.steps / total / 1e6
    line = {"impl": "reference", "metric": RAY_METRIC, "value": value, "unit": RAY_METRIC, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
            "config": {"workload": WORKLOAD, "rays_per_step": per_step, "triangles": N_TRIS},
            "cpu_baseline": {"value": value, "unit": RAY_METRIC, "cores": cores, "kind": "port",
                             "sample": f"{per_step} seeded rays of the 4M-ray set per step"},
            "e2e": {"value": value, "unit": RAY_METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    line = measure_raycast(args)
    if line is not None:
        print(json.dumps(line), flush=True)
    return 0


def measure_raycast(args, cpu_seconds=15.0):
    """The ray-cast configuration: 1M seeded random triangles (32-bin SAH ->
    BVH8), 4,194,304 seeded rays, exact closest hit. A step is one
    bc_raycast_device over all rays resident in HBM (ray ordering, the walk
    pass, the fp64 settlement pass, the re-trace pass); value = Mrays/s from
    CUDA events on the launching stream, L2 flushed between steps. Returns the
    JSON line on rank 0, None on the other ranks."""
    import numpy as np
    import torch
    import bcgx

    ws, rank, local = _dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from bcgx import scenes
    spec, rays = _make_workload()
    if rank:
        rays = rank_rays(rank)
    scene = scenes.to_scene(spec)
    ctx = bcgx.Context(local)
    if args.minblocks:
        ctx.set_option("raycast_minblocks", args.minblocks)
    if args.fast:
        ctx.set_option("raycast_exact", 0)
    if args.split is not None:
        ctx.set_option("raycast_split", args.split)
    ctx.upload(scene)
    stats = ctx.scene_stats()
    split = bool(ctx.get_option("raycast_split") and ctx.get_option("raycast_exact"))

    stream = torch.cuda.Stream(device=dev)
    d_rays = torch.from_numpy(rays).to(dev)
    d_t = torch.empty(N_RAYS, dtype=torch.float32, device=dev)
    d_p = torch.empty(N_RAYS, dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    tune = ctx.autotune_raycast(d_rays.data_ptr(), N_RAYS) if args.autotune else None

    def step():
        ctx.raycast_device(d_rays.data_ptr(), N_RAYS, d_t.data_ptr(), d_p.data_ptr(), stream.cuda_stream)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()  # L2 flush between steps, outside the events
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    kernel_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(kernel_ms)

    # any hit (bc_occluded_device) over the same rays: reported beside the metric
    d_occ = torch.empty(N_RAYS, dtype=torch.uint8, device=dev)
    ev_any = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
    with torch.cuda.stream(stream):
        ctx.occluded_device(d_rays.data_ptr(), N_RAYS, d_occ.data_ptr(), stream.cuda_stream)
        for a, b in ev_any:
            flush.zero_()
            a.record(stream)
            ctx.occluded_device(d_rays.data_ptr(), N_RAYS, d_occ.data_ptr(), stream.cuda_stream)
            b.record(stream)
    torch.cuda.synchronize()
    any_ms = sum(a.elapsed_time(b) for a, b in ev_any) / len(ev_any)

    # e2e: the host-buffer entry point, pinned host rays, copies inside the region
    h_rays = torch.from_numpy(rays).pin_memory()
    h_np = h_rays.numpy()
    h_t = torch.empty(N_RAYS, dtype=torch.float32).pin_memory().numpy()
    h_p = torch.empty(N_RAYS, dtype=torch.int32).pin_memory().numpy()
    e2e_steps = max(1, min(args.steps, 5))
    ctx.raycast(h_np, h_t, h_p)  # warm the device buffers
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.raycast(h_np, h_t, h_p)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    clk = clocks.stop()

    if dist:
        total_ms, e2e_s = max_over_ranks(dist, [total_ms, e2e_s], dev)
        dist.barrier()
    if rank != 0:
        ctx.close()
        if dist:
            dist.destroy_process_group()
        return None

    value = ws * N_RAYS * args.steps / (total_ms / 1e3) / 1e6
    e2e_value = ws * N_RAYS / e2e_s / 1e6
    peak, peak_kind = _peaks()
    if args.no_cpu_baseline:
        cpu_v, cores, sample, bytes_per_ray, counters = None, 0, "skipped", float("nan"), {}
    else:
        cpu_v, cores, sample, bytes_per_ray, counters = cpu_baseline(spec, rays, seconds_target=cpu_seconds)
    avg_ms = total_ms / args.steps
    achieved = bytes_per_ray * N_RAYS / (avg_ms / 1e3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "k_exact_walk__raycast_1M_tris_4M_rays_traffic.json")
    if os.path.exists(tf):
        with open(tf) as f:
            traffic = json.load(f).get("dram_bytes_per_launch")
    line = {
        "metric": RAY_METRIC, "value": value, "unit": RAY_METRIC, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": avg_ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 traversal + f64 re-test", "data": DATA,
        "config": {"workload": WORKLOAD, "triangles": N_TRIS, "rays_per_gpu": N_RAYS,
                   "l2": "flushed between steps (256 MiB write)", "bvh8_nodes": stats["nodes8"],
                   "bvh8_depth": stats["depth8"], "scene_bytes": stats["device_bytes"]},
        "autotune": tune,
        "e2e": {"value": e2e_value, "unit": RAY_METRIC, "h2d_bytes_per_step": N_RAYS * 32,
                "d2h_bytes_per_step": N_RAYS * 8},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_ray": bytes_per_ray, **counters},
        "cpu_baseline": {"value": cpu_v, "unit": RAY_METRIC, "cores": cores, "kind": "port", "sample": sample},
        # per step: the trace kernel (split form: walk, settle, re-trace), plus the
        # four ray-order kernels (keys, two scans, scatter)
        "gpu_launches": args.steps * ((3 if split else 1) +
                                      (4 if ctx.get_option("raycast_sort") and N_RAYS >= 65536 else 0)),
        "raycast_minblocks": ctx.get_option("raycast_minblocks"),
        "raycast_split": ctx.get_option("raycast_split"),
        "any_hit": {"value": N_RAYS / (any_ms / 1e3) / 1e6, "unit": "Mrays/s", "ms": any_ms,
                    "call": "bc_occluded_device, same rays, L2 flushed"},
        "raycast_exact": ctx.get_option("raycast_exact"),
        "clocks": clk,
        "kernel_ms": [round(x, 4) for x in kernel_ms],
    }
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return line


def _render_roofline(stats, mseg_per_s):
    """Algorithmic bytes per path segment from the oracle's binary-BVH counters on
    the CPU sample (32 B per box test, 40 per triangle, 32 per sphere, 32 of ray in
    and hit out per query incl. shadow rays) plus 160 B of path state read and
    written and 32 B of material per segment; achieved = that x segments/s."""
    segs = max(1, stats["segments"])
    per_seg = (32 * stats["boxes"] + 40 * stats["tris"] + 32 * stats["spheres"] +
               32 * (stats["segments"] + stats["shadow"])) / segs + 160 + 32
    peak, kind = _peaks()
    achieved = per_seg * mseg_per_s * 1e6 / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "peak_kind": kind, "algorithmic_bytes_per_segment": per_seg,
            "scope": "whole frame (all kernels), not one kernel"}


CONVERGED_SPP = 16384


def rmse_vs_converged(scene, spec, cam, st, window, conv_spp=CONVERGED_SPP, threads=0):
    """RMSE of linear HDR radiance (per pixel and channel, post passes off) over a
    pixel window (x0, y0, w, h), against a converged image of that window
    rendered by the oracle (fp64 CPU restatement of the reference's integrator)
    at conv_spp samples per pixel. effectiveSPP caps a render at 4096 samples
    per pixel (renderer.go:2395-2417), so the converged image is the mean of
    conv_spp / 4096 renders of 4096 samples with distinct seeds. Reported at the
    configuration's own spp for the GPU wave engine, the GPU one-kernel form and
    the oracle (each with its own seed, independent of the converged image's),
    plus the GPU's own conv_spp image against the oracle's: with agreeing
    estimators that difference is the two images' residual noise. Equal spp
    gives equal RMSE when the estimators agree, so throughput ratios at equal
    spp are ratios at equal RMSE."""
    import numpy as np
    import bcgx
    import oracle
    x0, y0, w, h = window
    ref = oracle.OracleScene.from_spec(spec)
    flat = st.copy()
    flat.denoise, flat.bloom = False, 0
    conv = flat.copy()
    conv.spp = min(conv_spp, 4096)
    parts = max(1, conv_spp // conv.spp)
    t0 = time.perf_counter()
    cpu_conv = sum(ref.render(cam, conv, seed=0xC0417E + k, threads=threads, window=window)["linear"]
                   for k in range(parts)) / parts
    conv_s = time.perf_counter() - t0
    cpu_eq = ref.render(cam, flat, seed=7, threads=threads, window=window)["linear"]
    ctx = bcgx.Context(0)
    ctx.upload(scene)

    def gpu(settings):
        return ctx.render_rows(cam, settings, y0, h)[0][:, x0:x0 + w].astype(np.float64)

    gpu_eq = gpu(flat)
    ctx.set_option("render_engine", 1)
    one_kernel = gpu(flat)
    ctx.set_option("render_engine", 0)
    gpu_conv = 0.0
    for k in range(parts):
        gc = conv.copy()
        gc.seed = 0x600D + k
        gpu_conv = gpu_conv + gpu(gc)
    gpu_conv = gpu_conv / parts
    ctx.close()

    def rmse(a, b):
        return float(np.sqrt(np.mean((a - b) ** 2)))

    return {"converged": f"oracle (fp64 CPU), {parts * conv.spp} spp ({parts} x {conv.spp}), {w}x{h} pixels at "
                         f"({x0}, {y0}) of the {st.width}x{st.height} frame, {conv_s:.0f} s on "
                         f"{threads or os.cpu_count()} threads",
            "spp": st.spp, "mean_radiance": float(cpu_conv.mean()),
            "gpu": rmse(gpu_eq, cpu_conv), "gpu_one_kernel": rmse(one_kernel, cpu_conv),
            "cpu": rmse(cpu_eq, cpu_conv),
            f"gpu_{parts * conv.spp}spp_vs_converged": rmse(gpu_conv, cpu_conv)}

def measure_render(args):
    """The Cornell-box configuration (320x240, 16 spp, 5 bounces, RR from 3,
    Halton, MIS, power lights; `args.workload == "cornell"`), or the Ultra-shaped
    frame with wall-clock timing (`"ultra-wall"`). value = extension rays (path
    segments) / wall time of the synchronous frame call without readback (the
    device is idle before and after); e2e = the same frame with the linear
    image and RGBA8 read back into pinned host buffers (mean of up to ten
    frames after one untimed read-back frame). Returns the JSON line."""
    import numpy as np
    import torch
    import bcgx
    from bcgx import scenes
    if args.workload == "cornell":
        spec, cam, st = scenes.cornell_box()
        workload = "cornell box: 36 tris, 320x240, 16 spp, 5 bounces, RR from bounce 3, Halton, MIS, power lights"
    else:
        spec, cam, st = scenes.icosphere_grid()
        workload = ("ultra-realism shape: 2,048,130 tris (64x64 displaced icospheres + ground + 64 emissive quads), "
                    "2560x1440, 256 spp, 16 bounces, RR from bounce 6, denoise x3, bloom 1, ACES")
    if args.spp:
        st.spp = args.spp
    if args.adaptive is not None:  # the preset's own adaptive stop (threshold), off for equal-spp measurement
        st.adaptive_sampling, st.adaptive_threshold = True, args.adaptive
    scene = scenes.to_scene(spec)
    ctx = bcgx.Context(0)
    if args.wave_cap:
        ctx.set_option("render_wave_cap", args.wave_cap)
    if args.extend is not None:
        ctx.set_option("render_extend", args.extend)
    ctx.upload(scene)
    L = bcgx.lib()
    import ctypes as C
    cc, sc = cam.c(), st.c()

    W, H = st.width, st.height
    # e2e host outputs: pinned, as a caller that streams frames would hold them
    h_lin = torch.empty((H, W, 3), dtype=torch.float32).pin_memory().numpy()
    h_rgba = torch.empty((H, W), dtype=torch.int32).pin_memory().numpy().view(np.uint32)

    def frame(readback):
        rays = C.c_int64(0)
        lin = h_lin if readback else None
        rgba = h_rgba if readback else None
        t0 = time.perf_counter()
        bcgx._lib.check(L.bc_render_frame(ctx.handle, C.byref(cc), C.byref(sc), bcgx._lib.ptr(lin, C.c_float), None,
                                          bcgx._lib.ptr(rgba, C.c_uint32), C.byref(rays)), ctx.handle)
        return time.perf_counter() - t0, rays.value, lin

    for _ in range(args.warmup):
        frame(False)
    clocks = ClockSampler(0)
    clocks.start()
    times, rays = [], 0
    for _ in range(args.steps):
        dt, r, _ = frame(False)
        times.append(dt)
        rays += r
    frame(True)  # first read-back call: its host-side setup stays out of the e2e figure
    e2e_t, e2e_r = 0.0, 0
    for _ in range(max(1, min(args.steps, 10))):
        dt, r, lin = frame(True)
        e2e_t += dt
        e2e_r += r
    plain = None
    if args.plain_steps > 0:
        # the plain form: one kernel per view, a thread per pixel looping over
        # samples and bounces (the reference's OpenCL kernel shape), same samples
        ctx.set_option("render_engine", 1)
        frame(False)
        pt, pr = [], 0
        for _ in range(args.plain_steps):
            dt, r, _ = frame(False)
            pt.append(dt)
            pr += r
        ctx.set_option("render_engine", 0)
        plain = {"value": pr / sum(pt) / 1e6, "unit": METRIC, "ms_per_step": 1e3 * sum(pt) / len(pt),
                 "steps": len(pt), "form": "one kernel launch per view, thread per pixel (same samples)"}
    clk = clocks.stop()
    value = rays / sum(times) / 1e6
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (float-float primary rays)", "data": "synthetic, seeded",
            "config": {"workload": workload, "spp": st.spp, "segments_per_frame": rays // max(1, args.steps),
                       "extend_variant": ctx.get_option("render_extend"),
                       "shade_block": ctx.get_option("render_shade_block")},
            "e2e": {"value": e2e_r / e2e_t / 1e6, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": st.width * st.height * 16},
            "gpu_launches": None, "clocks": clk}
    if plain:
        line["plain"] = plain
        line["wave_over_plain"] = value / plain["value"]
    if not args.no_cpu_baseline:
        import oracle
        ref = oracle.OracleScene.from_spec(spec)
        cst = st.copy()
        if args.workload != "cornell":  # bounded sample: the full frame at 4 spp
            cst.spp = 4
        else:  # the Cornell frame is tiny: several frames' worth of samples
            cst.spp = 512
        t0 = time.perf_counter()
        out = ref.render(cam, cst, seed=7, threads=0)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": out["stats"]["segments"] / dt / 1e6, "unit": METRIC,
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{cst.width}x{cst.height} at {cst.spp} spp, {dt:.1f} s"}
        line["roofline"] = _render_roofline(out["stats"], value)
    if args.rmse:
        if args.workload == "cornell":
            window = (0, 0, st.width, st.height)  # the whole frame
        else:  # a crop of spheres, ground and emitters around the frame centre
            window = (st.width // 2 - 64, st.height // 2 - 36, 128, 72)
        line["rmse"] = rmse_vs_converged(scene, spec, cam, st, window)
    ctx.close()
    return line


def run_render(args):
    print(json.dumps(measure_render(args)), flush=True)
    return 0


def sum_over_ranks(dist, values, device):
    """Element-wise sum of per-rank values over the process group."""
    import torch
    t = torch.tensor([float(v) for v in values], device=device, dtype=torch.float64)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return [float(x) for x in t]


def _frame_call(ctx, cam, st, seed, lin=None, rgba=None):
    """One bc_render_frame call; returns (wall seconds, extension rays, bc_last_timing)."""
    import bcgx
    q = st.copy()
    q.seed = seed
    cc, sc = cam.c(), q.c()
    rays = C.c_int64(0)
    L = bcgx.lib()
    t0 = time.perf_counter()
    bcgx._lib.check(L.bc_render_frame(ctx.handle, C.byref(cc), C.byref(sc), bcgx._lib.ptr(lin, C.c_float), None,
                                      bcgx._lib.ptr(rgba, C.c_uint32), C.byref(rays)), ctx.handle)
    wall = time.perf_counter() - t0
    return wall, rays.value, ctx.last_timing()


def rmse_gpu_converged(ctx, ref, cam, st, window, conv_spp=CONVERGED_SPP, threads=0):
    """RMSE of linear HDR radiance (post passes off) over a pixel window
    (x0, y0, w, h) against a converged image of that window rendered by the GPU
    wave engine at conv_spp samples per pixel (effectiveSPP caps a render at
    4096, renderer.go:2395-2417, so it is the mean of conv_spp / 4096 renders
    with distinct seeds). Reported at the configuration's spp for the wave
    engine, the one-kernel form (the same samples: equal RMSE by construction)
    and the oracle (an independent seed), each independent of the converged
    image's seeds."""
    import numpy as np
    x0, y0, w, h = window
    flat = st.copy()
    flat.denoise, flat.bloom = False, 0

    def gpu(settings):
        return ctx.render_rows(cam, settings, y0, h)[0][:, x0:x0 + w].astype(np.float64)

    conv = flat.copy()
    conv.spp = min(conv_spp, 4096)
    parts = max(1, conv_spp // conv.spp)
    t0 = time.perf_counter()
    acc = 0.0
    for k in range(parts):
        q = conv.copy()
        q.seed = 0xC0417E + k
        acc = acc + gpu(q)
    conv_img = acc / parts
    conv_s = time.perf_counter() - t0
    eq = flat.copy()
    eq.seed = 7
    wave = gpu(eq)
    ctx.set_option("render_engine", 1)
    try:
        plain = gpu(eq)
    finally:
        ctx.set_option("render_engine", 0)
    t0 = time.perf_counter()
    cpu = ref.render(cam, eq, seed=8, threads=threads, window=window)["linear"]
    cpu_s = time.perf_counter() - t0

    def rmse(a, b):
        return float(np.sqrt(np.mean((a - b) ** 2)))

    return {"converged": f"GPU wave engine, {parts * conv.spp} spp ({parts} x {conv.spp}), {w}x{h} pixels at "
                         f"({x0}, {y0}) of the {st.width}x{st.height} frame, {conv_s:.1f} s",
            "spp": st.spp, "mean_radiance": float(conv_img.mean()),
            "gpu": rmse(wave, conv_img), "gpu_one_kernel": rmse(plain, conv_img), "cpu": rmse(cpu, conv_img),
            "cpu_seconds": round(cpu_s, 2)}


def _kernel_roofline(stats, t, segments):
    """k_extend's roofline: algorithmic bytes per extension query (oracle
    binary-BVH counters: 32 B per box test, 40 per triangle test, 32 per
    sphere test, 24 ray in + 8 hit out) times the frame's queries, over the
    kernel's device time in that frame."""
    queries = max(1, stats["segments"] + stats["shadow"])
    per_query = (32 * stats["boxes"] + 40 * stats["tris"] + 32 * stats["spheres"]) / queries + 32
    peak, kind = _peaks()
    achieved = per_query * segments / (t["extend_ms"] / 1e3) / 1e9
    traffic = None
    tf = os.path.join(ROOT, "profiles", "k_extend__ultra_2560x1440_traffic.json")
    if os.path.exists(tf) and t["extend_launches"]:
        with open(tf) as f:
            per_seg = json.load(f).get("dram_bytes_per_segment")
        if per_seg:
            traffic = per_seg * segments / t["extend_launches"]
    return {"kernel": "k_extend", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "peak_kind": kind,
            "algorithmic_bytes_per_query": per_query,
            "algorithmic_bytes_per_launch": per_query * segments / max(1, t["extend_launches"]),
            "avg_launch_ms": t["extend_ms"] / max(1, t["extend_launches"]),
            "box_tests_per_query": stats["boxes"] / queries, "tri_tests_per_query": stats["tris"] / queries}


def _extras(args):
    """The other configurations, measured in the same run with fewer steps."""
    out = {}
    a = copy.copy(args)
    a.steps, a.warmup, a.rmse, a.autotune = max(3, min(args.steps, 10)), 3, False, False
    try:
        r = measure_raycast(a, cpu_seconds=3.0)
        out["raycast"] = {k: r[k] for k in ("metric", "value", "unit", "ms_per_step", "e2e", "roofline",
                                             "cpu_baseline", "any_hit", "gpu_launches", "clocks")}
        out["raycast"]["workload"] = r["config"]["workload"]
    except Exception as e:  # an extra line never hides the headline
        out["raycast"] = {"error": repr(e)}
    try:
        c = copy.copy(a)
        c.workload, c.steps, c.plain_steps = "cornell", max(10, a.steps), 2
        r = measure_render(c)
        out["cornell"] = {k: r.get(k) for k in ("metric", "value", "unit", "ms_per_step", "e2e", "plain",
                                                 "wave_over_plain", "cpu_baseline", "clocks")}
        out["cornell"]["workload"] = r["config"]["workload"]
    except Exception as e:
        out["cornell"] = {"error": repr(e)}
    try:
        b = copy.copy(a)
        b.steps, b.warmup, b.plain_steps, b.views = 2, 1, 1, 64
        r = measure_batch(b)
        out["batch"] = {k: r.get(k) for k in ("metric", "value", "unit", "ms_per_step", "e2e", "plain",
                                               "batched_over_plain", "plain_one_kernel", "batched_over_one_kernel",
                                               "cpu_baseline", "clocks")}
        out["batch"]["workload"] = r["config"]["workload"]
    except Exception as e:
        out["batch"] = {"error": repr(e)}
    try:
        d = copy.copy(a)
        d.steps, d.warmup = 5, 1
        r = measure_diff(d)
        out["adjoint"] = {k: r.get(k) for k in ("metric", "value", "unit", "forward_s", "backward_s",
                                                 "loss_first_last", "cpu_baseline", "clocks")}
        out["adjoint"]["workload"] = r["config"]["workload"]
    except Exception as e:
        out["adjoint"] = {"error": repr(e)}
    return out


def measure_ultra(args):
    """The headline line (see the module docstring); None on ranks other than 0."""
    import numpy as np
    import torch
    import bcgx
    from bcgx import scenes
    ws, rank, local = _dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    spec, cam, st = scenes.icosphere_grid()
    if args.spp:
        st.spp = args.spp
    if args.adaptive is not None:  # the preset's own adaptive stop (threshold), off for equal-spp measurement
        st.adaptive_sampling, st.adaptive_threshold = True, args.adaptive
    t0 = time.perf_counter()
    scene = scenes.to_scene(spec)
    build_s = time.perf_counter() - t0
    ctx = bcgx.Context(local)
    if args.wave_cap:
        ctx.set_option("render_wave_cap", args.wave_cap)
    if args.extend is not None:
        ctx.set_option("render_extend", args.extend)
    ctx.upload(scene)
    stats = ctx.scene_stats()
    W, H = st.width, st.height
    seed0 = 0x5EED0000 + 7919 * rank  # every rank renders its own samples
    for k in range(args.warmup):
        _frame_call(ctx, cam, st, seed0 + k)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    dev_ms, walls, rays, launches = [], [], 0, 0
    for k in range(args.steps):
        w, r, t = _frame_call(ctx, cam, st, seed0 + 1000 + k)
        dev_ms.append(t["device_ms"])
        walls.append(w)
        rays += r
        launches += t["launches"]
    torch.cuda.synchronize()
    clk = clocks.stop()
    if dist:
        dist.barrier()
    # device time per kernel class of one more frame (an event before every launch)
    ctx.set_option("render_timing", 1)
    try:
        _, kr, kt = _frame_call(ctx, cam, st, seed0 + 1000)
    finally:
        ctx.set_option("render_timing", 0)
    # the plain one-kernel form on the first timed frames' seeds: the same samples
    plain = None
    if args.plain_steps > 0:
        ctx.set_option("render_engine", 1)
        try:
            _frame_call(ctx, cam, st, seed0 + 999)
            pms, pr = [], 0
            for k in range(args.plain_steps):
                _, r, t = _frame_call(ctx, cam, st, seed0 + 1000 + k)
                pms.append(t["device_ms"])
                pr += r
        finally:
            ctx.set_option("render_engine", 0)
        plain = {"value": pr / sum(pms) / 1e3, "unit": METRIC, "ms_per_step": sum(pms) / len(pms),
                 "steps": len(pms), "segments_per_step": pr // len(pms),
                 "form": "one kernel launch per view, thread per pixel looping over samples and bounces "
                         "(the reference OpenCL kernel's shape), same seeds as the first timed frames"}
    # e2e: the reference-facing call with host outputs (pinned), copies inside the region
    lin = torch.empty((H, W, 3), dtype=torch.float32).pin_memory().numpy()
    rgba = torch.empty((H, W), dtype=torch.int32).pin_memory().numpy().view(np.uint32)
    _frame_call(ctx, cam, st, seed0 + 4000, lin, rgba)
    e2e_steps = max(1, min(args.steps, 3))
    ew, er = [], 0
    for k in range(e2e_steps):
        w, r, _ = _frame_call(ctx, cam, st, seed0 + 5000 + k, lin, rgba)
        ew.append(w)
        er += r
    total_ms, e2e_s = sum(dev_ms), sum(ew)
    all_rays, all_e2e_rays = float(rays), float(er)
    if dist:
        total_ms, e2e_s = max_over_ranks(dist, [total_ms, e2e_s], dev)
        all_rays, all_e2e_rays = sum_over_ranks(dist, [rays, er], dev)
        dist.barrier()
    if rank != 0:
        ctx.close()
        if dist:
            dist.destroy_process_group()
        return None
    value = all_rays / (total_ms / 1e3) / 1e6
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (float-float primary rays)", "data": ULTRA_DATA,
            "config": {"workload": ULTRA_WORKLOAD, "spp": st.spp, "segments_per_step": rays // args.steps,
                       "triangles": spec.n_triangles(), "bvh8_nodes": stats["nodes8"],
                       "scene_bytes": stats["device_bytes"], "host_bvh_build_s": round(build_s, 2),
                       "l2": "not flushed: path state (128 Mi paths x 100 B) and scene exceed the 126 MB L2",
                       "wave_cap": ctx.get_option("render_wave_cap"),
                       "extend_variant": ctx.get_option("render_extend"),
                       "shade_block": ctx.get_option("render_shade_block"),
                       "parallelism": f"replicas x{ws}"},
            "wall_ms_per_step": 1e3 * sum(walls) / args.steps,
            "e2e": {"value": all_e2e_rays / e2e_s / 1e6,
                    "unit": METRIC, "steps": e2e_steps,
                    "h2d_bytes_per_step": C.sizeof(bcgx._lib.CameraC) + C.sizeof(bcgx._lib.SettingsC),
                    "d2h_bytes_per_step": W * H * 16,
                    "call": "bc_render_frame, linear HDR + RGBA8 into pinned host buffers, wall clock"},
            "gpu_launches": launches,
            "kernel_times_ms": {k: round(kt[k], 3) for k in ("device_ms", "generate_ms", "extend_ms", "shade_ms",
                                                              "connect_ms", "accumulate_ms", "post_ms", "other_ms")},
            "kernel_share": {k[:-3]: round(kt[k] / max(1e-9, kt["device_ms"]), 4)
                             for k in ("generate_ms", "extend_ms", "shade_ms", "connect_ms", "accumulate_ms",
                                       "post_ms", "other_ms")},
            "clocks": clk,
            "frame_ms": [round(x, 2) for x in dev_ms]}
    if plain:
        line["plain"] = plain
        line["wave_over_plain"] = value / plain["value"]
    ref = None
    if not args.no_cpu_baseline:
        import oracle
        ref = oracle.OracleScene.from_spec(spec)
        cst = st.copy()
        cst.spp = CPU_SPP_ULTRA
        t0 = time.perf_counter()
        out = ref.render(cam, cst, seed=7, threads=0)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": out["stats"]["segments"] / dt / 1e6, "unit": METRIC,
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": f"the full {W}x{H} frame at {cst.spp} spp, {dt:.1f} s"}
        line["roofline"] = _kernel_roofline(out["stats"], kt, kr)
        line["frame_roofline"] = _render_roofline(out["stats"], value)
    if not args.no_rmse and ref is not None:
        line["rmse"] = rmse_gpu_converged(ctx, ref, cam, st, (W // 2 - 64, H // 2 - 36, 128, 72))
    ctx.close()
    if dist:
        dist.destroy_process_group()
    if ws == 1 and not args.no_extras:
        line["configs"] = _extras(args)
    return line


def run_headline(args):
    line = measure_ultra(args)
    if line is not None:
        print(json.dumps(line), flush=True)
    return 0


def run_reference_ultra(args):
    """The reference arm on the headline configuration: the oracle (the
    reference's CPU integrator restated in C++ fp64) on all host cores; a step
    is the full 2560x1440 frame at REF_SPP_ULTRA spp with a new seed."""
    ws, rank, _ = _dist_env()
    if rank != 0:
        return 0
    import oracle
    from bcgx import scenes
    spec, cam, st = scenes.icosphere_grid()
    ref = oracle.OracleScene.from_spec(spec)
    cores = os.cpu_count() or 1
    cst = st.copy()
    cst.spp = REF_SPP_ULTRA
    for k in range(args.warmup):
        ref.render(cam, cst, seed=100 + k, threads=0)
    times, segs = [], 0
    for k in range(args.steps):
        t0 = time.perf_counter()
        out = ref.render(cam, cst, seed=1000 + k, threads=0)
        times.append(time.perf_counter() - t0)
        segs += out["stats"]["segments"]
    value = segs / sum(times) / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": ULTRA_DATA,
            "config": {"workload": ULTRA_WORKLOAD, "spp_per_step": cst.spp, "segments_per_step": segs // args.steps},
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "port",
                             "sample": f"the full {cst.width}x{cst.height} frame at {cst.spp} spp per step"},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_reference(args):
    if args.workload == "raycast":
        return run_reference_raycast(args)
    return run_reference_ultra(args)


def measure_batch(args):
    """Batching workload: 4 resident scenes (10k / 50k / 200k / 500k random
    triangles + one emissive quad each), 64 views (log-uniform 128x128 ..
    1920x1080, spp U{4..64}, 8 bounces). Batched form = one bc_render_batch
    call over all 64 views (one wave engine, captured wave graph); plain form =
    64 sequential one-view calls of the same engine. Both render the same
    samples, so their images are bit-identical (equal RMSE by construction).
    value = path segments / wall time of the batched call without readback
    (the call returns after the device is idle); e2e = the batched call with
    every view's linear image read back to host memory."""
    import numpy as np
    import bcgx
    from bcgx import scenes
    n_views = args.views
    specs, views = scenes.batch_views(n_views=n_views)
    t0 = time.perf_counter()
    built = [scenes.to_scene(s) for s in specs]
    build_s = time.perf_counter() - t0
    ctx = bcgx.Context(0)
    if args.wave_cap:
        ctx.set_option("render_wave_cap", args.wave_cap)
    if args.extend is not None:
        ctx.set_option("render_extend", args.extend)
    ctx.upload_set(built)
    px = sum(st.width * st.height for _, _, st in views)
    paths = sum(st.width * st.height * st.spp for _, _, st in views)

    def batched(readback=False):
        t = time.perf_counter()
        _, r = ctx.render_batch(views, readback=readback)
        return time.perf_counter() - t, r

    def plain():
        t = time.perf_counter()
        r = 0
        for v in views:
            r += ctx.render_batch([v], readback=False)[1]
        return time.perf_counter() - t, r

    tune = ctx.autotune_render(views) if args.autotune else None
    for _ in range(args.warmup):
        batched()
    plain()
    clocks = ClockSampler(0)
    clocks.start()
    bt, br = [], 0
    for _ in range(args.steps):
        dt, r = batched()
        bt.append(dt)
        br += r
    pt, pr = [], 0
    for _ in range(args.steps):
        dt, r = plain()
        pt.append(dt)
        pr += r
    e2e_t, e2e_r = batched(readback=True)
    kernel_form = None
    if args.plain_steps > 0:  # one kernel launch per view (thread per pixel), same samples
        ctx.set_option("render_engine", 1)
        batched()
        kt, kr = [], 0
        for _ in range(args.plain_steps):
            dt, r = batched()
            kt.append(dt)
            kr += r
        ctx.set_option("render_engine", 0)
        kernel_form = {"value": kr / sum(kt) / 1e6, "unit": METRIC, "ms_per_step": 1e3 * sum(kt) / len(kt),
                       "form": f"{n_views} one-kernel launches (thread per pixel looping samples and bounces)"}
    clk = clocks.stop()
    value = br / sum(bt) / 1e6
    plain_v = pr / sum(pt) / 1e6
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(bt) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (float-float primary rays)",
            "data": "synthetic, seeded (seed 0xBEAC0004)",
            "config": {"workload": f"batch: {n_views} views over 4 resident scenes (10k/50k/200k/500k tris), "
                                   "128x128..1920x1080, spp U{4..64}, 8 bounces",
                       "pixels": px, "paths": paths, "segments_per_step": br // max(1, args.steps),
                       "host_bvh_build_s": round(build_s, 2),
                       "wave_cap": ctx.get_option("render_wave_cap"),
                       "extend_variant": ctx.get_option("render_extend"),
                       "shade_block": ctx.get_option("render_shade_block")},
            "plain": {"value": plain_v, "unit": METRIC, "ms_per_step": 1e3 * sum(pt) / args.steps,
                      "form": f"{n_views} sequential one-view bc_render_batch calls"},
            "batched_over_plain": value / plain_v,
            "autotune": tune,
            "plain_one_kernel": kernel_form,
            "batched_over_one_kernel": (value / kernel_form["value"]) if kernel_form else None,
            "e2e": {"value": e2e_r / e2e_t / 1e6, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": px * 12},
            "gpu_launches": None, "clocks": clk}
    if not args.no_cpu_baseline:
        import oracle
        t_all, segs = 0.0, 0
        agg = {"segments": 0, "shadow": 0, "boxes": 0, "tris": 0, "spheres": 0}
        sample = []
        for v in range(4):  # one view of each scene, 1 spp
            k, cam, st = views[v]
            ref = oracle.OracleScene.from_spec(specs[k])
            cst = st.copy()
            cst.spp = 1
            t0 = time.perf_counter()
            out = ref.render(cam, cst, seed=7, threads=0)
            t_all += time.perf_counter() - t0
            segs += out["stats"]["segments"]
            for key in agg:
                agg[key] += out["stats"][key]
            sample.append(f"{cst.width}x{cst.height}")
        line["cpu_baseline"] = {"value": segs / t_all / 1e6, "unit": METRIC, "cores": os.cpu_count(), "kind": "port",
                                "sample": f"views 0-3 (one per scene: {', '.join(sample)}) at 1 spp, {t_all:.1f} s"}
        line["roofline"] = _render_roofline(agg, value)
    if args.rmse:
        # one view of the 500k-triangle scene; a view renders the same image in a
        # batch as alone (bit-identical), so this is its RMSE in the batch too
        v = next(i for i, (k, _, _) in enumerate(views) if k == 3)
        k, cam, st = views[v]
        window = (st.width // 2 - 32, st.height // 2 - 32, 64, 64)
        line["rmse"] = {"view": v, "size": f"{st.width}x{st.height}",
                        **rmse_vs_converged(built[k], specs[k], cam, st, window)}
    ctx.close()
    return line


def run_batch(args):
    print(json.dumps(measure_batch(args)), flush=True)
    return 0


def measure_diff(args):
    """Differentiation workload: 200k random triangles on 256 diffuse material
    slots + 8 emissive quads, 512x512, 64 spp, 8 bounces (Russian roulette
    off). Target = the true parameters at 1024 spp (rendered once, untimed).
    A step is one iteration: bc_forward (parameters in, image + L2 loss) and
    bc_backward (path replay, 256x3 albedo + 8x3 emission gradients out), plus a
    sign-descent update on the host. value = seconds per iteration."""
    import numpy as np
    import bcgx
    from bcgx import scenes
    pb = scenes.diff_scene()
    t0 = time.perf_counter()
    scene = scenes.to_scene(pb.spec)
    build_s = time.perf_counter() - t0
    ctx = bcgx.Context(0)
    ctx.upload(scene)
    st_t = pb.settings.copy()
    st_t.spp = 1024
    ctx.diff_configure(pb.cam, st_t, pb.albedo_materials, pb.emission_materials)
    target, _ = ctx.forward(pb.true_params, 0xBEAC0005)
    ctx.diff_configure(pb.cam, pb.settings, pb.albedo_materials, pb.emission_materials)
    ctx.diff_set_target(target)
    params = pb.init_params.copy()
    na = len(pb.albedo_materials)

    def iteration(it):
        t = time.perf_counter()
        _, loss = ctx.forward(params, 0xBEAC0005 + 1 + it, want_image=False)
        tf = time.perf_counter()
        ga, ge = ctx.backward()
        tb = time.perf_counter()
        params[:na] = np.clip(params[:na] - 0.01 * np.sign(ga), 0.01, 0.99)
        params[na:] = np.maximum(params[na:] - 0.1 * np.sign(ge), 0.0)
        return tb - t, tf - t, tb - tf, loss

    for it in range(args.warmup):
        iteration(it)
    clocks = ClockSampler(0)
    clocks.start()
    times, tfs, tbs, losses = [], [], [], []
    for it in range(args.steps):
        dt, tf, tb, loss = iteration(args.warmup + it)
        times.append(dt)
        tfs.append(tf)
        tbs.append(tb)
        losses.append(loss)
    clk = clocks.stop()
    s_iter = sum(times) / args.steps
    line = {"metric": "adjoint s/iter", "value": s_iter, "unit": "s/iter", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * s_iter, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 paths, f64 gradient sums", "data": "synthetic, seeded (seed 0xBEAC0005)",
            "config": {"workload": "differentiation: 200k tris, 256 albedo slots + 8 emitters, 512x512, 64 spp, "
                                   "8 bounces, RR off, L2 loss vs 1024-spp target",
                       "host_bvh_build_s": round(build_s, 2)},
            "forward_s": sum(tfs) / args.steps, "backward_s": sum(tbs) / args.steps,
            "loss_first_last": [losses[0], losses[-1]],
            "e2e": {"value": s_iter, "unit": "s/iter", "h2d_bytes_per_step": 4 * params.size,
                    "d2h_bytes_per_step": 4 * params.size + 8},
            "gpu_launches": None, "clocks": clk}
    if not args.no_cpu_baseline:
        import oracle
        ref = oracle.OracleScene.from_spec(pb.spec)
        cst = pb.settings.copy()
        cst.spp = 4
        t0 = time.perf_counter()
        out = ref.render(pb.cam, cst, seed=7, threads=0)
        dt = time.perf_counter() - t0
        fwd_s = dt * pb.settings.spp / cst.spp
        line["cpu_baseline"] = {"value": 2 * fwd_s, "unit": "s/iter", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"oracle forward 512x512 at 4 spp ({dt:.1f} s, "
                                          f"{out['stats']['segments'] / dt / 1e6:.1f} Mseg/s), scaled to 64 spp; "
                                          "an iteration counted as two forwards (forward + replay)"}
    if args.rmse:  # the forward's image at the initial parameters
        st = pb.settings
        line["rmse"] = rmse_vs_converged(scene, pb.spec, pb.cam, st, (st.width // 2 - 24, st.height // 2 - 24, 48, 48))
    ctx.close()
    return line


def run_diff(args):
    print(json.dumps(measure_diff(args)), flush=True)
    return 0


def run_refit(args):
    """Geometry-only update of the ray-cast scene (1M random triangles): 1% of
    the triangles move, Scene.Refit (host builder) refits the node boxes, and
    bc_scene_upload takes the device path (primitives and boxes copied up,
    slots rewritten, every BVH8 node re-quantized on the GPU). Compared with a
    full upload of the same scene (host validation, BVH8 collapse, packing).
    Time per step = wall time of the bc_scene_upload call (host refit excluded)."""
    import numpy as np
    import bcgx
    from bcgx import scenes
    spec = scenes.random_triangles(N_TRIS)
    scene = scenes.to_scene(spec)
    ctx = bcgx.Context(0)
    ctx.upload(scene)
    rng = np.random.default_rng(0xBEAC0106)
    geo, full, refit_s = [], [], []
    for k in range(args.warmup + args.steps):
        for i in rng.choice(N_TRIS, N_TRIS // 100, replace=False):
            scene.translate_primitive(int(i), rng.normal(0.0, 0.002, 3))
        t0 = time.perf_counter()
        scene.refit()
        t1 = time.perf_counter()
        ctx.upload(scene)
        t2 = time.perf_counter()
        ctx.upload(scene, scene_id=0x5EED0000 + k)  # full path
        t3 = time.perf_counter()
        ctx.upload(scene)  # back to the tracked id for the next drag (full path again)
        if k >= args.warmup:
            refit_s.append(t1 - t0)
            geo.append(t2 - t1)
            full.append(t3 - t2)
    stats = ctx.scene_stats()
    line = {"metric": "geometry update ms", "value": 1e3 * statistics.median(geo), "unit": "ms",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(geo),
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64 in, f32/f64 records",
            "data": "synthetic, seeded (tris seed 0xBEAC0002)",
            "config": {"workload": f"refit: {N_TRIS} random tris, 1% moved per step", "bvh8_nodes": stats["nodes8"],
                       "binary_nodes": stats["binary_nodes"]},
            "full_upload_ms": 1e3 * statistics.median(full),
            "host_refit_ms": 1e3 * statistics.median(refit_s),
            "geometry_updates": stats["geometry_updates"],
            "e2e": {"value": 1e3 * statistics.median(geo), "unit": "ms",
                    "h2d_bytes_per_step": 8 * (16 * N_TRIS + 6 * stats["binary_nodes"]), "d2h_bytes_per_step": 0},
            "gpu_launches": 2 * args.steps}
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def run_build(args):
    """Binned SAH build (32 bins, leaf 4) of the ray-cast scene (1M random
    triangles) and of the Ultra-shaped scene (2,048,130 triangles): the host
    builder (the reference's buildNodeSAH restated in C++, one thread) vs the
    device build (bc_build_sah: same nodes and Order, bit for bit; host-side
    light distribution and array copies included in its time)."""
    import numpy as np
    import bcgx
    from bcgx import scenes
    ctx = bcgx.Context(0)
    out = {}
    for name, spec in (("random_1M", scenes.random_triangles(N_TRIS)), ("ultra_2M", scenes.icosphere_grid()[0])):
        host = scenes.to_scene(spec, build=False)
        dev = scenes.to_scene(spec, build=False)
        for s_ in (host, dev):
            s_.bvh_mode, s_.bvh_bins, s_.bvh_leaf = "SAH", 32, 4
        th, td = [], []
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            dev.build_device(ctx)
            t1 = time.perf_counter()
            if k >= args.warmup:
                td.append(t1 - t0)
        for k in range(max(1, min(args.steps, 2))):
            t0 = time.perf_counter()
            host.build()
            th.append(time.perf_counter() - t0)
        same = all(np.array_equal(x, y) for x, y in zip(
            (host.arrays().node_left, host.arrays().order), (dev.arrays().node_left, dev.arrays().order)))
        out[name] = {"prims": spec.n_triangles(), "device_ms": 1e3 * statistics.median(td),
                     "host_ms": 1e3 * statistics.median(th), "identical": bool(same)}
    value = out["ultra_2M"]["device_ms"]
    line = {"metric": "SAH build ms", "value": value, "unit": "ms", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": value, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic, seeded",
            "config": {"workload": "binned SAH build, 32 bins, leaf 4: Ultra-shaped scene (value) and 1M random tris"},
            "builds": out,
            "cpu_baseline": {"value": out["ultra_2M"]["host_ms"], "unit": "ms", "cores": 1, "kind": "port",
                             "sample": "the host builder (buildNodeSAH restated), whole Ultra-shaped scene"},
            "e2e": {"value": value, "unit": "ms", "h2d_bytes_per_step": 72 * out["ultra_2M"]["prims"],
                    "d2h_bytes_per_step": 4 * out["ultra_2M"]["prims"] + 2 * out["ultra_2M"]["prims"] * 64},
            "gpu_launches": None}
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def _bench_settings(w, h, spp, bounces):
    """benchmarkSettings (benchmark.go:71-94): Draft with adaptive sampling, post
    and upscaling off, Random sampler, MIS, power-weighted lights, 16-bin SAH."""
    import bcgx
    q = bcgx.quality("Draft")
    q.width, q.height, q.spp, q.bounces = w, h, spp, bounces
    q.adaptive_sampling, q.denoise = False, False
    q.fxaa, q.taa, q.tsaa, q.txaa, q.hbao, q.hbao_plus, q.bloom = 0, 0, 0, 0, 0, 0, 0
    q.msaa, q.sampler, q.mis, q.power_light_sampling = 1, "Random", True, True
    q.bvh_mode, q.bvh_bins, q.bvh_leaf_size = "SAH", 16, 4
    return q


def run_integrators(args):
    """The reference's integrator comparison (benchmarkIntegrators,
    benchmark.go:202-216): the Cornell-like room at 384x216, 2 spp, 5 bounces,
    for the path, recursive and photon-mapping integrators (PhotonMapping 1).
    A step is one frame through bc_render_frame (post off) with a new seed, so
    the photon integrator rebuilds its photon map every frame as Start does.
    value = rays (path segments, plus the photon map's) / frame time. One JSON
    line per integrator; `large` repeats the frame at 1920x1080, 64 spp."""
    import ctypes as C
    import numpy as np
    import bcgx
    from bcgx import scenes
    spec, cam = scenes.cornell_reference_scene()
    ctx = bcgx.Context(0)
    ctx.upload(scenes.to_scene(spec))
    L = bcgx.lib()
    cc = cam.c()

    def frames(st, n, seed0, readback=False):
        times, rays = [], 0
        for k in range(n):
            q = st.copy()
            q.seed = seed0 + k
            sc = q.c()
            r = C.c_int64(0)
            lin = np.empty((q.height, q.width, 3), np.float32) if readback else None
            t0 = time.perf_counter()
            bcgx._lib.check(L.bc_render_frame(ctx.handle, C.byref(cc), C.byref(sc), bcgx._lib.ptr(lin, C.c_float),
                                              None, None, C.byref(r)), ctx.handle)
            times.append(time.perf_counter() - t0)
            rays += r.value
        return times, rays

    for integ in (bcgx.INTEGRATOR_PATH, bcgx.INTEGRATOR_RECURSIVE, bcgx.INTEGRATOR_PHOTON):
        st = _bench_settings(384, 216, 2, 5)
        st.integrator = integ
        if integ == bcgx.INTEGRATOR_PHOTON:
            st.photon_mapping = 1
        frames(st, args.warmup, 1000)
        clocks = ClockSampler(0)
        clocks.start()
        times, rays = frames(st, args.steps, 2000)
        big = st.copy()
        big.width, big.height, big.spp = 1920, 1080, 64
        frames(big, 1, 3000)
        bt, br = frames(big, 2, 3100)
        clk = clocks.stop()
        frames(st, 1, 3900, readback=True)  # the first read-back frame after the large one sets up buffers
        et, er = frames(st, 5, 4000, readback=True)
        value = rays / sum(times) / 1e6
        line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": 1, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 (float-float primary rays)",
                "data": "synthetic, seeded",
                "config": {"workload": f"integrator comparison: Cornell-like room, 384x216, 2 spp, 5 bounces, "
                                       f"{integ}" + (", PhotonMapping 1" if st.photon_mapping else ""),
                           "rays_per_frame": rays // max(1, args.steps)},
                "large": {"value": br / sum(bt) / 1e6, "unit": METRIC, "ms_per_frame": 1e3 * sum(bt) / len(bt),
                          "frame": "1920x1080, 64 spp"},
                "e2e": {"value": er / sum(et) / 1e6, "unit": METRIC, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": st.width * st.height * 12},
                "gpu_launches": None, "clocks": clk}
        if not args.no_cpu_baseline:
            import oracle
            ref = oracle.OracleScene.from_spec(spec)
            cst = st.copy()
            cst.spp = 2048
            t0 = time.perf_counter()
            out = ref.render(cam, cst, seed=7, threads=0)
            dt = time.perf_counter() - t0
            segs = out["stats"]["segments"] + out["stats"]["photon_rays"]
            line["cpu_baseline"] = {"value": segs / dt / 1e6, "unit": METRIC, "cores": os.cpu_count(),
                                    "kind": "port", "sample": f"384x216 at 2048 spp, {dt:.1f} s"}
            line["roofline"] = _render_roofline(out["stats"], value)
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def run_calibration(args):
    """CPU-baseline calibration: the oracle on the reference's published CPU case
    (GIGA suite "CPU scaling", benchmarkSettings(448, 252, 4, 6, workers) on
    NewStressScene: 902,710 rays, 2.70 Mray/s on 1 worker and 4.91 on 2 of an
    unnamed 5-CPU container), on 1 and 2 threads of this host. No GPU work."""
    import oracle
    from bcgx import scenes
    spec, cam = scenes.stress_scene()
    ref = oracle.OracleScene.from_spec(spec)
    q = _bench_settings(448, 252, 4, 6)
    out = {"metric": "Mrays/s per worker", "impl": "oracle", "workload":
           "Stress scene 448x252, 4 spp, 6 bounces (benchmarkSettings)",
           "reference_published": {"1": 2.70, "2": 4.91, "rays": 902710}}
    for th in (1, 2):
        best = None
        for _ in range(3):
            t0 = time.perf_counter()
            r = ref.render(cam, q, seed=1, threads=th)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        out[str(th)] = r["stats"]["segments"] / best / 1e6
        out["rays"] = r["stats"]["segments"]
    print(json.dumps(out), flush=True)
    return 0


def main():
    global N_TRIS, N_RAYS
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--tris", type=int, default=N_TRIS, help="ray cast: smaller case for profiling")
    ap.add_argument("--rays", type=int, default=N_RAYS, help="ray cast: smaller case for profiling")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU leg (profiling runs)")
    ap.add_argument("--no-rmse", action="store_true", help="headline: skip the RMSE leg")
    ap.add_argument("--no-extras", action="store_true", help="headline: skip the other configurations")
    ap.add_argument("--minblocks", type=int, default=0, help="ray-cast register variant (1, 6, 8; 0 = library default)")
    ap.add_argument("--split", type=int, default=None, help="ray cast: raycast_split 0 or 1 (default: library default)")
    ap.add_argument("--fast", action="store_true", help="plain fp32 closest hit instead of the exact contract")
    ap.add_argument("--workload", default="ultra",
                    choices=["ultra", "raycast", "cornell", "ultra-wall", "batch", "diff", "refit", "build",
                             "integrators", "calibration"],
                    help="ultra (default: the headline line) or another configuration")
    ap.add_argument("--spp", type=int, default=0, help="override spp of a render workload")
    ap.add_argument("--extend", type=int, default=None, help="render workloads: render_extend variant 0, 1 or 2")
    ap.add_argument("--rmse", action="store_true",
                    help="cornell/batch/diff: RMSE against an oracle-converged image (slow)")
    ap.add_argument("--views", type=int, default=64, help="batch workload: number of views")
    ap.add_argument("--adaptive", type=float, default=None,
                    help="render workloads: turn the adaptive stop on with this threshold (Ultra preset: 8e-5)")
    ap.add_argument("--wave-cap", type=int, default=0, help="render workloads: paths per wave (0 = library default)")
    ap.add_argument("--autotune", action="store_true",
                    help="raycast and batch workloads: run the autotuner on the workload before timing")
    ap.add_argument("--plain-steps", type=int, default=2,
                    help="render workloads: frames timed with the one-kernel form (0 = skip)")
    args = ap.parse_args()
    N_TRIS, N_RAYS = args.tris, args.rays
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    runners = {"ultra": run_headline, "raycast": run_gpu, "cornell": run_render, "ultra-wall": run_render,
               "batch": run_batch, "diff": run_diff, "refit": run_refit, "build": run_build,
               "integrators": run_integrators, "calibration": run_calibration}
    return runners[args.workload](args)


if __name__ == "__main__":
    sys.exit(main())

#!/usr/bin/env python
"""Benchmark of the raster hot path on GB300.

Default workload (one JSON line on stdout): the fused stencil -- hillshade +
slope (degrees) + profile and planform curvature, float32 outputs -- over a
32768 x 32768 float32 fBm DEM (Hurst 0.7, 0-4000 m, 5 m pixels, ~2 % NoData
disks) cut into 4096^2 tiles with an 8 px halo, all tiles in one launch.

  value      Mpix/s with the DEM resident in HBM (device-timed, CUDA events)
  e2e        Mpix/s through the C ABI with host (pinned) buffers
             (fsg_stencil_host): the per-tile H2D copies of the DEM windows
             and the D2H copies of the four planes are inside the timed region
  roofline   the fused kernel against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle (NumPy/SciPy restatement of the reference's
             block functions) on a bounded sample, on the host cores

``--impl reference`` times the reference's CPU algorithm (the oracle port;
the reference itself is CuPy-only and cannot run on the host) with all host
cores on the same workload definition.

The line also carries ``extra``, each section device-timed (``--no-extra``
skips them; ``--workload <section>`` prints one section alone):
  topousm_fast       the tile loop at 32768^2, radii 2..2048
  openness           16384^2, 16 directions, R = 256: the reference's 10-sample
                     rays, and the dense every-step march on a 4096^2 crop
  ambient_occlusion  16384^2, 16 samples x 4 rings, radius 10 and 30
  prepare            NoData detection and void fill of a 32768^2 DEM
  openness_surrogate the CNN surrogate against the exact kernels
  spatial            spatial (multi-radius) mode of the stencil products and
                     openness at 8192^2
  batched            uneven tiles over a 3-level overview pyramid (hillshade,
                     topousm_fast, openness) as prepared plans replayed in one
                     CUDA graph
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpix/s on 32k² DEM; exact vs surrogate openness at ≤2° MAE; % of HBM roofline"


# ----------------------------------------------------------------- utilities
def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), float(d.get("bf16_tflops", 1900.0)), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        # wait for the first sample: nvidia-smi's NVML start-up must not overlap the timed region
        t0 = time.time()
        while self.proc is not None and time.time() - t0 < 10.0:
            try:
                if os.path.getsize(self.path) > 0:
                    break
            except OSError:
                pass
            time.sleep(0.05)
        time.sleep(0.3)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                    power.append(float(parts[3]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power) if power else None}


def dist_setup(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], device="cuda", dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------- CPU oracle baseline
# The CPU legs use the GPU workload's NoData law: disks of radius U(10, 200) px
# at 122 disks per 16384^2 (~2 % of the pixels), i.e. 2 disks per 2048^2 tile.
CPU_TILE = 2048
CPU_NODATA = {"disks": (2, 10.0, 200.0)}
CPU_NODATA_NOTE = "NoData: 2 disks of radius U(10,200) px per tile (the GPU workload's 122 per 16384^2)"
def _cpu_tile_job(args):
    """One tile of the reference's CPU algorithm (oracle port), returns core pixels."""
    kind, seed, core, pad, params = args
    import numpy as np
    from fujishadergpu_gb300 import synth
    from oracle import restated as R
    n = core + 2 * pad
    dem = synth.fbm(n, n, hurst=0.7, seed=seed, lo=0.0, hi=4000.0)
    disks = params.get("disks", (2, 10.0, 60.0))  # (count, rmin, rmax) of the NoData disks
    dem[synth.nodata_disks(n, n, count=disks[0], seed=seed + 1, rmin=disks[1], rmax=disks[2])] = np.nan
    t0 = time.perf_counter()
    if kind == "stencil":
        kw = dict(pixel_size=5.0, psx=5.0, psy=-5.0)
        R.hillshade(dem, **kw)
        R.slope(dem, **kw)
        R.curvature(dem, curvature_type="profile", **kw)
        R.curvature(dem, curvature_type="planform", **kw)
    elif kind == "topousm":
        R.topousm_block(dem, radii=params["radii"], weights=params["weights"], pixel_size=params["px"])
    elif kind == "openness":
        R.openness(dem, openness_type="positive", num_directions=16, max_distance=params["md"],
                   pixel_size=5.0, psx=5.0, psy=-5.0)
    elif kind == "ambient_occlusion":
        R.ambient_occlusion(dem, num_samples=16, radius=params["radius"], pixel_size=5.0, psx=5.0, psy=-5.0)
    elif kind == "prepare":
        R.prepare_dem(dem, fill_mode="enclosed", coarse_max=params["coarse_max"])
    return core * core, time.perf_counter() - t0


def cpu_oracle_rate(kind: str, *, procs: int, tiles: int, core: int, pad: int, params=None, seed=100):
    """Mpix/s of the oracle over ``tiles`` tiles on ``procs`` processes (spawned)."""
    jobs = [(kind, seed + 7 * i, core, pad, params or {}) for i in range(tiles)]
    if procs <= 1:
        t0 = time.perf_counter()
        px = sum(_cpu_tile_job(j)[0] for j in jobs)
        return px / (time.perf_counter() - t0) / 1e6
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        pool.map(_cpu_tile_job, jobs[:procs])  # warm the workers (imports, FFT plans)
        t0 = time.perf_counter()
        res = pool.map(_cpu_tile_job, jobs)
        wall = time.perf_counter() - t0
    return sum(r[0] for r in res) / wall / 1e6


# ----------------------------------------------------------- stencil workload
def stencil_workload(args, rank, world, out_dtype="float32"):
    import numpy as np
    import torch

    from fujishadergpu_gb300 import _arrays, _native, synth
    from fujishadergpu_gb300.algorithms import _stencil as S
    from fujishadergpu_gb300.core import tile_loop

    H = W = args.size
    tile, halo = args.tile, args.halo
    torch.manual_seed(0)
    # one raster for the whole job: every rank generates it and computes its band of tile rows
    dem = synth.fbm_device(H, W, hurst=0.7, seed=2, lo=0.0, hi=4000.0)
    ndisks = max(1, int(round(122 * (H * W) / (16384.0 * 16384.0))))
    synth.nodata_disks_device(dem, count=ndisks, seed=3)
    nodata_frac = float(torch.isnan(dem).float().mean().item())
    names = ["hillshade", "slope", "curvature_profile", "curvature_planform"]
    from fujishadergpu_gb300.io.output_encoding import quantize_params
    tdt = torch.float32 if out_dtype == "float32" else torch.uint8
    esz = 4 if out_dtype == "float32" else 1
    qps = {n: (None if out_dtype == "float32" else
               quantize_params(0.0, 90.0 if n == "slope" else 1.0, out_dtype)) for n in names}
    alg_bytes = 4 + 4 * esz   # DEM read + the four planes written, per pixel
    outs = {n: torch.empty((H, W), device="cuda", dtype=tdt) for n in names}
    view = _arrays.as_device_f32_2d(dem)
    params = S.make_params(azimuth=315.0, altitude=45.0, pixel_size=5.0)
    planes = {S.OUTPUT_INDEX[n]: S.make_plane(outs[n], out_dtype, qps[n]) for n in names}
    from fujishadergpu_gb300.core.sharding import shard_tiles
    infos = shard_tiles(tile_loop.tile_grid(H, W, tile, halo), world, rank)
    tiles = tile_loop.make_tiles(infos, pixel_scale_x=5.0, pixel_scale_y=-5.0)
    px_rank = sum(t.core_h * t.core_w for t in infos)
    stream = torch.cuda.current_stream()
    sh = int(stream.cuda_stream)

    def step():
        S.launch(view, tiles, params, planes, stream=sh)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    n0 = _native.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with _native.kernel_timer(max_launches=args.steps) as kt:  # the streaming pass of each step (CUDA events)
        e0.record(stream)
        for _ in range(args.steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    launches = _native.launch_count() - n0
    fast_ms = kt.ms / max(1, kt.launches)
    barrier(world)
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    ms = max_over_ranks(ms, world)
    px = H * W                 # the job: one raster over all ranks (strong scaling)
    value = px / (ms * 1e-3) / 1e6
    hbm, _, peak_kind = peaks()
    # dominant kernel: the streaming pass of this rank over its band (px_rank pixels)
    achieved = alg_bytes * px_rank / (fast_ms * 1e-3) / 1e9
    step_gbs = alg_bytes * px_rank / (e0.elapsed_time(e1) / args.steps * 1e-3) / 1e9  # whole step

    # ---- e2e: host (pinned) buffers through the C ABI (fsg_stencil_host): this rank's band
    # of the DEM and of the four planes in host memory; per row band of tiles one H2D
    # block, one kernel call, one D2H block per plane, overlapped on three streams
    wy0 = min(int(t.win_y0) for t in tiles)
    wy1 = max(int(t.win_y0) + int(t.win_h) for t in tiles)
    cy0 = min(int(t.core_y0) for t in tiles)
    cy1 = max(int(t.core_y0) + int(t.core_h) for t in tiles)
    host_dem = torch.empty((wy1 - wy0, W), dtype=torch.float32, pin_memory=True)
    host_dem.copy_(dem[wy0:wy1])
    host_out = {n: torch.empty((cy1 - cy0, W), dtype=tdt, pin_memory=True) for n in names}
    hplanes = {S.OUTPUT_INDEX[n]: S.host_plane(host_out[n], out_dtype, qps[n]) for n in names}
    htiles = []
    for t in tiles:  # the same tiles in the coordinates of the host buffers
        u = _native.Tile()
        u.win_y0, u.win_x0, u.win_h, u.win_w = t.win_y0 - wy0, t.win_x0, t.win_h, t.win_w
        u.core_y0, u.core_x0, u.core_h, u.core_w = t.core_y0 - wy0, t.core_x0, t.core_h, t.core_w
        u.out_y0, u.out_x0 = t.out_y0 - cy0, t.out_x0
        u.pixel_scale_x, u.pixel_scale_y = t.pixel_scale_x, t.pixel_scale_y
        htiles.append(u)
    # the host loop copies each row band's window union once (one block per band)
    bands = {}
    for t in htiles:
        k = (int(t.core_y0), int(t.win_y0), int(t.win_h))
        x0, x1 = bands.get(k, (1 << 30, -1))
        bands[k] = (min(x0, int(t.win_x0)), max(x1, int(t.win_x0) + int(t.win_w)))
    h2d_bytes = sum(k[2] * (x1 - x0) * 4 for k, (x0, x1) in bands.items())
    d2h_bytes = px_rank * esz * len(names)

    def e2e_step():
        S.launch_host(host_dem, htiles, params, hplanes, stream=sh)

    for _ in range(max(1, min(args.warmup, 2))):
        e2e_step()
    torch.cuda.synchronize()
    barrier(world)
    e2e_steps = max(2, min(args.steps, 5))
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(e2e_steps + 1)]
    e0.record(stream)
    marks[0].record(stream)
    for i in range(e2e_steps):
        e2e_step()
        marks[i + 1].record(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1) / e2e_steps, world)
    # per-step times: single steps have run up to ~40 % slower than the steady ones
    e2e_each = [round(marks[i].elapsed_time(marks[i + 1]), 2) for i in range(e2e_steps)]
    # correctness spot check of the host path against the device planes
    ok = all(torch.equal(host_out[n][::4097, ::4097].cuda().float().nan_to_num(-7.0),
                         outs[n][cy0:cy1][::4097, ::4097].float().nan_to_num(-7.0)) for n in names)
    link = host_link(host_out[names[0]], outs[names[0]][cy0:cy1], host_dem, dem[wy0:wy1], stream)
    link["floor_ms"] = round(max(d2h_bytes / (link["d2h_gbs"] * 1e9), h2d_bytes / (link["h2d_gbs"] * 1e9)) * 1e3, 2)
    link["e2e_frac_of_floor"] = round(link["floor_ms"] / e2e_ms, 3)
    del host_dem, host_out

    line = {
        "metric": METRIC,
        "value": round(value, 1),
        "unit": "Mpix/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms, 4),
        "higher_is_better": True,
        "scaling": "strong",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded spectral fBm, Hurst 0.7, 0-4000 m, NoData disks)",
        "config": {"workload": f"fused hillshade+slope(deg)+profile+planform curvature, {out_dtype} planes",
                   "raster": [H, W], "pixel_m": 5.0, "tile": tile, "halo": halo, "tiles": len(tiles),
                   "nodata_frac": round(nodata_frac, 4), "outputs": names,
                   "l2": "inputs larger than L2 (DEM %.1f GiB, no flush)" % (px * 4 / 2 ** 30),
                   "parallelism": (f"one {H}x{W} raster; each of the {world} GPUs computes a band of tile rows"
                                   " (no data-path collective)")},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "peak_kind": peak_kind + " (burst copy)",
                     "kernel": "stencil_fast_kernel (fused streaming pass)", "kernel_ms": round(fast_ms, 4),
                     "algorithmic_bytes_per_px": alg_bytes,
                     "algorithmic_bytes_per_launch": alg_bytes * px_rank,
                     "traffic": (profiled_traffic("stencil_fast_kernel_fused4_f32", px_rank)
                                 if out_dtype == "float32" else None),
                     "step_achieved": round(step_gbs, 1), "step_frac": round(step_gbs / hbm, 4)},
        "e2e": {"value": round(px / (e2e_ms * 1e-3) / 1e6, 1), "unit": "Mpix/s",
                "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": d2h_bytes,
                "ms_per_step": round(e2e_ms, 3), "ms_each_step": e2e_each, "matches_device_path": bool(ok),
                "path": "fsg_stencil_host (C ABI): pinned host DEM and planes; per row band of tiles one "
                        "H2D block, one kernel call, one D2H block per plane, overlapped on 3 streams",
                "host_link": link},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    return line


def host_link(host_a, dev_a, host_b, dev_b, stream) -> dict:
    """Copy bandwidth of the host link in this process: one device-to-host copy of
    ``dev_a`` into pinned ``host_a`` and one host-to-device copy of pinned ``host_b``
    into ``dev_b``, each alone (best of three, CUDA events on ``stream``).  The e2e
    floor is the larger of (D2H bytes / D2H rate, H2D bytes / H2D rate): the two
    directions overlap."""
    import torch

    def best(fn):
        t = []
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            t.append(e0.elapsed_time(e1))
        return min(t)

    with torch.cuda.stream(stream):
        d2h = best(lambda: host_a.copy_(dev_a, non_blocking=True))
        h2d = best(lambda: dev_b.copy_(host_b, non_blocking=True))
    nb_a = host_a.numel() * host_a.element_size()
    nb_b = host_b.numel() * host_b.element_size()
    return {"d2h_gbs": round(nb_a / (d2h * 1e-3) / 1e9, 1), "h2d_gbs": round(nb_b / (h2d * 1e-3) / 1e9, 1),
            "probe_bytes": [nb_a, nb_b]}


def profiled_value(kind: str, key: str):
    """The number on the ``key:`` line of the committed ncu summary profiles/<kind>.txt."""
    p = os.path.join(ROOT, "profiles", f"{kind}.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.strip().startswith(key + ":"):
                return float(line.split(":", 1)[1].split()[0])
    return None


def clocks_max_mhz():
    """clocks.max.sm of GPU 0 from nvidia-smi, or None."""
    try:
        r = subprocess.run(["nvidia-smi", "--query-gpu=clocks.max.sm", "--format=csv,noheader,nounits", "-i", "0"],
                           capture_output=True, text=True, timeout=20)
        return float(r.stdout.strip().splitlines()[0])
    except Exception:
        return None


def profiled_traffic(kind: str, px: int):
    """DRAM read+write bytes of the dominant kernel's launch, scaled to ``px`` pixels from
    the ``dram_bytes_per_px:`` line of the committed ncu summary (None if absent)."""
    p = os.path.join(ROOT, "profiles", f"{kind}.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.strip().startswith("dram_bytes_per_px:"):
                return int(round(float(line.split(":", 1)[1].split()[0]) * px))
    return None


# ------------------------------------------------------------ extra sections
def _time_ms(fn, steps, warmup, stream):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def tc_issued_flops(radii_full, n_tiles):
    """Tensor FLOPs the tcgen05 topousm kernel issues: per 128 x 192 CTA tile and
    full-resolution radius r, pass 1 = two column halves x the K steps (16 input rows)
    the band reaches x 3 digit MMAs of 128 x 128 x 16; pass 2 = the K steps (16 input
    columns) x 3 split MMAs of 128 x 192 x 16 (the K-step ranges of fsg_topousm_tc.cu)."""
    def ceil_div(a, b):
        return -((-a) // b)
    per = 0
    for r in radii_full:
        j1lo, j1hi = max(0, ceil_div(17 - r, 16)), min(11, (159 + r) // 16)
        j2lo, j2hi = max(0, ceil_div(17 - r, 16)), min(15, (223 + r) // 16)
        per += 2 * (j1hi - j1lo + 1) * 3 * 2 * 128 * 128 * 16
        per += (j2hi - j2lo + 1) * 3 * 2 * 128 * 192 * 16
    return per * n_tiles


def topousm_section(args):
    """topousm_fast on a 32768^2 fBm+ridged DEM (Hurst 0.8, 0-3500 m, 10 m), radii 2..2048 with
    2^n weights, 4096^2 tiles.  One step = the whole tile loop with the global scale known: NaN-aware
    overview + large-radius coarse field + every tile's small-radius pass and normalisation.
    Both arithmetic paths of the full-resolution box means are timed: "exact" (64-bit fixed-point
    running sums on the CUDA cores) and "tensor" (split-BF16 banded products on tcgen05), each
    with its error against the float64 oracle on one 4096^2 tile window."""
    import numpy as np
    import torch
    from fujishadergpu_gb300 import _native, synth
    from fujishadergpu_gb300.algorithms import _impl_topousm_fast as TU
    from fujishadergpu_gb300.core import tile_loop
    n = args.topousm_size
    dem = synth.fbm_ridged_device(n, n, hurst=0.8, seed_fbm=3, seed_ridged=4, lo=0.0, hi=3500.0)
    radii = [2, 8, 32, 128, 512, 2048]
    w = [2.0 ** (5 - i) for i in range(6)]
    w = [x / sum(w) for x in w]
    kw = dict(tile_size=4096, pixel_size=10.0, radii=radii, weights=w)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = tile_loop.process_dem_array(dem, "topousm_fast", **kw)
    torch.cuda.synchronize()
    first_s = time.perf_counter() - t0
    stats, pad = res.stats, res.padding
    del res
    stream = torch.cuda.current_stream()
    px = n * n
    hbm, _, _ = peaks()
    pk = {}
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
    except OSError:
        pass
    bf16 = float(pk.get("bf16_tflops", 1900.0))
    # CTA tiles of the tensor kernel: 128 x 192 over every 4096^2 core
    ntile_rows = -(-min(4096, n) // 128)
    ntile_cols = -(-min(4096, n) // 192)
    n_cta = (-(-n // 4096)) ** 2 * ntile_rows * ntile_cols
    small = [r for r in radii if r <= max(256, 4096 // 16)]
    full_res = [r for r in small if TU.downsample_factor(r, 10.0) == 1]
    out = {"workload": f"topousm_fast {n}x{n} fBm+ridged, radii {radii}, 2^n weights, 10 m, 4096^2 tiles",
           "first_call_s_incl_stats_prepass": round(first_s, 3),
           "p99_scale": float(stats[0]) if stats else None, "dtype": "f32"}
    for path in ("exact", "tensor"):
        with _native.kernel_timer(max_launches=args.extra_steps + 2) as kt:
            ms = _time_ms(lambda: tile_loop.process_dem_array(dem, "topousm_fast", global_stats=stats,
                                                              topousm_path=path, **kw),
                          args.extra_steps, 2, stream)
        kms = kt.ms / max(1, kt.launches)
        gbs = 8.0 * px / (ms * 1e-3) / 1e9
        kgbs = 8.0 * px / (kms * 1e-3) / 1e9
        sec = {"value": round(px / (ms * 1e-3) / 1e6, 1), "unit": "Mpix/s", "ms_per_step": round(ms, 3),
               "roofline": {"bound": "hbm", "achieved": round(kgbs, 1), "peak": hbm, "unit": "GB/s",
                            "frac": round(kgbs / hbm, 4), "algorithmic_bytes_per_px": 8,
                            "kernel": ("topousm_hybrid (exact fixed-point full-resolution radii + epilogue)"
                                       if path == "exact" else
                                       "topousm_tc (tcgen05 split-BF16 banded box means + epilogue)"),
                            "kernel_ms": round(kms, 3), "step_achieved": round(gbs, 1),
                            "step_frac": round(gbs / hbm, 4)}}
        if path == "exact":
            # the kernel is bound by instruction issue (64-bit integer box sums), so the
            # HBM fraction above is small by construction: its issue roofline from the
            # profiled instructions per pixel and the SM count and clock
            ipx = profiled_value("topousm_hybrid_8k", "issue_slots_per_px")
            if ipx:
                import torch
                prop = torch.cuda.get_device_properties(torch.cuda.current_device())
                clk_ghz = float((clocks_max_mhz() or 2070.0)) / 1e3
                peak_ti = prop.multi_processor_count * 4 * 32 * clk_ghz  # lane issue slots / ns
                ach = ipx * px / (kms * 1e-3) / 1e12                     # T lane issue slots / s
                sec["issue_roofline"] = {"bound": "issue", "issue_slots_per_px": ipx,
                                         "achieved": round(ach, 2), "peak": round(peak_ti / 1e3, 2),
                                         "unit": "T lane-slots/s", "frac": round(ach / (peak_ti / 1e3), 4),
                                         "peak_kind": "SMs x 4 schedulers x 32 lanes x max SM clock"}
        if path == "tensor":
            fl = tc_issued_flops(full_res, n_cta)
            tf = fl / (kms * 1e-3) / 1e12
            sec["tensor_roofline"] = {"bound": "tensor", "issued_tflop_per_launch": round(fl / 1e12, 3),
                                      "achieved": round(tf, 1), "peak": bf16, "unit": "TFLOP/s",
                                      "frac": round(tf / bf16, 4), "peak_kind": "measured bf16 (burst)",
                                      "cta_tiles": n_cta}
        out[path] = sec
    out["tensor_speedup_kernel"] = round(out["exact"]["roofline"]["kernel_ms"] /
                                         max(1e-9, out["tensor"]["roofline"]["kernel_ms"]), 3)
    out["tensor_speedup_step"] = round(out["exact"]["ms_per_step"] / max(1e-9, out["tensor"]["ms_per_step"]), 3)
    # error against float64: the per-tile radii of one interior tile window, both paths
    if not getattr(args, "no_fp64_check", False):
        from oracle import restated as R
        t = tile_loop.tile_grid(n, n, 4096, pad)[min(len(tile_loop.tile_grid(n, n, 4096, pad)) - 1, 9)]
        win = dem[t.win_y:t.win_y + t.win_h, t.win_x:t.win_x + t.win_w].contiguous()
        sw = [w[radii.index(r)] for r in small]
        ref64 = R.topousm_block(win.cpu().numpy().astype(np.float64), radii=small, weights=sw, pixel_size=10.0)
        sc = R.topousm_scale(ref64)[0]
        for path in ("exact", "tensor"):
            g = TU.compute_topousm_fast_efficient_block(win, radii=small, weights=sw, pixel_size=10.0,
                                                        path=path).cpu().numpy().astype(np.float64)
            e = float(np.nanmax(np.abs(g - ref64)))
            out[path]["fp64_error"] = {"max_abs_m": e, "rel_to_p99": e / sc,
                                       "window": [t.win_y, t.win_x, t.win_h, t.win_w],
                                       "radii": small, "p99_m": sc}
    del dem
    return out


def openness_section(args):
    """Exact openness (positive, 16 directions, R = 256, 5 m) on a 16384^2 fBm+ridged DEM with the
    reference's 10 samples per ray; the dense every-step ray-march on a 4096^2 crop."""
    import torch
    from fujishadergpu_gb300 import _arrays, synth
    from fujishadergpu_gb300.algorithms import _impl_openness as OP
    from fujishadergpu_gb300.core import tile_loop
    n = args.openness_size
    dem = synth.fbm_ridged_device(n, n, hurst=0.7, seed_fbm=5, seed_ridged=6, lo=0.0, hi=3000.0)
    v = _arrays.as_device_f32_2d(dem)
    tiles = tile_loop.make_tiles(tile_loop.tile_grid(n, n, 4096, 256), pixel_scale_x=5.0, pixel_scale_y=-5.0)
    out = torch.empty((n, n), device="cuda")
    stream = torch.cuda.current_stream()
    from fujishadergpu_gb300.algorithms._stencil import make_plane
    res = {}
    for mode, size in (("reference", n), ("dense", min(n, 4096))):
        params = OP.make_params(max_distance=256, pixel_size=5.0, sampling=mode)
        if mode == "dense":
            sub = dem[:size, :size].contiguous()
            vv = _arrays.as_device_f32_2d(sub)
            tt = tile_loop.make_tiles(tile_loop.tile_grid(size, size, 4096, 256), pixel_scale_x=5.0,
                                      pixel_scale_y=-5.0)
            o = out[:size, :size]
        else:
            vv, tt, o = v, tiles, out
        plane = make_plane(o)
        ms = _time_ms(lambda: OP.run_openness(vv, tt, params, plane, None, stream=int(stream.cuda_stream)),
                      max(1, args.extra_steps // 2), 1, stream)
        px = size * size
        samples = 160 if mode == "reference" else 16 * 256
        res[mode] = {"raster": [size, size], "value": round(px / (ms * 1e-3) / 1e6, 1), "unit": "Mpix/s",
                     "ms_per_step": round(ms, 3), "samples_per_px": samples,
                     "gsamples_per_s": round(px * samples / (ms * 1e-3) / 1e9, 1)}
    del dem, out
    return {"workload": f"openness positive, 16 dirs, R=256, 5 m, {n}x{n} (reference sampling)", **res}


def ambient_occlusion_section(args):
    """Ambient occlusion (16 samples x 4 rings, radius 10 and 30, 5 m) on a 16384^2 fBm+ridged DEM
    in 4096^2 tiles with the tile loop's 64 px halo: one step = the field kernel (the samples)
    and the finish kernel (Gaussian, gamma, stretch, store) over all tiles."""
    import torch
    from fujishadergpu_gb300 import _arrays, _native, synth
    from fujishadergpu_gb300.algorithms import _impl_ambient_occlusion as AO
    from fujishadergpu_gb300.algorithms._stencil import make_plane
    from fujishadergpu_gb300.core import tile_loop
    n = args.openness_size
    dem = synth.fbm_ridged_device(n, n, hurst=0.7, seed_fbm=5, seed_ridged=6, lo=0.0, hi=3000.0)
    v = _arrays.as_device_f32_2d(dem)
    tiles = tile_loop.make_tiles(tile_loop.tile_grid(n, n, 4096, 64), pixel_scale_x=5.0, pixel_scale_y=-5.0)
    out = torch.empty((n, n), device="cuda")
    plane = make_plane(out)
    stream = torch.cuda.current_stream()
    res = {}
    for radius in (10.0, 30.0):
        params = AO.make_params(radius=radius, pixel_size=5.0, stretch=(0.5, 0.45))
        steps = max(1, args.extra_steps // 2)
        fn = lambda: AO.run_ambient_occlusion(v, tiles, params, plane, stream=int(stream.cuda_stream))  # noqa: E731
        with _native.kernel_timer(max_launches=steps + 1) as kt:
            ms = _time_ms(fn, steps, 1, stream)
        field_ms = kt.ms / max(1, kt.launches)
        res[f"radius_{int(radius)}"] = {"value": round(n * n / (ms * 1e-3) / 1e6, 1), "unit": "Mpix/s",
                                        "ms_per_step": round(ms, 3), "field_kernel_ms": round(field_ms, 3),
                                        "samples_per_px": 64,
                                        "gsamples_per_s": round(n * n * 64 / (field_ms * 1e-3) / 1e9, 1)}
    del dem, out
    if not args.no_cpu_baseline:
        procs = max(1, os.cpu_count() or 1)
        rate = cpu_oracle_rate("ambient_occlusion", procs=procs, tiles=procs, core=1024, pad=16,
                               params={"radius": 10.0})
        res["cpu_baseline"] = {"value": round(rate, 2), "unit": "Mpix/s", "cores": procs, "kind": "port",
                               "sample": f"{procs} tiles of 1056^2, oracle compute_ambient_occlusion_block "
                                         "(radius 10), one tile per process"}
    return {"workload": f"ambient occlusion, 16 samples x 4 rings, 5 m, {n}x{n}, 4096^2 tiles", **res}


def prepare_section(args):
    """The prepare step (NoData detection and void fill) on a 32768^2 fBm DEM with ~2 % NaN
    disks, an undeclared 0-valued exterior frame and a declared -32768 patch: the whole
    prepare_dem call (coarse sample, host detection rules, coarse average, push-pull,
    exterior mask, full-resolution fill), and its full-resolution kernel alone against
    the HBM roofline (4 B read + 4 B written per pixel)."""
    import torch
    from fujishadergpu_gb300 import _native, synth
    from fujishadergpu_gb300.io import dem_preprocess as P
    n = args.size
    dem = synth.fbm_device(n, n, hurst=0.8, seed=9, lo=50.0, hi=3000.0)
    synth.nodata_disks_device(dem, count=max(1, int(200 * (n / 16384) ** 2)), seed=10, rmin=10.0, rmax=200.0)
    dem[: n // 50, :] = 0.0
    dem[:, -n // 40:] = 0.0
    out = torch.empty_like(dem)
    stream = torch.cuda.current_stream()
    steps = max(1, args.extra_steps // 2)
    fn = lambda: P.prepare_dem(dem, nodata=-32768.0, fill_mode="enclosed", out=out)  # noqa: E731
    with _native.kernel_timer(max_launches=steps + 1) as kt:
        ms = _time_ms(fn, steps, 1, stream)
    kms = kt.ms / max(1, kt.launches)
    hbm, _, src = peaks()
    gbs = n * n * 8 / (kms * 1e-3) / 1e9
    res = {"raster": [n, n], "value": round(n * n / (ms * 1e-3) / 1e6, 1), "unit": "Mpix/s",
           "ms_per_step": round(ms, 3), "fill_kernel_ms": round(kms, 3),
           "fill_kernel_roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": hbm, "peak_source": src,
                                    "unit": "GB/s", "frac": round(gbs / hbm, 4)}}
    del dem, out
    if not args.no_cpu_baseline:
        procs = max(1, os.cpu_count() or 1)
        rate = cpu_oracle_rate("prepare", procs=procs, tiles=procs, core=2048, pad=0,
                               params={"coarse_max": 128})
        res["cpu_baseline"] = {"value": round(rate, 2), "unit": "Mpix/s", "cores": procs, "kind": "port",
                               "sample": f"{procs} rasters of 2048^2 (2 NaN disks each), oracle prepare "
                                         "(coarse_max 128, the same 16x ratio), one raster per process"}
    return {"workload": f"prepare (fill_mode enclosed, coarse_max 2048), {n}x{n}", **res}


def spatial_section(args):
    """Spatial (multi-radius) mode on an 8192^2 fBm+ridged DEM (5 m, 4096^2 tiles): hillshade,
    slope and curvature with radii 2, 8, 32, 128 and openness with distances 4, 16, 64, 256
    (decimated 1x, 1x, 2x, 8x), weights 0.4, 0.3, 0.2, 0.1.  One step = the whole tile loop:
    per tile and radius the reflect-padded window, the smoothing / decimated ray-march, the
    product, the weighted combination and the masked store."""
    import torch
    from fujishadergpu_gb300 import synth
    from fujishadergpu_gb300.core import tile_loop
    n = args.spatial_size
    dem = synth.fbm_ridged_device(n, n, hurst=0.75, seed_fbm=7, seed_ridged=8, lo=0.0, hi=2500.0)
    stream = torch.cuda.current_stream()
    w = [0.4, 0.3, 0.2, 0.1]
    res = {}
    for algo, radii, extra in (("hillshade", [2, 8, 32, 128], {}), ("slope", [2, 8, 32, 128], {}),
                               ("curvature", [2, 8, 32, 128], {"curvature_type": "profile"}),
                               ("openness", [4, 16, 64, 256], {"global_stats": (0.5, 0.4)})):
        kw = dict(tile_size=4096, pixel_size=5.0, pixel_scale_x=5.0, pixel_scale_y=-5.0, mode="spatial",
                  radii=radii, weights=w, **extra)
        ms = _time_ms(lambda: tile_loop.process_dem_array(dem, algo, **kw), max(1, args.extra_steps // 2), 1,
                      stream)
        res[algo] = {"radii": radii, "value": round(n * n / (ms * 1e-3) / 1e6, 1), "unit": "Mpix/s",
                     "ms_per_step": round(ms, 3)}
    del dem
    return {"workload": f"spatial mode, {n}x{n} fBm+ridged, 5 m, 4096^2 tiles, weights {w}", **res}


def surrogate_section(args):
    """Openness (positive, 16 dirs, R = 256, 5 m) on a 16384^2 fBm+ridged DEM three ways over the
    same 4096^2 tiles (halo 288): exact reference sampling, exact dense ray-march, and the CNN
    surrogate with its exact check block per tile (tiles over 2 degrees MAE redone exactly)."""
    import torch
    from fujishadergpu_gb300 import synth
    from fujishadergpu_gb300.algorithms import _impl_openness as OP
    from fujishadergpu_gb300.core import tile_loop
    from fujishadergpu_gb300.surrogate import openness_cnn as S
    n = args.openness_size
    model = S.load_default()
    if model is None:
        return {"unavailable": "no trained surrogate weights (fujishadergpu_gb300/surrogate/openness_r256.npz)"}
    dem = synth.fbm_ridged_device(n, n, hurst=0.7, seed_fbm=5, seed_ridged=6, lo=0.0, hi=3000.0)
    pad = tile_loop.required_padding("openness", {"mode": "local", "max_distance": 256}, 10.0, 4096)
    infos = tile_loop.tile_grid(n, n, 4096, pad)
    tiles = tile_loop.make_tiles(infos, pixel_scale_x=5.0, pixel_scale_y=-5.0)
    from fujishadergpu_gb300 import _arrays
    v = _arrays.as_device_f32_2d(dem)
    res = {"workload": f"openness positive, 16 dirs, R=256, 5 m, {n}x{n}, 4096^2 tiles, halo {pad}",
           "params": model.n_params()}
    exact = {}
    for mode in ("reference", "dense"):
        raw = torch.empty((n, n), device="cuda")
        params = OP.make_params(max_distance=256, pixel_size=5.0, sampling=mode)
        stream = torch.cuda.current_stream()
        ms = _time_ms(lambda: OP.run_openness(v, tiles, params, None, raw, stream=int(stream.cuda_stream)), 1, 1,
                      stream)
        exact[mode] = raw
        res[f"exact_{mode}"] = {"value": round(n * n / (ms * 1e-3) / 1e6, 1), "unit": "Mpix/s",
                                "ms_per_step": round(ms, 2)}
    stream = torch.cuda.current_stream()
    out = {}
    ms = _time_ms(lambda: out.update(S.surrogate_tile_loop(dem, infos, model, pixel_size=5.0)), 1, 1, stream)
    plane = out["plane"]
    d = (plane - exact["reference"]).abs()
    mae = float(d[torch.isfinite(d)].mean().item())
    res["surrogate"] = {"value": round(n * n / (ms * 1e-3) / 1e6, 1), "unit": "Mpix/s", "ms_per_step": round(ms, 2),
                        "mae_vs_exact_reference_deg": round(mae, 3), "tiles": out["tiles"],
                        "tiles_redone_exactly": out["exact_redone"],
                        "check_block_mae_deg": out["check_mae_deg"],
                        "speedup_vs_exact_dense": round(res["exact_dense"]["ms_per_step"] / ms, 2),
                        "speedup_vs_exact_reference": round(res["exact_reference"]["ms_per_step"] / ms, 3)}
    del dem, plane, exact
    return res


def batched_section(args):
    """Batched uneven tiles: a geographic fBm DEM (1 arcsec columns, latitudes 45 -> 30 deg, 0-5000 m,
    ~1 % NoData disks) and its 2x / 4x overviews in one atlas, each level cut into its own tile grid with
    autotuned tile sizes (candidates 256 .. 4096), through hillshade, topousm_fast (radii 2..512, 2^n
    weights, per-level coarse field and scale) and exact openness (16 dirs, R = 256, reference sampling)
    as prepared launches captured into one CUDA graph; one step = one graph replay."""
    import tempfile

    import torch
    from fujishadergpu_gb300 import synth
    from fujishadergpu_gb300.core.autotune import Autotuner
    from fujishadergpu_gb300.core.batch import BatchConfig, BatchedTiles
    H, W = args.batched_rows, 2 * args.batched_rows
    dem = synth.fbm_device(H, W, hurst=0.75, seed=9, lo=0.0, hi=5000.0)
    ndisks = max(1, int(round(60 * (H * W) / (16384.0 * 16384.0))))
    synth.nodata_disks_device(dem, count=ndisks, seed=10)
    nodata_frac = float(torch.isnan(dem).float().mean().item())
    T6 = (1.0 / 3600.0, 0.0, 135.0, 0.0, -(45.0 - 30.0) / H, 45.0)
    tune_path = os.path.join(tempfile.gettempdir(), "fsg_bench_autotune.json")
    t0 = time.perf_counter()
    b = BatchedTiles(dem, T6, config=BatchConfig(levels=3), tuner=Autotuner(path=tune_path))
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    del dem
    stream = torch.cuda.current_stream()
    eager_ms = _time_ms(b.step, max(1, args.extra_steps // 2), 1, stream)
    b.capture()
    graph_ms = _time_ms(b.replay, args.extra_steps, 2, stream)
    per_product = b.product_graph_ms(args.extra_steps)
    px = b.pyr.pixels
    res = {"workload": f"batched uneven tiles: {H}x{W} geographic fBm (1 arcsec columns, lat 45-30), 3 overview "
                       "levels, hillshade + topousm_fast (radii 2..512) + openness (R=256, 16 dirs) per tile",
           "pixels_all_levels": px, "levels": [[L.h, L.w] for L in b.pyr.levels],
           "nodata_frac": round(nodata_frac, 4), "tile_sizes": b.tile_sizes, "tiles": b.tile_counts,
           "plans": len(b.plans),
           "value": round(px / (graph_ms * 1e-3) / 1e6, 1), "unit": "Mpix/s (all levels, 3 products)",
           "ms_per_step_graph": round(graph_ms, 2), "ms_per_step_eager": round(eager_ms, 2),
           "ms_per_product_graph": {k: round(v, 2) for k, v in per_product.items()},
           "scheduling": "each product's units popped from a device-side atomic queue by persistent CTAs / warps",
           "setup_s_incl_autotune_and_stats": round(setup_s, 2),
           "autotune_costs_ns_per_px": {k: {c: round(v * 1e6, 4) for c, v in cv.items()}
                                        for k, cv in b.tuner.measured.items()}}
    b.close()
    return res


# --------------------------------------------------------------------- main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["stencil", "topousm", "openness", "ambient_occlusion", "surrogate",
                                           "spatial", "batched", "prepare"],
                    default="stencil",
                    help="stencil: the headline line; topousm / openness: that section alone (profiling)")
    ap.add_argument("--size", type=int, default=32768)
    ap.add_argument("--tile", type=int, default=4096)
    ap.add_argument("--halo", type=int, default=8)
    ap.add_argument("--stencil-dtype", choices=["float32", "uint8"], default="float32",
                    help="plane type of the headline stencil line (uint8: the extra section's workload alone)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the topousm / openness sections")
    ap.add_argument("--no-fp64-check", action="store_true",
                    help="skip the float64 error statement of the topousm section (host oracle on one tile)")
    ap.add_argument("--topousm-size", type=int, default=32768)
    ap.add_argument("--openness-size", type=int, default=16384)
    ap.add_argument("--spatial-size", type=int, default=8192)
    ap.add_argument("--extra-steps", type=int, default=4)
    ap.add_argument("--batched-rows", type=int, default=32768, help="rows of the batched workload's DEM (2x columns)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    if args.impl == "reference":
        return reference_arm(args)

    rank, world, _ = dist_setup(args.gpus)
    if args.workload != "stencil":
        sec = {"topousm": topousm_section, "openness": openness_section,
               "ambient_occlusion": ambient_occlusion_section, "surrogate": surrogate_section,
               "prepare": prepare_section,
               "spatial": spatial_section, "batched": batched_section}[args.workload](args)
        if rank == 0:
            print(json.dumps({"section": args.workload, **sec}))
        return
    line = stencil_workload(args, rank, world, out_dtype=args.stencil_dtype)
    if not args.no_extra:
        import torch
        torch.cuda.empty_cache()
        u8 = stencil_workload(args, rank, world, out_dtype="uint8")
        line["extra"] = {"stencil_uint8": {k: u8[k] for k in ("value", "unit", "ms_per_step", "config", "roofline",
                                                               "e2e", "gpu_launches")}}
        torch.cuda.empty_cache()
        line["extra"]["topousm_fast"] = topousm_section(args)
        torch.cuda.empty_cache()
        line["extra"]["openness"] = openness_section(args)
        torch.cuda.empty_cache()
        line["extra"]["ambient_occlusion"] = ambient_occlusion_section(args)
        torch.cuda.empty_cache()
        line["extra"]["prepare"] = prepare_section(args)
        torch.cuda.empty_cache()
        line["extra"]["openness_surrogate"] = surrogate_section(args)
        torch.cuda.empty_cache()
        line["extra"]["spatial"] = spatial_section(args)
        torch.cuda.empty_cache()
        line["extra"]["batched"] = batched_section(args)
    if rank == 0:
        if not args.no_cpu_baseline and world == 1:
            procs = max(1, os.cpu_count() or 1)
            rate = cpu_oracle_rate("stencil", procs=procs, tiles=procs, core=CPU_TILE, pad=8, params=CPU_NODATA)
            line["cpu_baseline"] = {"value": round(rate, 2), "unit": "Mpix/s", "cores": procs, "kind": "port",
                                    "sample": f"{procs} tiles of {CPU_TILE}^2 (+8 px halo), oracle hillshade+slope+"
                                              "profile+planform, one tile per process; " + CPU_NODATA_NOTE}
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def reference_arm(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    procs = max(1, os.cpu_count() or 1)
    rates = []
    for i in range(args.warmup + args.steps):
        r = cpu_oracle_rate("stencil", procs=procs, tiles=procs, core=CPU_TILE, pad=8, seed=200 + 31 * i,
                            params=CPU_NODATA)
        if i >= args.warmup:
            rates.append(r)
    v = statistics.median(rates)
    px_step = procs * CPU_TILE * CPU_TILE
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": round(v, 2),
        "unit": "Mpix/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(px_step / (v * 1e6) * 1e3, 1),
        "higher_is_better": True,
        "scaling": "strong",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded spectral fBm, Hurst 0.7, 0-4000 m, NoData disks)",
        "config": {"workload": "fused hillshade+slope(deg)+profile+planform curvature, float32 planes",
                   "raster": [args.size, args.size], "tile": args.tile, "halo": args.halo,
                   "sample_per_step": f"{procs} tiles of {CPU_TILE}^2"},
        "cpu_baseline": {"value": round(v, 2), "unit": "Mpix/s", "cores": procs, "kind": "port",
                         "sample": f"{procs} tiles of {CPU_TILE}^2 per step, one per process; " + CPU_NODATA_NOTE},
        "e2e": {"value": round(v, 2), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference is CuPy-only; its CPU algorithm is timed through the NumPy/SciPy oracle port",
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()

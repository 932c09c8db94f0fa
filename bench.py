#!/usr/bin/env python
"""Benchmark of the projection/backprojection hot path (one JSON line on rank 0).

Workload (default "ossart512"): a 512 x 256 x 512 (W x H x D) float32 volume of
60 seeded ellipsoids; 61 projections of 512 x 256 at -60..+60 deg with seeded
per-tilt shifts U(-5,5) px and in-plane rotations U(-1,1) deg; one step is one
whole reconstruction job on the resident tilt-series: Hamming-ramp WBP, then
OS-SART with update 7 (9 subsets of 61 tilts) for 20 iterations.  The metric
is voxel-updates/s: one update is one (voxel, tilt) pair of one pass, so a step
is Nvox * Nproj * (1 + 20) updates.  Inputs are larger than L2 (the volume is
268 MB), so no flush is needed between steps.

Arms:
  default            the GB300 engine through its C ABI (device-resident inputs)
  --impl reference   the reference's CPU algorithm (C restatement, all host
                     threads) on a bounded sample of the same workload
Multi-GPU (torchrun): every rank reconstructs its own series (weak scaling, no
collective on the data path); value = all ranks' updates / max rank time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "ossart512": dict(W=512, H=256, D=512, n=61, amax=60.0, ellipsoids=60, shifts=5.0, rot=1.0, noise=0.0,
                      wbp="hamming_ramp", n_iter=20, update=7, relax=1.0, seed=1235),
    "sirt256": dict(W=256, H=64, D=256, n=61, amax=60.0, ellipsoids=20, shifts=0.0, rot=0.0, noise=0.01,
                    wbp="ramp", n_iter=10, update=0, relax=1.0, seed=1234),
}
METRIC = "SIRT voxel-updates/s + served recon p50/p99 vs plain FP32 GPU, ≤1e-3 rel-L2"
FALLBACK_HBM_GBS = 6800.0


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def want(args, leg):
    """Whether the extra leg `leg` runs (not --no-extra, and named by --legs or --legs all).
    The extra legs characterise one GPU: a multi-rank run (scaling) times the main job only."""
    if args.no_extra or int(os.environ.get("WORLD_SIZE", "1")) > 1:
        return False
    return args.legs == "all" or leg in args.legs.split(",")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ----------------------------------------------------------------------------- inputs
def make_inputs(wl, project_fn):
    from tomoj_gb300 import phantom as P
    t0 = time.time()
    vol = P.ellipsoid_phantom(wl["W"], wl["H"], wl["D"], wl["ellipsoids"], wl["seed"])
    angles = np.linspace(-wl["amax"], wl["amax"], wl["n"])
    ideal = project_fn(vol, angles)
    n = wl["n"]
    if wl["shifts"] or wl["rot"]:
        T = P.misalignment(n, wl["seed"] + 1, wl["shifts"], wl["rot"])
        series = np.array([P.unalign(ideal[i], T[i]) for i in range(n)], np.float32)
    else:
        T = np.tile(np.array([1.0, 0, 0, 1, 0, 0]), (n, 1))
        series = ideal
    if wl["noise"]:
        series = P.add_gaussian_noise(series, wl["noise"], wl["seed"] + 2)
    log(f"[bench] inputs ready in {time.time() - t0:.1f}s")
    return vol, angles, np.ascontiguousarray(T), np.ascontiguousarray(series, np.float32)


def euler_y(angles):
    from tomoj_gb300.tiltseries import euler_angles_to_matrix
    return np.ascontiguousarray([euler_angles_to_matrix(0.0, a, -0.0) for a in angles], np.float64)


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------------------- CPU arm
def cpu_sample(wl, rows, threads, steps=1):
    """Time the C restatement of the reference's CPU path on `rows` volume rows of the
    workload: the same W, D, tilts, phantom density, misalignment, noise, WBP filter and
    subsets.  One step is what the reference does for one WBP pass and one OS-SART
    iteration: align the projections (average fill for WBP, NaN fill for the iterative
    pass), weight and backproject them, then the iteration.
    Returns (updates/s, seconds, updates)."""
    from oracle import oracle as O
    from tomoj_gb300 import phantom as P
    O.build()
    O.set_threads(threads)
    W, D, n = wl["W"], wl["D"], wl["n"]
    H = rows
    g = O.Geom(W, H, D, W, H)
    vol = P.ellipsoid_phantom(W, H, D, wl["ellipsoids"], wl["seed"])
    angles = np.linspace(-wl["amax"], wl["amax"], n)
    eul = np.array([O.euler_tilt_y(a) for a in angles])
    ideal = np.nan_to_num(np.array([O.project(vol, g, e)[0] for e in eul], np.float32))
    if wl["shifts"] or wl["rot"]:
        T = P.misalignment(n, wl["seed"] + 1, wl["shifts"], wl["rot"])
        series = np.array([P.unalign(ideal[i], T[i]) for i in range(n)], np.float32)
    else:
        T = np.tile(np.array([1.0, 0, 0, 1, 0, 0]), (n, 1))
        series = ideal
    if wl["noise"]:
        series = P.add_gaussian_noise(series, wl["noise"], wl["seed"] + 2)
    stats = np.array([[series[i].mean(dtype=np.float64), series[i].std(dtype=np.float64)] for i in range(n)])
    mask = O.ramp_mask(W, H, angles, hamming=(wl["wbp"] == "hamming_ramp"))
    order = O.order_shuffle(eul, 0)
    upd = wl["update"]
    ups = W * H * D * n * 2
    t0 = time.perf_counter()
    for _ in range(steps):
        avg = np.array([O.align(series[i], T[i], False, stats[i, 0], stats[i, 1], O.FILL_AVG) for i in range(n)],
                       np.float32)
        meas = np.array([O.align(series[i], T[i], fill=O.FILL_NAN) for i in range(n)], np.float32)
        rec = np.zeros((D, H, W), np.float32)
        O.wbp(rec, g, eul, avg, mask)
        O.ossart_iteration(rec, g, eul, meas, order, wl["relax"], upd)
    dt = time.perf_counter() - t0
    return ups * steps / dt, dt, ups * steps


def config_of(args, wl, world):
    """The `config` object both arms print for the workload."""
    W, H, D, n = wl["W"], wl["H"], wl["D"], wl["n"]
    return {"workload": args.workload, "W": W, "H": H, "D": D, "nproj": n, "proj": f"{W}x{H}", "wbp": wl["wbp"],
            "shifts_px": wl["shifts"], "rot_deg": wl["rot"], "noise": wl["noise"], "ellipsoids": wl["ellipsoids"],
            "n_iter": wl["n_iter"], "update": wl["update"], "updates_per_step": W * H * D * n * (1 + wl["n_iter"]),
            "l2": f"inputs larger than L2 (volume {W * H * D * 4 // 10**6} MB)", "parallelism": f"replicas{world}"}


def cpu_plan(wl, threads, target_s):
    """(rows, passes) of the workload whose CPU sample takes about target_s seconds:
    calibrated on 16 rows (the per-tilt barriers make smaller samples unrepresentative),
    capped at the whole volume, with repeated passes when the whole volume is faster."""
    rows0 = min(16, wl["H"])
    _, dt, _ = cpu_sample(wl, rows0, threads)
    per_row = dt / rows0
    rows = int(max(rows0, min(wl["H"], round(target_s / max(per_row, 1e-6)))))
    passes = int(max(1, round(target_s / max(per_row * rows, 1e-6))))
    return rows, passes


def run_reference(args, wl):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # steps are bounded samples: about cpu_seconds / steps of CPU work each
    rows, passes = cpu_plan(wl, threads, max(2.0, args.cpu_seconds / max(args.steps, 1)))
    for _ in range(args.warmup):
        cpu_sample(wl, min(rows, 16), threads)
    vals, secs = [], 0.0
    for _ in range(args.steps):
        rate, dt, _ = cpu_sample(wl, rows, threads, passes)
        vals.append(rate)
        secs += dt
    value = float(np.mean(vals))
    sample = (f"{wl['W']}x{rows}x{wl['D']} rows of the workload: {passes} x (1 WBP pass + 1 OS-SART iteration "
              f"(update {wl['update']})) per step, {wl['n']} tilts")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "voxel-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * secs / max(args.steps, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_of(args, wl, world),
        "cpu_baseline": {"value": value, "unit": "voxel-updates/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "voxel-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU arm
def run_engine(args, wl):
    import torch
    from tomoj_gb300 import _abi
    from tomoj_gb300.build import build

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if rank == 0:
        build()
    if world > 1:
        torch.distributed.barrier()
    lib = _abi.load()
    stream = torch.cuda.current_stream()
    W, H, D, n = wl["W"], wl["H"], wl["D"], wl["n"]

    def create(normalize=False):
        g = _abi.make_geom(W, H, D, W, H, n)
        p = _abi.make_params(fill=_abi.FILL_NAN, normalize=normalize)
        h = C.c_void_p()
        _abi.check(lib.tomo_create(C.byref(g), C.byref(p), C.byref(h)))
        _abi.check(lib.tomo_set_stream(h, C.c_void_p(stream.cuda_stream)))
        return h

    eul = euler_y(np.linspace(-wl["amax"], wl["amax"], n))

    def project_fn(vol, angles):
        h = create()
        try:
            zeros = np.zeros((n, H, W), np.float32)
            _abi.check(lib.tomo_load_series(h, zeros.ctypes.data, 0, _abi.ptr(eul, C.c_double), None, None))
            v = np.ascontiguousarray(vol)
            _abi.check(lib.tomo_set_volume(h, v.ctypes.data, 0, 0, H))
            for i in range(n):
                _abi.check(lib.tomo_add_projection(h, i))
            _abi.check(lib.tomo_project(h, 0, H))
            out = np.empty((n, H, W), np.float32)
            for i in range(n):
                _abi.check(lib.tomo_get_projection(h, i, _abi.ptr(out[i])))
            return np.nan_to_num(out)
        finally:
            lib.tomo_destroy(h)

    _, angles, T, series = make_inputs(wl, project_fn)
    wkind = {"ramp": _abi.WEIGHT_RAMP, "hamming_ramp": _abi.WEIGHT_HAMMING_RAMP}[wl["wbp"]]

    # per-tilt ROI statistics (TiltSeries.getImageStatistics) for the FILL_AVG of the WBP pass
    from tomoj_gb300.tiltseries import TiltSeries
    ts = TiltSeries(series, angles)
    for i in range(n):
        ts.getAlignment().setTransform(i, T[i])
    ts.getAlignment().setCombineTransforms(False)
    stats = np.ascontiguousarray(ts.statistics(), np.float64)

    h = create()

    def load(pixels):
        _abi.check(lib.tomo_load_series(h, pixels.ctypes.data, 0, _abi.ptr(eul, C.c_double),
                                        _abi.ptr(T, C.c_double), _abi.ptr(stats, C.c_double)))
        _abi.check(lib.tomo_set_weighting(h, wkind, 0.0, None, None))

    load(series)
    nvox = W * H * D
    updates_per_step = nvox * n * (1 + wl["n_iter"])
    # kernel shapes for this series from the engine's autotuner (one update, 3 launches per
    # candidate; the volume is put back), as a caller would run it once per series
    tune = np.zeros(4)
    _abi.check(lib.tomo_set_fill(h, _abi.FILL_NAN))
    _abi.check(lib.tomo_autotune(h, wl["update"], 3, _abi.ptr(tune, C.c_double)))
    autotune = {"tilts_per_cta": int(tune[0]) or "auto", "bp_rows": int(tune[1]) or "auto",
                "fp_ms": float(tune[2]), "bp_ms": float(tune[3])}

    def step(errs=None):
        # WBP on FILL_AVG projections, then OS-SART on FILL_NAN projections, as the
        # reference's WBP and iterative applications set them
        _abi.check(lib.tomo_fill_volume(h, 0.0))
        _abi.check(lib.tomo_set_fill(h, _abi.FILL_AVG))
        _abi.check(lib.tomo_run_wbp(h, 0, H))
        _abi.check(lib.tomo_set_fill(h, _abi.FILL_NAN))
        _abi.check(lib.tomo_run_ossart(h, wl["n_iter"], wl["relax"], wl["update"], wl["seed"], 0, H, 1,
                                       None if errs is None else _abi.ptr(errs, C.c_double)))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    # ---- timed region: device-resident inputs ----
    _abi.check(lib.tomo_set_profiling(h, 1))
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = lib.tomo_kernel_launches()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    errs = np.zeros((wl["n_iter"], 5))
    for _ in range(args.steps):
        step(errs)
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = lib.tomo_kernel_launches() - launches0
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    prof = np.zeros(4)
    _abi.check(lib.tomo_profile_read(h, _abi.ptr(prof, C.c_double)))
    _abi.check(lib.tomo_set_profiling(h, 0))
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = updates_per_step * args.steps * world / (ms / 1000.0)

    # ---- end to end through the C ABI with pinned host buffers ----
    series_pin = torch.empty(series.shape, dtype=torch.float32, pin_memory=True).numpy()
    series_pin[...] = series
    vol_pin = torch.empty((D, H, W), dtype=torch.float32, pin_memory=True).numpy()
    h2d = series_pin.nbytes + eul.nbytes + T.nbytes + stats.nbytes
    d2h = vol_pin.nbytes
    e2e_steps = max(1, min(args.steps, 3))
    phase = {"load_s": 0.0, "job_s": 0.0, "readback_s": 0.0}
    # first use of the two pinned buffers outside the timed region (a reused staging
    # buffer, as a caller keeps one)
    load(series_pin)
    _abi.check(lib.tomo_get_volume(h, vol_pin.ctypes.data, 0, 0, H))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ta = time.perf_counter()
        load(series_pin)  # synchronous: series H2D, geometry tables, alignment
        tb = time.perf_counter()
        step()
        torch.cuda.synchronize()
        tc = time.perf_counter()
        _abi.check(lib.tomo_get_volume(h, vol_pin.ctypes.data, 0, 0, H))
        td = time.perf_counter()
        phase["load_s"] += tb - ta
        phase["job_s"] += tc - tb
        phase["readback_s"] += td - tc
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_value = updates_per_step * e2e_steps * world / e2e_s
    phase = {k: v / e2e_steps for k, v in phase.items()}

    # ---- the same job with its OS-SART iterations on two row streams (opt-in engine
    # option: the forward projection of one row range overlaps the backprojection of
    # the other; bitwise the same volume) ----
    row_leg = None
    if want(args, "row_streams"):
        _abi.check(lib.tomo_set_row_streams(h, 2))
        for _ in range(2):
            step()
        torch.cuda.synchronize()
        ra, rb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ra.record(stream)
        for _ in range(args.steps):
            step()
        rb.record(stream)
        torch.cuda.synchronize()
        rms = ra.elapsed_time(rb)
        _abi.check(lib.tomo_set_row_streams(h, 1))
        row_leg = {"row_streams": 2, "ms_per_step": rms / args.steps,
                   "voxel_updates_per_s": updates_per_step * args.steps / (rms / 1000.0),
                   "speedup_vs_one_stream": (ms / args.steps) / (rms / args.steps)}

    # ---- the compressed-sensing end-of-iteration filter on the same volume (FP64 wavelet
    # transform, threshold search, soft threshold, inverse; default levels from the width) ----
    cs_leg = None
    if want(args, "compressed_sensing"):
        _abi.check(lib.tomo_set_compressed_sensing(h, 3, 3.0, 0.0, 0.95, None, 1))
        _abi.check(lib.tomo_end_iteration(h))
        ca, cb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 3
        ca.record(stream)
        for _ in range(reps):
            _abi.check(lib.tomo_end_iteration(h))
        cb.record(stream)
        torch.cuda.synchronize()
        cms = ca.elapsed_time(cb) / reps
        _abi.check(lib.tomo_set_compressed_sensing(h, 0, 0.0, 0.0, 0.0, None, 0))
        levels = 1
        while 64 << (levels - 1) < W:
            levels += 1
        cs_leg = {"wavelet": "B-spline, degree 3", "levels": [levels] * 3, "fraction_zeros": 0.95,
                  "ms_per_filter": cms, "voxels_per_s": nvox / (cms / 1000.0),
                  "vs_one_plain_iteration": cms / (ms / args.steps / (1 + wl["n_iter"]))}

    # ---- roofline of the dominant kernel ----
    # Both kernels keep the tilts of a launch on chip (a staged plane serves every tilt; a
    # voxel is loaded once for all tilts), so DRAM carries about one volume read (+ write)
    # per launch and the ceiling that binds is the shared-memory data path: one 128-byte
    # wavefront per SM clock.  Wavefront and DRAM byte counts per launch come from the ncu
    # capture summarised in profiles/kernels_ossart512.json (same workload, same launches);
    # launch durations are this run's CUDA events.
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        hbm_peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "measured"
    else:
        hbm_peak, peak_src = FALLBACK_HBM_GBS, "fallback"
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
    smem_peak = 128.0 * sms * sm_mhz * 1e6 / 1e9  # GB/s
    fp_ms, fp_n, bp_ms, bp_n = prof
    upd = n if wl["update"] == 0 else wl["update"]
    nsub = (n + upd - 1) // upd
    tilts_per_launch = n / nsub
    npix = W * H
    updates_per_launch = nvox * tilts_per_launch
    rays = tilts_per_launch * npix
    ncu = {}
    kpath = os.path.join(ROOT, "profiles", "kernels_ossart512.json")
    if os.path.exists(kpath) and args.workload == "ossart512":
        ncu = json.load(open(kpath))["kernels"]
    # unfused-equivalent bytes (a projector streaming the volume once per tilt, FP32): FP 4 B
    # per voxel-update + 16 B per ray; BP 8 B per voxel-update + 4 B per ray
    unfused = {"fp_separable": 4.0 * updates_per_launch + 16.0 * rays,
               "bp_separable": 8.0 * updates_per_launch + 4.0 * rays}
    compulsory = {"fp_separable": 4.0 * nvox + 16.0 * rays, "bp_separable": 8.0 * nvox + 4.0 * rays}
    kernels = {}
    for k, ms_tot, cnt in (("fp_separable", fp_ms, fp_n), ("bp_separable", bp_ms, bp_n)):
        avg_s = ms_tot / max(cnt, 1) / 1000.0
        nk = ncu.get(k, {})
        dram = nk.get("dram_bytes_per_launch", compulsory[k])
        kv = {"avg_ms": avg_s * 1000.0, "launches": int(cnt),
              "hbm_GBs": dram / avg_s / 1e9, "hbm_frac": dram / avg_s / 1e9 / hbm_peak,
              "dram_bytes_per_launch": dram, "dram_bytes_source": "ncu" if "dram_bytes_per_launch" in nk else "compulsory",
              "unfused_equivalent_GBs": unfused[k] / avg_s / 1e9}
        if "smem_wavefronts_per_launch" in nk:
            sb = 128.0 * nk["smem_wavefronts_per_launch"]
            kv.update({"smem_GBs": sb / avg_s / 1e9, "smem_frac": sb / avg_s / 1e9 / smem_peak})
        kernels[k] = kv
    dom = max(kernels, key=lambda k: kernels[k]["avg_ms"] * kernels[k]["launches"])
    kd = kernels[dom]
    if "smem_frac" in kd:
        roofline = {"bound": "smem", "kernel": dom, "achieved": kd["smem_GBs"], "peak": smem_peak, "unit": "GB/s",
                    "frac": kd["smem_frac"], "peak_source": f"128 B per SM clock x {sms} SMs x {sm_mhz:.0f} MHz"}
    else:
        roofline = {"bound": "hbm", "kernel": dom, "achieved": kd["hbm_GBs"], "peak": hbm_peak, "unit": "GB/s",
                    "frac": kd["hbm_frac"], "peak_source": peak_src}
    roofline.update({
        "traffic": kd["dram_bytes_per_launch"], "avg_launch_ms": kd["avg_ms"],
        "updates_per_launch": updates_per_launch,
        "hbm": {"achieved": kd["hbm_GBs"], "peak": hbm_peak, "unit": "GB/s", "frac": kd["hbm_frac"],
                "peak_source": peak_src, "bytes": kd["dram_bytes_source"]},
        "counts_source": "profiles/kernels_ossart512.json" if ncu else None,
        "kernels": kernels,
        # the plain-form accounting of a projector streaming the volume once per tilt: 12 B per
        # voxel-update; above 1 only because the fused kernels never move those bytes
        "unfused_equivalent": {"bytes_per_update": 12, "achieved_GBs": value * 12.0 / 1e9 / world,
                               "frac_of_hbm": value * 12.0 / 1e9 / world / hbm_peak},
    })

    # ---- CPU baseline (rank 0, N=1 only) ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rows, passes = cpu_plan(wl, threads, args.cpu_seconds)
        rate, dt, ups = cpu_sample(wl, rows, threads, passes)
        cpu = {"value": rate, "unit": "voxel-updates/s", "cores": threads, "kind": "port",
               "sample": f"{W}x{rows}x{D} rows of the workload, {passes} x (1 WBP pass + 1 OS-SART iteration), "
                         f"{dt:.1f} s"}

    lib.tomo_destroy(h)
    config1 = None if (not want(args, "config1") or args.no_cpu or rank != 0 or world != 1) else run_config1_leg(lib, args)
    batched = run_batched_leg(lib, args) if want(args, "batched") else None
    serving = run_serving_leg(args) if want(args, "serving") else None
    precision = run_precision_leg(lib, args) if want(args, "precision") else None
    tv = run_tv_leg(lib, args) if want(args, "tv") else None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "voxel-updates/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": config_of(args, wl, world),
            "e2e": {"value": e2e_value, "unit": "voxel-updates/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "steps": e2e_steps, "phases_s": phase},
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": int(launches),
            "row_streams": row_leg, "compressed_sensing": cs_leg, "config1_full": config1, "batched": batched,
            "serving": serving, "precision": precision, "tv_denoise": tv, "autotune": autotune,
            "sirt_error_last_iteration": float(errs[-1, 0]),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def _project_series(lib, vol, W, H, D, eul, stream):
    """FP32 forward projection by the engine of a (D, H, W) device phantom at the given
    Euler matrices: the ideal tilt-series (n, H, W) float32 on the host."""
    from tomoj_gb300 import _abi
    n = eul.shape[0]
    g = _abi.make_geom(W, H, D, W, H, n)
    prm = _abi.make_params(fill=_abi.FILL_NAN)
    h = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(g), C.byref(prm), C.byref(h)))
    series = np.zeros((n, H, W), np.float32)
    try:
        _abi.check(lib.tomo_set_stream(h, C.c_void_p(stream.cuda_stream)))
        _abi.check(lib.tomo_load_series(h, series.ctypes.data, 0, _abi.ptr(eul, C.c_double), None, None))
        stream.synchronize()
        _abi.check(lib.tomo_set_volume(h, C.c_void_p(vol.data_ptr()), 1, 0, H))
        for i in range(n):
            _abi.check(lib.tomo_add_projection(h, i))
        _abi.check(lib.tomo_project(h, 0, H))
        for i in range(n):
            _abi.check(lib.tomo_get_projection(h, i, _abi.ptr(series[i])))
    finally:
        lib.tomo_destroy(h)
    return np.nan_to_num(series)


def run_batched_leg(lib, args):
    """BASELINE config 3: 64 independent series (W in {256,384,512,768,1024}, H 64, D in
    [64,256], 41/61/81/121 tilts over +/-50..70 deg in uniform, Saxton or dose-symmetric
    order), each the engine's projection of its own seeded ellipsoid phantom; 30 SIRT
    iterations.  Every member's kernel shapes come from the autotuner (tomo_autotune).
    Timed with CUDA events on one stream: the 64 handles one by one, the batch (one launch
    per kernel variant, the iteration a CUDA graph), the same batch in persistent form (one
    forward launch per CTA size and one backprojection launch per iteration), and the batch
    with FP16 volume storage."""
    import torch
    from tomoj_gb300 import _abi
    from tomoj_gb300 import phantom as P
    stream = torch.cuda.current_stream()
    g = np.random.Generator(np.random.PCG64(3))
    specs = []
    for m in range(64):
        W = int(g.choice([256, 384, 512, 768, 1024]))
        H, D, n = 64, int(g.integers(64, 257)), int(g.choice([41, 61, 81, 121]))
        amax = float(g.uniform(50, 70))
        scheme = int(g.integers(0, 3))
        angles = (np.linspace(-amax, amax, n) if scheme == 0 else
                  P.saxton_tilts(amax, n) if scheme == 1 else P.dose_symmetric_tilts(amax, n))
        specs.append((W, H, D, n, euler_y(angles), 1000 + m))
    t_in = time.time()
    series = []
    for W, H, D, n, eul, seed in specs:
        vol = phantom_on_device(W, H, D, P.n_ellipsoids_for(W, H, D), seed, "cuda")
        series.append(_project_series(lib, vol, W, H, D, eul, stream))
        del vol
    torch.cuda.empty_cache()
    ups = sum(W * H * D * n for W, H, D, n, _, _ in specs)
    n_iter = 30
    sp = C.c_void_p(stream.cuda_stream)

    def make(prec):
        hs = []
        for (W, H, D, n, eul, _), ser in zip(specs, series):
            geo = _abi.make_geom(W, H, D, W, H, n)
            prm = _abi.make_params(precision=prec)
            h = C.c_void_p()
            _abi.check(lib.tomo_create(C.byref(geo), C.byref(prm), C.byref(h)))
            _abi.check(lib.tomo_load_series(h, ser.ctypes.data, 0, _abi.ptr(eul, C.c_double), None, None))
            hs.append(h)
        return hs

    def tune(hs):
        shapes = {}
        t0 = time.time()
        for h in hs:
            out = np.zeros(4)
            _abi.check(lib.tomo_autotune(h, 0, 2, _abi.ptr(out, C.c_double)))
            key = f"tilts_per_cta={int(out[0]) or 'auto'},bp_rows={int(out[1]) or 'auto'}"
            shapes[key] = shapes.get(key, 0) + 1
        return shapes, time.time() - t0

    def timed(fn):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stream.synchronize()
        ev0.record(stream)
        k0 = lib.tomo_kernel_launches()
        fn()
        ev1.record(stream)
        ev1.synchronize()
        return ev0.elapsed_time(ev1) / 1000.0, lib.tomo_kernel_launches() - k0

    def batch_of(hs, persistent):
        b = C.c_void_p()
        _abi.check(lib.tomo_batch_create(C.byref(b)))
        _abi.check(lib.tomo_batch_set_stream(b, sp))
        _abi.check(lib.tomo_batch_set_persistent(b, persistent))
        arr = (C.c_void_p * len(hs))(*[h.value for h in hs])
        _abi.check(lib.tomo_batch_set(b, arr, len(hs)))
        return b

    rel = np.ones(64)
    upd = np.zeros(64, np.int32)

    def iterate(b, ks):
        for k in ks:
            first = np.array([lib.tomo_first_index(1, k, sp_[3]) for sp_ in specs], np.int32)
            _abi.check(lib.tomo_batch_iteration(b, _abi.ptr(rel, C.c_double), _abi.ptr(upd, C.c_int32),
                                                _abi.ptr(first, C.c_int32), 1, None))

    out = {"workload": "64 heterogeneous series (seeded ellipsoid phantoms), SIRT, 30 iterations",
           "iterations": n_iter, "updates_per_iteration": ups}
    hs = make(_abi.PREC_FP32)
    try:
        shapes, tune_s = tune(hs)
        out["autotuned_shapes"] = shapes
        out["autotune_s"] = tune_s
        for h in hs:
            _abi.check(lib.tomo_set_stream(h, sp))
        for h in hs[:2]:
            _abi.check(lib.tomo_run_ossart(h, 1, 1.0, 0, 1, 0, 64, 1, None))
        for h in hs:
            _abi.check(lib.tomo_fill_volume(h, 0.0))
        sec, _ = timed(lambda: [_abi.check(lib.tomo_run_ossart(h, n_iter, 1.0, 0, 1, 0, 64, 1, None)) for h in hs])
        out["one_by_one_voxel_updates_per_s"] = ups * n_iter / sec
        for h in hs:
            _abi.check(lib.tomo_set_stream(h, None))
        for persistent, key in ((0, "per_variant"), (1, "persistent")):
            for h in hs:
                _abi.check(lib.tomo_fill_volume(h, 0.0))
            b = batch_of(hs, persistent)
            try:
                iterate(b, [0])  # plan, graph
                sec, launches = timed(lambda: iterate(b, range(n_iter)))
            finally:
                lib.tomo_batch_destroy(b)
            out[key] = {"voxel_updates_per_s": ups * n_iter / sec, "launches_per_iteration": launches / n_iter}
    finally:
        for h in hs:
            lib.tomo_destroy(h)
    hs = make(_abi.PREC_FP16)
    try:
        tune(hs)
        b = batch_of(hs, 0)
        try:
            iterate(b, [0])
            for h in hs:
                _abi.check(lib.tomo_fill_volume(h, 0.0))
            sec, launches = timed(lambda: iterate(b, range(n_iter)))
        finally:
            lib.tomo_batch_destroy(b)
        out["fp16"] = {"voxel_updates_per_s": ups * n_iter / sec, "launches_per_iteration": launches / n_iter}
    finally:
        for h in hs:
            lib.tomo_destroy(h)
    one = out["one_by_one_voxel_updates_per_s"]
    out["voxel_updates_per_s"] = out["per_variant"]["voxel_updates_per_s"]
    out["speedup_vs_one_by_one"] = out["per_variant"]["voxel_updates_per_s"] / one
    out["persistent_speedup_vs_one_by_one"] = out["persistent"]["voxel_updates_per_s"] / one
    out["fp16_speedup_vs_one_by_one"] = out["fp16"]["voxel_updates_per_s"] / one
    out["inputs_s"] = time.time() - t_in
    return out


def run_tv_leg(lib, args):
    """The TV denoise of a TVM iteration (TVMProjector3D.endOfIteration: 5 inner steps,
    theta 25, g 1, dt = lambda = 0.01) timed alone with CUDA events on a args.tv_size volume of
    uniform random values, FP32 and FP16 storage (16-bit: unpack and pack included), with the
    inner step's algorithmic DRAM rate (28 B per voxel: f and p read, p written)."""
    import torch
    from tomoj_gb300 import _abi
    W, H, D = args.tv_size
    stream = torch.cuda.current_stream()
    out = {"volume": f"{W}x{H}x{D}", "inner_steps": 5}
    for name, prec in (("fp32", _abi.PREC_FP32), ("fp16", _abi.PREC_FP16)):
        g = _abi.make_geom(W, H, D, W, H, 3)
        prm = _abi.make_params(precision=prec)
        h = C.c_void_p()
        _abi.check(lib.tomo_create(C.byref(g), C.byref(prm), C.byref(h)))
        try:
            _abi.check(lib.tomo_set_stream(h, C.c_void_p(stream.cuda_stream)))
            vol = torch.rand((D, H, W), device="cuda", dtype=torch.float32, generator=torch.Generator("cuda").manual_seed(5))
            _abi.check(lib.tomo_set_volume(h, C.c_void_p(vol.data_ptr()), 1, 0, H))
            del vol
            _abi.check(lib.tomo_set_tvm(h, 25.0, 1.0, 0.01, 5))
            _abi.check(lib.tomo_end_iteration(h))  # warm-up
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            reps = 3
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(reps):
                _abi.check(lib.tomo_end_iteration(h))
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / reps
            out[name] = {"ms_per_denoise": ms, "step_GBs_upper_bound": 28.0 * W * H * D * 5 / (ms / 1000.0) / 1e9}
        finally:
            lib.tomo_destroy(h)
            torch.cuda.empty_cache()
    return out


def _serving_costs(lib, precision):
    """Per-unit GPU costs of each request kind for the serving replay, measured on one
    1024 x 1024 x 256 request with 61 tilts in the leg's storage precision: seconds per
    voxel-update of a SIRT, OS-SART (update ceil(61/10)) and WBP pass, and seconds per voxel
    of a TV-denoise step (TVM iteration minus SIRT iteration)."""
    from tomoj_gb300.serving import OSSART, SIRT, TVM, WBP, CostModel, EngineAdapter, synthetic_requests
    eng = EngineAdapter(lanes=1)
    base = synthetic_requests(1, seed=7, sizes=(1024,), thick=(256,), tilts=(61,), precision=precision)[0]
    ups = base.updates_per_iteration()
    out = {}
    try:
        for kind, n_it in ((WBP, 1), (SIRT, 4), (OSSART, 4), (TVM, 4)):
            base.kind = kind
            hd = eng.create(base)
            try:
                upd = 7 if kind == OSSART else 0
                run = (lambda k: eng.run_wbp(hd, base)) if kind == WBP else \
                    (lambda k: _abi_mod().check(lib.tomo_run_ossart(hd, k, 1.0, upd, 3, 0, base.H, 1, None)))
                run(1)  # warm-up (tables, graph)
                t0 = time.perf_counter()
                run(n_it)
                out[kind] = (time.perf_counter() - t0) / n_it
            finally:
                eng.destroy(hd)
    finally:
        eng.close()
    nvox = base.W * base.H * base.D
    return CostModel({SIRT: out[SIRT] / ups, OSSART: out[OSSART] / ups, WBP: out[WBP] / ups},
                     tv_s_per_voxel=max(out[TVM] - out[SIRT], 0.0) / nvox)


def run_serving_leg(args):
    """BASELINE config 5: Poisson arrivals (4/s) of series of {512,1024,2048}^2 x {128,256,512}
    with {41,61,121} tilts, WBP 30 % / SIRT 40 % / OS-SART 20 % / TVM 10 %, 5-50 iterations,
    volumes stored in FP16; continuous batching in three lanes with HBM admission.  Served:
    the first args.serve_requests requests of the seeded schedule (p50/p99 overall, per method
    and per size, offered load).  Replayed in virtual time with per-unit costs measured here:
    the same requests (against the served figures) and the whole 1000-request schedule.  The
    p50 drift check serves one short schedule at the start and again at the end."""
    import torch
    from tomoj_gb300 import _abi
    from tomoj_gb300.serving import EngineAdapter, Server, lane_summary, simulate, summarize, synthetic_requests
    prec = _abi.PREC_FP16
    # admission is by free HBM: hand back what earlier legs left in torch's allocator cache
    torch.cuda.empty_cache()
    lib = _abi_mod().load()
    cost = _serving_costs(lib, prec)

    def serve(reqs):
        eng = EngineAdapter(lanes=3)
        try:
            srv = Server(eng, max_active=64)
            t0 = time.perf_counter()
            res = srv.run(reqs)
            wall = time.perf_counter() - t0
        finally:
            eng.close()
        s = summarize(res, requests=reqs)
        s["wall_s"] = wall
        s["lanes_observed"] = lane_summary(srv.lane_log, wall)
        return s

    def short(s):
        return {k: s[k] for k in ("requests", "p50_s", "p99_s", "mean_s", "voxel_updates_per_s") if k in s}

    drift_reqs = synthetic_requests(24, seed=9, sizes=(512, 1024), precision=prec)
    drift0 = serve(drift_reqs)
    reqs = synthetic_requests(args.serve_requests, seed=42, precision=prec)
    out = serve(reqs)
    drift1 = serve(drift_reqs)
    del reqs
    sim_same = summarize(simulate(synthetic_requests(args.serve_requests, seed=42, precision=prec, with_series=False),
                                  cost), requests=None)
    full = synthetic_requests(1000, seed=42, precision=prec, with_series=False)
    sim_full = summarize(simulate(full, cost), requests=full)
    out["unit"] = "seconds (time to reconstruction)"
    out["precision"] = "fp16"
    out["lanes"] = "3 (iteration < 8e9, < 6e10, larger voxel-updates); WBP on a worker at top priority"
    out["replay"] = {
        "cost_model": {"s_per_update": cost.s_per_update, "tv_s_per_voxel": cost.tv_s_per_voxel,
                       "measured_on": "1024x1024x256, 61 tilts, fp16"},
        "same_requests": short(sim_same),
        "schedule_1000": {k: sim_full[k] for k in ("requests", "p50_s", "p99_s", "mean_s", "makespan_s",
                                                   "voxel_updates_per_s", "offered_load", "per_kind", "per_size")},
    }
    out["p50_drift_check"] = {"schedule": "24 requests of 512^2 / 1024^2 (seed 9), served before and after the "
                                          "main leg in the same process",
                              "before": short(drift0), "after": short(drift1)}
    return out


def run_config1_leg(lib, args):
    """The 256 x 64 x 256 workload (20 ellipsoids, 61 tilts of 256 x 64 at -60..60 deg made
    by the oracle's projector, 1 % Gaussian noise; ramp-filtered WBP start, then 10 SIRT
    iterations, relaxation 1), timed in full on both sides: the engine (CUDA events, device
    resident) and the C restatement of the reference's CPU path on all host threads."""
    import torch
    from oracle import oracle as O
    from tomoj_gb300 import phantom as P
    wl = WORKLOADS["sirt256"]
    W, H, D, n = wl["W"], wl["H"], wl["D"], wl["n"]
    threads = os.cpu_count() or 1
    O.build()
    O.set_threads(threads)
    g = O.Geom(W, H, D, W, H)
    vol = P.ellipsoid_phantom(W, H, D, wl["ellipsoids"], wl["seed"])
    angles = np.linspace(-wl["amax"], wl["amax"], n)
    eul = np.array([O.euler_tilt_y(a) for a in angles])
    series = np.nan_to_num(np.array([O.project(vol, g, e)[0] for e in eul], np.float32))
    series = np.ascontiguousarray(P.add_gaussian_noise(series, wl["noise"], wl["seed"] + 2), np.float32)
    ups = W * H * D * n * (1 + wl["n_iter"])
    seed = 5
    # engine
    stream = torch.cuda.current_stream()
    geo = _abi_mod().make_geom(W, H, D, W, H, n)
    prm = _abi_mod().make_params(fill=_abi_mod().FILL_NAN)
    h = C.c_void_p()
    _abi_mod().check(lib.tomo_create(C.byref(geo), C.byref(prm), C.byref(h)))
    e = np.ascontiguousarray(eul, np.float64)
    try:
        _abi_mod().check(lib.tomo_set_stream(h, C.c_void_p(stream.cuda_stream)))
        _abi_mod().check(lib.tomo_load_series(h, series.ctypes.data, 0, _abi_mod().ptr(e, C.c_double), None, None))

        def job():
            _abi_mod().check(lib.tomo_fill_volume(h, 0.0))
            _abi_mod().check(lib.tomo_set_weighting(h, _abi_mod().WEIGHT_RAMP, 0.0, None, None))
            _abi_mod().check(lib.tomo_run_wbp(h, 0, H))
            _abi_mod().check(lib.tomo_set_weighting(h, _abi_mod().WEIGHT_NONE, 0.0, None, None))
            _abi_mod().check(lib.tomo_run_ossart(h, wl["n_iter"], wl["relax"], 0, seed, 0, H, 1, None))

        for _ in range(3):
            job()
        reps = 10
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(reps):
            job()
        ev1.record(stream)
        torch.cuda.synchronize()
        gpu_s = ev0.elapsed_time(ev1) / 1000.0 / reps
    finally:
        lib.tomo_destroy(h)
    # CPU: the whole job once
    mask = O.ramp_mask(W, H, angles, hamming=False)
    order = O.order_shuffle(eul, 0)
    t0 = time.perf_counter()
    rec = np.zeros((D, H, W), np.float32)
    O.wbp(rec, g, eul, series, mask)
    for _ in range(wl["n_iter"]):
        O.ossart_iteration(rec, g, eul, series, order, wl["relax"], 0)
    cpu_s = time.perf_counter() - t0
    return {"workload": "sirt256: 256x64x256, 61 tilts of 256x64, ramp WBP + 10 SIRT iterations",
            "updates": ups, "engine_s": gpu_s, "engine_voxel_updates_per_s": ups / gpu_s,
            "cpu_s": cpu_s, "cpu_voxel_updates_per_s": ups / cpu_s, "cpu_cores": threads,
            "cpu_kind": "port", "speedup": cpu_s / gpu_s}


def phantom_on_device(W, H, D, n_ell, seed, device):
    """The seeded ellipsoid phantom of tomoj_gb300.phantom (same parameter draws),
    evaluated on the GPU for volumes too large for the host generator."""
    import math
    import torch
    from tomoj_gb300 import phantom as P
    g = P.rng(seed)
    vol = torch.zeros((D, H, W), dtype=torch.float32, device=device)
    dims = np.array([W, H, D], np.float64)
    for _ in range(n_ell):
        axes = g.uniform(0.05, 0.25, 3) * dims
        centre = np.clip(g.uniform(0.0, 1.0, 3) * (dims - 2 * axes) + axes, 0, dims - 1)
        a, b, c = g.uniform(0, 2 * np.pi, 3)
        ca, sa, cb, sb, cc, sc = math.cos(a), math.sin(a), math.cos(b), math.sin(b), math.cos(c), math.sin(c)
        Rm = (np.array([[ca, -sa, 0], [sa, ca, 0], [0, 0, 1]]) @ np.array([[cb, 0, sb], [0, 1, 0], [-sb, 0, cb]])
              @ np.array([[cc, -sc, 0], [sc, cc, 0], [0, 0, 1]])).astype(np.float32)
        dens = float(g.uniform(0.0, 1.0))
        r = float(np.max(axes)) + 1
        x0, x1 = int(max(0, centre[0] - r)), int(min(W, centre[0] + r + 1))
        y0, y1 = int(max(0, centre[1] - r)), int(min(H, centre[1] + r + 1))
        z0, z1 = int(max(0, centre[2] - r)), int(min(D, centre[2] + r + 1))
        if x0 >= x1 or y0 >= y1 or z0 >= z1:
            continue
        px = (torch.arange(x0, x1, device=device, dtype=torch.float32) - float(centre[0]))[None, None, :]
        py = (torch.arange(y0, y1, device=device, dtype=torch.float32) - float(centre[1]))[None, :, None]
        pz = (torch.arange(z0, z1, device=device, dtype=torch.float32) - float(centre[2]))[:, None, None]
        q = 0
        for k in range(3):
            t = (float(Rm[0, k]) * px + float(Rm[1, k]) * py + float(Rm[2, k]) * pz) / float(axes[k])
            q = q + t * t
        vol[z0:z1, y0:y1, x0:x1] += (q <= 1.0).to(torch.float32) * dens
    return vol


def _config4_series(lib, W, H, D, n, seed, stream):
    """The tilt-series of the reduced-precision workload: the seeded ellipsoid phantom
    (evaluated on the GPU), its FP32 forward projection by the engine at -60..+60 deg in
    equal steps, then Poisson noise at 50 e-/px.  Returns (series float32 (n, H, W), eulers)."""
    import torch
    from tomoj_gb300 import _abi
    from tomoj_gb300 import phantom as P
    eul = euler_y(np.linspace(-60.0, 60.0, n))
    vol = phantom_on_device(W, H, D, P.n_ellipsoids_for(W, H, D), seed, "cuda")
    g = _abi.make_geom(W, H, D, W, H, n)
    prm = _abi.make_params(fill=_abi.FILL_NAN)
    h = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(g), C.byref(prm), C.byref(h)))
    series = np.empty((n, H, W), np.float32)
    try:
        _abi.check(lib.tomo_set_stream(h, C.c_void_p(stream.cuda_stream)))
        _abi.check(lib.tomo_load_series(h, series.ctypes.data, 0, _abi.ptr(eul, C.c_double), None, None))
        torch.cuda.synchronize()
        _abi.check(lib.tomo_set_volume(h, C.c_void_p(vol.data_ptr()), 1, 0, H))
        for i in range(n):
            _abi.check(lib.tomo_add_projection(h, i))
        _abi.check(lib.tomo_project(h, 0, H))
        for i in range(n):
            _abi.check(lib.tomo_get_projection(h, i, _abi.ptr(series[i])))
    finally:
        lib.tomo_destroy(h)
    del vol
    torch.cuda.empty_cache()
    return P.add_poisson_noise(np.nan_to_num(series), 50.0, seed + 1), eul


def _device_rel_l2(a, b, chunk=64):
    """||a - b|| / ||b|| of two (D, H, W) float32 device tensors, accumulated in FP64 by plane chunks."""
    num = den = 0.0
    for z in range(0, a.shape[0], chunk):
        x, y = a[z:z + chunk].double(), b[z:z + chunk].double()
        num += float(((x - y) ** 2).sum())
        den += float((y ** 2).sum())
    return (num / max(den, 1e-300)) ** 0.5


def _schedule(lib, W, H, D, series, eul, prec, n_sirt, n_tvm, seed, stream):
    """n_sirt SIRT iterations then n_tvm TVM iterations (SIRT + TV denoise: theta 25, g 1,
    dt = lambda = 0.01, 5 inner steps) on one handle; both parts timed with CUDA events on the
    handle's stream.  Returns (figures, volume after SIRT, final volume) with the volumes as
    FP32 device tensors."""
    import torch
    from tomoj_gb300 import _abi
    n = series.shape[0]
    g = _abi.make_geom(W, H, D, W, H, n)
    prm = _abi.make_params(fill=_abi.FILL_NAN, precision=prec)
    h = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(g), C.byref(prm), C.byref(h)))
    try:
        _abi.check(lib.tomo_set_stream(h, C.c_void_p(stream.cuda_stream)))
        _abi.check(lib.tomo_load_series(h, series.ctypes.data, 0, _abi.ptr(eul, C.c_double), None, None))
        _abi.check(lib.tomo_run_ossart(h, 1, 1.0, 0, seed, 0, H, 1, None))  # warm-up: tables, graph
        _abi.check(lib.tomo_fill_volume(h, 0.0))
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        torch.cuda.synchronize()
        ev[0].record(stream)
        _abi.check(lib.tomo_run_ossart(h, n_sirt, 1.0, 0, seed, 0, H, 1, None))
        ev[1].record(stream)
        after_sirt = torch.empty((D, H, W), dtype=torch.float32, device="cuda")
        _abi.check(lib.tomo_get_volume(h, C.c_void_p(after_sirt.data_ptr()), 1, 0, H))
        _abi.check(lib.tomo_set_tvm(h, 25.0, 1.0, 0.01, 5))
        ev[1].synchronize()
        ev[2].record(stream)
        _abi.check(lib.tomo_run_ossart(h, n_tvm, 1.0, 0, seed, 0, H, 1, None))
        ev3 = torch.cuda.Event(enable_timing=True)
        ev3.record(stream)
        torch.cuda.synchronize()
        final = torch.empty((D, H, W), dtype=torch.float32, device="cuda")
        _abi.check(lib.tomo_get_volume(h, C.c_void_p(final.data_ptr()), 1, 0, H))
        torch.cuda.synchronize()
    finally:
        lib.tomo_destroy(h)
    sirt_ms = ev[0].elapsed_time(ev[1])
    tvm_ms = ev[2].elapsed_time(ev3)
    ups = W * H * D * n
    fig = {"sirt_voxel_updates_per_s": ups * n_sirt / (sirt_ms / 1000.0), "sirt_ms_per_iteration": sirt_ms / n_sirt,
           "tvm_ms_per_iteration": tvm_ms / max(n_tvm, 1),
           "schedule_voxel_updates_per_s": ups * (n_sirt + n_tvm) / ((sirt_ms + tvm_ms) / 1000.0),
           "volume_bytes": W * H * D * (4 if prec == _abi.PREC_FP32 else 2)}
    return fig, after_sirt, final


def _fp64_reference(series, eul, W, H, D, n_sirt, n_tvm, seed, threads):
    """The FP64 oracle (oracle/oracle64.py) on the same schedule, whole volume."""
    from oracle import oracle as O
    from oracle import oracle64 as O64
    lib = _abi_mod().load()
    n = series.shape[0]
    O64.set_threads(threads)
    g = O.Geom(W, H, D, W, H)
    meas = np.ascontiguousarray(series, np.float64)
    vol = np.zeros((D, H, W), np.float64)
    for it in range(n_sirt):
        O64.ossart_iteration(vol, g, eul, meas, O.order_shuffle(eul, int(lib.tomo_first_index(seed, it, n))), 1.0, 0)
    after_sirt = vol.copy()
    for it in range(n_tvm):
        O64.ossart_iteration(vol, g, eul, meas, O.order_shuffle(eul, int(lib.tomo_first_index(seed, it, n))), 1.0, 0)
        O64.tv_denoise(vol, 25.0, 1.0, 0.01, 5)
    return after_sirt, vol


def run_precision_leg(lib, args):
    """BASELINE config 4 at its schedule: a W x H x D = 2048 x 512 x 2048 phantom, 121
    projections of 2048 x 512 at -60..+60 deg in 1 deg steps with Poisson noise at 50 e-/px;
    50 SIRT iterations, then 20 TVM iterations (SIRT + TV denoise, lambda = dt = 0.01), with
    the volume stored in FP32, BF16 and FP16 (per-row slab scales, Kahan-compensated FP32
    backprojection sums, FP64 residual norms).  Reports per storage its voxel-updates/s and
    its relative L2 against the FP32 form (whole volume, after the SIRT part and at the end).

    The FP64 oracle costs ~20 ns per voxel-update per core (about 18 min per volume row of
    this size for the 50 SIRT iterations), so the relative L2 against FP64 is measured on the
    same schedule, tilts, noise and phantom generator at args.prec_check (384 x 32 x 384 by
    default), whole volume, with the oracle running on all host cores beside the GPU work."""
    import threading
    import torch
    from tomoj_gb300 import _abi
    stream = torch.cuda.current_stream()
    n, seed = 121, 5
    n_sirt, n_tvm = args.prec_sirt, args.prec_tvm
    forms = (("fp32", _abi.PREC_FP32), ("bf16", _abi.PREC_BF16), ("fp16", _abi.PREC_FP16))
    out = {"schedule": f"{n_sirt} SIRT + {n_tvm} TVM iterations (TV: theta 25, g 1, dt 0.01, 5 inner steps)"}
    # --- FP64 check on the scaled volume: inputs, then the oracle on a host thread ---
    cW, cH, cD = args.prec_check
    t0 = time.time()
    cser, ceul = _config4_series(lib, cW, cH, cD, n, 4321, stream)
    ref64 = {}
    threads = os.cpu_count() or 1

    def oracle_job():
        t = time.time()
        ref64["sirt"], ref64["final"] = _fp64_reference(cser, ceul, cW, cH, cD, n_sirt, n_tvm, seed, threads)
        ref64["seconds"] = time.time() - t

    th = threading.Thread(target=oracle_job, daemon=True)
    th.start()
    check = {}
    for name, prec in forms:
        fig, a, f = _schedule(lib, cW, cH, cD, cser, ceul, prec, n_sirt, n_tvm, seed, stream)
        check[name] = (a.cpu().numpy().astype(np.float64), f.cpu().numpy().astype(np.float64))
        del a, f
    # --- full size ---
    W, H, D = args.prec_size
    series, eul = _config4_series(lib, W, H, D, n, 1238, stream)
    log(f"[bench] precision inputs ready in {time.time() - t0:.1f}s")
    ref_sirt = ref_final = None
    for name, prec in forms:
        fig, a, f = _schedule(lib, W, H, D, series, eul, prec, n_sirt, n_tvm, seed, stream)
        if name == "fp32":
            ref_sirt, ref_final = a, f
        else:
            fig["rel_l2_vs_fp32_after_sirt"] = _device_rel_l2(a, ref_sirt)
            fig["rel_l2_vs_fp32"] = _device_rel_l2(f, ref_final)
            fig["speedup_vs_fp32"] = fig["sirt_voxel_updates_per_s"] / out["fp32"]["sirt_voxel_updates_per_s"]
            del a, f
        out[name] = fig
        torch.cuda.empty_cache()
    del ref_sirt, ref_final
    torch.cuda.empty_cache()
    th.join()

    def rel(x, y):
        return float(np.linalg.norm(x - y) / max(np.linalg.norm(y), 1e-300))

    for name, _ in forms:
        a, f = check[name]
        out[name]["rel_l2_vs_fp64_after_sirt"] = rel(a, ref64["sirt"])
        out[name]["rel_l2_vs_fp64"] = rel(f, ref64["final"])
        out[name]["meets_1e-3_vs_fp64"] = out[name]["rel_l2_vs_fp64"] <= 1e-3
    out["workload"] = f"{W}x{H}x{D} phantom, {n} tilts of {W}x{H} at -60..60 deg (1 deg), Poisson 50 e-/px"
    out["fp64_check"] = {"volume": f"{cW}x{cH}x{cD}", "tilts": n, "oracle": "oracle/oracle64 (FP64), whole volume",
                         "cpu_threads": threads, "oracle_seconds": ref64.get("seconds")}
    return out


def _abi_mod():
    from tomoj_gb300 import _abi
    return _abi


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="ossart512", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the batched, serving and precision legs")
    ap.add_argument("--legs", default="all",
                    help="comma list of extra legs to run: row_streams, compressed_sensing, config1, batched, "
                         "serving, precision, tv (default all)")
    ap.add_argument("--tv-size", type=int, nargs=3, default=[2048, 512, 2048], metavar=("W", "H", "D"),
                    help="volume of the TV denoise leg")
    ap.add_argument("--serve-requests", type=int, default=128)
    ap.add_argument("--prec-size", type=int, nargs=3, default=[2048, 512, 2048], metavar=("W", "H", "D"),
                    help="volume of the reduced-precision leg")
    ap.add_argument("--prec-check", type=int, nargs=3, default=[384, 32, 384], metavar=("W", "H", "D"),
                    help="volume on which the reduced-precision schedule is checked against the FP64 oracle")
    ap.add_argument("--prec-sirt", type=int, default=50)
    ap.add_argument("--prec-tvm", type=int, default=20)
    args = ap.parse_args()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, wl)
    else:
        run_engine(args, wl)


if __name__ == "__main__":
    main()

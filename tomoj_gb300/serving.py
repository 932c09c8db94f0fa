"""Continuous-batching reconstruction server.

Requests (a tilt-series plus a method: WBP, SIRT, OS-SART or TVM, with its
iteration count) arrive over time.  The server keeps every admitted request's
volume, series and residuals resident in HBM and advances all active iterative
requests together, one batched iteration per tick (tomo_batch_iteration: one
launch per kernel variant covers every member).  Requests join at the next
tick after their series is uploaded and leave when their last iteration is
done, so requests that arrive while others run share the GPU with them.

Admission is by free HBM: a request is admitted when the engine can allocate
its buffers (tomo_create's admission control, TOMO_ERR_NOMEM otherwise) and an
active slot is free; otherwise it waits until a running request completes and
releases its memory.  Handle creation and the series upload run on an
admission thread, so the host-to-device copy overlaps the running batch.

Reported: per request time-to-reconstruction (completion - arrival), p50/p99,
and aggregate voxel-updates/s.  Because a batched iteration is bitwise the
same as running the request alone, a request's result does not depend on the
mix it ran in.
"""
from __future__ import annotations

import ctypes as C
import heapq
import queue
import threading
from concurrent.futures import ThreadPoolExecutor
import time
from dataclasses import dataclass, field

import numpy as np

from . import _abi


def _release_torch_cache() -> bool:
    """Admission is by free HBM: blocks that torch's allocator keeps cached in this process
    count as used.  When torch is loaded with CUDA, hand them back; True if it was."""
    import sys
    torch = sys.modules.get("torch")
    if torch is None or not torch.cuda.is_initialized():
        return False
    torch.cuda.empty_cache()
    return True
from .tiltseries import euler_angles_to_matrix

WBP, SIRT, OSSART, TVM = "WBP", "SIRT", "OS-SART", "TVM"


@dataclass
class Request:
    rid: int
    arrival: float               # seconds after the server starts
    kind: str                    # WBP | SIRT | OS-SART | TVM
    series: np.ndarray           # (N, h, w) float32, unaligned
    angles: np.ndarray           # (N,) degrees
    W: int
    H: int
    D: int
    n_iter: int = 1
    update: int = 0              # 0 = SIRT
    relax: float = 1.0
    seed: int = 0
    transforms: np.ndarray | None = None   # (N, 6) AffineTransform matrices
    tvm: tuple = (25.0, 1.0, 0.01, 5)      # theta, g, dt (lambda), inner iterations
    weighting: int = _abi.WEIGHT_HAMMING_RAMP
    keep_volume: bool = False

    def updates(self) -> int:
        passes = 1 if self.kind == WBP else self.n_iter
        return self.W * self.H * self.D * len(self.angles) * passes


@dataclass
class Result:
    rid: int
    kind: str
    arrival: float
    admitted: float
    completed: float
    updates: int
    errors: list = field(default_factory=list)
    volume: np.ndarray | None = None

    @property
    def latency(self) -> float:
        return self.completed - self.arrival


class EngineAdapter:
    """The engine calls the server needs (a fake with the same methods tests the scheduling on CPU).

    The active requests iterate as `split` batches (alternate members), each on its own
    stream and driven from its own host thread, so that one batch's forward projections
    run beside another's backprojections."""

    def __init__(self, split: int = 2):
        self.lib = _abi.load()
        self.batches = []
        for _ in range(max(1, split)):
            b = C.c_void_p()
            _abi.check(self.lib.tomo_batch_create(C.byref(b)))
            self.batches.append(b)
        self.pool = ThreadPoolExecutor(max_workers=len(self.batches)) if len(self.batches) > 1 else None

    def close(self):
        if self.pool is not None:
            self.pool.shutdown()
        for b in self.batches:
            self.lib.tomo_batch_destroy(b)

    def create(self, req: Request):
        """Handle with the request's series loaded; None if HBM is short (TOMO_ERR_NOMEM)."""
        lib = self.lib
        N, h, w = req.series.shape
        g = _abi.make_geom(req.W, req.H, req.D, w, h, N)
        fill = _abi.FILL_AVG if req.kind == WBP else _abi.FILL_NAN
        p = _abi.make_params(fill=fill)
        hd = C.c_void_p()
        rc = lib.tomo_create(C.byref(g), C.byref(p), C.byref(hd))
        if rc == _abi.ERR_NOMEM and _release_torch_cache():
            rc = lib.tomo_create(C.byref(g), C.byref(p), C.byref(hd))
        if rc == _abi.ERR_NOMEM:
            return None
        _abi.check(rc)
        try:
            eul = np.ascontiguousarray([euler_angles_to_matrix(0.0, a, -0.0) for a in req.angles], np.float64)
            T = None if req.transforms is None else np.ascontiguousarray(req.transforms, np.float64)
            pix = np.ascontiguousarray(req.series, np.float32)
            _abi.check(lib.tomo_load_series(hd, pix.ctypes.data, 0, _abi.ptr(eul, C.c_double),
                                            None if T is None else _abi.ptr(T, C.c_double), None))
            if req.kind == WBP:
                _abi.check(lib.tomo_set_weighting(hd, req.weighting, 0.5, None, None))
            if req.kind == TVM:
                th, gg, dt, it = req.tvm
                _abi.check(lib.tomo_set_tvm(hd, th, gg, dt, it))
        except Exception:
            lib.tomo_destroy(hd)
            raise
        return hd

    def run_wbp(self, hd, req: Request):
        _abi.check(self.lib.tomo_run_wbp(hd, 0, req.H))

    def set_members(self, handles):
        k = len(self.batches)
        for i, b in enumerate(self.batches):
            part = handles[i::k]
            arr = (C.c_void_p * max(len(part), 1))(*[h.value for h in part])
            _abi.check(self.lib.tomo_batch_set(b, arr, len(part)))

    def iterate(self, handles, reqs, iteration):
        M, k = len(handles), len(self.batches)
        relax = np.array([r.relax for r in reqs], np.float64)
        upd = np.array([0 if r.kind in (SIRT, TVM) else r.update for r in reqs], np.int32)
        first = np.array([self.lib.tomo_first_index(r.seed, it, len(r.angles)) for r, it in zip(reqs, iteration)],
                         np.int32)
        err = np.zeros((M, 5))

        def run(i):
            idx = np.arange(i, M, k)
            if idx.size == 0:
                return
            r, u, f = (np.ascontiguousarray(x[idx]) for x in (relax, upd, first))
            e = np.zeros((idx.size, 5))
            _abi.check(self.lib.tomo_batch_iteration(self.batches[i], _abi.ptr(r, C.c_double),
                                                     _abi.ptr(u, C.c_int32), _abi.ptr(f, C.c_int32), 1,
                                                     _abi.ptr(e, C.c_double)))
            err[idx] = e

        if self.pool is None:
            run(0)
        else:
            list(self.pool.map(run, range(k)))
        return err

    def read_volume(self, hd, req: Request):
        out = np.empty((req.D, req.H, req.W), np.float32)
        _abi.check(self.lib.tomo_get_volume(hd, out.ctypes.data, 0, 0, req.H))
        return out

    def destroy(self, hd):
        self.lib.tomo_destroy(hd)


class Server:
    def __init__(self, engine=None, max_active: int = 64):
        self.engine = engine if engine is not None else EngineAdapter()
        self.max_active = max_active

    def run(self, requests: list[Request], time_scale: float = 1.0) -> list[Result]:
        """Serve `requests` (arrival times scaled by time_scale) to completion."""
        eng = self.engine
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0  # noqa: E731
        pending = [(r.arrival * time_scale, r.rid, r) for r in requests]
        heapq.heapify(pending)
        arrived: queue.Queue = queue.Queue()      # arrived, not yet admitted (FIFO)
        ready: queue.Queue = queue.Queue()        # admitted handles waiting to join
        freed = threading.Event()
        stop = threading.Event()
        results: dict[int, Result] = {}
        slots = threading.Semaphore(self.max_active)
        errors: list[BaseException] = []
        inflight = [0]  # admitted requests not yet completed (guarded by lock)
        lock = threading.Lock()

        def admitter():
            while not stop.is_set():
                try:
                    req = arrived.get(timeout=0.01)
                except queue.Empty:
                    continue
                slots.acquire()
                while True:
                    try:
                        hd = eng.create(req)
                    except BaseException as e:  # surfaced to the caller
                        errors.append(e)
                        slots.release()
                        hd = "failed"
                        break
                    if hd is not None:
                        break
                    with lock:
                        alone = inflight[0] == 0
                    if alone:  # nothing running will free memory: the request can never fit
                        errors.append(_abi.NoMemoryError(-3, f"request {req.rid} does not fit in free HBM"))
                        slots.release()
                        hd = "failed"
                        break
                    freed.clear()
                    freed.wait(0.05)  # HBM short: wait for a completion
                    if stop.is_set():
                        slots.release()
                        return
                if hd != "failed":
                    with lock:
                        inflight[0] += 1
                    ready.put((req, hd, now()))

        th = threading.Thread(target=admitter, daemon=True)
        th.start()
        active = []          # [req, handle, admitted, iterations done, errors]
        members_dirty = False
        n_total = len(requests)
        try:
            while len(results) < n_total:
                if errors:
                    raise errors[0]
                t = now()
                while pending and pending[0][0] <= t:
                    arrived.put(heapq.heappop(pending)[2])
                joined = False
                while True:
                    try:
                        req, hd, adm = ready.get_nowait()
                    except queue.Empty:
                        break
                    if req.kind == WBP:
                        eng.run_wbp(hd, req)
                        vol = eng.read_volume(hd, req) if req.keep_volume else None
                        eng.destroy(hd)
                        with lock:
                            inflight[0] -= 1
                        slots.release()
                        freed.set()
                        results[req.rid] = Result(req.rid, req.kind, req.arrival * time_scale, adm, now(),
                                                  req.updates(), [], vol)
                    else:
                        active.append([req, hd, adm, 0, []])
                        joined = True
                if joined:
                    members_dirty = True
                if not active:
                    time.sleep(0.001)
                    continue
                if members_dirty:
                    eng.set_members([a[1] for a in active])
                    members_dirty = False
                err = eng.iterate([a[1] for a in active], [a[0] for a in active], [a[3] for a in active])
                done = []
                for a, e in zip(active, err):
                    a[3] += 1
                    a[4].append(list(e))
                    if a[3] >= a[0].n_iter:
                        done.append(a)
                if done:
                    for a in done:
                        req, hd = a[0], a[1]
                        vol = eng.read_volume(hd, req) if req.keep_volume else None
                        active.remove(a)
                        results[req.rid] = Result(req.rid, req.kind, req.arrival * time_scale, a[2], now(),
                                                  req.updates(), a[4], vol)
                    # the batch must forget the finished handles before they are destroyed
                    eng.set_members([a[1] for a in active])
                    members_dirty = False
                    for a in done:
                        eng.destroy(a[1])
                        with lock:
                            inflight[0] -= 1
                        slots.release()
                    freed.set()
        finally:
            stop.set()
            th.join(timeout=5)
        return [results[r.rid] for r in requests]


def summarize(results: list[Result], wall_s: float | None = None) -> dict:
    lat = np.array([r.latency for r in results])
    t_first = min(r.arrival for r in results)
    t_last = max(r.completed for r in results)
    span = wall_s if wall_s is not None else (t_last - t_first)
    ups = sum(r.updates for r in results)
    return {"requests": len(results), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "makespan_s": float(span), "voxel_updates_per_s": ups / span if span else 0.0,
            "kinds": {k: int(sum(1 for r in results if r.kind == k)) for k in (WBP, SIRT, OSSART, TVM)}}


def synthetic_requests(n: int, seed: int, rate: float = 4.0, sizes=(512, 1024, 2048), thick=(128, 256, 512),
                       tilts=(41, 61, 121), mix=((WBP, 0.3), (SIRT, 0.4), (OSSART, 0.2), (TVM, 0.1)),
                       iters=(5, 50), keep_volume=False) -> list[Request]:
    """Poisson arrivals (mean `rate` per second) of seeded synthetic tilt-series with the
    serving configuration's size, tilt-count and method distributions."""
    g = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    cache: dict[tuple, np.ndarray] = {}
    kinds, probs = zip(*mix)
    for rid in range(n):
        t += g.exponential(1.0 / rate)
        N = int(g.choice(sizes))
        D = int(g.choice(thick))
        nt = int(g.choice(tilts))
        kind = str(g.choice(kinds, p=probs))
        amax = 60.0
        angles = np.linspace(-amax, amax, nt)
        key = (N, nt)
        if key not in cache:
            # smooth synthetic projections: a few Gaussian blobs, shifted per tilt
            yy, xx = np.mgrid[0:N, 0:N].astype(np.float32)
            base = np.zeros((N, N), np.float32)
            for _ in range(6):
                cx, cy, s = g.uniform(0.2, 0.8) * N, g.uniform(0.2, 0.8) * N, g.uniform(0.03, 0.1) * N
                base += np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / (2 * s * s)) * np.float32(D * 0.2)
            cache[key] = np.stack([np.roll(base, int(round(N * 0.1 * np.sin(np.deg2rad(a)))), axis=1)
                                   for a in angles]).astype(np.float32)
        n_iter = 1 if kind == WBP else int(g.integers(iters[0], iters[1] + 1))
        update = 0 if kind in (SIRT, TVM, WBP) else -(-nt // 10)  # "10 subsets": subset size ceil(N / 10)
        out.append(Request(rid, t, kind, cache[key], angles, N, N, D, n_iter, update, 1.0, int(g.integers(0, 1 << 30)),
                           keep_volume=keep_volume))
    return out

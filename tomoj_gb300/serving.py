"""Continuous-batching reconstruction server.

Requests (a tilt-series plus a method: WBP, SIRT, OS-SART or TVM, with its
iteration count and volume storage precision) arrive over time.  The server keeps
every admitted request's volume, series and residuals resident in HBM.

* Admission (one host thread): requests queue in arrival order per lane (below);
  the head of the most urgent lane that fits is admitted when its lane has a free
  active slot and the engine can allocate its buffers (a free-HBM check first,
  leaving a per-lane headroom for more urgent lanes, then tomo_create's admission
  by free HBM, TOMO_ERR_NOMEM otherwise; handle buffers come from the engine's
  stream-ordered pool, so a retired request's memory is reused without a
  device-wide synchronisation).  A large request waiting for HBM therefore does
  not hold back smaller ones; under sustained overload large requests wait
  longest.  The series upload runs on the admission thread, beside the GPU work
  of the running requests.
* Iterative requests (SIRT, OS-SART, TVM) join a lane by the size of one of their
  iterations (voxel-updates).  Each lane is one batch (tomo_batch_iteration: one
  launch per kernel variant covers every member, the iteration replayed as a CUDA
  graph) driven by its own host thread, on its own stream, at its own priority:
  lanes iterate independently, so a 512^2 request is not paced by the iterations
  of 2048^2 ones, and the lanes of smaller requests are more urgent: their CTAs
  are dispatched first as SMs free up (measured: a 10.5 ms iteration of five
  512^2 series takes 10.9 ms beside a 2048^2 x 512 iteration of 200 ms).  Requests join a lane between two of its
  iterations and leave when their last iteration is done.
* WBP requests (one weighted backprojection) run on a worker thread per lane, each
  on its handle's own stream at the most urgent priority.

Reported: per request time-to-reconstruction (completion - arrival), p50/p99 over
all requests and per method and size, aggregate voxel-updates/s, and the offered
load (arrival rate x mean work) against the throughput achieved.  Because a
batched iteration is bitwise the same as running the request alone, a request's
result does not depend on the mix it ran in.

`simulate` replays the same policy in virtual time with per-iteration costs from
measured rates, for schedules too long to serve in a benchmark run.
"""
from __future__ import annotations

import ctypes as C
import heapq
import queue
import threading
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .tiltseries import euler_angles_to_matrix

WBP, SIRT, OSSART, TVM = "WBP", "SIRT", "OS-SART", "TVM"
KINDS = (WBP, SIRT, OSSART, TVM)

# Lane boundaries in voxel-updates per iteration (W * H * D * tilts): below 8e9 (e.g.
# 512^2 x 256 x 61), below 6e10 (1024^2 x 512 x 121 and smaller), the rest.
DEFAULT_LANE_BOUNDS = (8e9, 6e10)


def _release_torch_cache() -> bool:
    """Admission is by free HBM: blocks that torch's allocator keeps cached in this process
    count as used.  When torch is loaded with CUDA, hand them back; True if it was."""
    import sys
    torch = sys.modules.get("torch")
    if torch is None or not torch.cuda.is_initialized():
        return False
    torch.cuda.empty_cache()
    return True


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
    precision: int = _abi.PREC_FP32        # volume storage (PREC_*)

    def updates_per_iteration(self) -> int:
        return self.W * self.H * self.D * len(self.angles)

    def updates(self) -> int:
        passes = 1 if self.kind == WBP else self.n_iter
        return self.updates_per_iteration() * passes


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
    size: int = 0
    lane: int = -1               # -1: WBP worker
    create_s: float = 0.0        # handle creation and series upload

    @property
    def latency(self) -> float:
        return self.completed - self.arrival


def lane_of(req: Request, bounds) -> int:
    u = req.updates_per_iteration()
    for i, b in enumerate(bounds):
        if u < b:
            return i
    return len(bounds)


class EngineAdapter:
    """The engine calls the server needs (a fake with the same methods tests the scheduling
    on CPU): one batch per lane, lane 0 on the most urgent stream priority."""

    def __init__(self, lanes: int = 3):
        self.lib = _abi.load()
        self.n_lanes = max(1, int(lanes))
        self.batches = []
        for i in range(self.n_lanes):
            b = C.c_void_p()
            _abi.check(self.lib.tomo_batch_create(C.byref(b)))
            self.batches.append(b)
            _abi.check(self.lib.tomo_batch_set_priority(b, self.n_lanes - 1 - i))
        self.top_priority = self.n_lanes

    def close(self):
        for b in self.batches:
            self.lib.tomo_batch_destroy(b)
        self.batches = []

    def fits(self, req: Request, headroom: float = 0.0) -> bool:
        """Whether free HBM (with the engine pool's idle blocks) holds the request's estimated
        footprint and still leaves `headroom` (a fraction of the device's HBM): a cheap test
        before tomo_create, which would otherwise allocate and release most of a request
        that cannot be admitted yet."""
        free, total = C.c_uint64(), C.c_uint64()
        if self.lib.tomo_device_memory(C.byref(free), C.byref(total)) != _abi.OK:
            return True
        return request_bytes(req) + headroom * total.value <= free.value

    def create(self, req: Request):
        """Handle with the request's series loaded; None if HBM is short (TOMO_ERR_NOMEM)."""
        lib = self.lib
        N, h, w = req.series.shape
        g = _abi.make_geom(req.W, req.H, req.D, w, h, N)
        fill = _abi.FILL_AVG if req.kind == WBP else _abi.FILL_NAN
        p = _abi.make_params(fill=fill, precision=req.precision)
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
            # the series tables and the TV scratch are allocated here too: HBM short for
            # them defers the request like a short tomo_create
            rc = lib.tomo_load_series(hd, pix.ctypes.data, 0, _abi.ptr(eul, C.c_double),
                                      None if T is None else _abi.ptr(T, C.c_double), None)
            if rc == _abi.ERR_NOMEM:
                lib.tomo_destroy(hd)
                return None
            _abi.check(rc)
            if req.kind == WBP:
                _abi.check(lib.tomo_set_weighting(hd, req.weighting, 0.5, None, None))
                _abi.check(lib.tomo_set_priority(hd, self.top_priority))
            if req.kind == TVM:
                th, gg, dt, it = req.tvm
                rc = lib.tomo_set_tvm(hd, th, gg, dt, it)
                if rc == _abi.ERR_NOMEM:
                    lib.tomo_destroy(hd)
                    return None
                _abi.check(rc)
        except Exception:
            lib.tomo_destroy(hd)
            raise
        return hd

    def run_wbp(self, hd, req: Request):
        _abi.check(self.lib.tomo_run_wbp(hd, 0, req.H))

    def set_members(self, handles, lane: int = 0):
        arr = (C.c_void_p * max(len(handles), 1))(*[h.value for h in handles])
        _abi.check(self.lib.tomo_batch_set(self.batches[lane], arr, len(handles)))

    def iterate(self, handles, reqs, iteration, lane: int = 0):
        M = len(handles)
        relax = np.ascontiguousarray([r.relax for r in reqs], np.float64)
        upd = np.ascontiguousarray([0 if r.kind in (SIRT, TVM) else r.update for r in reqs], np.int32)
        first = np.ascontiguousarray([self.lib.tomo_first_index(r.seed, it, len(r.angles))
                                      for r, it in zip(reqs, iteration)], np.int32)
        err = np.zeros((M, 5))
        _abi.check(self.lib.tomo_batch_iteration(self.batches[lane], _abi.ptr(relax, C.c_double),
                                                 _abi.ptr(upd, C.c_int32), _abi.ptr(first, C.c_int32), 1,
                                                 _abi.ptr(err, C.c_double)))
        return err

    def read_volume(self, hd, req: Request):
        out = np.empty((req.D, req.H, req.W), np.float32)
        _abi.check(self.lib.tomo_get_volume(hd, out.ctypes.data, 0, 0, req.H))
        return out

    def destroy(self, hd):
        self.lib.tomo_destroy(hd)


class Server:
    def __init__(self, engine=None, max_active: int = 64, lane_bounds=None, headroom=None):
        """max_active: active requests per lane.  headroom: per lane, the fraction of HBM its
        admissions must leave free for more urgent lanes (default 0 for the most urgent lane,
        0.05 for the next, 0.15 for the others).  After run(), `lane_log` holds one
        (lane, start, end, members, voxel-updates) tuple per batched iteration."""
        self.engine = engine if engine is not None else EngineAdapter()
        self.max_active = max_active
        self.lane_log: list[tuple] = []
        n = getattr(self.engine, "n_lanes", 1)
        bounds = DEFAULT_LANE_BOUNDS if lane_bounds is None else tuple(lane_bounds)
        if len(bounds) < n - 1:
            raise ValueError(f"{n} lanes need {n - 1} lane bounds")
        self.bounds = tuple(bounds[:n - 1])
        self.headroom = tuple(headroom) if headroom is not None else tuple(
            0.0 if i == 0 else 0.05 if i == 1 else 0.15 for i in range(n))

    def run(self, requests: list[Request], time_scale: float = 1.0) -> list[Result]:
        """Serve `requests` (arrival times scaled by time_scale) to completion."""
        eng = self.engine
        n_lanes = len(self.bounds) + 1
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0  # noqa: E731
        pending = [(r.arrival * time_scale, r.rid, r) for r in requests]
        heapq.heapify(pending)
        arrived = [queue.Queue() for _ in range(n_lanes)]  # per lane: arrived, not yet admitted (FIFO)
        inbox = [queue.Queue() for _ in range(n_lanes)]
        wbp_q = [queue.Queue() for _ in range(n_lanes)]
        freed = threading.Event()  # a completion: the admitter retries
        stop = threading.Event()
        all_done = threading.Event()
        results: dict[int, Result] = {}
        created: dict[int, float] = {}
        # active slots per lane (WBP requests count in their size's lane), so that large
        # requests filling their lane's slots never hold back smaller ones
        slots = [threading.Semaphore(self.max_active) for _ in range(n_lanes)]
        errors: list[BaseException] = []
        inflight = [0]  # admitted requests not yet completed (guarded by lock)
        lock = threading.Lock()
        n_total = len(requests)
        self.lane_log = []
        if n_total == 0:
            return []

        def finish(res: Result, hd, req: Request):
            res.create_s = created.get(res.rid, 0.0)
            eng.destroy(hd)
            with lock:
                inflight[0] -= 1
                results[res.rid] = res
                if len(results) == n_total:
                    all_done.set()
            slots[lane_of(req, self.bounds)].release()
            freed.set()

        def fail(e: BaseException):
            errors.append(e)
            all_done.set()

        def admitter():
            # one FIFO per lane (WBP requests by their size too); the most urgent lane whose
            # head fits is admitted first, so small requests are not held behind a large one
            # that waits for HBM.  One thread: concurrent series uploads slowed each other
            # (measured: 0.5 s median creation of a 512^2 request with one admission thread
            # per lane, p50 over all requests 18 s instead of 9.6 s).
            queues = [deque() for _ in range(n_lanes)]
            while not stop.is_set():
                for li in range(n_lanes):
                    while True:
                        try:
                            queues[li].append(arrived[li].get_nowait())
                        except queue.Empty:
                            break
                if not any(queues):
                    time.sleep(0.002)
                    continue
                admitted = False
                for li, q in enumerate(queues):
                    if not q:
                        continue
                    if not slots[li].acquire(blocking=False):
                        continue
                    req = q[0]
                    fits = getattr(eng, "fits", None)
                    with lock:
                        alone = inflight[0] == 0
                    if fits is not None and not alone and not fits(req, self.headroom[li]):
                        slots[li].release()  # HBM short for this head: try the next lane
                        continue
                    t_create = time.perf_counter()
                    try:
                        hd = eng.create(req)
                    except BaseException as e:  # surfaced to the caller
                        slots[li].release()
                        fail(e)
                        return
                    if hd is None:  # HBM short for this head: try the next lane
                        slots[li].release()
                        with lock:
                            alone = inflight[0] == 0
                        if alone:  # nothing running will free memory: the request can never fit
                            fail(_abi.NoMemoryError(-3, f"request {req.rid} does not fit in free HBM"))
                            return
                        continue
                    created[req.rid] = time.perf_counter() - t_create
                    q.popleft()
                    with lock:
                        inflight[0] += 1
                    item = (req, hd, now())
                    if req.kind == WBP:
                        wbp_q[li].put(item)
                    else:
                        inbox[li].put(item)
                    admitted = True
                    break  # start again from the most urgent lane
                if not admitted:
                    freed.clear()
                    freed.wait(0.02)  # wait for a completion (or a new arrival)

        def wbp_worker(li: int):
            while not stop.is_set():
                try:
                    req, hd, adm = wbp_q[li].get(timeout=0.01)
                except queue.Empty:
                    continue
                try:
                    eng.run_wbp(hd, req)
                    vol = eng.read_volume(hd, req) if req.keep_volume else None
                    finish(Result(req.rid, req.kind, req.arrival * time_scale, adm, now(), req.updates(), [], vol,
                                  req.W, -1), hd, req)
                except BaseException as e:
                    fail(e)
                    return

        def lane_worker(li: int):
            active = []          # [req, handle, admitted, iterations done, errors]
            dirty = False
            try:
                while not stop.is_set():
                    while True:
                        try:
                            req, hd, adm = inbox[li].get_nowait() if active else inbox[li].get(timeout=0.01)
                        except queue.Empty:
                            break
                        active.append([req, hd, adm, 0, []])
                        dirty = True
                    if not active:
                        continue
                    if dirty:
                        eng.set_members([a[1] for a in active], lane=li)
                        dirty = False
                    t_it = now()
                    err = eng.iterate([a[1] for a in active], [a[0] for a in active], [a[3] for a in active],
                                      lane=li)
                    self.lane_log.append((li, t_it, now(), len(active),
                                          sum(a[0].updates_per_iteration() for a in active)))
                    done = []
                    for a, e in zip(active, err):
                        a[3] += 1
                        a[4].append(list(e))
                        if a[3] >= a[0].n_iter:
                            done.append(a)
                    if done:
                        vols = {id(a): (eng.read_volume(a[1], a[0]) if a[0].keep_volume else None) for a in done}
                        t_done = now()
                        for a in done:
                            active.remove(a)
                        # the batch must forget the finished handles before they are destroyed
                        eng.set_members([a[1] for a in active], lane=li)
                        dirty = False
                        for a in done:
                            req = a[0]
                            finish(Result(req.rid, req.kind, req.arrival * time_scale, a[2], t_done, req.updates(),
                                          a[4], vols[id(a)], req.W, li), a[1], req)
            except BaseException as e:
                fail(e)

        threads = [threading.Thread(target=admitter, daemon=True)]
        for i in range(n_lanes):
            threads += [threading.Thread(target=wbp_worker, args=(i,), daemon=True),
                        threading.Thread(target=lane_worker, args=(i,), daemon=True)]
        for th in threads:
            th.start()
        try:
            while not all_done.is_set():
                t = now()
                while pending and pending[0][0] <= t:
                    r = heapq.heappop(pending)[2]
                    arrived[lane_of(r, self.bounds)].put(r)
                wait = (pending[0][0] - now()) if pending else 0.05
                all_done.wait(min(max(wait, 0.0005), 0.05))
            if errors:
                raise errors[0]
        finally:
            stop.set()
            for th in threads:
                th.join(timeout=30)
        return [results[r.rid] for r in requests]


def lane_summary(lane_log: list, span: float) -> dict:
    """Per lane: iterations, fraction of the span with an iteration in flight, mean members,
    mean seconds per iteration and voxel-updates/s while iterating."""
    out = {}
    for li in sorted({x[0] for x in lane_log}):
        xs = [x for x in lane_log if x[0] == li]
        busy = sum(x[2] - x[1] for x in xs)
        out[str(li)] = {"iterations": len(xs), "busy_fraction": busy / span if span > 0 else 0.0,
                        "mean_members": float(np.mean([x[3] for x in xs])),
                        "mean_iteration_s": busy / len(xs),
                        "voxel_updates_per_s_while_busy": sum(x[4] for x in xs) / busy if busy > 0 else 0.0}
    return out


def _pcts(res: list) -> dict:
    """Latency percentiles of results, with the median wait for admission (admitted -
    arrival) and median time from admission to completion."""
    lat = np.array([r.latency for r in res], np.float64)
    wait = np.array([r.admitted - r.arrival for r in res], np.float64)
    serv = np.array([r.completed - r.admitted for r in res], np.float64)
    return {"n": int(lat.size), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "wait_p50_s": float(np.percentile(wait, 50)),
            "service_p50_s": float(np.percentile(serv, 50)),
            "create_p50_s": float(np.percentile([r.create_s for r in res], 50))}


def summarize(results: list[Result], wall_s: float | None = None, requests: list[Request] | None = None) -> dict:
    """p50/p99 over all requests, per method and per size; aggregate voxel-updates/s over the
    makespan; with the requests, the offered load: updates offered per second of arrivals
    (total updates / arrival span) over the updates per second achieved."""
    lat = np.array([r.latency for r in results])
    t_first = min(r.arrival for r in results)
    t_last = max(r.completed for r in results)
    span = wall_s if wall_s is not None else (t_last - t_first)
    ups = sum(r.updates for r in results)
    out = {"requests": len(results), "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
           "mean_s": float(lat.mean()), "makespan_s": float(span), "voxel_updates_per_s": ups / span if span else 0.0,
           "kinds": {k: int(sum(1 for r in results if r.kind == k)) for k in KINDS}}
    out["per_kind"] = {k: _pcts([r for r in results if r.kind == k]) for k in KINDS if any(r.kind == k for r in results)}
    sizes = sorted({r.size for r in results if r.size})
    if sizes:
        out["per_size"] = {str(s): _pcts([r for r in results if r.size == s]) for s in sizes}
    if requests:
        arr = sorted(r.arrival for r in requests)
        arr_span = arr[-1] - arr[0] if len(arr) > 1 else 0.0
        if arr_span > 0 and out["voxel_updates_per_s"] > 0:
            offered = sum(r.updates() for r in requests) / arr_span
            out["offered_voxel_updates_per_s"] = offered
            out["offered_load"] = offered / out["voxel_updates_per_s"]
    return out


def synthetic_requests(n: int, seed: int, rate: float = 4.0, sizes=(512, 1024, 2048), thick=(128, 256, 512),
                       tilts=(41, 61, 121), mix=((WBP, 0.3), (SIRT, 0.4), (OSSART, 0.2), (TVM, 0.1)),
                       iters=(5, 50), keep_volume=False, precision=_abi.PREC_FP32,
                       with_series: bool = True) -> list[Request]:
    """Poisson arrivals (mean `rate` per second) of seeded synthetic tilt-series with the
    serving configuration's size, tilt-count and method distributions.  with_series=False
    leaves the projections empty (shape only), for simulation."""
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
                if with_series:
                    base += np.exp(-((xx - cx) ** 2 + (yy - cy) ** 2) / (2 * s * s)) * np.float32(D * 0.2)
            if with_series:
                cache[key] = np.stack([np.roll(base, int(round(N * 0.1 * np.sin(np.deg2rad(a)))), axis=1)
                                       for a in angles]).astype(np.float32)
            else:
                cache[key] = np.lib.stride_tricks.as_strided(np.zeros(1, np.float32), (nt, N, N), (0, 0, 0))
        n_iter = 1 if kind == WBP else int(g.integers(iters[0], iters[1] + 1))
        update = 0 if kind in (SIRT, TVM, WBP) else -(-nt // 10)  # "10 subsets": subset size ceil(N / 10)
        out.append(Request(rid, t, kind, cache[key], angles, N, N, D, n_iter, update, 1.0, int(g.integers(0, 1 << 30)),
                           keep_volume=keep_volume, precision=precision))
    return out


# ---------------------------------------------------------------------------------------
# Virtual-time replay of the policy above
# ---------------------------------------------------------------------------------------

@dataclass
class CostModel:
    """Seconds of GPU time per unit of work, from measured runs: one voxel-update of a SIRT,
    OS-SART or WBP pass, one voxel of a TV-denoise step (a TVM iteration is a SIRT iteration
    plus one denoise), plus a fixed cost per batched iteration and per WBP request (launch
    and host work).  Upload: host-to-device bytes per second of the series."""
    s_per_update: dict
    tv_s_per_voxel: float
    iteration_overhead_s: float = 2e-4
    wbp_overhead_s: float = 2e-3
    h2d_bytes_per_s: float = 2.0e10

    def iteration_s(self, req: Request) -> float:
        kind = SIRT if req.kind == TVM else req.kind
        t = req.updates_per_iteration() * self.s_per_update[kind]
        if req.kind == TVM:
            t += req.W * req.H * req.D * self.tv_s_per_voxel
        return t

    def wbp_s(self, req: Request) -> float:
        return req.updates_per_iteration() * self.s_per_update[WBP] + self.wbp_overhead_s

    def upload_s(self, req: Request) -> float:
        return req.series.shape[0] * req.series.shape[1] * req.series.shape[2] * 4 / self.h2d_bytes_per_s


def request_bytes(req: Request) -> int:
    """Device bytes of a request's handle, as the engine allocates them (volume in its storage
    type, the series, three projection-sized work buffers, the per-tilt tables; a TVM
    request adds its TV scratch: six FP32 volumes of dual variables, and an FP32 copy of a
    16-bit volume)."""
    N, h, w = req.series.shape
    nvox = req.W * req.H * req.D
    red = req.precision != _abi.PREC_FP32
    vol = nvox * (2 if red else 4)
    tv = nvox * 4 * (7 if red else 6) if req.kind == TVM else 0
    return vol + tv + 4 * N * h * w * 4 + 64 * N * w


def simulate(requests: list[Request], cost: CostModel, max_active: int = 64, lane_bounds=DEFAULT_LANE_BOUNDS,
             hbm_bytes: float = 2.6e11, headroom=None) -> list[Result]:
    """Replays the server's policy in virtual time: admission by slots and HBM from one FIFO
    per lane, most urgent lane first, each lane leaving its headroom of HBM free for more
    urgent ones (a request joins its work when its upload ends), lanes that iterate independently with strict
    priority on the GPU (smallest lane first; WBP requests above all lanes, one at a time), a
    member joining or leaving between two of its lane's iterations.  The GPU is shared as a
    fluid: the most urgent runnable job gets all of it."""
    bounds = tuple(lane_bounds)
    n_lanes = len(bounds) + 1
    room = tuple(headroom) if headroom is not None else tuple(
        0.0 if i == 0 else 0.05 if i == 1 else 0.15 for i in range(n_lanes))
    reqs = sorted(requests, key=lambda r: (r.arrival, r.rid))
    t = 0.0
    i_arr = 0
    waiting = [deque() for _ in range(n_lanes)]  # arrived, not admitted (FIFO per lane)
    used = 0.0
    n_active = [0] * n_lanes  # per lane, WBP requests in their size's lane
    joining = [[] for _ in range(n_lanes)]  # (ready time, req, admitted)
    members = [[] for _ in range(n_lanes)]  # [req, admitted, iterations done]
    work = [0.0] * n_lanes                  # GPU seconds left of the lane's current iteration
    running = [False] * n_lanes
    wbp_q: list = []                        # (ready time, req, admitted)
    wbp_cur = None                          # [req, admitted, seconds left]
    results: dict[int, Result] = {}
    INF = float("inf")

    def admit():
        nonlocal used
        progress = True
        while progress:
            progress = False
            for li, q in enumerate(waiting):  # most urgent lane first; a head short of HBM lets the next lane try
                if not q or n_active[li] >= max_active:
                    continue
                r = q[0]
                need = request_bytes(r)
                if need > hbm_bytes:
                    raise _abi.NoMemoryError(-3, f"request {r.rid} does not fit in HBM")
                if used + need + room[li] * hbm_bytes > hbm_bytes and used > 0:
                    continue
                q.popleft()
                used += need
                n_active[li] += 1
                ready = t + cost.upload_s(r)
                if r.kind == WBP:
                    wbp_q.append((ready, r, t))
                else:
                    joining[lane_of(r, bounds)].append((ready, r, t))
                progress = True
                break

    def release(r: Request):
        nonlocal used
        used -= request_bytes(r)
        n_active[lane_of(r, bounds)] -= 1

    def start_iterations():
        for li in range(n_lanes):
            if running[li]:
                continue
            stay = []
            for item in joining[li]:
                if item[0] <= t:
                    members[li].append([item[1], item[2], 0])
                else:
                    stay.append(item)
            joining[li] = stay
            if members[li]:
                running[li] = True
                work[li] = sum(cost.iteration_s(m[0]) for m in members[li]) + cost.iteration_overhead_s

    while len(results) < len(reqs):
        while i_arr < len(reqs) and reqs[i_arr].arrival <= t:
            waiting[lane_of(reqs[i_arr], bounds)].append(reqs[i_arr])
            i_arr += 1
        admit()
        if wbp_cur is None:
            ready = [x for x in wbp_q if x[0] <= t]
            if ready:
                x = ready[0]
                wbp_q.remove(x)
                wbp_cur = [x[1], x[2], cost.wbp_s(x[1])]
        start_iterations()
        # the most urgent runnable job holds the GPU
        job = "wbp" if wbp_cur is not None else next((li for li in range(n_lanes) if running[li]), None)
        t_next = reqs[i_arr].arrival if i_arr < len(reqs) else INF
        for x in wbp_q:
            if x[0] > t:
                t_next = min(t_next, x[0])
        for li in range(n_lanes):
            for x in joining[li]:
                if x[0] > t and not running[li]:
                    t_next = min(t_next, x[0])
        if job is None:
            if t_next == INF:
                raise RuntimeError("simulation stalled")
            t = t_next
            continue
        left = wbp_cur[2] if job == "wbp" else work[job]
        dt = min(left, t_next - t)
        t += dt
        if job == "wbp":
            wbp_cur[2] -= dt
            if wbp_cur[2] <= 1e-12:
                r = wbp_cur[0]
                results[r.rid] = Result(r.rid, r.kind, r.arrival, wbp_cur[1], t, r.updates(), [], None, r.W, -1)
                release(r)
                wbp_cur = None
        else:
            work[job] -= dt
            if work[job] <= 1e-12:
                running[job] = False
                keep = []
                for m in members[job]:
                    m[2] += 1
                    if m[2] >= m[0].n_iter:
                        r = m[0]
                        results[r.rid] = Result(r.rid, r.kind, r.arrival, m[1], t, r.updates(), [], None, r.W, job)
                        release(r)
                    else:
                        keep.append(m)
                members[job] = keep
    return [results[r.rid] for r in requests]

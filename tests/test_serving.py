"""Serving loop scheduling on CPU with a fake engine: continuous batching (requests join
and leave between iterations), slot limits, admission by free memory (an allocation
failure makes a request wait for a completion), lanes by iteration size that iterate
independently, WBP requests beside the lanes, latency and offered-load accounting,
failure reporting for a request that can never fit, and the virtual-time replay of the
same policy."""
from __future__ import annotations

import threading
import time

import numpy as np
import pytest

from tomoj_gb300 import _abi
from tomoj_gb300.serving import (OSSART, SIRT, TVM, WBP, CostModel, Request, Server, lane_of, request_bytes, simulate,
                                 summarize, synthetic_requests)


class FakeEngine:
    """Iterations sleep tick_s per member plus cost_s per 1e6 voxel-updates of the lane."""

    def __init__(self, budget, tick_s=0.002, lanes=1, cost_s=0.0):
        self.budget = budget
        self.used = 0
        self.tick_s = tick_s
        self.cost_s = cost_s
        self.n_lanes = lanes
        self.members = {i: [] for i in range(lanes)}
        self.max_members = 0
        self.live = 0
        self.iterations = {}
        self.lock = threading.Lock()
        self.created = 0
        self.refused = 0
        self.wbp_during_iteration = 0
        self.iterating = 0

    def create(self, req):
        need = req.W * req.H * req.D
        with self.lock:
            if self.used + need > self.budget:
                self.refused += 1
                return None
            self.used += need
            self.created += 1
        return ("h", req.rid, need)

    def run_wbp(self, hd, req):
        with self.lock:
            self.wbp_during_iteration += self.iterating > 0
        time.sleep(self.tick_s)
        self.iterations[req.rid] = 1

    def set_members(self, handles, lane=0):
        with self.lock:
            self.members[lane] = list(handles)
            self.max_members = max(self.max_members, sum(len(m) for m in self.members.values()))

    def iterate(self, handles, reqs, iteration, lane=0):
        assert list(handles) == self.members[lane]
        for r, it in zip(reqs, iteration):
            assert self.iterations.get(r.rid, 0) == it
            self.iterations[r.rid] = it + 1
        with self.lock:
            self.iterating += 1
        time.sleep(self.tick_s + self.cost_s * sum(r.updates_per_iteration() for r in reqs) / 1e6)
        with self.lock:
            self.iterating -= 1
        return np.zeros((len(handles), 5))

    def read_volume(self, hd, req):
        return np.full((req.D, req.H, req.W), float(req.rid), np.float32)

    def destroy(self, hd):
        with self.lock:
            self.used -= hd[2]


def req(rid, arrival, kind, n_iter, size=4, tilts=3):
    series = np.zeros((tilts, size, size), np.float32)
    return Request(rid, arrival, kind, series, np.linspace(-10.0, 10.0, tilts), size, size, size, n_iter,
                   0 if kind != OSSART else 1, keep_volume=True)


def test_requests_join_and_leave_between_iterations():
    reqs = [req(0, 0.0, SIRT, 5), req(1, 0.005, OSSART, 3), req(2, 0.01, WBP, 1), req(3, 0.02, TVM, 4)]
    eng = FakeEngine(budget=10 ** 9)
    res = Server(eng, max_active=8).run(reqs)
    assert [r.rid for r in res] == [0, 1, 2, 3]
    for r, q in zip(res, reqs):
        assert r.completed >= r.admitted >= r.arrival
        assert eng.iterations[q.rid] == q.n_iter
        assert np.all(r.volume == q.rid)
        assert len(r.errors) == (0 if q.kind == WBP else q.n_iter)
    assert eng.max_members >= 2  # the SIRT and OS-SART requests overlapped
    assert eng.used == 0
    s = summarize(res, requests=reqs)
    assert s["requests"] == 4 and s["p99_s"] >= s["p50_s"] > 0
    assert set(s["per_kind"]) == {SIRT, OSSART, WBP, TVM} and s["per_kind"][SIRT]["n"] == 1
    assert s["offered_load"] > 0


def test_admission_waits_for_memory_and_respects_slots():
    reqs = [req(i, 0.0, SIRT, 3) for i in range(6)]
    per = 4 ** 3
    eng = FakeEngine(budget=2 * per)  # room for two at a time
    res = Server(eng, max_active=8).run(reqs)
    assert len(res) == 6 and eng.refused > 0 and eng.max_members <= 2 and eng.used == 0
    eng2 = FakeEngine(budget=10 ** 9)
    Server(eng2, max_active=3).run([req(i, 0.0, SIRT, 2) for i in range(7)])
    assert eng2.max_members <= 3


def test_request_that_never_fits_is_reported():
    eng = FakeEngine(budget=10)
    with pytest.raises(_abi.NoMemoryError):
        Server(eng).run([req(0, 0.0, SIRT, 2)])


def test_lanes_iterate_independently():
    """A small request that arrives after a large one has started runs in its own lane and
    finishes first; a WBP request runs while a lane iterates."""
    big = req(0, 0.0, SIRT, 6, size=40, tilts=21)          # 1.3e6 updates per iteration
    small = req(1, 0.03, SIRT, 3, size=8, tilts=5)          # 2.6e3
    wbp = req(2, 0.04, WBP, 1, size=8, tilts=5)
    assert lane_of(big, (1e5,)) == 1 and lane_of(small, (1e5,)) == 0
    eng = FakeEngine(budget=10 ** 9, lanes=2, cost_s=0.05)  # ~65 ms per iteration of the large request
    res = Server(eng, max_active=8, lane_bounds=(1e5,)).run([big, small, wbp])
    rb, rs, rw = res
    assert (rb.lane, rs.lane, rw.lane) == (1, 0, -1)
    assert rs.completed < rb.completed and rw.completed < rb.completed
    assert rs.latency < 0.2 < rb.latency
    assert eng.wbp_during_iteration >= 1
    for q in (big, small):
        assert eng.iterations[q.rid] == q.n_iter


def test_lane_bounds_must_cover_the_lanes():
    with pytest.raises(ValueError):
        Server(FakeEngine(budget=1, lanes=3), lane_bounds=(1e6,))


def _cost():
    return CostModel({SIRT: 1e-12, OSSART: 1.2e-12, WBP: 0.5e-12}, tv_s_per_voxel=7e-11, iteration_overhead_s=1e-4,
                     wbp_overhead_s=1e-3, h2d_bytes_per_s=2e10)


def test_simulation_of_one_request_is_its_work():
    cost = _cost()
    r = synthetic_requests(1, seed=3, with_series=False)[0]
    r.kind, r.n_iter, r.arrival = SIRT, 7, 0.5
    res = simulate([r], cost)[0]
    expect = cost.upload_s(r) + 7 * (cost.iteration_s(r) + cost.iteration_overhead_s)
    assert res.latency == pytest.approx(expect, rel=1e-9)
    r.kind = TVM
    assert cost.iteration_s(r) == pytest.approx(r.updates_per_iteration() * 1e-12 + r.W * r.H * r.D * 7e-11)


def test_simulation_priority_and_admission():
    cost = _cost()
    reqs = synthetic_requests(200, seed=11, rate=4.0, with_series=False)
    res = simulate(reqs, cost, max_active=64)
    assert [x.rid for x in res] == [r.rid for r in reqs]
    for x, r in zip(res, reqs):
        assert x.completed >= x.admitted >= x.arrival
        assert x.latency >= (cost.wbp_s(r) if r.kind == WBP else r.n_iter * cost.iteration_s(r)) - 1e-9
    s = summarize(res, requests=reqs)
    assert s["requests"] == 200 and s["offered_load"] > 0
    # the smallest lane's requests wait less than the largest lane's
    lat = {0: [], 2: []}
    for x in res:
        if x.lane in lat:
            lat[x.lane].append(x.latency)
    assert np.median(lat[0]) < np.median(lat[2])
    # an HBM budget that holds one large request at a time serialises them, and still finishes
    import dataclasses
    big0 = next(r for r in reqs if r.W == 2048)
    big = [dataclasses.replace(big0, rid=k, arrival=0.0) for k in range(4)]
    one = simulate(big, cost, hbm_bytes=1.5 * request_bytes(big0))
    ends = sorted(x.completed for x in one)
    starts = sorted(x.admitted for x in one)
    assert all(starts[i + 1] >= ends[i] - 1e-9 for i in range(3))
    with pytest.raises(_abi.NoMemoryError):
        simulate(big[:1], cost, hbm_bytes=10.0)


def test_small_request_is_not_held_behind_a_large_one_waiting_for_memory():
    big0 = req(0, 0.0, SIRT, 4, size=40, tilts=21)
    big1 = req(1, 0.001, SIRT, 4, size=40, tilts=21)       # waits: HBM holds one large request
    small = req(2, 0.01, SIRT, 2, size=8, tilts=5)
    eng = FakeEngine(budget=40 ** 3 + 8 ** 3, lanes=2, cost_s=0.05)
    res = Server(eng, max_active=8, lane_bounds=(1e5,)).run([big0, big1, small])
    r0, r1, r2 = res
    assert r1.admitted >= r0.completed - 1e-3     # the second large request waited for the first
    assert r2.admitted < r0.completed and r2.completed < r0.completed
    assert eng.refused > 0 and eng.used == 0


def test_lane_summary_and_per_class_statistics():
    from tomoj_gb300.serving import Result, lane_summary
    log = [(0, 0.0, 0.5, 2, 1e9), (0, 1.0, 1.5, 1, 5e8), (1, 0.0, 2.0, 3, 4e9)]
    s = lane_summary(log, span=4.0)
    assert s["0"]["iterations"] == 2 and s["0"]["busy_fraction"] == pytest.approx(0.25)
    assert s["0"]["voxel_updates_per_s_while_busy"] == pytest.approx(1.5e9)
    assert s["1"]["mean_members"] == 3 and s["1"]["mean_iteration_s"] == pytest.approx(2.0)
    res = [Result(0, SIRT, 0.0, 1.0, 3.0, 10, size=512, lane=0, create_s=0.2),
           Result(1, WBP, 0.5, 0.5, 0.7, 5, size=512, lane=-1, create_s=0.1),
           Result(2, SIRT, 1.0, 4.0, 9.0, 40, size=2048, lane=2, create_s=0.5)]
    out = summarize(res)
    assert out["per_size"]["512"]["n"] == 2 and out["per_size"]["2048"]["wait_p50_s"] == pytest.approx(3.0)
    assert out["per_kind"][SIRT]["service_p50_s"] == pytest.approx(3.5)
    assert out["per_size"]["512"]["create_p50_s"] == pytest.approx(0.15)
    assert out["voxel_updates_per_s"] == pytest.approx(55 / 9.0)

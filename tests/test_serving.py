"""Serving loop scheduling on CPU with a fake engine: continuous batching (requests join
and leave between iterations), slot limits, admission by free memory (an allocation
failure makes a request wait for a completion), latency accounting, and failure
reporting for a request that can never fit."""
from __future__ import annotations

import threading
import time

import numpy as np
import pytest

from tomoj_gb300 import _abi
from tomoj_gb300.serving import OSSART, SIRT, TVM, WBP, Request, Server, summarize


class FakeEngine:
    def __init__(self, budget, tick_s=0.002):
        self.budget = budget
        self.used = 0
        self.tick_s = tick_s
        self.members = []
        self.max_members = 0
        self.iterations = {}
        self.lock = threading.Lock()
        self.created = 0
        self.refused = 0

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
        self.iterations[req.rid] = 1

    def set_members(self, handles):
        self.members = list(handles)
        self.max_members = max(self.max_members, len(handles))

    def iterate(self, handles, reqs, iteration):
        assert list(handles) == self.members
        for r, it in zip(reqs, iteration):
            assert self.iterations.get(r.rid, 0) == it
            self.iterations[r.rid] = it + 1
        time.sleep(self.tick_s)
        return np.zeros((len(handles), 5))

    def read_volume(self, hd, req):
        return np.full((req.D, req.H, req.W), float(req.rid), np.float32)

    def destroy(self, hd):
        with self.lock:
            self.used -= hd[2]


def req(rid, arrival, kind, n_iter, size=4):
    series = np.zeros((3, size, size), np.float32)
    return Request(rid, arrival, kind, series, np.array([-10.0, 0.0, 10.0]), size, size, size, n_iter,
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
    s = summarize(res)
    assert s["requests"] == 4 and s["p99_s"] >= s["p50_s"] > 0


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

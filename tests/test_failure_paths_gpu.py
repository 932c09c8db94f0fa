"""Failure handling of the real engine, without faulting, trapping or hanging the GPU.

* Cancellation (TomoReconstruction2.interrupt, polled by the iteration loop,
  TomoReconstruction2.java:137-140, 587-598): tomo_cancel from another host thread
  ends tomo_run_ossart between iterations with TOMO_ERR_CANCELLED; the handle
  keeps working.
* Admission control (the reference reports an out-of-memory reconstruction,
  ReconstructionThreadManager.java:186-192): a library-wide memory limit below a
  request's size makes tomo_create answer TOMO_ERR_NOMEM; the serving loop defers
  such a request and admits it once a running request has finished.
* Bounded waits: with the forward projector's first plane copies held back
  (tomo_debug_hold_first_copy) every CTA's first mbarrier wait runs out, the
  kernel records the timeout in the device status word and returns with nothing
  in flight; the call reports TOMO_ERR_DEVICE and the same handle then projects
  correctly.
"""
from __future__ import annotations

import ctypes as C
import threading
import time

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import rel_l2, series_case
from tomoj_gb300 import _abi
from tomoj_gb300.serving import SIRT, EngineAdapter, Request, Server

pytestmark = pytest.mark.gpu


def _create(lib, c):
    g = _abi.make_geom(c["W"], c["H"], c["D"], c["w"], c["h"], c["n"])
    p = _abi.make_params(fill=_abi.FILL_NAN)
    h = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(g), C.byref(p), C.byref(h)))
    eul = np.ascontiguousarray(c["eul"], np.float64)
    series = np.ascontiguousarray(c["series"], np.float32)
    _abi.check(lib.tomo_load_series(h, series.ctypes.data, 0, _abi.ptr(eul, C.c_double), None, None))
    return h


@pytest.fixture(scope="module")
def case():
    return series_case(W=64, H=8, D=48, n=15, seed=31)


def test_cancel_set_before_the_run_stops_at_the_first_iteration(engine, case):
    h = _create(engine, case)
    try:
        _abi.check(engine.tomo_cancel(h))
        rc = engine.tomo_run_ossart(h, 5, 1.0, 0, 1, 0, case["H"], 1, None)
        assert rc == _abi.ERR_CANCELLED, rc
        # the request was consumed: the next run completes
        _abi.check(engine.tomo_run_ossart(h, 1, 1.0, 0, 1, 0, case["H"], 1, None))
    finally:
        engine.tomo_destroy(h)


def test_cancel_from_another_thread_ends_a_long_run(engine, case):
    h = _create(engine, case)
    try:
        n_iter = 20000
        errs = np.zeros((n_iter, 5))
        out = {}

        def run():
            t0 = time.perf_counter()
            out["rc"] = engine.tomo_run_ossart(h, n_iter, 1.0, 0, 1, 0, case["H"], 1, _abi.ptr(errs, C.c_double))
            out["s"] = time.perf_counter() - t0

        th = threading.Thread(target=run)
        th.start()
        time.sleep(0.3)
        _abi.check(engine.tomo_cancel(h))
        th.join(timeout=120)
        assert not th.is_alive()
        assert out["rc"] == _abi.ERR_CANCELLED, out
        done = int(np.count_nonzero(errs[:, 0]))
        assert 0 < done < n_iter, done  # stopped between iterations, after some had run
        # the volume is that of the completed iterations and the handle keeps working
        _abi.check(engine.tomo_run_ossart(h, 1, 1.0, 0, 1, 0, case["H"], 1, None))
    finally:
        engine.tomo_destroy(h)


def _footprint(lib, c):
    """Device bytes one handle of the case holds after a batched iteration."""
    before = lib.tomo_memory_in_use()
    h = _create(lib, c)
    try:
        b = C.c_void_p()
        _abi.check(lib.tomo_batch_create(C.byref(b)))
        try:
            arr = (C.c_void_p * 1)(h.value)
            _abi.check(lib.tomo_batch_set(b, arr, 1))
            rel, upd, first = np.ones(1), np.zeros(1, np.int32), np.zeros(1, np.int32)
            _abi.check(lib.tomo_batch_iteration(b, _abi.ptr(rel, C.c_double), _abi.ptr(upd, C.c_int32),
                                                _abi.ptr(first, C.c_int32), 1, None))
            _abi.check(lib.tomo_batch_set(b, arr, 0))
        finally:
            lib.tomo_batch_destroy(b)
        return lib.tomo_memory_in_use() - before
    finally:
        lib.tomo_destroy(h)


def test_memory_limit_refuses_a_handle(engine, case):
    need = _footprint(engine, case)
    base = engine.tomo_memory_in_use()
    try:
        _abi.check(engine.tomo_set_memory_limit(base + need // 2))
        g = _abi.make_geom(case["W"], case["H"], case["D"], case["w"], case["h"], case["n"])
        p = _abi.make_params()
        h = C.c_void_p()
        rc = engine.tomo_create(C.byref(g), C.byref(p), C.byref(h))
        assert rc == _abi.ERR_NOMEM, rc
        assert b"memory limit" in engine.tomo_last_error()
        assert engine.tomo_memory_in_use() == base  # the partial allocation was released
    finally:
        _abi.check(engine.tomo_set_memory_limit(0))
    h = _create(engine, case)
    engine.tomo_destroy(h)


def test_serving_defers_a_request_until_memory_frees(engine, case):
    """Two identical requests under a limit that holds one: the second is admitted only
    after the first has completed, and both results equal a run alone."""
    need = _footprint(engine, case)
    n_iter = 4
    angles = case["angles"]
    reqs = [Request(k, 0.0, SIRT, np.ascontiguousarray(case["series"], np.float32), angles, case["W"], case["H"],
                    case["D"], n_iter, 0, 1.0, 17 + k, keep_volume=True) for k in range(2)]
    eng = EngineAdapter(lanes=1)
    base = engine.tomo_memory_in_use()
    try:
        _abi.check(engine.tomo_set_memory_limit(base + need + need // 2))
        res = Server(eng, max_active=4).run(reqs)
    finally:
        _abi.check(engine.tomo_set_memory_limit(0))
        eng.close()
    first, second = sorted(res, key=lambda r: r.admitted)
    assert second.admitted >= first.completed - 1e-3, (first, second)
    for r, q in zip(res, reqs):
        h = _create(engine, case)
        try:
            _abi.check(engine.tomo_run_ossart(h, n_iter, 1.0, 0, q.seed, 0, case["H"], 1, None))
            alone = np.empty((case["D"], case["H"], case["W"]), np.float32)
            _abi.check(engine.tomo_get_volume(h, alone.ctypes.data, 0, 0, case["H"]))
        finally:
            engine.tomo_destroy(h)
        assert np.array_equal(r.volume, alone), q.rid


def test_expired_wait_reports_device_error_and_handle_recovers(engine, oracle_lib, case):
    c = case
    assert (c["W"] * 4) % 16 == 0  # rows staged with bulk copies: the hook applies
    vol = np.ascontiguousarray(c["vol"])
    h = _create(engine, c)
    try:
        _abi.check(engine.tomo_set_volume(h, vol.ctypes.data, 0, 0, c["H"]))
        for i in range(c["n"]):
            _abi.check(engine.tomo_add_projection(h, i))
        _abi.check(engine.tomo_debug_hold_first_copy(h, 1))
        rc = engine.tomo_project(h, 0, c["H"])
        assert rc == _abi.ERR_DEVICE, rc
        assert b"bounded wait" in engine.tomo_last_error()
        # the graph-captured driver reports it too
        rc = engine.tomo_run_ossart(h, 2, 1.0, 0, 1, 0, c["H"], 1, None)
        assert rc == _abi.ERR_DEVICE, rc
        _abi.check(engine.tomo_debug_hold_first_copy(h, 0))
        # same handle, status cleared: a correct projection
        _abi.check(engine.tomo_set_volume(h, vol.ctypes.data, 0, 0, c["H"]))
        _abi.check(engine.tomo_clear_projections(h))
        for i in range(c["n"]):
            _abi.check(engine.tomo_add_projection(h, i))
        _abi.check(engine.tomo_project(h, 0, c["H"]))
        for i in range(c["n"]):
            got = np.empty((c["h"], c["w"]), np.float32)
            _abi.check(engine.tomo_get_projection(h, i, _abi.ptr(got)))
            ref, _ = O.project(vol, c["g"], c["eul"][i])
            assert rel_l2(got, ref) <= 1e-5, i
    finally:
        engine.tomo_destroy(h)

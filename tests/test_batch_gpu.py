"""Batched iterations of heterogeneous tilt-series equal the same handles run one by one
(same kernels, same orderings: bitwise), including mixed SIRT / OS-SART update sizes,
positivity and TVM members, with and without the captured graph."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from tests.cases import series_case
from tests.test_parity_gpu import Handle
from tomoj_gb300 import _abi

pytestmark = pytest.mark.gpu

SPECS = [
    dict(W=64, H=10, D=40, n=15, seed=1, misalign=True),
    dict(W=96, H=6, D=24, n=21, seed=2),
    dict(W=48, H=8, D=64, n=9, seed=3, amax=50.0),
]


@pytest.mark.parametrize("use_graph", [0, 1])
def test_batch_iterations_equal_individual_runs(engine, use_graph):
    cases = [series_case(**s) for s in SPECS]
    updates = [0, 4, 3]
    relax = [1.0, 0.8, 1.0]
    seeds = [11, 12, 13]
    n_iter = 3
    opts = [dict(), dict(positivity=True), dict()]
    # one by one
    ref_vol, ref_err = [], []
    for c, u, r, sd, o in zip(cases, updates, relax, seeds, opts):
        hd = Handle(engine, c, **o)
        try:
            if c is cases[2]:
                _abi.check(engine.tomo_set_tvm(hd.h, 25.0, 1.0, 0.01, 3))
            err = np.zeros((n_iter, 5))
            _abi.check(engine.tomo_run_ossart(hd.h, n_iter, r, u, sd, 0, c["H"], 1, _abi.ptr(err, C.c_double)))
            ref_vol.append(hd.volume())
            ref_err.append(err)
        finally:
            hd.close()
    # batched
    hds = [Handle(engine, c, **o) for c, o in zip(cases, opts)]
    b = C.c_void_p()
    _abi.check(engine.tomo_batch_create(C.byref(b)))
    try:
        _abi.check(engine.tomo_set_tvm(hds[2].h, 25.0, 1.0, 0.01, 3))
        arr = (C.c_void_p * len(hds))(*[h.h.value for h in hds])
        _abi.check(engine.tomo_batch_set(b, arr, len(hds)))
        rel = np.array(relax)
        upd = np.array(updates, np.int32)
        errs = []
        for it in range(n_iter):
            first = np.array([engine.tomo_first_index(sd, it, c["n"]) for sd, c in zip(seeds, cases)], np.int32)
            e = np.zeros((len(hds), 5))
            _abi.check(engine.tomo_batch_iteration(b, _abi.ptr(rel, C.c_double), _abi.ptr(upd, C.c_int32),
                                                   _abi.ptr(first, C.c_int32), use_graph, _abi.ptr(e, C.c_double)))
            errs.append(e)
        for m, hd in enumerate(hds):
            assert np.array_equal(hd.volume(), ref_vol[m]), m
            got = np.array([errs[it][m] for it in range(n_iter)])
            assert np.allclose(got, ref_err[m], rtol=1e-12), m
    finally:
        engine.tomo_batch_destroy(b)
        for hd in hds:
            hd.close()


PERSIST_SPECS = [  # widths on both CTA sizes (256 threads: QP 1, 2; 512 threads: QP 2, 4), FP32 and FP16
    (dict(W=200, H=5, D=24, n=11, seed=21), _abi.PREC_FP16, 4),
    (dict(W=300, H=4, D=20, n=9, seed=22), _abi.PREC_FP32, 0),
    (dict(W=700, H=4, D=16, n=7, seed=23), _abi.PREC_FP16, 3),
    (dict(W=1100, H=3, D=12, n=5, seed=24), _abi.PREC_FP32, 0),
]


def _prec_handle(lib, c, prec):
    g = _abi.make_geom(c["W"], c["H"], c["D"], c["w"], c["h"], c["n"])
    p = _abi.make_params(precision=prec)
    h = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(g), C.byref(p), C.byref(h)))
    eul = np.ascontiguousarray(c["eul"], np.float64)
    series = np.ascontiguousarray(c["series"], np.float32)
    _abi.check(lib.tomo_load_series(h, series.ctypes.data, 0, _abi.ptr(eul, C.c_double), None, None))
    return h


@pytest.mark.parametrize("use_graph", [0, 1])
def test_persistent_launches_equal_per_variant_launches(engine, use_graph):
    """The persistent form (one forward launch per CTA size, one backprojection launch per
    storage type, items pulled from a list) computes bitwise what one launch per kernel
    variant with a CTA per item computes, with fewer launches per iteration."""
    cases = [(series_case(**s), prec, u) for s, prec, u in PERSIST_SPECS]
    n_iter, seeds = 2, [5, 6, 7, 8]
    vols, launches = {}, {}
    for persistent in (0, 1):
        hs = [_prec_handle(engine, c, prec) for c, prec, _ in cases]
        b = C.c_void_p()
        _abi.check(engine.tomo_batch_create(C.byref(b)))
        try:
            _abi.check(engine.tomo_batch_set_persistent(b, persistent))
            arr = (C.c_void_p * len(hs))(*[h.value for h in hs])
            _abi.check(engine.tomo_batch_set(b, arr, len(hs)))
            rel = np.ones(len(hs))
            upd = np.array([u for _, _, u in cases], np.int32)
            for it in range(n_iter):
                first = np.array([engine.tomo_first_index(sd, it, c["n"]) for sd, (c, _, _) in zip(seeds, cases)],
                                 np.int32)
                k0 = engine.tomo_kernel_launches()
                _abi.check(engine.tomo_batch_iteration(b, _abi.ptr(rel, C.c_double), _abi.ptr(upd, C.c_int32),
                                                       _abi.ptr(first, C.c_int32), use_graph, None))
                launches[persistent] = engine.tomo_kernel_launches() - k0
            vols[persistent] = []
            for h, (c, _, _) in zip(hs, cases):
                out = np.empty((c["D"], c["H"], c["W"]), np.float32)
                _abi.check(engine.tomo_get_volume(h, out.ctypes.data, 0, 0, c["H"]))
                vols[persistent].append(out)
        finally:
            engine.tomo_batch_destroy(b)
            for h in hs:
                engine.tomo_destroy(h)
    for m in range(len(cases)):
        assert np.array_equal(vols[0][m], vols[1][m]), m
        assert np.isfinite(vols[1][m]).all() and np.abs(vols[1][m]).max() > 0, m
    assert launches[1] < launches[0], launches


def test_batch_stream_and_priority_do_not_change_results(engine):
    """A batch on a caller's stream at a more urgent priority, and a handle whose own stream
    was recreated at a priority, compute bitwise what the defaults compute."""
    torch = pytest.importorskip("torch")
    c = series_case(W=64, H=6, D=24, n=11, seed=41)
    vols = []
    for variant in (0, 1):
        hs = [_prec_handle(engine, c, _abi.PREC_FP32) for _ in range(2)]
        b = C.c_void_p()
        _abi.check(engine.tomo_batch_create(C.byref(b)))
        side = torch.cuda.Stream()
        try:
            if variant:
                _abi.check(engine.tomo_batch_set_priority(b, 2))
                _abi.check(engine.tomo_batch_set_stream(b, C.c_void_p(side.cuda_stream)))
                _abi.check(engine.tomo_set_priority(hs[1], 1))
            arr = (C.c_void_p * 1)(hs[0].value)
            _abi.check(engine.tomo_batch_set(b, arr, 1))
            rel, upd = np.ones(1), np.zeros(1, np.int32)
            for it in range(2):
                first = np.array([engine.tomo_first_index(3, it, c["n"])], np.int32)
                _abi.check(engine.tomo_batch_iteration(b, _abi.ptr(rel, C.c_double), _abi.ptr(upd, C.c_int32),
                                                       _abi.ptr(first, C.c_int32), 1, None))
            _abi.check(engine.tomo_run_ossart(hs[1], 2, 1.0, 0, 3, 0, c["H"], 1, None))
            out = []
            for h in hs:
                v = np.empty((c["D"], c["H"], c["W"]), np.float32)
                _abi.check(engine.tomo_get_volume(h, v.ctypes.data, 0, 0, c["H"]))
                out.append(v)
            vols.append(out)
        finally:
            engine.tomo_batch_destroy(b)
            for h in hs:
                engine.tomo_destroy(h)
    assert np.array_equal(vols[0][0], vols[1][0]) and np.array_equal(vols[0][1], vols[1][1])

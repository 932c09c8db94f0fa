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

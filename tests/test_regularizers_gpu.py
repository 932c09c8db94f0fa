"""Regularised projectors on the GPU against the oracle: BayesianVoxelProjector3D
(distance volume seeded by the 27-point stencil, differences backprojected into it,
alpha times it added at the end of each iteration).  Tolerance as for OS-SART
iterations: <= 1e-4 relative L2 after two iterations."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import rel_l2, series_case
from tests.test_parity_gpu import Handle, oracle_aligned
from tomoj_gb300 import _abi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("update,positivity,use_graph", [(0, False, 1), (4, True, 0), (3, False, 1)])
def test_bayesian_iterations_match_oracle(engine, oracle_lib, update, positivity, use_graph):
    c = series_case(W=48, H=6, D=32, n=13, seed=41)
    lam, alpha, seed, n_iter = 0.05, 0.7, 9, 2
    hd = Handle(engine, c, positivity=positivity)
    try:
        # start from a non-trivial volume so that the stencil term matters
        start = (0.5 * c["vol"]).astype(np.float32)
        hd.set_volume(start)
        _abi.check(engine.tomo_set_bayesian(hd.h, lam, alpha, 1))
        err = np.zeros((n_iter, 5))
        _abi.check(engine.tomo_run_ossart(hd.h, n_iter, 1.0, update, seed, 0, c["H"], use_graph,
                                          _abi.ptr(err, C.c_double)))
        got = hd.volume()
        g = O.Geom(c["W"], c["H"], c["D"], c["w"], c["h"], positivity=positivity)
        ref = start.copy()
        meas = oracle_aligned(c)
        for it in range(n_iter):
            order = O.order_shuffle(c["eul"], int(engine.tomo_first_index(seed, it, c["n"])))
            e5 = O.bayesian_iteration(ref, g, c["eul"], meas, order, 1.0, update, lam, alpha)
            assert np.allclose(err[it, [0, 1, 3]], e5[[0, 1, 3]], rtol=1e-4)
        assert rel_l2(got, ref) <= 1e-4, rel_l2(got, ref)
    finally:
        hd.close()


def test_bayesian_needs_fp32_storage(engine):
    c = series_case(W=32, H=4, D=16, n=5, seed=3)
    g = _abi.make_geom(c["W"], c["H"], c["D"], c["w"], c["h"], c["n"])
    p = _abi.make_params(precision=_abi.PREC_FP16)
    h = C.c_void_p()
    _abi.check(engine.tomo_create(C.byref(g), C.byref(p), C.byref(h)))
    try:
        assert engine.tomo_set_bayesian(h, 0.1, 0.1, 1) == _abi.ERR_UNSUPPORTED
    finally:
        engine.tomo_destroy(h)


@pytest.mark.parametrize("dark_bg,do_median", [(1, 1), (0, 0)])
def test_bgart_iterations_match_oracle(engine, oracle_lib, dark_bg, do_median):
    c = series_case(W=40, H=6, D=28, n=11, seed=43)
    k, seed, n_iter, update = 1.5, 4, 2, 0
    hd = Handle(engine, c)
    try:
        start = (0.8 * c["vol"]).astype(np.float32)
        hd.set_volume(start)
        ref = start.copy()
        _abi.check(engine.tomo_set_bgart(hd.h, k, dark_bg, do_median, float("nan"), 1))
        O.bgart_collapse(ref, k, bool(dark_bg))  # the constructor's collapse
        assert np.array_equal(hd.volume(), ref)
        _abi.check(engine.tomo_run_ossart(hd.h, n_iter, 1.0, update, seed, 0, c["H"], 1, None))
        got = hd.volume()
        meas = oracle_aligned(c)
        for it in range(n_iter):
            if do_median:
                O.bgart_median_cross(ref)
            order = O.order_shuffle(c["eul"], int(engine.tomo_first_index(seed, it, c["n"])))
            O.ossart_iteration(ref, c["g"], c["eul"], meas, order, 1.0, update)
            O.bgart_collapse(ref, k, bool(dark_bg))
        # the collapse snaps whole histogram bins: a voxel within rounding of a threshold
        # may land on the other side, so compare the fraction of differing voxels too
        diff = np.abs(got - ref) > 1e-4 * max(1.0, float(np.abs(ref).max()))
        assert diff.mean() < 1e-3, diff.mean()
        assert rel_l2(got[~diff], ref[~diff]) <= 1e-4
    finally:
        hd.close()

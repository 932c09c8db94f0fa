"""Edge cases on the GPU against the oracle: calls with no projections added, a
single-tilt series, a one-row volume with one-row projections (FFTWeighting's 1-D
path, FFTWeighting.java:87-91, 114-134), and a series of all-NaN images."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import rel_l2, series_case
from tomoj_gb300 import _abi

pytestmark = pytest.mark.gpu


def make(lib, c, fill=_abi.FILL_NAN):
    g = _abi.make_geom(c["W"], c["H"], c["D"], c["w"], c["h"], c["n"])
    p = _abi.make_params(fill=fill)
    hd = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(g), C.byref(p), C.byref(hd)))
    eul = np.ascontiguousarray(c["eul"], np.float64)
    s = np.ascontiguousarray(c["series"], np.float32)
    _abi.check(lib.tomo_load_series(hd, s.ctypes.data, 0, _abi.ptr(eul, C.c_double), None, None))
    return hd


def volume(lib, hd, c):
    out = np.empty((c["D"], c["H"], c["W"]), np.float32)
    _abi.check(lib.tomo_get_volume(hd, out.ctypes.data, 0, 0, c["H"]))
    return out


def test_calls_with_no_projections_leave_the_volume(engine):
    c = series_case(W=32, H=4, D=16, n=5, seed=2)
    hd = make(engine, c)
    try:
        start = np.random.default_rng(1).random((c["D"], c["H"], c["W"]), dtype=np.float32)
        _abi.check(engine.tomo_set_volume(hd, start.ctypes.data, 0, 0, c["H"]))
        assert engine.tomo_projection_count(hd) == 0
        _abi.check(engine.tomo_project(hd, 0, c["H"]))
        _abi.check(engine.tomo_backproject(hd, 0, c["H"]))
        err = np.zeros(1)
        _abi.check(engine.tomo_project_and_difference(hd, 1.0, 0, c["H"], _abi.ptr(err, C.c_double)))
        assert np.array_equal(volume(engine, hd, c), start)
    finally:
        engine.tomo_destroy(hd)


def test_single_tilt_series_matches_oracle(engine, oracle_lib):
    c = series_case(W=40, H=6, D=24, n=1, amax=0.0, seed=3)
    hd = make(engine, c)
    try:
        err = np.zeros((3, 5))
        _abi.check(engine.tomo_run_ossart(hd, 3, 1.0, 0, 1, 0, c["H"], 1, _abi.ptr(err, C.c_double)))
        got = volume(engine, hd, c)
    finally:
        engine.tomo_destroy(hd)
    ref = np.zeros_like(c["vol"])
    for it in range(3):
        e5, _ = O.ossart_iteration(ref, c["g"], c["eul"], c["series"], np.array([0]), 1.0, 0)
        assert np.allclose(err[it, [0, 1, 3]], e5[[0, 1, 3]], rtol=1e-4)
    assert rel_l2(got, ref) <= 1e-4, rel_l2(got, ref)


@pytest.mark.parametrize("w", [64, 45])
def test_one_row_wbp_matches_oracle(engine, oracle_lib, w):
    # h = 1: the reference weights with its 1-D transform (weighting1D)
    c = series_case(W=w, H=1, D=32, n=11, seed=4, noise=0.0)
    hd = make(engine, c, fill=_abi.FILL_AVG)
    try:
        _abi.check(engine.tomo_set_weighting(hd, _abi.WEIGHT_RADERMACHER, 0.5, None, None))
        _abi.check(engine.tomo_run_wbp(hd, 0, 1))
        got = volume(engine, hd, c)
    finally:
        engine.tomo_destroy(hd)
    ref = np.zeros_like(c["vol"])
    O.wbp(ref, c["g"], c["eul"], c["series"], O.weighting_mask(c["w"], 1, c["angles"], None, 0.5 * c["w"]))
    assert rel_l2(got, ref) <= 1e-5, rel_l2(got, ref)


def test_all_nan_series_leaves_the_volume_at_zero(engine, oracle_lib):
    c = series_case(W=24, H=4, D=16, n=5, seed=6)
    c["series"] = np.full_like(c["series"], np.nan)
    hd = make(engine, c)
    try:
        err = np.zeros((2, 5))
        _abi.check(engine.tomo_run_ossart(hd, 2, 1.0, 2, 1, 0, c["H"], 1, _abi.ptr(err, C.c_double)))
        got = volume(engine, hd, c)
    finally:
        engine.tomo_destroy(hd)
    ref = np.zeros_like(c["vol"])
    for it in range(2):
        order = O.order_shuffle(c["eul"], int(engine.tomo_first_index(1, it, c["n"])))
        O.ossart_iteration(ref, c["g"], c["eul"], c["series"], order, 1.0, 2)
    assert np.array_equal(got, ref)
    assert not np.any(got)

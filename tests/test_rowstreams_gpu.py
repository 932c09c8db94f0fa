"""Row streams: an OS-SART iteration split into 2 to 4 row ranges on as many streams
(volume rows are independent with a vertical tilt axis) gives bitwise the volume and
residuals of the one-stream iteration."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from tests.cases import series_case
from tomoj_gb300 import _abi

pytestmark = pytest.mark.gpu


def run(lib, c, k, use_graph, update=5, positivity=False):
    g = _abi.make_geom(c["W"], c["H"], c["D"], c["w"], c["h"], c["n"])
    p = _abi.make_params(positivity=positivity)
    hd = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(g), C.byref(p), C.byref(hd)))
    try:
        eul = np.ascontiguousarray(c["eul"], np.float64)
        T = np.ascontiguousarray(c["T"], np.float64)
        s = np.ascontiguousarray(c["series"], np.float32)
        _abi.check(lib.tomo_load_series(hd, s.ctypes.data, 0, _abi.ptr(eul, C.c_double), _abi.ptr(T, C.c_double),
                                        None))
        _abi.check(lib.tomo_set_row_streams(hd, k))
        err = np.zeros((3, 5))
        _abi.check(lib.tomo_run_ossart(hd, 3, 1.0, update, 11, 0, c["H"], use_graph, _abi.ptr(err, C.c_double)))
        out = np.empty((c["D"], c["H"], c["W"]), np.float32)
        _abi.check(lib.tomo_get_volume(hd, out.ctypes.data, 0, 0, c["H"]))
        return out, err
    finally:
        lib.tomo_destroy(hd)


@pytest.mark.parametrize("k", [2, 3, 4])
@pytest.mark.parametrize("use_graph", [1, 0])
def test_row_streams_equal_one_stream(engine, k, use_graph):
    # enough rows that the one-stream forward launch fills the GPU (no depth split)
    c = series_case(W=64, H=400, D=48, n=13, seed=9, misalign=True)
    v1, e1 = run(engine, c, 1, use_graph)
    vk, ek = run(engine, c, k, use_graph)
    assert np.array_equal(v1, vk)
    assert np.array_equal(e1, ek)


def test_row_streams_with_positivity_and_sirt(engine):
    c = series_case(W=48, H=320, D=40, n=9, seed=4, misalign=True)
    v1, e1 = run(engine, c, 1, 1, update=0, positivity=True)
    v3, e3 = run(engine, c, 3, 1, update=0, positivity=True)
    assert np.array_equal(v1, v3)
    assert np.array_equal(e1, e3)


def test_row_streams_count_is_checked(engine):
    c = series_case(W=16, H=4, D=8, n=3, seed=1)
    g = _abi.make_geom(c["W"], c["H"], c["D"], c["w"], c["h"], c["n"])
    hd = C.c_void_p()
    _abi.check(engine.tomo_create(C.byref(g), None, C.byref(hd)))
    try:
        assert engine.tomo_set_row_streams(hd, 0) == _abi.ERR_INVALID
        assert engine.tomo_set_row_streams(hd, 5) == _abi.ERR_INVALID
    finally:
        engine.tomo_destroy(hd)

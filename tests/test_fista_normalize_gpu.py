"""GPU parity of two reference features the benchmark configurations leave off.

* FISTA momentum (FistaProjector3D.endOfIteration, FistaProjector3D.java:40-72):
  after every OS-SART iteration t <- (1 + sqrt(1 + 4 t^2)) / 2 and
  rec += ((t_prev - 1) / t) (rec - previous iteration's rec), with t0 = 0 so that
  the first step returns to the starting volume.
* Normalised projections (TiltSeries.setNormalize, AffineAlignment.applyTransformOnImage,
  AffineAlignment.java:148-151, 210-224): (x - mean) / stdDev per tilt, with the
  statistics of the tilt-dependent central region (TiltSeries.getImageStatistics,
  TiltSeries.java:809-835) computed by the host mirror and handed to both sides.

Tolerances as the plain form: <= 1e-5 relative L2 per pass, <= 1e-4 after several
iterations.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import rel_l2, series_case
from tomoj_gb300 import _abi
from tomoj_gb300.tiltseries import TiltSeries

pytestmark = pytest.mark.gpu


def _create(lib, c, normalize=False, stats=None, fill=_abi.FILL_NAN):
    g = _abi.make_geom(c["W"], c["H"], c["D"], c["w"], c["h"], c["n"])
    p = _abi.make_params(fill=fill, normalize=normalize)
    h = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(g), C.byref(p), C.byref(h)))
    eul = np.ascontiguousarray(c["eul"], np.float64)
    T = np.ascontiguousarray(c["T"], np.float64)
    series = np.ascontiguousarray(c["series"], np.float32)
    st = None if stats is None else np.ascontiguousarray(stats, np.float64)
    _abi.check(lib.tomo_load_series(h, series.ctypes.data, 0, _abi.ptr(eul, C.c_double), _abi.ptr(T, C.c_double),
                                    None if st is None else _abi.ptr(st, C.c_double)))
    return h


def _volume(lib, h, c):
    out = np.empty((c["D"], c["H"], c["W"]), np.float32)
    _abi.check(lib.tomo_get_volume(h, out.ctypes.data, 0, 0, c["H"]))
    return out


def test_fista_iterations_match_oracle(engine, oracle_lib):
    c = series_case(W=64, H=10, D=40, n=19, seed=21)
    n_iter, seed = 5, 3
    h = _create(engine, c)
    try:
        _abi.check(engine.tomo_set_fista(h, 1))
        _abi.check(engine.tomo_run_ossart(h, n_iter, 1.0, 5, seed, 0, c["H"], 1, None))
        got = _volume(engine, h, c)
    finally:
        engine.tomo_destroy(h)
    ref = np.zeros((c["D"], c["H"], c["W"]), np.float32)
    meas = np.ascontiguousarray(c["series"], np.float32)
    t = 0.0
    for it in range(n_iter):
        order = O.order_shuffle(c["eul"], int(engine.tomo_first_index(seed, it, c["n"])))
        prev = ref.copy()  # FistaProjector3D.startOfIteration keeps a copy of rec
        O.ossart_iteration(ref, c["g"], c["eul"], meas, order, 1.0, 5)
        t = O.fista_step(ref, prev, t)
    assert np.linalg.norm(ref) > 0
    err = rel_l2(got, ref)
    assert err <= 1e-4, err


def test_fista_first_step_returns_to_start(engine):
    """t0 = 0 makes the first momentum factor -1 (FistaProjector3D.java:47-49): one
    iteration from a given volume ends on that volume."""
    c = series_case(W=48, H=6, D=32, n=11, seed=4)
    h = _create(engine, c)
    try:
        start = np.ascontiguousarray(c["vol"] * np.float32(0.5))
        _abi.check(engine.tomo_set_volume(h, start.ctypes.data, 0, 0, c["H"]))
        _abi.check(engine.tomo_set_fista(h, 1))
        _abi.check(engine.tomo_run_ossart(h, 1, 1.0, 0, 1, 0, c["H"], 1, None))
        got = _volume(engine, h, c)
    finally:
        engine.tomo_destroy(h)
    # rec + (-1)(rec - start) rounds back to start up to one float rounding per voxel
    assert rel_l2(got, start) <= 1e-6


@pytest.fixture(scope="module")
def norm_case():
    c = series_case(W=64, H=12, D=48, n=21, misalign=True, seed=9)
    ts = TiltSeries(np.ascontiguousarray(c["series"], np.float32), c["angles"])
    for i in range(c["n"]):
        ts.getAlignment().setTransform(i, c["T"][i])
    ts.getAlignment().setCombineTransforms(False)
    c["stats"] = np.ascontiguousarray(ts.statistics(), np.float64)
    assert np.all(c["stats"][:, 1] > 0)
    return c


@pytest.mark.parametrize("fill", [_abi.FILL_NAN, _abi.FILL_AVG])
def test_normalized_alignment_matches_oracle(engine, oracle_lib, norm_case, fill):
    c = norm_case
    h = _create(engine, c, normalize=True, stats=c["stats"], fill=fill)
    try:
        ofill = {_abi.FILL_NAN: O.FILL_NAN, _abi.FILL_AVG: O.FILL_AVG}[fill]
        for i in range(c["n"]):
            got = np.empty((c["h"], c["w"]), np.float32)
            _abi.check(engine.tomo_get_aligned(h, i, _abi.ptr(got)))
            mean, std = c["stats"][i]
            ref = O.align(c["series"][i], c["T"][i], normalize=True, mean=mean, std=std, fill=ofill)
            assert np.array_equal(np.isnan(got), np.isnan(ref)), i
            ok = ~np.isnan(ref)
            assert np.abs(got[ok] - ref[ok]).max() <= 1e-6 * max(1.0, np.abs(ref[ok]).max()), i
            # the normalised image really is centred and scaled by the ROI statistics
            raw = O.align(c["series"][i], c["T"][i], False, mean, std, fill=ofill)  # average fill = the mean
            assert np.allclose(ref[ok], (raw[ok] - mean) / std, rtol=1e-5, atol=1e-5)
    finally:
        engine.tomo_destroy(h)


def test_normalized_ossart_iteration_matches_oracle(engine, oracle_lib, norm_case):
    c = norm_case
    h = _create(engine, c, normalize=True, stats=c["stats"])
    try:
        _abi.check(engine.tomo_run_ossart(h, 2, 1.0, 7, 11, 0, c["H"], 1, None))
        got = _volume(engine, h, c)
    finally:
        engine.tomo_destroy(h)
    meas = np.array([O.align(c["series"][i], c["T"][i], normalize=True, mean=c["stats"][i][0],
                             std=c["stats"][i][1], fill=O.FILL_NAN) for i in range(c["n"])], np.float32)
    ref = np.zeros((c["D"], c["H"], c["W"]), np.float32)
    for it in range(2):
        order = O.order_shuffle(c["eul"], int(engine.tomo_first_index(11, it, c["n"])))
        O.ossart_iteration(ref, c["g"], c["eul"], meas, order, 1.0, 7)
    assert np.linalg.norm(ref) > 0
    err = rel_l2(got, ref)
    assert err <= 1e-5 * 2, err

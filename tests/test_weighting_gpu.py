"""WBP weighting on the GPU against the oracle's 2-D DFT form of FFTWeighting
(FFTWeighting.java:31-112): the 2-D mask for a tilt axis that is not vertical
(radix-2 and Bluestein transform lengths, tilted and vertical Euler matrices), and
the reference's spreading of a non-finite pixel over its whole image by the 2-D
transform, for the row filter as well.  Tolerance 1e-5 relative L2 per pass."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import rel_l2
from tomoj_gb300 import _abi
from tomoj_gb300 import phantom as P

pytestmark = pytest.mark.gpu

TOL_PASS = 1e-5


def make_case(W, H, D, w, h, n, axis, euler_axis, seed):
    """euler_axis: tilt axis of the Euler matrices (0 = the series was rotated to a
    vertical axis, as TiltSeries.setTiltAxis does); axis: ts.getTiltAxis() for the mask."""
    vol = P.ellipsoid_phantom(W, H, D, 6, seed)
    angles = np.linspace(-60, 60, n)
    eul = np.array([O.euler(euler_axis, a, -euler_axis) for a in angles])
    g = O.Geom(W, H, D, w, h)
    series = np.nan_to_num(np.array([O.project(vol, g, eul[i])[0] for i in range(n)], np.float32))
    series = P.add_gaussian_noise(series, 0.01, seed + 1)
    return dict(vol=vol, eul=eul, g=g, series=series, angles=angles, axes=np.full(n, float(axis)),
                W=W, H=H, D=D, w=w, h=h, n=n)


def run_wbp(lib, c, radius, tilt_deg=True):
    g = _abi.make_geom(c["W"], c["H"], c["D"], c["w"], c["h"], c["n"])
    p = _abi.make_params(fill=_abi.FILL_NAN)
    h = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(g), C.byref(p), C.byref(h)))
    try:
        eul = np.ascontiguousarray(c["eul"], np.float64)
        series = np.ascontiguousarray(c["series"], np.float32)
        _abi.check(lib.tomo_load_series(h, series.ctypes.data, 0, _abi.ptr(eul, C.c_double), None, None))
        ang = np.ascontiguousarray(c["angles"], np.float64)
        axes = np.ascontiguousarray(c["axes"], np.float64)
        _abi.check(lib.tomo_set_weighting(h, _abi.WEIGHT_RADERMACHER, radius,
                                          _abi.ptr(ang, C.c_double) if tilt_deg else None,
                                          _abi.ptr(axes, C.c_double)))
        _abi.check(lib.tomo_run_wbp(h, 0, c["H"]))
        out = np.empty((c["D"], c["H"], c["W"]), np.float32)
        _abi.check(lib.tomo_get_volume(h, out.ctypes.data, 0, 0, c["H"]))
        return out
    finally:
        lib.tomo_destroy(h)


def oracle_wbp(c, radius):
    ref = np.zeros((c["D"], c["H"], c["W"]), np.float32)
    mask = O.weighting_mask(c["w"], c["h"], c["angles"], c["axes"], radius * c["w"])
    O.wbp(ref, c["g"], c["eul"], c["series"], mask)
    return ref


CASES = {
    # (W, H, D, w, h, n, mask axis, Euler axis)
    "tilted_bluestein": (40, 10, 30, 40, 10, 9, 7.0, 7.0),      # generic kernels, both lengths Bluestein
    "vertical_pow2": (64, 32, 40, 64, 32, 11, 30.0, 0.0),       # XZ-plane kernels, radix-2 both ways
    "vertical_mixed": (64, 24, 40, 64, 24, 11, -12.5, 0.0),     # radix-2 rows, Bluestein columns
    "vertical_odd": (45, 17, 33, 45, 17, 7, 80.0, 0.0),         # odd lengths
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_wbp_2d_weighting_matches_oracle(engine, oracle_lib, name):
    W, H, D, w, h, n, axis, eaxis = CASES[name]
    c = make_case(W, H, D, w, h, n, axis, eaxis, seed=11)
    radius = 0.5
    got = run_wbp(engine, c, radius)
    ref = oracle_wbp(c, radius)
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    assert rel_l2(got, ref) <= TOL_PASS, rel_l2(got, ref)


def test_wbp_row_filter_from_tilt_angles_equals_euler_form(engine, oracle_lib):
    # zero axis: tilt angles given or read from the Euler matrices give the same filter
    c = make_case(48, 8, 32, 48, 8, 9, 0.0, 0.0, seed=3)
    a = run_wbp(engine, c, 0.4, tilt_deg=True)
    b = run_wbp(engine, c, 0.4, tilt_deg=False)
    assert rel_l2(a, b) <= 1e-6
    assert rel_l2(a, oracle_wbp(c, 0.4)) <= TOL_PASS


@pytest.mark.parametrize("axis,w", [(0.0, 64), (0.0, 48), (25.0, 48)])
def test_wbp_weighting_spreads_non_finite_pixels_over_the_image(engine, oracle_lib, axis, w):
    # FFTWeighting's 2-D transform turns an image holding one NaN or Inf into NaN
    # everywhere, and the backprojection skips NaN samples: such an image adds nothing.
    c = make_case(w, 8, 32, w, 8, 9, axis, 0.0, seed=5)
    s = c["series"]
    s[2, 3, 5] = np.nan
    s[6, 0, w - 1] = np.inf
    got = run_wbp(engine, c, 0.5)
    ref = oracle_wbp(c, 0.5)
    keep = [i for i in range(c["n"]) if i not in (2, 6)]
    without = np.zeros_like(ref)
    mask = O.weighting_mask(c["w"], c["h"], c["angles"], c["axes"], 0.5 * c["w"])
    O.wbp(without, c["g"], c["eul"][keep], c["series"][keep], mask)
    assert np.array_equal(ref, without)
    assert rel_l2(got, ref) <= TOL_PASS, rel_l2(got, ref)


def test_ramp_filters_need_a_zero_tilt_axis(engine):
    c = make_case(32, 4, 16, 32, 4, 5, 10.0, 0.0, seed=1)
    g = _abi.make_geom(c["W"], c["H"], c["D"], c["w"], c["h"], c["n"])
    p = _abi.make_params()
    h = C.c_void_p()
    _abi.check(engine.tomo_create(C.byref(g), C.byref(p), C.byref(h)))
    try:
        eul = np.ascontiguousarray(c["eul"], np.float64)
        series = np.ascontiguousarray(c["series"], np.float32)
        _abi.check(engine.tomo_load_series(h, series.ctypes.data, 0, _abi.ptr(eul, C.c_double), None, None))
        axes = np.ascontiguousarray(c["axes"], np.float64)
        st = engine.tomo_set_weighting(h, _abi.WEIGHT_RAMP, 0.0, None, _abi.ptr(axes, C.c_double))
        assert st == _abi.ERR_UNSUPPORTED
    finally:
        engine.tomo_destroy(h)

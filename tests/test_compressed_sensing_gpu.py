"""CompressedSensingProjector on the GPU against the oracle (oracle/wavelet_oracle.py):
the end-of-iteration wavelet filter alone (FP64 on both sides: the threshold must agree
to rounding and the volume to 1e-6), for the three wavelet types, power-of-two and
Bluestein line lengths and explicit level counts; OS-SART iterations with the filter
through ReconstructionParameters.createCompressedSensingParameters, getProjector and
TomoReconstruction2.OSSART (<= 1e-4 after the iterations); and the refusals."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from oracle import wavelet_oracle as WO
from tests.cases import rel_l2
from tomoj_gb300 import _abi
from tomoj_gb300 import phantom as P
from tomoj_gb300 import reconstruction as R
from tomoj_gb300.projector import first_index
from tomoj_gb300.tiltseries import TiltSeries

pytestmark = pytest.mark.gpu


def handle(lib, W, H, D, prec=_abi.PREC_FP32):
    g = _abi.make_geom(W, H, D, W, H, 3)
    p = _abi.make_params(precision=prec)
    hd = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(g), C.byref(p), C.byref(hd)))
    return hd


def set_cs(lib, hd, kind, alpha, tau, frac, levels):
    lv = None if levels is None else (C.c_int32 * 3)(*levels)
    return lib.tomo_set_compressed_sensing(hd, kind, alpha, tau, frac, lv, 1)


@pytest.mark.parametrize("W,H,D,kind,alpha,tau,frac,levels", [
    (64, 8, 48, WO.BSPLINE, 3.0, 0.0, 0.95, None),        # default levels (1), Bluestein along z
    (96, 12, 40, WO.ORTHONORMAL, 1.5, 0.25, 0.8, (2, 2, 1)),  # no power-of-two line at all
    (128, 16, 64, WO.DUAL, 3.0, 0.0, 0.95, None),         # two levels, powers of two
    (32, 6, 20, WO.BSPLINE, 0.5, -0.3, 0.5, (1, 1, 2)),
])
def test_wavelet_filter_matches_oracle(engine, W, H, D, kind, alpha, tau, frac, levels):
    rng = np.random.default_rng(W + H + D)
    vol = (P.ellipsoid_phantom(W, H, D, 6, 11) + 0.05 * rng.standard_normal((D, H, W))).astype(np.float32)
    hd = handle(engine, W, H, D)
    try:
        _abi.check(engine.tomo_set_volume(hd, vol.ctypes.data, 0, 0, H))
        _abi.check(set_cs(engine, hd, kind, alpha, tau, frac, levels))
        _abi.check(engine.tomo_end_iteration(hd))
        got = np.empty_like(vol)
        _abi.check(engine.tomo_get_volume(hd, got.ctypes.data, 0, 0, H))
        t = C.c_double()
        _abi.check(engine.tomo_compressed_sensing_threshold(hd, C.byref(t)))
    finally:
        engine.tomo_destroy(hd)
    ref = vol.copy()
    t_ref = WO.cs_filter(ref, frac, kind, alpha, tau, levels)
    assert np.isclose(t.value, t_ref, rtol=1e-12, atol=0.0), (t.value, t_ref)
    assert rel_l2(got, ref) <= 1e-6, rel_l2(got, ref)
    assert not np.array_equal(got, vol)


def test_compressed_sensing_iterations_match_oracle(engine, oracle_lib):
    W, H, D, n = 64, 8, 32, 13
    vol = P.ellipsoid_phantom(W, H, D, 6, 23)
    angles = np.linspace(-60.0, 60.0, n)
    eul = np.array([O.euler_tilt_y(a) for a in angles])
    g = O.Geom(W, H, D, W, H)
    pix = np.nan_to_num(np.array([O.project(vol, g, e)[0] for e in eul], np.float32))
    pix = P.add_gaussian_noise(pix, 0.01, 4)
    ts = TiltSeries(pix, angles)
    ts.setNormalize(False)
    ts.setFillType(O.FILL_NAN)
    n_iter, relax, frac, seed = 3, 0.7, 0.9, 5
    params = R.ReconstructionParameters.createCompressedSensingParameters(W, H, D, n_iter, relax, frac,
                                                                         WO.BSPLINE, 3.0, 0.0)
    rec = R.TomoReconstruction2(W, H, D)
    proj = params.getProjector(ts, rec)
    try:
        assert proj.getWaveletsIterations() == [1, 1, 1]
        errs = rec.OSSART(ts, proj, params, seed=seed)
        got = rec.getVolume()
        t_last = proj.getLastThreshold()
    finally:
        proj.close()
    ref = np.zeros((D, H, W), np.float32)
    for it in range(n_iter):
        order = O.order_shuffle(eul, first_index(seed, it, n))
        e5, _ = O.ossart_iteration(ref, g, eul, pix, order, relax, 0)
        assert np.isclose(errs[it][0], e5[0], rtol=1e-4)
        t_ref = WO.cs_filter(ref, frac, WO.BSPLINE, 3.0, 0.0, (1, 1, 1))
    assert np.isclose(t_last, t_ref, rtol=1e-3)
    assert rel_l2(got, ref) <= 1e-4, rel_l2(got, ref)


def test_compressed_sensing_refusals(engine):
    hd = handle(engine, 64, 6, 32)
    try:
        assert set_cs(engine, hd, 2, 3.0, 0.0, 0.9, None) == _abi.ERR_INVALID        # no such type
        assert set_cs(engine, hd, 3, -0.6, 0.0, 0.9, None) == _abi.ERR_INVALID       # degree <= -0.5
        assert set_cs(engine, hd, 3, 3.0, 0.0, 1.5, None) == _abi.ERR_INVALID        # fraction > 1
        assert set_cs(engine, hd, 3, 3.0, 0.0, 0.9, (1, 2, 1)) == _abi.ERR_UNSUPPORTED  # 6 -> 3: odd
        assert set_cs(engine, hd, 3, 3.0, 0.0, 0.9, None) == _abi.OK
        assert engine.tomo_set_compressed_sensing(hd, 0, 0.0, 0.0, 0.0, None, 0) == _abi.OK
    finally:
        engine.tomo_destroy(hd)
    hb = handle(engine, 64, 6, 32, prec=_abi.PREC_BF16)
    try:
        assert set_cs(engine, hb, 3, 3.0, 0.0, 0.9, None) == _abi.ERR_UNSUPPORTED
    finally:
        engine.tomo_destroy(hb)


def test_long_lines_and_a_second_handle(engine):
    # 3072-voxel lines (Bluestein over 8192 points: 180 KB of shared memory per CTA), then a
    # handle with short lines is set up before the first filters again
    W, H, D = 3072, 2, 4
    vol = np.random.default_rng(8).standard_normal((D, H, W)).astype(np.float32)
    big = handle(engine, W, H, D)
    small = handle(engine, 32, 6, 20)
    try:
        _abi.check(engine.tomo_set_volume(big, vol.ctypes.data, 0, 0, H))
        _abi.check(set_cs(engine, big, WO.ORTHONORMAL, 3.0, 0.0, 0.9, (1, 1, 1)))
        _abi.check(set_cs(engine, small, WO.BSPLINE, 3.0, 0.0, 0.9, None))
        _abi.check(engine.tomo_end_iteration(small))
        _abi.check(engine.tomo_end_iteration(big))
        got = np.empty_like(vol)
        _abi.check(engine.tomo_get_volume(big, got.ctypes.data, 0, 0, H))
    finally:
        engine.tomo_destroy(small)
        engine.tomo_destroy(big)
    ref = vol.copy()
    WO.cs_filter(ref, 0.9, WO.ORTHONORMAL, 3.0, 0.0, (1, 1, 1))
    assert rel_l2(got, ref) <= 1e-6, rel_l2(got, ref)

"""Any geometry on the GPU against the oracle: a tilt axis that is not vertical
(full Euler matrices, generic kernels), and on the XZ-plane kernels with blended
rows: scale != 1 (projections finer or coarser than the volume grid, with
backprojection tiles spanning up to 192 image columns) and a half-pixel offset
between projection and volume centres.  The generic kernels
follow the reference's double arithmetic step by step, so norms and NaN patterns
must match exactly and values to float rounding (tolerance 1e-5 per pass, 1e-4
after iterations)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import rel_l2
from tomoj_gb300 import _abi
from tomoj_gb300 import phantom as P

pytestmark = pytest.mark.gpu

CASES = {
    # generic kernels (full Euler matrices)
    "tilt_axis_7deg": dict(W=40, H=10, D=30, w=40, h=10, axis=7.0, scale=1.0),
    # vertical axis with blended rows on the XZ-plane kernels
    "scale_2": dict(W=24, H=6, D=20, w=48, h=12, axis=0.0, scale=2.0),
    "scale_2_tiles": dict(W=80, H=5, D=72, w=160, h=10, axis=0.0, scale=2.0),
    "scale_half": dict(W=48, H=8, D=32, w=24, h=4, axis=0.0, scale=0.5),
    "half_pixel_rows": dict(W=36, H=8, D=24, w=36, h=9, axis=0.0, scale=1.0),
}


def make_case(name, n=7, seed=5):
    s = CASES[name]
    W, H, D, w, h = s["W"], s["H"], s["D"], s["w"], s["h"]
    vol = P.ellipsoid_phantom(W, H, D, 6, seed)
    angles = np.linspace(-55, 55, n)
    eul = np.array([O.euler(s["axis"], a, -s["axis"]) for a in angles])
    g = O.Geom(W, H, D, w, h, scale=s["scale"])
    series = np.nan_to_num(np.array([O.project(vol, g, eul[i])[0] for i in range(n)], np.float32))
    series = P.add_gaussian_noise(series, 0.01, seed + 1)
    return dict(vol=vol, eul=eul, g=g, series=series, W=W, H=H, D=D, w=w, h=h, n=n, scale=s["scale"])


class GHandle:
    def __init__(self, lib, c):
        self.lib, self.c = lib, c
        g = _abi.make_geom(c["W"], c["H"], c["D"], c["w"], c["h"], c["n"], scale=c["scale"])
        p = _abi.make_params(fill=_abi.FILL_NAN)
        h = C.c_void_p()
        _abi.check(lib.tomo_create(C.byref(g), C.byref(p), C.byref(h)))
        self.h = h
        eul = np.ascontiguousarray(c["eul"], np.float64)
        series = np.ascontiguousarray(c["series"], np.float32)
        _abi.check(lib.tomo_load_series(h, series.ctypes.data, 0, _abi.ptr(eul, C.c_double), None, None))

    def set_volume(self, v):
        v = np.ascontiguousarray(v, np.float32)
        _abi.check(self.lib.tomo_set_volume(self.h, v.ctypes.data, 0, 0, self.c["H"]))

    def volume(self):
        c = self.c
        out = np.empty((c["D"], c["H"], c["W"]), np.float32)
        _abi.check(self.lib.tomo_get_volume(self.h, out.ctypes.data, 0, 0, c["H"]))
        return out

    def slot(self, fn, k):
        out = np.empty((self.c["h"], self.c["w"]), np.float32)
        _abi.check(fn(self.h, k, _abi.ptr(out)))
        return out

    def close(self):
        self.lib.tomo_destroy(self.h)


@pytest.mark.parametrize("name", sorted(CASES))
def test_generic_forward_projection_matches_oracle(engine, oracle_lib, name):
    c = make_case(name)
    vol = c["vol"] + np.float32(0.05) * np.random.default_rng(3).random(c["vol"].shape, dtype=np.float32)
    hd = GHandle(engine, c)
    try:
        hd.set_volume(vol)
        for i in range(c["n"]):
            _abi.check(engine.tomo_add_projection(hd.h, i))
        _abi.check(engine.tomo_project(hd.h, 0, c["H"]))
        for i in range(c["n"]):
            p_ref, n_ref = O.project(vol, c["g"], c["eul"][i])
            p = hd.slot(engine.tomo_get_projection, i)
            n = hd.slot(engine.tomo_get_norm, i)
            assert np.array_equal(np.isnan(p), np.isnan(p_ref)), i
            assert np.array_equal(n, n_ref), i
            assert rel_l2(p, p_ref) <= 1e-5, (i, rel_l2(p, p_ref))
    finally:
        hd.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_generic_backprojection_matches_oracle(engine, oracle_lib, name):
    c = make_case(name)
    rng = np.random.default_rng(12)
    imgs = rng.normal(0, 1, (c["n"], c["h"], c["w"])).astype(np.float32)
    c2 = dict(c, series=imgs)
    hd = GHandle(engine, c2)
    try:
        start = rng.random((c["D"], c["H"], c["W"]), dtype=np.float32)
        hd.set_volume(start)
        order = [4, 0, 6, 2]
        for i in order:
            _abi.check(engine.tomo_add_projection(hd.h, i))
        _abi.check(engine.tomo_backproject(hd.h, 0, c["H"]))
        got = hd.volume()
        ref = start.copy()
        for i in order:
            O.backproject(ref, c["g"], c["eul"][i], imgs[i])
        assert rel_l2(got - start, ref - start) <= 1e-5, rel_l2(got - start, ref - start)
    finally:
        hd.close()


@pytest.mark.parametrize("name", sorted(CASES))
def test_generic_sirt_matches_oracle(engine, oracle_lib, name):
    c = make_case(name)
    hd = GHandle(engine, c)
    try:
        n_iter, seed, update = 3, 7, 3
        err = np.zeros((n_iter, 5))
        _abi.check(engine.tomo_run_ossart(hd.h, n_iter, 1.0, update, seed, 0, c["H"], 1, _abi.ptr(err, C.c_double)))
        got = hd.volume()
        ref = np.zeros_like(c["vol"])
        meas = np.array([O.align(c["series"][i], np.array([1.0, 0, 0, 1, 0, 0]), fill=O.FILL_NAN)
                         for i in range(c["n"])], np.float32)
        for it in range(n_iter):
            order = O.order_shuffle(c["eul"], int(engine.tomo_first_index(seed, it, c["n"])))
            e5, _ = O.ossart_iteration(ref, c["g"], c["eul"], meas, order, 1.0, update)
            assert np.allclose(err[it, [0, 1, 3]], e5[[0, 1, 3]], rtol=1e-4)
        assert rel_l2(got, ref) <= 1e-4, rel_l2(got, ref)
    finally:
        hd.close()


def test_generic_geometry_rejects_16bit_storage(engine):
    c = make_case("scale_2", n=3)
    g = _abi.make_geom(c["W"], c["H"], c["D"], c["w"], c["h"], c["n"], scale=c["scale"])
    p = _abi.make_params(precision=_abi.PREC_FP16)
    h = C.c_void_p()
    _abi.check(engine.tomo_create(C.byref(g), C.byref(p), C.byref(h)))
    try:
        eul = np.ascontiguousarray(c["eul"], np.float64)
        series = np.ascontiguousarray(c["series"], np.float32)
        st = engine.tomo_load_series(h, series.ctypes.data, 0, _abi.ptr(eul, C.c_double), None, None)
        assert st == _abi.ERR_UNSUPPORTED
    finally:
        engine.tomo_destroy(h)

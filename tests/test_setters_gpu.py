"""VoxelProjector3D setters on a created handle (VoxelProjector3D.java:78-104):
setScale, setPositivityConstraint and setLongObjectCompensation give bitwise the
results of a handle created with those settings."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tomoj_gb300 import _abi
from tomoj_gb300 import phantom as P

pytestmark = pytest.mark.gpu

W, H, D, w, h, n = 24, 6, 20, 48, 12, 7


def make_series(scale):
    vol = P.ellipsoid_phantom(W, H, D, 4, 8)
    eul = np.array([O.euler_tilt_y(a) for a in np.linspace(-50, 50, n)])
    g = O.Geom(W, H, D, w, h, scale=scale)
    s = np.nan_to_num(np.array([O.project(vol, g, e)[0] for e in eul], np.float32))
    return vol, eul, s


def handle(lib, scale, positivity=False, long_object=False):
    g = _abi.make_geom(W, H, D, w, h, n, scale=scale)
    p = _abi.make_params(positivity=positivity, long_object=long_object)
    hd = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(g), C.byref(p), C.byref(hd)))
    return hd


def load(lib, hd, eul, series):
    e = np.ascontiguousarray(eul, np.float64)
    s = np.ascontiguousarray(series, np.float32)
    _abi.check(lib.tomo_load_series(hd, s.ctypes.data, 0, _abi.ptr(e, C.c_double), None, None))


def run(lib, hd, vol):
    v = np.ascontiguousarray(vol, np.float32)
    _abi.check(lib.tomo_set_volume(hd, v.ctypes.data, 0, 0, H))
    _abi.check(lib.tomo_run_ossart(hd, 2, 1.0, 3, 4, 0, H, 1, None))
    out = np.empty((D, H, W), np.float32)
    _abi.check(lib.tomo_get_volume(hd, out.ctypes.data, 0, 0, H))
    norms = []
    for i in range(n):
        _abi.check(lib.tomo_add_projection(hd, i))
    _abi.check(lib.tomo_project(hd, 0, H))
    for i in range(n):
        m = np.empty((h, w), np.float32)
        _abi.check(lib.tomo_get_norm(hd, i, _abi.ptr(m)))
        norms.append(m)
    _abi.check(lib.tomo_clear_projections(hd))
    return out, np.array(norms)


@pytest.mark.parametrize("positivity,long_object", [(False, False), (True, False), (False, True), (True, True)])
def test_setters_equal_creation_settings(engine, positivity, long_object):
    vol, eul, series = make_series(2.0)
    start = vol - np.float32(0.3)  # negative voxels: positivity matters
    ref_h = handle(engine, 2.0, positivity, long_object)
    hd = handle(engine, 1.0)
    try:
        load(engine, ref_h, eul, series)
        load(engine, hd, eul, series)
        _abi.check(engine.tomo_set_scale(hd, 2.0))
        _abi.check(engine.tomo_set_positivity(hd, int(positivity)))
        _abi.check(engine.tomo_set_long_object(hd, int(long_object)))
        v_ref, n_ref = run(engine, ref_h, start)
        v, nm = run(engine, hd, start)
        assert np.array_equal(v, v_ref)
        assert np.array_equal(nm, n_ref)
    finally:
        engine.tomo_destroy(ref_h)
        engine.tomo_destroy(hd)


def test_set_scale_rejects_nonpositive(engine):
    hd = handle(engine, 1.0)
    try:
        assert engine.tomo_set_scale(hd, 0.0) == _abi.ERR_INVALID
        assert engine.tomo_set_scale(hd, -1.0) == _abi.ERR_INVALID
    finally:
        engine.tomo_destroy(hd)


def test_set_centers_equals_creation_centres(engine):
    # volume centre off by 1.5 columns / 0.5 planes, tilt axis 2 pixels right of the
    # projection centre: blended rows and shifted tables, as a handle created with them
    vol, eul, series = make_series(2.0)
    vc = np.array([(W - 1) / 2.0 + 1.5, (H - 1) / 2.0, (D - 1) / 2.0 - 0.5])
    pc = np.array([(w - 1) / 2.0, (h - 1) / 2.0, (w - 1) / 2.0 + 2.0, (h - 1) / 2.0])
    g = _abi.make_geom(W, H, D, w, h, n, vol_center=tuple(vc), proj_center=tuple(pc), scale=2.0)
    p = _abi.make_params()
    ref_h = C.c_void_p()
    _abi.check(engine.tomo_create(C.byref(g), C.byref(p), C.byref(ref_h)))
    hd = handle(engine, 2.0)
    try:
        load(engine, ref_h, eul, series)
        load(engine, hd, eul, series)
        _abi.check(engine.tomo_set_centers(hd, _abi.ptr(np.ascontiguousarray(vc), C.c_double),
                                           _abi.ptr(np.ascontiguousarray(pc), C.c_double)))
        v_ref, n_ref = run(engine, ref_h, vol)
        v, nm = run(engine, hd, vol)
        assert np.array_equal(v, v_ref)
        assert np.array_equal(nm, n_ref)
    finally:
        engine.tomo_destroy(ref_h)
        engine.tomo_destroy(hd)


def test_project_volume_matches_oracle(engine, oracle_lib):
    from tomoj_gb300.reconstruction import project_volume
    vol = P.ellipsoid_phantom(32, 8, 24, 4, 3)
    projs, angles = project_volume(vol, -30.0, 30.0, 7.5)
    assert angles.size == 9 and projs.shape == (9, 8, 32)
    g = O.Geom(32, 8, 24, 32, 8)
    for i, a in enumerate(angles):
        ref, _ = O.project(vol, g, O.euler_tilt_y(a))
        assert np.array_equal(np.isnan(projs[i]), np.isnan(ref))
        ok = ~np.isnan(ref)
        assert np.allclose(projs[i][ok], ref[ok], rtol=1e-5, atol=1e-5)

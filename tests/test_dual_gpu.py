"""Dual-axis drivers on the GPU against the oracle: two tilt-series (a vertical tilt
axis and a 90 degree axis, the second on the generic kernels) reconstructed into one
volume by two projectors built on the same TomoReconstruction2 (TomoReconstruction2
.ADASIRT / ADOSSART / ADASIRT2Single, TomoReconstruction2.java:880-1181, 1282-1428),
plus the lifetime of a shared device volume.  Tolerance 1e-4 after the iterations."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import rel_l2
from tomoj_gb300 import phantom as P
from tomoj_gb300.projector import VoxelProjector3D, first_index
from tomoj_gb300.reconstruction import ReconstructionParameters, TomoReconstruction2
from tomoj_gb300.tiltseries import TiltSeries

pytestmark = pytest.mark.gpu

W, H, D = 24, 24, 16


def series(axis, angles, vol, seed):
    eul = np.array([O.euler(axis, a, -axis) for a in angles])
    g = O.Geom(W, H, D, W, H)
    pix = np.nan_to_num(np.array([O.project(vol, g, e)[0] for e in eul], np.float32))
    pix = P.add_gaussian_noise(pix, 0.01, seed)
    ts = TiltSeries(pix, angles)
    ts.setNormalize(False)
    ts.setFillType(O.FILL_NAN)
    if axis != 0.0:
        ts.getAlignment().setTiltAxis(axis)
        ts.getAlignment().setTiltAxisVertical(False)
    return ts, eul, g


@pytest.fixture(scope="module")
def dual():
    vol = P.ellipsoid_phantom(W, H, D, 5, 31)
    ts1, e1, g1 = series(0.0, np.linspace(-60, 60, 11), vol, 1)
    ts2, e2, g2 = series(90.0, np.linspace(-50, 50, 9), vol, 2)
    return dict(ts1=ts1, e1=e1, g1=g1, ts2=ts2, e2=e2, g2=g2)


def projectors(c):
    rec = TomoReconstruction2(W, H, D)
    p1 = VoxelProjector3D(c["ts1"], rec)
    p2 = VoxelProjector3D(c["ts2"], rec)
    return rec, p1, p2


def test_adossart_matches_oracle(engine, oracle_lib, dual):
    c = dual
    params = ReconstructionParameters.createOSSARTParameters(W, H, D, 3, 1.0, 3)
    rec, p1, p2 = projectors(c)
    try:
        errs = rec.ADOSSART(c["ts1"], p1, c["ts2"], p2, params, seed=5)
        got = rec.getVolume()
    finally:
        p2.close()
        p1.close()
    ref = np.zeros((D, H, W), np.float32)
    m1, m2 = c["ts1"].pixels, c["ts2"].pixels
    n1, n2 = m1.shape[0], m2.shape[0]
    ref_errs = []
    for i in range(len(errs)):
        o1 = O.order_shuffle(c["e1"], first_index(5, 2 * i, n1))
        o2 = O.order_shuffle(c["e2"], first_index(5, 2 * i + 1, n2))
        e5 = O.ossart_iteration_dual(ref, c["g1"], c["e1"], m1, o1, c["g2"], c["e2"], m2, o2, 1.0, 3)
        ref_errs.append(e5[0])
    assert len(errs) == 3
    assert np.allclose(errs, ref_errs, rtol=1e-4)
    assert rel_l2(got, ref) <= 1e-4, rel_l2(got, ref)


def test_adasirt_matches_oracle(engine, oracle_lib, dual):
    c = dual
    params = ReconstructionParameters.createOSSARTParameters(W, H, D, 2, 0.5, 0)
    rec, p1, p2 = projectors(c)
    try:
        errs = rec.ADASIRT(c["ts1"], p1, c["ts2"], p2, params, seed=9)
        got = rec.getVolume()
    finally:
        p1.close()
        p2.close()
    ref = np.zeros((D, H, W), np.float32)
    m1, m2 = c["ts1"].pixels, c["ts2"].pixels
    n1, n2 = m1.shape[0], m2.shape[0]
    for i in range(len(errs)):
        O.ossart_iteration(ref, c["g1"], c["e1"], m1, O.order_shuffle(c["e1"], first_index(9, 2 * i, n1)), 0.5, 0)
        e5, _ = O.ossart_iteration(ref, c["g2"], c["e2"], m2, O.order_shuffle(c["e2"], first_index(9, 2 * i + 1, n2)),
                                   0.5, 0)
        assert np.isclose(errs[i], e5[0], rtol=1e-4)
    assert rel_l2(got, ref) <= 1e-4, rel_l2(got, ref)


def test_adasirt2single_matches_surface_ossart(engine, oracle_lib, dual):
    c = dual
    params = ReconstructionParameters.createOSSARTParameters(W, H, D, 2, 1.0, 4)
    rec = TomoReconstruction2(W, H, D)
    p = VoxelProjector3D(c["ts2"], rec)
    try:
        errs = rec.ADASIRT2Single(c["ts2"], p, params, seed=3)
        got = rec.getVolume()
    finally:
        p.close()
    ref = np.zeros((D, H, W), np.float32)
    n = c["ts2"].pixels.shape[0]
    for i in range(len(errs)):
        e5, _ = O.ossart_iteration(ref, c["g2"], c["e2"], c["ts2"].pixels,
                                   O.order_shuffle(c["e2"], first_index(3, i, n)), 1.0, 4)
        assert np.isclose(errs[i], e5[0], rtol=1e-4)
    assert rel_l2(got, ref) <= 1e-4, rel_l2(got, ref)


def test_shared_volume_survives_its_owner(engine, dual):
    c = dual
    rec, p1, p2 = projectors(c)
    start = np.random.default_rng(4).random((D, H, W), dtype=np.float32)
    rec.setVolume(start)
    try:
        # both projectors see one volume: a backprojection through p2 is seen by p1
        p2.addProjection(0)
        p2.backproject(0, H)
        p2.clearAllProjections()
        after = rec.getVolume()
        assert not np.array_equal(after, start)
        assert np.array_equal(p1._get_volume(), p2._get_volume())
        # closing the owner hands the device volume to the sharer
        p1.close()
        assert np.array_equal(rec.getVolume(), after)
        assert np.array_equal(p2._get_volume(), after)
        p2.addProjection(1)
        p2.backproject(0, H)
        assert not np.array_equal(rec.getVolume(), after)
    finally:
        p1.close()
        p2.close()


def test_a_sharer_follows_its_owners_stream(engine, dual):
    from tomoj_gb300 import _abi
    rec, p1, p2 = projectors(dual)
    try:
        assert engine.tomo_set_stream(p2.handle, None) == _abi.ERR_STATE
        assert engine.tomo_set_stream(p1.handle, None) == _abi.OK
    finally:
        p2.close()
        p1.close()

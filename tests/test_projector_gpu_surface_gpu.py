"""The reference's OpenCL projector surface (ProjectorGPU / VoxelProjector3DGPU) on the
engine: the slab flow of ReconstructionThreadManagerGPU.doGPURec (initForIterative per row
slab, OS-SART on those rows, updateFromGPU, releaseCL_Memory) gives the volume of one
whole-volume OS-SART run; initForBP starts a backprojection from zero rows; the host copy
only changes through updateFromGPU."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import rel_l2
from tomoj_gb300 import phantom as P
from tomoj_gb300.projector import VoxelProjector3D, VoxelProjector3DGPU
from tomoj_gb300.reconstruction import ReconstructionParameters, TomoReconstruction2
from tomoj_gb300.tiltseries import TiltSeries

pytestmark = pytest.mark.gpu

W, H, D, n = 48, 10, 32, 11


@pytest.fixture(scope="module")
def series():
    vol = P.ellipsoid_phantom(W, H, D, 6, 29)
    angles = np.linspace(-60.0, 60.0, n)
    g = O.Geom(W, H, D, W, H)
    pix = np.nan_to_num(np.array([O.project(vol, g, O.euler_tilt_y(a))[0] for a in angles], np.float32))
    return P.add_gaussian_noise(pix, 0.01, 6), angles


def tilt_series(s):
    ts = TiltSeries(s[0], s[1])
    ts.setNormalize(False)
    ts.setFillType(O.FILL_NAN)
    return ts


def test_slab_flow_equals_one_whole_run(engine, series):
    params = ReconstructionParameters.createOSSARTParameters(W, H, D, 2, 0.8, 4)
    start = np.random.default_rng(2).random((D, H, W), dtype=np.float32)
    ts = tilt_series(series)
    rec = TomoReconstruction2(W, H, D, start)
    proj = VoxelProjector3D(ts, rec)
    try:
        rec.OSSART(ts, proj, params, seed=7)
        whole = rec.getVolume().copy()
    finally:
        proj.close()

    rec = TomoReconstruction2(W, H, D, start)
    gp = VoxelProjector3DGPU(ts, rec, None, None)
    assert 0 < gp.computeMaximumSizeForVolume()
    for y0, y1 in ((0, 4), (4, 10)):
        gp.initForIterative(y0, y1, 4, VoxelProjector3DGPU.SEPARATE_PROJ_DIFF, False)
        rec.OSSART(ts, gp, params, startY=y0, endY=y1, seed=7)
        gp.updateFromGPU(y0, y1)
    gp.releaseCL_Memory()
    assert rel_l2(rec.getVolume(), whole) <= 1e-6, rel_l2(rec.getVolume(), whole)


def test_init_for_bp_starts_from_zero_rows(engine, series):
    ts = tilt_series(series)
    ones = np.ones((D, H, W), np.float32)
    rec = TomoReconstruction2(W, H, D, ones)
    gp = VoxelProjector3DGPU(ts, rec, None, None)
    try:
        gp.initForBP(2, 7, n)
        for i in range(n):
            gp.addProjection(i)
            gp.backproject(2, 7)
            gp.clearAllProjections()
        gp.updateFromGPU(0, H, 2, 7)
    finally:
        gp.releaseCL_Memory()
    got = rec.getVolume()
    assert np.array_equal(got[:, :2], ones[:, :2]) and np.array_equal(got[:, 7:], ones[:, 7:])

    rec0 = TomoReconstruction2(W, H, D)
    p0 = VoxelProjector3D(ts, rec0)
    try:
        for i in range(n):
            p0.addProjection(i)
            p0.backproject(2, 7)
            p0.clearAllProjections()
        ref = rec0.getVolume()
    finally:
        p0.close()
    assert np.array_equal(got[:, 2:7], ref[:, 2:7])


def test_host_copy_changes_only_through_update(engine, series):
    ts = tilt_series(series)
    start = np.full((D, H, W), 0.5, np.float32)
    rec = TomoReconstruction2(W, H, D, start)
    gp = VoxelProjector3DGPU(ts, rec, None, None)
    gp.initForBP(0, H, n)   # device rows zeroed, nothing downloaded
    with pytest.raises(NotImplementedError):
        gp.initForIterative(0, H, n, 0, True)
    gp.releaseCL_Memory()
    assert np.array_equal(rec.getVolume(), start)

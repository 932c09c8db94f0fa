"""AdvancedReconstructionParameters factories through getProjector and
TomoReconstruction2.OSSART (AdvancedReconstructionParameters.java:135-221): the Bayesian
type against the oracle's Bayesian iteration (alpha carried by the relaxation
coefficient), and BgART bitwise against a BgARTVoxelProjector3D built by hand."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import rel_l2
from tomoj_gb300 import phantom as P
from tomoj_gb300 import reconstruction as R
from tomoj_gb300.projector import BgARTVoxelProjector3D, first_index
from tomoj_gb300.tiltseries import TiltSeries

pytestmark = pytest.mark.gpu

W, H, D, n = 32, 6, 24, 11


@pytest.fixture(scope="module")
def case():
    vol = P.ellipsoid_phantom(W, H, D, 5, 17)
    angles = np.linspace(-60.0, 60.0, n)
    eul = np.array([O.euler_tilt_y(a) for a in angles])
    g = O.Geom(W, H, D, W, H)
    pix = np.nan_to_num(np.array([O.project(vol, g, e)[0] for e in eul], np.float32))
    pix = P.add_gaussian_noise(pix, 0.01, 5)
    return dict(vol=vol, angles=angles, eul=eul, g=g, pix=pix)


def tilt_series(c):
    ts = TiltSeries(c["pix"], c["angles"])
    ts.setNormalize(False)
    ts.setFillType(O.FILL_NAN)
    return ts


def test_bayesian_parameters_match_oracle(engine, oracle_lib, case):
    c = case
    alpha, lam, n_iter, seed = 0.6, 0.05, 2, 7
    params = R.ReconstructionParameters.createBayesianParameters(W, H, D, n_iter, alpha, lam)
    assert params.getRegularizationWeight() == lam
    ts = tilt_series(c)
    start = (0.5 * c["vol"]).astype(np.float32)
    rec = R.TomoReconstruction2(W, H, D, start.copy())
    proj = params.getProjector(ts, rec)
    try:
        assert proj.regularizationAlpha == alpha and proj.regularizationLambda == lam
        errs = rec.OSSART(ts, proj, params, seed=seed)
        got = rec.getVolume()
    finally:
        proj.close()
    ref = start.copy()
    for it in range(n_iter):
        order = O.order_shuffle(c["eul"], first_index(seed, it, n))
        # the relaxation coefficient carries alpha into both the OS-SART step and the
        # end-of-iteration regularisation; update 0 is SIRT
        e5 = O.bayesian_iteration(ref, c["g"], c["eul"], c["pix"], order, alpha, 0, lam, alpha)
        assert np.isclose(errs[it][0], e5[0], rtol=1e-4)
    assert rel_l2(got, ref) <= 1e-4, rel_l2(got, ref)


@pytest.mark.parametrize("median,dark", [(True, True), (False, False)])
def test_bgart_parameters_equal_a_hand_built_projector(engine, case, median, dark):
    c = case
    k, n_iter, seed = 1.5, 2, 3
    params = R.ReconstructionParameters.createBgARTParameters(W, H, D, n_iter, 0.8, 3, k, median, dark)
    start = (0.8 * c["vol"]).astype(np.float32)
    out = []
    for build in (lambda ts, rec: params.getProjector(ts, rec),
                  lambda ts, rec: BgARTVoxelProjector3D(ts, rec, None, k, dark, median)):
        ts = tilt_series(c)
        rec = R.TomoReconstruction2(W, H, D, start.copy())
        proj = build(ts, rec)
        try:
            errs = rec.OSSART(ts, proj, params, seed=seed)
            out.append((rec.getVolume(), np.asarray(errs)))
        finally:
            proj.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert not np.array_equal(out[0][0], start)



def test_thread_manager_runs_the_parameters(engine, case):
    # ReconstructionThreadManager.reconstruct: the same volume as driving the projector by
    # hand; a second call on the same sizes adds iterations to the same volume
    c = case
    params = R.ReconstructionParameters.createOSSARTParameters(W, H, D, 2, 0.9, 4)
    mgr = R.ReconstructionThreadManager(None, tilt_series(c))
    mgr.seed = 3
    try:
        rec = mgr.reconstruct(params)
        first = rec.getVolume().copy()
        errs = mgr.getReconstructionDissimilarities()
        assert len(errs) == 2 and mgr.getNumberofsteps() == n * 2 * 2
        assert mgr.reconstruct(params) is rec
        second = rec.getVolume().copy()
        proj5 = mgr.getProjection(5)
    finally:
        mgr.close()
    ts = tilt_series(c)
    ref = R.TomoReconstruction2(W, H, D)
    p = params.getProjector(ts, ref)
    try:
        ref_errs = ref.OSSART(ts, p, params, seed=3)
        assert np.array_equal(ref.getVolume(), first)
        assert np.array_equal(np.asarray(errs), np.asarray(ref_errs))
        ref.OSSART(ts, p, params, seed=3)
        assert np.array_equal(ref.getVolume(), second)
        p.addProjection(5)
        p.project(0, H)
        assert np.array_equal(p.getProjection(0), proj5)
        p.clearAllProjections()
    finally:
        p.close()
    wbp = R.ReconstructionParameters.createWBPParameters(W, H, D, 0.5)
    mgr = R.ReconstructionThreadManager(None, tilt_series(c))
    try:
        rec = mgr.reconstruct(wbp)
        assert mgr.getReconstructionDissimilarities() is None and np.any(rec.getVolume())
    finally:
        mgr.close()

"""ResolutionEstimation on the engine: even / odd half reconstructions (WBP and SIRT)
against the oracle's, and their Fourier shell correlation."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import rel_l2, series_case
from tomoj_gb300 import _abi
from tomoj_gb300 import resolution as R
from tomoj_gb300.reconstruction import ReconstructionParameters
from tomoj_gb300.tiltseries import TiltSeries

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", ["wbp", "sirt"])
def test_half_reconstructions_and_fsc(engine, oracle_lib, method):
    c = series_case(W=48, H=8, D=32, n=21, seed=61, noise=0.02)
    ts = TiltSeries(c["series"], c["angles"])
    ts.setNormalize(False)
    if method == "wbp":
        ts.setFillType(_abi.FILL_AVG)
        params = ReconstructionParameters.createWBPParameters(c["W"], c["H"], c["D"], 0.5)
    else:
        ts.setFillType(_abi.FILL_NAN)
        params = ReconstructionParameters.createOSSARTParameters(c["W"], c["H"], c["D"], 3, 1.0, 0)
    est = R.ResolutionEstimation(ts, params, seed=3)
    curve = est.fsc()
    for half, rec in ((R.EVEN_PROJECTIONS, est.recFSCeven), (R.ODD_PROJECTIONS, est.recFSCodd)):
        idx = R.available_indexes(c["n"], half)
        eul = c["eul"][idx]
        series = c["series"][idx]
        ref = np.zeros_like(c["vol"])
        if method == "wbp":
            stats = np.asarray(ts.statistics())[idx]
            meas = np.array([O.align(series[k], np.array([1.0, 0, 0, 1, 0, 0]), mean=stats[k][0],
                                     std=stats[k][1], fill=O.FILL_AVG) for k in range(idx.size)], np.float32)
            mask = O.weighting_mask(c["w"], c["h"], c["angles"][idx], None, 0.5 * c["w"])
            O.wbp(ref, c["g"], eul, meas, mask)
        else:
            meas = np.array([O.align(series[k], np.array([1.0, 0, 0, 1, 0, 0]), fill=O.FILL_NAN)
                             for k in range(idx.size)], np.float32)
            for it in range(3):
                from tomoj_gb300.projector import first_index
                order = O.order_shuffle(eul, first_index(3, it, idx.size))
                O.ossart_iteration(ref, c["g"], eul, meas, order, 1.0, 0)
        assert rel_l2(rec, ref) <= 1e-4, (half, rel_l2(rec, ref))
    # both halves image the same object: strong correlation at low frequency
    assert curve.shape == (4, c["W"] // 2 + 1)
    assert np.nanmean(curve[1][1:4]) > 0.5


def test_ssnr_on_the_engine(engine):
    c = series_case(W=48, H=8, D=32, n=21, seed=62, noise=0.02)
    ts = TiltSeries(c["series"], c["angles"])
    ts.setNormalize(False)
    ts.setFillType(_abi.FILL_NAN)
    params = ReconstructionParameters.createOSSARTParameters(c["W"], c["H"], c["D"], 2, 1.0, 0)
    est = R.ResolutionEstimation(ts, params, seed=5)
    table = est.SSNR(ring_width=4, computeVSSNR=True)
    assert table.shape == (9, c["W"] // 2 + 1)
    # volumetric SSNR: the per-tilt SSNR images reconstructed like the data
    assert est.tsVSSNR.pixels.shape == c["series"].shape
    assert est.recVSSNR.shape == (c["D"], c["H"], c["W"]) and np.abs(est.recVSSNR).max() > 0
    assert est.recSignal.shape == (c["D"], c["H"], c["W"]) and est.recNoise.shape == est.recSignal.shape
    # the phantom's reprojections carry far more low-frequency power than the noise series'
    assert np.all(np.isfinite(table[3][1:5])) and np.nanmean(table[3][1:5]) > np.nanmean(table[6][1:5])

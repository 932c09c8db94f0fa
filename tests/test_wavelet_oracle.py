"""The compressed-sensing oracle on its own (CPU): the restated fractional spline wavelet
filter banks reconstruct perfectly for every type, degree and shift (power-of-two and
other lengths), the orthonormal type keeps the energy, the autocorrelation obeys its
two-scale relation, and findThreshold / the soft threshold follow
CompressedSensingProjector.java:80-125 on hand-checked cases."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import wavelet_oracle as WO


@pytest.mark.parametrize("kind", [WO.ORTHONORMAL, WO.BSPLINE, WO.DUAL])
@pytest.mark.parametrize("alpha,tau", [(3.0, 0.0), (1.5, 0.25), (0.2, -0.1)])
def test_transform_inverts(kind, alpha, tau):
    rng = np.random.default_rng(3)
    for shape, iters in (((16, 8, 32), (2, 2, 2)), ((20, 6, 24), (2, 1, 1))):
        v = rng.standard_normal(shape)
        b = v.copy()
        WO.transform3d(b, iters, kind, alpha, tau)
        assert not np.allclose(b, v)
        WO.inverse3d(b, iters, kind, alpha, tau)
        assert np.abs(b - v).max() < 1e-12


def test_orthonormal_transform_keeps_energy():
    v = np.random.default_rng(4).standard_normal((8, 16, 16))
    b = v.copy()
    WO.transform3d(b, (2, 2, 1), WO.ORTHONORMAL, 3.0, 0.0)
    assert np.isclose(np.sum(b * b), np.sum(v * v), rtol=1e-12)


def test_autocorrelation_two_scale_relation():
    # A(2w) = (|H(w)|^2 A(w) + |H(w + pi)|^2 A(w + pi)) / 2, with |H|^2 = 2 |cos(w/2)|^(2a+2)
    w = np.linspace(-np.pi, np.pi, 37)
    for a in (0.0, 1.0, 3.0, 2.5):
        lhs = WO.autocorrelation(2 * w, a)
        h2 = 2 * np.abs(np.cos(w / 2)) ** (2 * a + 2)
        hp2 = 2 * np.abs(np.cos((w + np.pi) / 2)) ** (2 * a + 2)
        rhs = (h2 * WO.autocorrelation(w, a) + hp2 * WO.autocorrelation(w + np.pi, a)) / 2
        assert np.allclose(lhs, rhs, rtol=1e-9)
    assert WO.autocorrelation(np.array([0.0]), 3.0)[0] == 1.0


def test_best_iterations_follow_the_width():
    assert WO.best_iterations(64) == (1, 1, 1)
    assert WO.best_iterations(65) == (2, 2, 2)
    assert WO.best_iterations(512) == (4, 4, 4)


def test_threshold_refines_until_the_count_fits():
    # one coefficient at 1.0 and 99 at k * 1e-5 (k = 1..99), 50 % zeros.  Pass 1: histomax 1,
    # scale 256, all 99 small ones in bin 0: 99 > 1.01 * 50, so histomax = 1 / 256.  Pass 2:
    # scale 65536, k * 0.65536 -> bins; 48 values below bin 32, k = 49, 50 in it: exactly 50.
    buf = np.concatenate([np.arange(1, 100) * 1e-5, [1.0]]).reshape(1, 10, 10)
    assert WO.find_threshold(buf, 0.5) == 32 / 65536.0
    assert WO.abs_histogram(buf, 1 / 256.0)[:33].sum() == 50


def test_threshold_edge_cases():
    assert WO.find_threshold(np.zeros((2, 2, 2)), 0.9) == 0.0  # the reference loops forever here
    buf = np.full((1, 1, 4), 2.0)
    # no zeros asked: index -1, a negative threshold, as the reference computes it
    assert WO.find_threshold(buf, 0.0) == -1 / 128.0


def test_soft_threshold():
    b = np.array([-3.0, -1.0, 0.5, 1.0, 2.5])
    WO.soft_threshold(b, 1.0)
    assert b.tolist() == [-2.0, 0.0, 0.0, 0.0, 1.5]


def test_cs_filter_zeroes_the_small_coefficients():
    rng = np.random.default_rng(5)
    vol = rng.standard_normal((16, 8, 32)).astype(np.float32)
    out = vol.copy()
    t = WO.cs_filter(out, 0.9, WO.ORTHONORMAL, 3.0, 0.0, (1, 1, 1))
    assert t > 0 and out.dtype == np.float32
    b = out.astype(np.float64)
    WO.transform3d(b, (1, 1, 1), WO.ORTHONORMAL, 3.0, 0.0)
    # after the soft threshold about 90 % of the coefficients are (numerically) zero
    assert np.mean(np.abs(b) < 1e-5 * np.abs(b).max()) > 0.85

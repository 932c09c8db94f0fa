"""Seeded parity cases shared by the tests (sizes the CPU oracle finishes in seconds)."""
from __future__ import annotations

import numpy as np

from oracle import oracle as O
from tomoj_gb300 import phantom as P


def series_case(W=64, H=12, D=48, n=21, amax=60.0, seed=7, misalign=False, noise=0.01, w=None, h=None):
    """Phantom, its oracle tilt-series (optionally misaligned and noisy), angles, Eulers, transforms."""
    w = W if w is None else w
    h = H if h is None else h
    vol = P.ellipsoid_phantom(W, H, D, max(4, P.n_ellipsoids_for(W, H, D) // 2), seed)
    angles = np.linspace(-amax, amax, n)
    eul = np.array([O.euler_tilt_y(a) for a in angles])
    g = O.Geom(W, H, D, w, h)
    ideal = np.array([O.project(vol, g, eul[i])[0] for i in range(n)], np.float32)
    ideal = np.nan_to_num(ideal)
    T = np.tile(np.array([1, 0, 0, 1, 0, 0], np.float64), (n, 1))
    series = ideal
    if misalign:
        T = P.misalignment(n, seed + 1, max_shift=3.0, max_rot_deg=1.0)
        series = np.array([P.unalign(ideal[i], T[i]) for i in range(n)], np.float32)
    if noise:
        series = P.add_gaussian_noise(series, noise, seed + 2)
    return dict(vol=vol, angles=angles, eul=eul, T=T, series=series, g=g, W=W, H=H, D=D, w=w, h=h, n=n)


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    ok = np.isfinite(a) & np.isfinite(b)
    den = np.linalg.norm(b[ok])
    return float(np.linalg.norm(a[ok] - b[ok]) / (den if den > 0 else 1.0))

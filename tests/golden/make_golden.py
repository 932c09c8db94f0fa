"""Generates the committed golden fixtures of the projection path.

The reference ships no golden vectors, fixtures or tests for this path and
cannot run here (no JDK / ImageJ / ParallelColt), so the fixtures are produced
by the CPU oracle (oracle/tomo_oracle.c, a restatement of the reference's CPU
code) on small seeded inputs.  They pin the oracle against regressions and give
the GPU parity tests fixed inputs and outputs.  Run from the repository root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tomoj_gb300 import phantom as P  # noqa: E402


def case_small():
    """32 x 6 x 24 volume, 9 tilts of 32 x 6, misaligned + noisy series."""
    W, H, D, n = 32, 6, 24, 9
    vol = P.ellipsoid_phantom(W, H, D, 5, 2024)
    angles = np.linspace(-60, 60, n)
    eul = np.array([O.euler_tilt_y(a) for a in angles])
    g = O.Geom(W, H, D, W, H)
    ideal = np.nan_to_num(np.array([O.project(vol, g, e)[0] for e in eul], np.float32))
    T = P.misalignment(n, 2025, max_shift=2.0, max_rot_deg=1.0)
    series = P.add_gaussian_noise(np.array([P.unalign(ideal[i], T[i]) for i in range(n)], np.float32), 0.01, 2026)
    aligned = np.array([O.align(series[i], T[i], fill=O.FILL_NAN) for i in range(n)], np.float32)
    proj = np.zeros((n, H, W), np.float32)
    norm = np.zeros((n, H, W), np.float32)
    for i in range(n):
        proj[i], norm[i] = O.project(vol, g, eul[i])
    bp = np.zeros((D, H, W), np.float32)
    for i in (0, 4, 8):
        O.backproject(bp, g, eul[i], np.nan_to_num(aligned[i]))
    rec = np.zeros((D, H, W), np.float32)
    errs = []
    for it in range(3):
        order = O.order_shuffle(eul, it % n)
        e5, _ = O.ossart_iteration(rec, g, eul, aligned, order, 1.0, 3)
        errs.append(e5)
    mask = O.weighting_mask(W, H, angles, None, 0.5 * W)
    wbp = np.zeros((D, H, W), np.float32)
    O.wbp(wbp, g, eul, np.nan_to_num(aligned), mask)
    tv = vol.copy()
    O.tv_denoise(tv, 25.0, 1.0, 0.01, 5)
    return dict(vol=vol, angles=angles, eul=eul, T=T, series=series, aligned=aligned, proj=proj, norm=norm, bp=bp,
                rec=rec, errs=np.array(errs), mask=mask, wbp=wbp, tv=tv)


def main():
    out = os.path.join(HERE, "oracle_small.npz")
    np.savez_compressed(out, **case_small())
    print(out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()

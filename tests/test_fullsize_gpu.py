"""Parity at the full sizes of the benchmark workloads.

* 256x64x256 volume, 61 tilts of 256x64 (the CPU-runnable SIRT workload): ramp-filtered
  WBP start and 10 SIRT iterations, whole volume against the oracle (<= 1e-4).
* 512x256x512 volume, 61 misaligned tilts of 512x256 (the drop-in workload):
  Hamming-ramp WBP then OS-SART (update 7) on the engine at full size; sampled row
  slabs checked against the oracle run on each slab alone.
* 2048x512x2048 volume, 121 tilts of 2048x512 (the large workload, 8.6 GB): one SIRT
  iteration at full size, sampled row slabs against the oracle.

With a vertical tilt axis and whole-row centre offsets the volume rows are independent
(projection row j sees volume row j - offset only), so the oracle on rows [y0, y1) with
the full volume's centres in slab coordinates (tomoj_gb300.slabs) computes exactly those
rows of the full problem; a halo row keeps the last-row sampler rule off the slab edge.
"""
from __future__ import annotations

import ctypes as C
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import rel_l2
from tomoj_gb300 import _abi, slabs
from tomoj_gb300 import phantom as P

pytestmark = pytest.mark.gpu

TOL_PASS = 1e-5
TOL_ITER = 1e-4


def create(lib, W, H, D, w, h, n, fill=_abi.FILL_NAN):
    g = _abi.make_geom(W, H, D, w, h, n)
    p = _abi.make_params(fill=fill)
    hd = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(g), C.byref(p), C.byref(hd)))
    return hd


def get_rows(lib, hd, W, D, y0, y1):
    out = np.empty((D, y1 - y0, W), np.float32)
    _abi.check(lib.tomo_get_volume(hd, out.ctypes.data, 0, y0, y1))
    return out


def hash_rows(W, D, y0, y1):
    """A white-noise volume in [0, 1) defined per voxel by an integer hash, so any row
    slab is generated alone with the same values: [D][y1 - y0][W] float32."""
    z = np.arange(D, dtype=np.int64)[:, None, None]
    y = np.arange(y0, y1, dtype=np.int64)[None, :, None]
    x = np.arange(W, dtype=np.int64)[None, None, :]
    hv = (x * 73856093 + y * 19349663 + z * 83492791) & 0xFFFFFF
    return (hv.astype(np.float32) * np.float32(1.0 / (1 << 24))).astype(np.float32)


def slab_oracle(W, H, D, w, h, y0, y1, meas):
    """(oracle geometry, cropped measurements, slab) for volume rows [y0, y1)."""
    sl = slabs.slab(W, H, D, w, h, y0, y1)
    g = O.Geom(W, sl.rows, D, w, sl.proj_rows, vc=sl.vol_center, pc=sl.proj_center)
    return g, slabs.crop_series(meas, sl), sl


def on_threads(fn, items):
    """fn over items on host threads (the oracle's C calls release the GIL; its own
    worker pool stays off, so concurrent calls share nothing)."""
    O.set_threads(1)
    with ThreadPoolExecutor(max_workers=max(1, min(len(items), os.cpu_count() or 1))) as ex:
        return list(ex.map(fn, items))


def test_sirt10_full_volume_256x64x256(engine, oracle_lib):
    W, H, D, w, h, n = 256, 64, 256, 256, 64, 61
    angles = np.arange(-60.0, 60.0 + 1e-9, 2.0)
    eul = np.array([O.euler_tilt_y(a) for a in angles])
    g = O.Geom(W, H, D, w, h)
    vol = P.ellipsoid_phantom(W, H, D, 20, 1)
    series = np.nan_to_num(np.array([O.project(vol, g, e)[0] for e in eul], np.float32))
    series = P.add_gaussian_noise(series, 0.01, 2)
    hd = create(engine, W, H, D, w, h, n)
    try:
        e = np.ascontiguousarray(eul, np.float64)
        _abi.check(engine.tomo_load_series(hd, np.ascontiguousarray(series).ctypes.data, 0, _abi.ptr(e, C.c_double),
                                           None, None))
        ang = np.ascontiguousarray(angles, np.float64)
        _abi.check(engine.tomo_set_weighting(hd, _abi.WEIGHT_RAMP, 0.0, _abi.ptr(ang, C.c_double), None))
        _abi.check(engine.tomo_run_wbp(hd, 0, H))
        wbp = get_rows(engine, hd, W, D, 0, H)
        _abi.check(engine.tomo_set_weighting(hd, _abi.WEIGHT_NONE, 0.0, None, None))
        n_iter, seed = 10, 3
        err = np.zeros((n_iter, 5))
        _abi.check(engine.tomo_run_ossart(hd, n_iter, 1.0, 0, seed, 0, H, 1, _abi.ptr(err, C.c_double)))
        got = get_rows(engine, hd, W, D, 0, H)
        firsts = [int(engine.tomo_first_index(seed, it, n)) for it in range(n_iter)]
    finally:
        engine.tomo_destroy(hd)
    O.set_threads(os.cpu_count() or 1)
    try:
        ref = np.zeros((D, H, W), np.float32)
        O.wbp(ref, g, eul, series, O.ramp_mask(w, h, angles))
        assert rel_l2(wbp, ref) <= TOL_PASS, rel_l2(wbp, ref)
        for it in range(n_iter):
            e5, _ = O.ossart_iteration(ref, g, eul, series, O.order_shuffle(eul, firsts[it]), 1.0, 0)
            assert np.allclose(err[it, [0, 1, 3]], e5[[0, 1, 3]], rtol=1e-4), it
    finally:
        O.set_threads(1)
    assert rel_l2(got, ref) <= TOL_ITER, rel_l2(got, ref)


def test_ossart_slabs_full_size_512x256x512(engine, oracle_lib):
    W, H, D, w, h, n = 512, 256, 512, 512, 256, 61
    rng = np.random.default_rng(21)
    angles = np.linspace(-60.0, 60.0, n)
    eul = np.array([O.euler_tilt_y(a) for a in angles])
    T = np.zeros((n, 6))
    for i in range(n):
        a = np.deg2rad(rng.uniform(-1.0, 1.0))
        T[i] = [np.cos(a), np.sin(a), -np.sin(a), np.cos(a), rng.uniform(-5, 5), rng.uniform(-5, 5)]
    series = (rng.random((n, h, w), dtype=np.float32) + np.float32(0.5)).astype(np.float32)
    stats = np.array([[series[i].mean(dtype=np.float64), series[i].std(dtype=np.float64)] for i in range(n)])
    n_iter, update, seed = 2, 7, 9
    samples = [(0, 6), (125, 131), (250, 256)]
    hd = create(engine, W, H, D, w, h, n)
    try:
        # WBP on average-filled projections, OS-SART on NaN-filled ones (as the benchmark job)
        e = np.ascontiguousarray(eul, np.float64)
        _abi.check(engine.tomo_load_series(hd, series.ctypes.data, 0, _abi.ptr(e, C.c_double),
                                           _abi.ptr(np.ascontiguousarray(T), C.c_double),
                                           _abi.ptr(np.ascontiguousarray(stats), C.c_double)))
        _abi.check(engine.tomo_set_weighting(hd, _abi.WEIGHT_HAMMING_RAMP, 0.0, None, None))
        _abi.check(engine.tomo_set_fill(hd, _abi.FILL_AVG))
        _abi.check(engine.tomo_run_wbp(hd, 0, H))
        wbp = [get_rows(engine, hd, W, D, y0, y1) for y0, y1 in samples]
        _abi.check(engine.tomo_set_weighting(hd, _abi.WEIGHT_NONE, 0.0, None, None))
        _abi.check(engine.tomo_set_fill(hd, _abi.FILL_NAN))
        _abi.check(engine.tomo_run_ossart(hd, n_iter, 1.0, update, seed, 0, H, 1, None))
        got = [get_rows(engine, hd, W, D, y0, y1) for y0, y1 in samples]
        firsts = [int(engine.tomo_first_index(seed, it, n)) for it in range(n_iter)]
    finally:
        engine.tomo_destroy(hd)
    avg = np.array([O.align(series[i], T[i], False, stats[i, 0], stats[i, 1], O.FILL_AVG) for i in range(n)],
                   np.float32)
    meas = np.array([O.align(series[i], T[i], fill=O.FILL_NAN) for i in range(n)], np.float32)
    mask = O.ramp_mask(w, h, np.rad2deg(np.arctan2(eul[:, 2, 0], eul[:, 2, 2])), hamming=True)
    # WBP weights whole projections: weight, then crop per slab
    weighted = np.array([O.weighting_apply(avg[i], mask) for i in range(n)], np.float32)

    def one(k):
        y0, y1 = samples[k]
        g, sub, sl = slab_oracle(W, H, D, w, h, y0, y1, meas)
        ref = np.zeros((D, sl.rows, W), np.float32)
        O.wbp(ref, g, eul, slabs.crop_series(weighted, sl, halo_nan=False), None)
        ref_wbp = ref[:, :y1 - y0, :].copy()
        for it in range(n_iter):
            O.ossart_iteration(ref, g, eul, sub, O.order_shuffle(eul, firsts[it]), 1.0, update)
        return ref_wbp, ref[:, :y1 - y0, :]

    for k, (ref_wbp, ref) in enumerate(on_threads(one, list(range(len(samples))))):
        assert rel_l2(wbp[k], ref_wbp) <= TOL_PASS, (samples[k], rel_l2(wbp[k], ref_wbp))
        assert rel_l2(got[k], ref) <= TOL_ITER, (samples[k], rel_l2(got[k], ref))


def test_sirt_slabs_full_size_2048x512x2048(engine, oracle_lib):
    W, H, D, w, h, n = 2048, 512, 2048, 2048, 512, 121
    angles = np.linspace(-60.0, 60.0, n)
    eul = np.array([O.euler_tilt_y(a) for a in angles])
    rng = np.random.default_rng(33)
    series = (rng.random((n, h, w), dtype=np.float32) * np.float32(200.0)).astype(np.float32)
    # single rows: first, middle, last (each with the oracle on one thread: ~1e9 updates)
    samples = [(0, 1), (300, 301), (511, 512)]
    hd = create(engine, W, H, D, w, h, n)
    try:
        e = np.ascontiguousarray(eul, np.float64)
        _abi.check(engine.tomo_load_series(hd, series.ctypes.data, 0, _abi.ptr(e, C.c_double), None, None))
        for y0 in range(0, H, 8):
            rows = hash_rows(W, D, y0, min(H, y0 + 8))
            _abi.check(engine.tomo_set_volume(hd, rows.ctypes.data, 0, y0, min(H, y0 + 8)))
        _abi.check(engine.tomo_run_ossart(hd, 1, 1.0, 0, 4, 0, H, 1, None))
        got = [get_rows(engine, hd, W, D, y0, y1) for y0, y1 in samples]
        first = int(engine.tomo_first_index(4, 0, n))
    finally:
        engine.tomo_destroy(hd)
    order = O.order_shuffle(eul, first)

    def one(k):
        y0, y1 = samples[k]
        g, sub, sl = slab_oracle(W, H, D, w, h, y0, y1, series)
        ref = np.ascontiguousarray(hash_rows(W, D, y0, y1 + sl.halo))
        O.ossart_iteration(ref, g, eul, sub, order, 1.0, 0)
        return ref[:, :y1 - y0, :]

    for k, ref in enumerate(on_threads(one, list(range(len(samples))))):
        assert rel_l2(got[k], ref) <= TOL_ITER, (samples[k], rel_l2(got[k], ref))

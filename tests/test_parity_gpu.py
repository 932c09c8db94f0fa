"""GPU parity: the engine (through its C ABI) against the CPU oracle on the same seeded inputs.

Tolerances (plain FP32 form): <= 1e-5 relative L2 per forward / backprojection
pass and <= 1e-4 after 10 SIRT iterations; norms and NaN patterns exactly.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests.cases import rel_l2, series_case
from tomoj_gb300 import _abi

pytestmark = pytest.mark.gpu

TOL_PASS = 1e-5
TOL_SIRT10 = 1e-4


class Handle:
    def __init__(self, lib, case, positivity=False, long_object=False, fill=_abi.FILL_NAN, normalize=False,
                 vol=None):
        self.lib = lib
        self.c = case
        g = _abi.make_geom(case["W"], case["H"], case["D"], case["w"], case["h"], case["n"])
        p = _abi.make_params(positivity=positivity, long_object=long_object, fill=fill, normalize=normalize)
        h = C.c_void_p()
        _abi.check(lib.tomo_create(C.byref(g), C.byref(p), C.byref(h)))
        self.h = h
        eul = np.ascontiguousarray(case["eul"], np.float64)
        T = np.ascontiguousarray(case["T"], np.float64)
        series = np.ascontiguousarray(case["series"], np.float32)
        _abi.check(lib.tomo_load_series(h, series.ctypes.data, 0, _abi.ptr(eul, C.c_double),
                                        _abi.ptr(T, C.c_double), None))
        if vol is not None:
            self.set_volume(vol)

    def set_volume(self, vol):
        v = np.ascontiguousarray(vol, np.float32)
        _abi.check(self.lib.tomo_set_volume(self.h, v.ctypes.data, 0, 0, v.shape[1]))

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


def oracle_aligned(case, fill=O.FILL_NAN):
    return np.array([O.align(case["series"][i], case["T"][i], fill=fill) for i in range(case["n"])], np.float32)


@pytest.fixture(scope="module")
def case():
    return series_case(W=64, H=12, D=48, n=21, misalign=True)


def test_forward_projection_matches_oracle(engine, oracle_lib, case):
    vol = case["vol"] + np.float32(0.05) * np.random.default_rng(3).random(case["vol"].shape, dtype=np.float32)
    hd = Handle(engine, case, vol=vol)
    try:
        for i in range(case["n"]):
            _abi.check(engine.tomo_add_projection(hd.h, i))
        _abi.check(engine.tomo_project(hd.h, 0, case["H"]))
        for i in range(case["n"]):
            p_ref, n_ref = O.project(vol, case["g"], case["eul"][i])
            p = hd.slot(engine.tomo_get_projection, i)
            n = hd.slot(engine.tomo_get_norm, i)
            assert np.array_equal(np.isnan(p), np.isnan(p_ref)), f"NaN pattern differs at tilt {i}"
            assert np.array_equal(n, n_ref), f"norms differ at tilt {i}"
            assert rel_l2(p, p_ref) <= TOL_PASS, (i, rel_l2(p, p_ref))
    finally:
        hd.close()


def test_projection_difference_matches_oracle(engine, oracle_lib, case):
    hd = Handle(engine, case, vol=case["vol"] * np.float32(0.8))
    try:
        meas = oracle_aligned(case)
        idx = [3, 17, 0, 9]
        for i in idx:
            _abi.check(engine.tomo_add_projection(hd.h, i))
        factor = float(np.float32(1.0 / 7))
        err = np.zeros(len(idx))
        _abi.check(engine.tomo_project_and_difference(hd.h, factor, 0, case["H"], _abi.ptr(err, C.c_double)))
        for k, i in enumerate(idx):
            p_ref, n_ref = O.project(hd.c["vol"] * np.float32(0.8), case["g"], case["eul"][i])
            d_ref, e_ref = O.difference(meas[i], p_ref, n_ref, factor)
            d = hd.slot(engine.tomo_get_difference, k)
            assert rel_l2(d, d_ref) <= TOL_PASS, (i, rel_l2(d, d_ref))
            assert abs(err[k] - e_ref) <= 1e-5 * abs(e_ref), (err[k], e_ref)
    finally:
        hd.close()


@pytest.mark.parametrize("kind", ["smooth", "noise"])
def test_backprojection_matches_oracle(engine, oracle_lib, case, kind):
    rng = np.random.default_rng(11)
    hd = Handle(engine, case)
    try:
        if kind == "noise":
            imgs = rng.normal(0, 1, (case["n"], case["h"], case["w"])).astype(np.float32)
        else:
            imgs = oracle_aligned(case)
            imgs = np.nan_to_num(imgs)
        # backproject the images as "original projections": load them as the series, identity alignment
        c2 = dict(case, series=imgs, T=np.tile([1.0, 0, 0, 1, 0, 0], (case["n"], 1)))
        hd.close()
        hd = Handle(engine, c2)
        start = rng.random((case["D"], case["H"], case["W"]), dtype=np.float32)
        hd.set_volume(start)
        order = [5, 0, 20, 11, 2]
        for i in order:
            _abi.check(engine.tomo_add_projection(hd.h, i))
        _abi.check(engine.tomo_backproject(hd.h, 0, case["H"]))
        got = hd.volume()
        ref = start.copy()
        for i in order:
            O.backproject(ref, case["g"], case["eul"][i], imgs[i])
        assert rel_l2(got - start, ref - start) <= TOL_PASS, rel_l2(got - start, ref - start)
    finally:
        hd.close()


@pytest.mark.parametrize("positivity", [False, True])
@pytest.mark.parametrize("shape", [(64, 12, 48), (70, 7, 75)])
def test_backprojection_row_pairs_match_one_row_and_oracle(engine, oracle_lib, shape, positivity):
    """Two volume rows per backprojection thread (forced; the size rule would pick one row
    for volumes this small): bitwise the one-row kernel, and the oracle to 1e-5.  An odd
    row count leaves the last pair with one row; a sub-range of rows must leave the rows
    outside it untouched."""
    W, H, D = shape
    c = series_case(W=W, H=H, D=D, n=9, seed=17, noise=0.0)
    rng = np.random.default_rng(4)
    imgs = rng.normal(0, 1, (c["n"], c["h"], c["w"])).astype(np.float32)
    c2 = dict(c, series=imgs, T=np.tile([1.0, 0, 0, 1, 0, 0], (c["n"], 1)))
    start = rng.standard_normal((D, H, W)).astype(np.float32)
    order = [4, 0, 8, 2, 6, 1]
    y0, y1 = 1, H
    got = {}
    for rows in (1, 2):
        hd = Handle(engine, c2, positivity=positivity, vol=start)
        try:
            _abi.check(engine.tomo_set_bp_rows(hd.h, rows))
            for i in order:
                _abi.check(engine.tomo_add_projection(hd.h, i))
            _abi.check(engine.tomo_backproject(hd.h, y0, y1))
            got[rows] = hd.volume()
        finally:
            hd.close()
    assert np.array_equal(got[1].view(np.uint32), got[2].view(np.uint32))
    assert np.array_equal(got[2][:, :y0], start[:, :y0])
    ref = start.copy()
    g = O.Geom(W, H, D, W, H, positivity=positivity)
    for i in order:
        O.backproject(ref, g, c["eul"][i], imgs[i], y0, y1)
    assert rel_l2(got[2] - start, ref - start) <= TOL_PASS, rel_l2(got[2] - start, ref - start)


def test_alignment_matches_oracle(engine, oracle_lib, case):
    hd = Handle(engine, case)
    try:
        for i in range(case["n"]):
            ref = O.align(case["series"][i], case["T"][i], fill=O.FILL_NAN)
            got = hd.slot(engine.tomo_get_aligned, i)
            assert np.array_equal(np.isnan(got), np.isnan(ref))
            ok = ~np.isnan(ref)
            assert np.max(np.abs(got[ok] - ref[ok])) <= 1e-6 * max(1.0, np.max(np.abs(ref[ok])))
    finally:
        hd.close()


def test_sirt_10_iterations_matches_oracle(engine, oracle_lib):
    c = series_case(W=48, H=8, D=32, n=15, seed=21, misalign=False)
    hd = Handle(engine, c)
    try:
        n_iter, seed = 10, 99
        err = np.zeros((n_iter, 5))
        _abi.check(engine.tomo_run_ossart(hd.h, n_iter, 1.0, 0, seed, 0, c["H"], 1, _abi.ptr(err, C.c_double)))
        got = hd.volume()
        ref = np.zeros_like(c["vol"])
        meas = oracle_aligned(c)
        errs = []
        for it in range(n_iter):
            order = O.order_shuffle(c["eul"], int(engine.tomo_first_index(seed, it, c["n"])))
            e5, _ = O.ossart_iteration(ref, c["g"], c["eul"], meas, order, 1.0, 0)
            errs.append(e5)
        errs = np.array(errs)
        assert rel_l2(got, ref) <= TOL_SIRT10, rel_l2(got, ref)
        assert np.allclose(err[:, 0], errs[:, 0], rtol=1e-4)
    finally:
        hd.close()


def test_ossart_subsets_match_oracle(engine, oracle_lib, case):
    hd = Handle(engine, case)
    try:
        n_iter, seed, update = 2, 5, 4
        err = np.zeros((n_iter, 5))
        _abi.check(engine.tomo_run_ossart(hd.h, n_iter, 0.8, update, seed, 0, case["H"], 0,
                                          _abi.ptr(err, C.c_double)))
        got = hd.volume()
        ref = np.zeros_like(case["vol"])
        meas = oracle_aligned(case)
        for it in range(n_iter):
            order = O.order_shuffle(case["eul"], int(engine.tomo_first_index(seed, it, case["n"])))
            e5, _ = O.ossart_iteration(ref, case["g"], case["eul"], meas, order, 0.8, update)
            assert np.allclose(err[it, [0, 1, 3]], e5[[0, 1, 3]], rtol=1e-4)
            assert err[it, 2] == e5[2] and err[it, 4] == e5[4]
        assert rel_l2(got, ref) <= 1e-5 * 10, rel_l2(got, ref)
    finally:
        hd.close()


def test_graph_and_eager_iterations_are_bitwise_equal(engine, case):
    vols = []
    for use_graph in (0, 1):
        hd = Handle(engine, case)
        try:
            _abi.check(engine.tomo_run_ossart(hd.h, 3, 1.0, 5, 17, 0, case["H"], use_graph, None))
            vols.append(hd.volume())
        finally:
            hd.close()
    assert np.array_equal(vols[0], vols[1])


def test_wbp_radermacher_matches_oracle(engine, oracle_lib):
    c = series_case(W=64, H=8, D=40, n=21, seed=4, misalign=False, noise=0.0)
    hd = Handle(engine, c, fill=_abi.FILL_AVG)
    try:
        radius = 0.5
        _abi.check(engine.tomo_set_weighting(hd.h, _abi.WEIGHT_RADERMACHER, radius, None, None))
        _abi.check(engine.tomo_run_wbp(hd.h, 0, c["H"]))
        got = hd.volume()
        ref = np.zeros_like(c["vol"])
        mask = O.weighting_mask(c["w"], c["h"], c["angles"], None, radius * c["w"])
        O.wbp(ref, c["g"], c["eul"], c["series"], mask)
        assert rel_l2(got, ref) <= TOL_PASS, rel_l2(got, ref)
    finally:
        hd.close()


@pytest.mark.parametrize("W", [60, 100, 37])
def test_wbp_radermacher_any_width_matches_oracle(engine, oracle_lib, W):
    # widths that are not powers of two go through the circular-convolution row filter
    c = series_case(W=W, H=6, D=30, n=15, seed=6, misalign=False, noise=0.0)
    hd = Handle(engine, c, fill=_abi.FILL_AVG)
    try:
        radius = 0.45
        _abi.check(engine.tomo_set_weighting(hd.h, _abi.WEIGHT_RADERMACHER, radius, None, None))
        _abi.check(engine.tomo_run_wbp(hd.h, 0, c["H"]))
        got = hd.volume()
        ref = np.zeros_like(c["vol"])
        mask = O.weighting_mask(c["w"], c["h"], c["angles"], None, radius * c["w"])
        O.wbp(ref, c["g"], c["eul"], c["series"], mask)
        assert rel_l2(got, ref) <= TOL_PASS, rel_l2(got, ref)
    finally:
        hd.close()


def test_tvm_iteration_matches_oracle(engine, oracle_lib):
    c = series_case(W=40, H=8, D=24, n=11, seed=8)
    hd = Handle(engine, c)
    try:
        _abi.check(engine.tomo_set_tvm(hd.h, 25.0, 1.0, 0.01, 5))
        _abi.check(engine.tomo_run_ossart(hd.h, 2, 1.0, 0, 3, 0, c["H"], 1, None))
        got = hd.volume()
        ref = np.zeros_like(c["vol"])
        meas = oracle_aligned(c)
        for it in range(2):
            order = O.order_shuffle(c["eul"], int(engine.tomo_first_index(3, it, c["n"])))
            O.ossart_iteration(ref, c["g"], c["eul"], meas, order, 1.0, 0)
            O.tv_denoise(ref, 25.0, 1.0, 0.01, 5)
        assert rel_l2(got, ref) <= 1e-5 * 10, rel_l2(got, ref)
    finally:
        hd.close()


@pytest.mark.parametrize("shape", [(70, 19, 75), (33, 9, 33), (2, 3, 40)])
def test_tv_denoise_matches_oracle_bitwise(engine, oracle_lib, shape):
    """The fused TV step (one kernel per inner step, u rebuilt in shared memory) against
    TotalVariationDenoising_3D's updateP / updateU sequence: identical float expressions
    in the same order, so the denoised volume is the oracle's bit for bit.  The shapes
    cover several x / y / z tiles of the kernel, ragged tile edges and a two-column volume."""
    W, H, D = shape
    c = series_case(W=W, H=H, D=D, n=3, seed=21)
    rng = np.random.default_rng(5)
    vol = (rng.standard_normal((D, H, W)) * 3.0).astype(np.float32)
    hd = Handle(engine, c, vol=vol)
    try:
        _abi.check(engine.tomo_set_tvm(hd.h, 25.0, 1.0, 0.01, 5))
        _abi.check(engine.tomo_end_iteration(hd.h))
        got = hd.volume()
        ref = vol.copy()
        O.tv_denoise(ref, 25.0, 1.0, 0.01, 5)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), float(np.abs(got - ref).max())
    finally:
        hd.close()


@pytest.mark.parametrize("shape", [(30, 5, 17, 30, 5), (64, 8, 64, 64, 12), (20, 6, 9, 24, 6)])
def test_odd_shapes_positivity_long_object(engine, oracle_lib, shape):
    W, H, D, w, h = shape
    c = series_case(W=W, H=H, D=D, n=9, seed=13, w=w, h=h, noise=0.0)
    for pos, lo in ((True, False), (False, True)):
        hd = Handle(engine, c, positivity=pos, long_object=lo)
        try:
            g = O.Geom(W, H, D, w, h, positivity=pos, long_object=lo)
            meas = oracle_aligned(c)
            err = np.zeros((1, 5))
            _abi.check(engine.tomo_run_ossart(hd.h, 1, 1.0, 3, 1, 0, H, 0, _abi.ptr(err, C.c_double)))
            got = hd.volume()
            ref = np.zeros_like(c["vol"])
            order = O.order_shuffle(c["eul"], int(engine.tomo_first_index(1, 0, c["n"])))
            O.ossart_iteration(ref, g, c["eul"], meas, order, 1.0, 3)
            if h == H:
                assert rel_l2(got, ref) <= TOL_PASS * 10, (shape, pos, lo, rel_l2(got, ref))
            else:
                # h > H: the reference reports Inf errors for the uncomputed rows; volumes still agree
                assert rel_l2(got, ref) <= TOL_PASS * 10, (shape, pos, lo, rel_l2(got, ref))
        finally:
            hd.close()


def test_repeat_runs_are_bitwise_identical(engine, case):
    outs = []
    for _ in range(2):
        hd = Handle(engine, case)
        try:
            _abi.check(engine.tomo_run_ossart(hd.h, 2, 1.0, 0, 4, 0, case["H"], 1, None))
            outs.append(hd.volume())
        finally:
            hd.close()
    assert np.array_equal(outs[0], outs[1])

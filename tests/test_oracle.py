"""The CPU oracle: regression pin against the committed golden fixtures, analytic
known-answer cases, and agreement with the independent FP64 numpy twin.

Parity of the oracle with the reference itself is unpinned: the reference has no
golden vectors for this path and cannot be run here (no JDK / jars)."""
from __future__ import annotations

import os

import numpy as np
import pytest

from oracle import np_oracle as N
from oracle import oracle as O
from tests.cases import rel_l2, series_case
from tests.golden.make_golden import case_small

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz")


@pytest.fixture(scope="module")
def golden(oracle_lib):
    return dict(np.load(GOLDEN))


def test_oracle_reproduces_golden_fixtures(golden):
    # bitwise on the machine that wrote them; libm's sin/cos may differ by an ulp elsewhere
    fresh = case_small()
    for k, v in golden.items():
        assert np.array_equal(np.isnan(fresh[k]), np.isnan(v)), k
        assert rel_l2(fresh[k], v) <= 1e-6, k


def test_constant_volume_forward_projection_is_ray_length(oracle_lib):
    W, H, D = 24, 4, 16
    vol = np.ones((D, H, W), np.float32)
    g = O.Geom(W, H, D, W, H)
    p, n = O.project(vol, g, O.euler_tilt_y(0.0))
    assert np.all(p == D) and np.all(n == D)  # every ray crosses D unit voxels, normIncrement 1
    p, n = O.project(vol, g, O.euler_tilt_y(30.0))
    ok = ~np.isnan(p)
    ninc = 1.0 / np.cos(np.deg2rad(30.0))
    # count samples of 1 -> ray sum * ninc; the norm adds one more increment when the
    # ray leaves the volume through a side face (VoxelProjector3D.java:780-783)
    side = ~np.isclose(p[ok], n[ok], rtol=1e-6)
    assert np.allclose(p[ok][side], n[ok][side] - ninc, rtol=1e-5)
    assert side.any() and (~side).any()


def test_backprojection_of_constant_at_zero_tilt(oracle_lib):
    W, H, D = 20, 3, 10
    g = O.Geom(W, H, D, W, H)
    vol = np.zeros((D, H, W), np.float32)
    O.backproject(vol, g, O.euler_tilt_y(0.0), np.full((H, W), 2.5, np.float32))
    assert np.all(vol == 2.5)


def test_single_tilt_radermacher_mask_closed_form(oracle_lib):
    w, h, dm = 16, 4, 8.0
    m0 = O.weighting_mask(w, h, [0.0], None, dm)
    assert np.allclose(m0, 1.0 / dm)  # sinc(0) = 1 for every frequency
    th = 30.0
    m = O.weighting_mask(w, h, [th], None, dm)
    i = np.arange(w)
    ci = np.where(i > w / 2.0, i - w, i).astype(np.float64)
    v = dm * np.pi * ci * np.sin(np.deg2rad(th)) / w
    s = np.where(v == 0, 1.0, np.sin(v) / np.where(v == 0, 1, v))
    ref = (1.0 / (np.maximum(s, 0.005) * dm)).astype(np.float32)
    assert np.allclose(m, np.broadcast_to(ref, (h, w)), rtol=1e-6)


def test_tv_leaves_constant_volume_unchanged(oracle_lib):
    vol = np.full((6, 5, 7), 3.0, np.float32)
    out = vol.copy()
    O.tv_denoise(out, 25.0, 1.0, 0.1, 5)
    assert np.array_equal(out, vol)


def test_tv_step_function_against_hand_computed_step(oracle_lib):
    # two voxels along x: u = f = [0, 1]; one ROF step with theta=1, g=1, dt=1
    f = np.array([[[0.0, 1.0]]], np.float32)
    out = f.copy()
    O.tv_denoise(out, 1.0, 1.0, 1.0, 1)
    # updateP: dux(0) = 1, |grad| = 1, dd = 2 -> px(0) = (0 - 1) / 2 = -0.5, px(1) = 0
    # updateU: div(0) = px(0) = -0.5, div(1) = -px(1) = 0 -> u = f - div = [0.5, 1]
    assert np.allclose(out.ravel(), [0.5, 1.0])


@pytest.mark.parametrize("theta", [-60.0, -37.0, 0.0, 2.0, 45.0, 60.0])
def test_c_oracle_matches_fp64_twin_forward(oracle_lib, theta):
    c = series_case(W=40, H=6, D=30, n=3, noise=0.0)
    vol = c["vol"]
    g = c["g"]
    p, n = O.project(vol, g, O.euler_tilt_y(theta))
    p2, n2 = N.project(vol, g, N.euler_tilt_y(theta))
    assert np.array_equal(np.isnan(p), np.isnan(p2))
    assert rel_l2(p, p2) < 1e-6
    assert np.allclose(n, n2, rtol=1e-6)


def test_c_oracle_matches_fp64_twin_general_geometry(oracle_lib):
    c = series_case(W=40, H=10, D=30, n=3, noise=0.0)
    R = O.euler(10.0, 40.0, -10.0)
    p, _ = O.project(c["vol"], c["g"], R)
    p2, _ = N.project(c["vol"], c["g"], N.euler(10.0, 40.0, -10.0))
    ok = ~np.isnan(p) & ~np.isnan(p2)
    assert rel_l2(p[ok], p2[ok]) < 1e-6
    img = np.random.default_rng(1).normal(0, 1, (10, 40)).astype(np.float32)
    v1 = np.zeros_like(c["vol"])
    O.backproject(v1, c["g"], R, img)
    v2 = np.zeros(c["vol"].shape)
    N.backproject(v2, c["g"], R, img)
    assert rel_l2(v1, v2) < 1e-6


def test_c_oracle_matches_fp64_twin_backprojection_alignment_weighting(oracle_lib):
    rng = np.random.default_rng(0)
    W, H, D = 32, 6, 20
    g = O.Geom(W, H, D, W, H)
    img = rng.normal(0, 1, (H, W)).astype(np.float32)
    for th in (-55.0, 0.0, 33.0):
        v1 = np.zeros((D, H, W), np.float32)
        O.backproject(v1, g, O.euler_tilt_y(th), img)
        v2 = np.zeros((D, H, W))
        N.backproject(v2, g, N.euler_tilt_y(th), img)
        assert rel_l2(v1, v2) < 1e-6
    T = (np.cos(0.01), np.sin(0.01), -np.sin(0.01), np.cos(0.01), 1.3, -2.2)
    a1 = O.align(img, T)
    a2 = N.align(img, T)
    assert np.array_equal(np.isnan(a1), np.isnan(a2))
    assert np.nanmax(np.abs(a1 - a2)) < 1e-6
    tilts = np.arange(-60, 61, 3.0)
    m1 = O.weighting_mask(W, H, tilts, None, 0.5 * W)
    m2 = N.weighting_mask(W, H, tilts, None, 0.5 * W)
    assert np.allclose(m1, m2, rtol=1e-6)
    assert rel_l2(O.weighting_apply(img, m1), N.weighting_apply(img, m1.astype(np.float64))) < 1e-6


def test_c_oracle_matches_fp64_twin_tv(oracle_lib):
    vol = series_case(W=20, H=5, D=12, n=1, noise=0.0)["vol"]
    t1 = vol.copy()
    O.tv_denoise(t1, 25.0, 1.0, 0.1, 5)
    assert rel_l2(t1, N.tv_denoise(vol, 25.0, 1.0, 0.1, 5)) < 1e-6


def test_c_oracle_matches_fp64_twin_ossart(oracle_lib):
    c = series_case(W=32, H=4, D=20, n=9, seed=3, misalign=True)
    meas = np.array([O.align(c["series"][i], c["T"][i]) for i in range(c["n"])], np.float32)
    order = O.order_shuffle(c["eul"], 4)
    assert np.array_equal(order, N.order_shuffle(list(c["eul"]), 4))
    v1 = np.zeros_like(c["vol"])
    v2 = np.zeros(c["vol"].shape)
    for _ in range(2):
        e1, _ = O.ossart_iteration(v1, c["g"], c["eul"], meas, order, 1.0, 3)
        e2 = N.ossart_iteration(v2, c["g"], c["eul"], meas, order, 1.0, 3)
        assert np.allclose(e1[[0, 1, 3]], e2[[0, 1, 3]], rtol=1e-5)
        assert e1[2] == e2[2] and e1[4] == e2[4]
    assert rel_l2(v1, v2) < 1e-5


def test_multithreaded_oracle_is_bitwise_deterministic(oracle_lib):
    c = series_case(W=32, H=8, D=20, n=7, seed=9)
    outs = []
    for th in (1, 4):
        O.set_threads(th)
        v = np.zeros_like(c["vol"])
        order = O.order_shuffle(c["eul"], 0)
        O.ossart_iteration(v, c["g"], c["eul"], c["series"], order, 1.0, 0)
        outs.append(v)
    O.set_threads(1)
    assert np.array_equal(outs[0], outs[1])


def test_order_shuffle_picks_most_perpendicular(oracle_lib):
    eul = np.array([O.euler_tilt_y(a) for a in np.arange(-60, 61, 2.0)])
    idx = O.order_shuffle(eul, 30)  # 0 degrees first
    assert idx[0] == 30 and sorted(idx) == list(range(61))
    # from 0 deg the beam is most perpendicular to +-60 deg; the first of equals wins
    assert idx[1] == 0


def test_bayesian_stencil_is_zero_padded_mixed_second_difference(oracle_lib):
    # BayesianVoxelProjector3D.startOfIteration: -lambda * sum of the 3x3x3 neighbours weighted
    # by [1,-2,1]^3, out-of-volume neighbours 0 (getCubicNeightborhoodWithClamp reads getPixel)
    rng = np.random.default_rng(5)
    D, H, W = 6, 5, 7
    vol = rng.uniform(-1, 1, (D, H, W)).astype(np.float32)
    k1 = np.array([1.0, -2.0, 1.0])
    pad = np.pad(vol.astype(np.float64), 1)
    ref = np.zeros((D, H, W))
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                ref += k1[dz] * k1[dy] * k1[dx] * pad[dz:dz + D, dy:dy + H, dx:dx + W]
    lam = 0.3
    dist = np.zeros_like(vol)
    O.lib().or_bayes_start(vol.ctypes.data_as(O.C.POINTER(O.C.c_float)),
                           dist.ctypes.data_as(O.C.POINTER(O.C.c_float)), W, H, D, lam)
    assert np.allclose(dist, -lam * ref, rtol=1e-6, atol=1e-6)
    # a linear ramp has zero mixed second differences away from the border
    ramp = np.fromfunction(lambda z, y, x: x + 2 * y + 3 * z, (D, H, W)).astype(np.float32)
    O.lib().or_bayes_start(ramp.ctypes.data_as(O.C.POINTER(O.C.c_float)),
                           dist.ctypes.data_as(O.C.POINTER(O.C.c_float)), W, H, D, lam)
    assert np.all(dist[1:-1, 1:-1, 1:-1] == 0)


def test_bayesian_iteration_backprojects_into_the_distance_volume(oracle_lib):
    # with lambda = 0 and alpha = 1 one Bayesian iteration is a SIRT iteration whose
    # projections all see the volume at the start of the iteration: for update = nproj
    # (SIRT) that equals plain SIRT exactly
    c = series_case(W=32, H=4, D=24, n=7, seed=2, noise=0.0)
    meas = np.array([O.align(c["series"][i], c["T"][i], fill=O.FILL_NAN) for i in range(c["n"])], np.float32)
    order = O.order_shuffle(c["eul"], 0)
    a = np.zeros_like(c["vol"])
    b = np.zeros_like(c["vol"])
    O.ossart_iteration(a, c["g"], c["eul"], meas, order, 1.0, 0)
    O.bayesian_iteration(b, c["g"], c["eul"], meas, order, 1.0, 0, 0.0, 1.0)
    assert rel_l2(b, a) < 1e-6
    # with subsets the Bayesian form differs (later subsets project the unchanged volume)
    a2 = np.zeros_like(c["vol"])
    b2 = np.zeros_like(c["vol"])
    O.ossart_iteration(a2, c["g"], c["eul"], meas, order, 1.0, 2)
    O.bayesian_iteration(b2, c["g"], c["eul"], meas, order, 1.0, 2, 0.0, 1.0)
    assert rel_l2(b2, a2) > 1e-3


def _median_cross_numpy(vol):
    # BgARTVoxelProjector3D.medianFilter3Dcross written out independently
    D, H, W = vol.shape
    P = W * H
    out = np.empty_like(vol)
    flat = vol.reshape(D, P)
    for z in range(D):
        for idx in range(P):
            nb = [flat[z - 1, idx] if z > 0 else 0.0, flat[z + 1, idx] if z < D - 1 else 0.0, flat[z, idx],
                  flat[z, idx + 1] if idx + 1 < P else 0.0, flat[z, idx - 1] if idx - 1 > 0 else 0.0,
                  flat[z, idx - W] if idx - W > 0 else 0.0, flat[z, idx + W] if idx + W < P else 0.0]
            out.reshape(D, P)[z, idx] = sorted(nb)[3]
    return out


def test_bgart_median_cross_matches_its_definition(oracle_lib):
    rng = np.random.default_rng(8)
    vol = rng.normal(0, 1, (4, 5, 6)).astype(np.float32)
    ref = _median_cross_numpy(vol)
    got = O.bgart_median_cross(vol.copy())
    assert np.array_equal(got, ref)


def test_bgart_collapse_snaps_background_side_to_the_mode(oracle_lib):
    rng = np.random.default_rng(9)
    n = 20000
    v = np.zeros(n, np.float32)
    v[:12000] = rng.normal(0.0, 0.05, 12000)        # background around 0
    v[12000:] = rng.uniform(0.5, 1.0, n - 12000)    # object
    vol = v.reshape(10, 40, 50).copy()
    k = 2.0
    bg = O.bgart_collapse(vol, k, True)
    # recompute the thresholds from the stated histogram rules
    lo, hi = float(v.min()), float(v.max())
    b = np.minimum(((v.astype(np.float64) - lo) * (256.0 / (hi - lo))).astype(np.int64), 255)
    hist = np.bincount(b, minlength=256)
    mi = int(np.argmax(hist))
    binw = (hi - lo) / 256
    mode = lo + mi * binw
    centers = lo + np.arange(mi) * binw
    sigma = np.sqrt(np.sum((centers - mode) ** 2 * hist[:mi]) / hist[:mi].sum())
    assert bg == pytest.approx(mode)
    expect = np.where(v.astype(np.float64) < mode + k * sigma, np.float32(mode), v).reshape(vol.shape)
    assert np.array_equal(vol, expect)
    # bright-background variant keeps the dark side and snaps the rest
    vol2 = v.reshape(10, 40, 50).copy()
    O.bgart_collapse(vol2, k, False)
    expect2 = np.where(v.astype(np.float64) > mode - k * sigma, np.float32(mode), v).reshape(vol.shape)
    assert np.array_equal(vol2, expect2)


def test_dual_iteration_flushes_like_the_reference(oracle_lib, monkeypatch):
    # osartIterationDual with n1 = 5, n2 = 4, update = 3: two projections of each series
    # in turn, one shared counter; series 1's last projection is never reached (t < n1 - 1)
    flushed = []

    def record(vol, g, eul, meas, batch, factor, y0=0, y1=None):
        flushed.append((g.tag, list(batch)))
        return np.zeros(len(batch))

    monkeypatch.setattr(O, "update_step", record)
    g1, g2 = O.Geom(4, 2, 4, 4, 2), O.Geom(4, 2, 4, 4, 2)
    g1.tag, g2.tag = 1, 2
    o1, o2 = [10, 11, 12, 13, 14], [20, 21, 22, 23]
    vol = np.zeros((4, 2, 4), np.float32)
    O.ossart_iteration_dual(vol, g1, None, None, o1, g2, None, None, o2, 1.0, 3)
    assert flushed == [(2, [20]), (1, [10, 11, 12, 13]), (2, [21, 22, 23])]


def test_fp64_oracle_build_matches_numpy_fp64_twin():
    """The double build of the C oracle and the numpy FP64 twin are two FP64 restatements
    of the same OS-SART + TV sequence: they agree to rounding (1e-10 relative L2)."""
    from oracle import oracle64 as O64
    c = series_case(W=32, H=4, D=20, n=9, seed=3, misalign=True)
    meas = np.array([O.align(c["series"][i], c["T"][i]) for i in range(c["n"])], np.float32)
    order = O.order_shuffle(c["eul"], 4)
    v64 = np.zeros(c["vol"].shape)
    vnp = np.zeros(c["vol"].shape)
    for _ in range(3):
        e64 = O64.ossart_iteration(v64, c["g"], c["eul"], meas.astype(np.float64), order, 1.0, 3)
        enp = N.ossart_iteration(vnp, c["g"], c["eul"], meas, order, 1.0, 3)
        assert np.allclose(e64[[0, 1, 3]], enp[[0, 1, 3]], rtol=1e-9)
        O64.tv_denoise(v64, 25.0, 1.0, 0.01, 5)
        vnp = N.tv_denoise(vnp, 25.0, 1.0, 0.01, 5)
    assert rel_l2(v64, vnp) < 1e-10, rel_l2(v64, vnp)


def test_fp64_row_slab_sirt_matches_whole_volume():
    """A volume row solved alone (as the interior row of a two-row problem) equals that row
    of the whole-volume FP64 SIRT: rows are independent with a vertical tilt axis."""
    from oracle import oracle64 as O64
    c = series_case(W=40, H=6, D=24, n=11, seed=9, noise=0.0)
    meas = np.nan_to_num(c["series"]).astype(np.float64)
    orders = [O.order_shuffle(c["eul"], k % c["n"]) for k in range(4)]
    whole = np.zeros(c["vol"].shape)
    for order in orders:
        O64.ossart_iteration(whole, c["g"], c["eul"], meas, order, 1.0, 0)
    for r in (0, 2, 4):
        row = O64.row_slab_sirt(np.ascontiguousarray(meas[:, r:r + 2, :]), c["eul"], c["W"], c["D"], orders)
        assert rel_l2(row, whole[:, r, :]) < 1e-12, (r, rel_l2(row, whole[:, r, :]))

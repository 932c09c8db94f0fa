"""Resolution estimation (ResolutionEstimation.fsc / frc / frcSlices) on the host, and
the even / odd half-data reconstructions on the engine."""
from __future__ import annotations

import numpy as np
import pytest

from tomoj_gb300 import resolution as R


def _fsc_loops(even, odd):
    # the reference's loops written out directly (ResolutionEstimation.java:456-557)
    D, H, W = even.shape
    mask = np.zeros_like(even)
    for z in range(D):
        for y in range(H):
            for x in range(W):
                d = np.sqrt((x - W / 2.0) ** 2 + ((z - D / 2.0) ** 2 + (y - H / 2.0) ** 2))
                mask[z, y, x] = 1 if d < D else (np.float32((1 + np.cos((d - D) * np.pi / 20)) * .5) if d < D + 20 else 0)
    fe = np.fft.fftn((even * mask).astype(np.float64))
    fo = np.fft.fftn((odd * mask).astype(np.float64))
    nb = W // 2 + 1
    num, de, do, err, cnt = (np.zeros(nb) for _ in range(5))
    for z in range(D):
        for y in range(H):
            for x in range(W):
                w = np.sqrt(R.convert_to_frequency(x, W) ** 2 + R.convert_to_frequency(y, H) ** 2
                            + R.convert_to_frequency(z, D) ** 2)
                i = int(np.floor(w * W + 0.5))
                if i >= nb:
                    continue
                e, o = fe[z, y, x], fo[z, y, x]
                num[i] += (e * np.conj(o)).real
                de[i] += abs(e) ** 2
                do[i] += abs(o) ** 2
                err[i] += abs(e - o)
                cnt[i] += 1
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.array([np.arange(nb) / W, num / np.sqrt(de * do), 2 / np.sqrt(cnt), err / cnt])


def test_fsc_matches_the_reference_loops():
    rng = np.random.default_rng(0)
    a = rng.normal(0, 1, (6, 7, 8)).astype(np.float32)
    b = (a + 0.5 * rng.normal(0, 1, a.shape)).astype(np.float32)
    got = R.fsc(a, b)
    ref = _fsc_loops(a, b)
    assert np.allclose(got, ref, rtol=1e-9, atol=1e-12, equal_nan=True)


def test_fsc_of_identical_and_independent_volumes():
    rng = np.random.default_rng(1)
    a = rng.normal(0, 1, (16, 16, 16)).astype(np.float32)
    same = R.fsc(a, a)
    assert np.allclose(same[1][np.isfinite(same[1])], 1.0)
    b = rng.normal(0, 1, a.shape).astype(np.float32)
    ind = R.fsc(a, b)
    # independent data: |FSC| mostly inside the 2/sqrt(n) curve (skip the DC shell)
    inside = np.abs(ind[1][1:]) <= 2.5 * ind[2][1:]
    assert inside.mean() > 0.8


def test_frc_and_frc_slices_accumulate_like_the_reference():
    rng = np.random.default_rng(2)
    a = rng.normal(0, 1, (3, 20, 24)).astype(np.float32)
    b = (a + rng.normal(0, 1, a.shape)).astype(np.float32)
    s = R.frc_slices(a, b)
    assert s.shape == (3, 4, 24 // 2 + 1)
    # slice sums are cumulative: the count row of slice z is (z + 1) times slice 0's
    c0 = 4.0 / s[0, 2] ** 2
    c2 = 4.0 / s[2, 2] ** 2
    ok = np.isfinite(c0) & np.isfinite(c2)
    assert np.allclose(c2[ok], 3 * c0[ok])
    f = R.frc(a[0], a[0])
    assert np.allclose(f[1][np.isfinite(f[1])], 1.0)


@pytest.mark.parametrize("n,even,odd", [(7, [0, 2, 4], [1, 3, 5]), (6, [0, 2, 4], [1, 3, 5]),
                                        (5, [0, 2], [1, 3])])
def test_even_odd_available_indexes(n, even, odd):
    assert list(R.available_indexes(n, R.EVEN_PROJECTIONS)) == even
    assert list(R.available_indexes(n, R.ODD_PROJECTIONS)) == odd
    assert list(R.available_indexes(n, R.ALL_PROJECTIONS)) == list(range(n))


def _rings_loops(signal, th_s, noise, th_n, ring_width):
    H, W = signal.shape
    acc = [np.zeros(W) for _ in range(5)]
    ps = [np.abs(np.fft.fft2(x.astype(np.float64))) ** 2 for x in (th_s, signal - th_s, th_n, noise - th_n)]
    for y in range(H):
        for x in range(W):
            w = np.sqrt(R.convert_to_frequency(x, W) ** 2 + R.convert_to_frequency(y, H) ** 2) * W
            l0 = max(0, int(np.ceil(w - ring_width)))
            lf = int(np.floor(w))
            for l in range(l0, lf):
                for a, p in zip(acc, ps):
                    a[l] += p[y, x]
                acc[4][l] += 1
    return acc


def test_ssnr_rings_match_the_reference_loops():
    rng = np.random.default_rng(4)
    H, W = 10, 16
    s, ts, n, tn = (rng.normal(0, 1, (H, W)).astype(np.float32) for _ in range(4))
    acc = [np.zeros(W) for _ in range(5)]
    R.ssnr_rings(s, ts, n, tn, 4, acc)
    ref = _rings_loops(s, ts, n, tn, 4)
    for a, b in zip(acc, ref):
        assert np.allclose(a, b, rtol=1e-10, atol=1e-9)
    table = R.ssnr_table(acc)
    assert table.shape == (9, W // 2 + 1)


def _swap_loops(data, cx, cy):
    h, w = data.shape
    flat = data.ravel()
    out = np.zeros(h * w, data.dtype)
    for y in range(h):
        yy = y * w
        yyc = y + cy
        if yyc >= h:
            yyc -= h
        yyc *= w
        out[yyc + cx:yyc + 2 * cx] = flat[yy:yy + cx]
        out[yyc:yyc + cx] = flat[yy + cx:yy + 2 * cx]
    return out.reshape(h, w)


@pytest.mark.parametrize("h,w", [(8, 12), (7, 9), (5, 6)])
def test_swap_quadrant_matches_the_reference_copies(h, w):
    d = np.arange(h * w, dtype=np.float32).reshape(h, w) + 1
    out = R.swap_quadrant_2d(d, w // 2, h // 2)
    assert np.array_equal(out, _swap_loops(d, w // 2, h // 2))
    if w % 2:
        assert np.all(out[:, w - 1] == 0)


def test_vssnr_image_matches_the_reference_loop():
    rng = np.random.default_rng(9)
    H, W = 6, 10
    s, ts, n, tn = (rng.normal(0, 1, (H, W)).astype(np.float32) for _ in range(4))
    s[1, 2] = np.nan
    tn[:] = 0.0  # alpha = 0: ISSNR / 0 = Inf, the SSNR saturates to Inf dB
    tn[0, 0] = 1.0
    img = R.vssnr_image(s, ts, n, tn)
    s0 = np.nan_to_num(s, nan=0.0)
    ps = [np.abs(np.fft.fft2(x.astype(np.float64))) ** 2 for x in (s0 - ts, ts, n - tn, tn)]
    ref = np.zeros((H, W), np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        for y in range(H):
            for x in range(W):
                issnr = ps[1][y, x] / ps[0][y, x]
                alpha = ps[3][y, x] / ps[2][y, x]
                aux = issnr / alpha - 1.0
                v = np.nan if np.isnan(aux) else max(aux, 0.0)
                ref[y, x] = np.float32(10.0 * np.log10(v + 1.0))
    ref = _swap_loops(ref, W // 2, H // 2)
    assert np.array_equal(np.isnan(img), np.isnan(ref))
    ok = np.isfinite(ref)
    assert np.array_equal(img[ok], ref[ok]) and np.array_equal(np.isinf(img), np.isinf(ref))

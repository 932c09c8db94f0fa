"""Compressed-sensing regularisation of CompressedSensingProjector
(TomoJ_AdvancedReconstruction/src/main/java/fr/curie/tomoj/tomography/projectors/
CompressedSensingProjector.java:34-155) over the separable 3-D wavelet transform of
fr.curie.wavelets.WaveletProcessing (WaveletProcessing.java, doTransform3D / doInverse3D),
restated in numpy FP64.

TEST INFRASTRUCTURE ONLY: imported by tests/ to check the engine, never by the engine.

Parity: unpinned.  The wavelet filters come from the third-party library
jar.epfl:Fractional_Splines_Wavelets 1.0 (TomoJ_AdvancedReconstruction/pom.xml:22-26; Blu
and Unser's fractional spline wavelets, package `fractsplinewavelets`), which is not in
the reference tree.  They are restated from the published mathematics (M. Unser and
T. Blu, "Fractional splines and wavelets", SIAM Review 42(1), 2000; T. Blu and M. Unser,
"The fractional spline wavelet transform: definition and implementation", ICASSP 2000):

* refinement filter of the (alpha, tau) fractional B-spline, for w in (-pi, pi]:
  H(w) = sqrt(2) |cos(w/2)|^(alpha+1) exp(-i tau w);
* autocorrelation A(w) = |2 sin(w/2)|^(2 alpha+2) sum_k |w + 2 pi k|^-(2 alpha+2)
  (A(0) = 1), summed over |k| <= 256 with the tail from its integral and the first
  Euler-Maclaurin correction;
* ORTHONORMAL (type 0): analysis = synthesis, Ho(w) = H(w) sqrt(A(w) / A(2w)),
  Go(w) = exp(-i w) conj(Ho(w + pi));
* BSPLINE (type 3): synthesis H and G(w) = exp(-i w) conj(H(w + pi)) A(w + pi);
  analysis Ht(w) = H(w) A(w) / A(2w) and Gt(w) = exp(-i w) conj(H(w + pi)) / A(2w);
* DUAL (type 6): BSPLINE with analysis and synthesis exchanged.

One level along an axis of length n (even): c = ifft_{n/2}((X(k) conj(Ht(k)) +
X(k + n/2) conj(Ht(k + n/2))) / 2), likewise d with Gt, stored as [c | d]; synthesis
x = ifft_n(C(k mod n/2) H(k) + D(k mod n/2) G(k)).  The sign and circular position of the
detail band are conventions that the soft threshold commutes with, so the regularised
volume does not depend on them; the filter family and its normalisation do matter and
are what stays unpinned.  Levels run on the low-pass corner, x then y then z forward and
z, y, x backward, as WaveletProcessing does.
"""
from __future__ import annotations

import numpy as np

ORTHONORMAL, BSPLINE, DUAL = 0, 3, 6
_TAIL_K = 256


def autocorrelation(w: np.ndarray, alpha: float) -> np.ndarray:
    """A(w) of the fractional B-spline of degree alpha (float64, any w)."""
    p = 2.0 * alpha + 2.0
    w = np.remainder(np.asarray(w, np.float64) + np.pi, 2 * np.pi) - np.pi  # (-pi, pi]
    out = np.ones_like(w)
    nz = w != 0.0
    wn = w[nz]
    k = np.arange(1, _TAIL_K + 1, dtype=np.float64)[:, None]
    s = np.abs(wn) ** -p + np.sum(np.abs(wn + 2 * np.pi * k) ** -p + np.abs(wn - 2 * np.pi * k) ** -p, axis=0)
    # tail sum_{k > K} f(k), f(t) = |w +- 2 pi t|^-p: integral from K + 1/2 plus the
    # midpoint-rule Euler-Maclaurin term f'(K + 1/2) / 24
    a = 2 * np.pi * (_TAIL_K + 0.5)
    s += ((a + wn) ** (1 - p) + (a - wn) ** (1 - p)) / (2 * np.pi * (p - 1))
    s -= 2 * np.pi * p / 24 * ((a + wn) ** (-p - 1) + (a - wn) ** (-p - 1))
    out[nz] = np.abs(2 * np.sin(wn / 2)) ** p * s
    return out


def _freq(n: int) -> np.ndarray:
    k = np.arange(n, dtype=np.float64)
    return 2 * np.pi * np.where(k > n // 2, k - n, k) / n


def _refine(w: np.ndarray, alpha: float, tau: float) -> np.ndarray:
    w = np.remainder(w + np.pi, 2 * np.pi) - np.pi
    w = np.where(w == -np.pi, np.pi, w)
    return np.sqrt(2.0) * np.abs(np.cos(w / 2)) ** (alpha + 1) * np.exp(-1j * tau * w)


def filters(n: int, kind: int, alpha: float, tau: float):
    """(analysis low, analysis high, synthesis low, synthesis high) sampled at the n
    frequencies 2 pi k / n, complex128."""
    w = _freq(n)
    H = _refine(w, alpha, tau)
    Hp = _refine(w + np.pi, alpha, tau)
    A, Ap, A2 = autocorrelation(w, alpha), autocorrelation(w + np.pi, alpha), autocorrelation(2 * w, alpha)
    e = np.exp(-1j * w)
    if kind == ORTHONORMAL:
        Ho = H * np.sqrt(A / A2)
        Hop = Hp * np.sqrt(Ap / A2)
        Go = e * np.conj(Hop)
        return Ho, Go, Ho, Go
    if kind not in (BSPLINE, DUAL):
        raise ValueError("wavelet type must be 0 (orthonormal), 3 (B-spline) or 6 (dual)")
    syn_l, syn_h = H, e * np.conj(Hp) * Ap
    ana_l, ana_h = H * A / A2, e * np.conj(Hp) / A2
    if kind == BSPLINE:
        return ana_l, ana_h, syn_l, syn_h
    return syn_l, syn_h, ana_l, ana_h


def _analysis_lines(x: np.ndarray, fl, fh) -> np.ndarray:
    """One analysis level on the last axis (length n, even)."""
    n = x.shape[-1]
    m = n // 2
    X = np.fft.fft(x, axis=-1)
    lo = (X[..., :m] * np.conj(fl[:m]) + X[..., m:] * np.conj(fl[m:])) / 2
    hi = (X[..., :m] * np.conj(fh[:m]) + X[..., m:] * np.conj(fh[m:])) / 2
    return np.concatenate([np.fft.ifft(lo, axis=-1).real, np.fft.ifft(hi, axis=-1).real], axis=-1)


def _synthesis_lines(x: np.ndarray, fl, fh) -> np.ndarray:
    n = x.shape[-1]
    m = n // 2
    C = np.fft.fft(x[..., :m], axis=-1)
    Dd = np.fft.fft(x[..., m:], axis=-1)
    V = np.concatenate([C, C], axis=-1) * fl + np.concatenate([Dd, Dd], axis=-1) * fh
    return np.fft.ifft(V, axis=-1).real


def _on_axis(buf, axis, ext, fn):
    """Apply fn to the lines along `axis` of the corner buf[:ext[0], :ext[1], :ext[2]]
    (axes in [z][y][x] order)."""
    sl = tuple(slice(0, e) for e in ext)
    sub = np.moveaxis(buf[sl], axis, -1)
    buf[sl] = np.moveaxis(fn(sub), -1, axis)


def transform3d(buf: np.ndarray, iters, kind: int, alpha: float, tau: float) -> None:
    """doTransform3D on a float64 [D][H][W] buffer in place; iters = (x, y, z) levels."""
    D, H, W = buf.shape
    size = [W, H, D]
    for level in range(1, max(iters) + 1):
        for ax, vaxis in ((0, 2), (1, 1), (2, 0)):  # x, y, z
            if level > iters[ax]:
                continue
            n = size[ax]
            fl, fh, _, _ = filters(n, kind, alpha, tau)
            ext = [size[2], size[1], size[0]]
            _on_axis(buf, vaxis, ext, lambda s: _analysis_lines(s, fl, fh))
        for ax in range(3):
            if level <= iters[ax]:
                size[ax] //= 2


def inverse3d(buf: np.ndarray, iters, kind: int, alpha: float, tau: float) -> None:
    """doInverse3D on a float64 [D][H][W] buffer in place."""
    D, H, W = buf.shape
    full = [W, H, D]
    size = [full[a] >> iters[a] for a in range(3)]
    for level in range(max(iters), 0, -1):
        for ax in range(3):
            if level <= iters[ax]:
                size[ax] *= 2
        for ax, vaxis in ((2, 0), (1, 1), (0, 2)):  # z, y, x
            if level > iters[ax]:
                continue
            n = size[ax]
            _, _, fl, fh = filters(n, kind, alpha, tau)
            ext = [size[2], size[1], size[0]]
            _on_axis(buf, vaxis, ext, lambda s: _synthesis_lines(s, fl, fh))


def best_iterations(width: int):
    """findBestWaveletsIteration (CompressedSensingProjector.java:127-151): levels from
    64 doubling up to the width, the same count on all three axes (the reference sizes
    every axis from rec.getWidth())."""
    n, s = 1, 64
    while s < width:
        s *= 2
        n += 1
    return (n, n, n)


def abs_histogram(buf: np.ndarray, histomax: float) -> np.ndarray:
    """computeAbsHistogram (CompressedSensingProjector.java:112-125): 256 bins of |v| on
    [0, histomax), (int)(scale |v|) clamped to 255."""
    scale = 256.0 / histomax
    idx = np.minimum((scale * np.abs(buf)).astype(np.int64), 255)
    return np.bincount(idx.ravel(), minlength=256)


def find_threshold(buf: np.ndarray, fraction_zeros: float, max_passes: int = 16) -> float:
    """findThreshold (CompressedSensingProjector.java:80-110).  Two guards the reference
    lacks: an all-zero buffer gives 0 (the reference loops forever), and the refinement
    stops after max_passes or when histomax no longer shrinks."""
    histomax = float(max(abs(buf.min()), abs(buf.max())))
    if histomax == 0.0:
        return 0.0
    D, H, W = buf.shape
    nbpixels = int(fraction_zeros * W * H * D)  # evaluated left to right, as the reference
    for _ in range(max_passes):
        histoscale = 256.0 / histomax
        histo = abs_histogram(buf, histomax)
        total, index = 0, -1
        while total < nbpixels:
            index += 1
            total += int(histo[index])
        if nbpixels > 0 and total / nbpixels > 1.01:
            new_max = abs((index + 1) / histoscale)
            if new_max < histomax:
                histomax = new_max
                continue
        break
    return index / histoscale


def soft_threshold(buf: np.ndarray, t: float) -> None:
    """Soft threshold (CoefProcessing.doSoftThreshold3D): v - t above t, v + t below -t,
    0 between."""
    buf[:] = np.where(buf > t, buf - t, np.where(buf < -t, buf + t, 0.0))


def cs_filter(vol: np.ndarray, fraction_zeros=0.95, kind=BSPLINE, alpha=3.0, tau=0.0, iters=None) -> float:
    """filterInWavelets (CompressedSensingProjector.java:40-71) on a float32 [D][H][W]
    volume in place: FP64 buffer, forward transform, threshold, soft threshold, inverse,
    (float) back into the volume.  Returns the threshold."""
    iters = best_iterations(vol.shape[2]) if iters is None else tuple(iters)
    buf = vol.astype(np.float64)
    transform3d(buf, iters, kind, alpha, tau)
    t = find_threshold(buf, fraction_zeros)
    soft_threshold(buf, t)
    inverse3d(buf, iters, kind, alpha, tau)
    vol[:] = buf.astype(np.float32)
    return t

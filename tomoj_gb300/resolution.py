"""Resolution estimation: Fourier shell / ring correlation of two half-data
reconstructions.

Mirrors ResolutionEstimation (TomoJ_Base/src/main/java/fr/curie/tomoj/tomography/
ResolutionEstimation.java): the tilt-series is split into even and odd projections
as ReconstructionParameters.getAvailableIndexes does for EVEN_PROJECTIONS /
ODD_PROJECTIONS (ReconstructionParameters.java:212-256), each half is reconstructed
with the same parameters (here on the GPU engine), and the two volumes are compared
shell by shell:

  * fsc (:456-557): both volumes times a soft spherical mask (1 inside a radius of
    the stack depth, a 20-voxel raised-cosine edge), 3-D FFT, shells indexed by
    round(|f| * W) with f the signed frequency of each axis (convertToFrequency,
    :699-701); per shell: sum Re(E conj(O)), sum |E|^2, sum |O|^2, sum |E - O|,
    count; output rows {i / W, FSC, 2 / sqrt(count), mean |E - O|};
  * frc (:376-454): the same on one pair of images with a circular mask;
  * frcSlices (:275-374): per-slice 2-D FFTs with a cylinder mask; the shell sums
    are not reset between slices, so slice z reports the sums over slices 0..z
    (reproduced as the reference computes it);
  * SSNR (:167-273, 581-697): the series and a Gaussian-noise series of the same
    geometry are reconstructed and reprojected; per tilt the power spectra of the
    reprojections and of the residuals accumulate over rings of width ringWidth.

The reference transforms float data with ParallelColt (absent from the reference
tree); here the transforms are numpy's double-precision FFTs.  The result agrees
to FP32 rounding, and that correspondence is not pinned by any reference test.
"""
from __future__ import annotations

import numpy as np

from .reconstruction import BP, WBP, ReconstructionParameters, TomoReconstruction2
from .tiltseries import TiltSeries

ALL_PROJECTIONS, EVEN_PROJECTIONS, ODD_PROJECTIONS = 0, 11, 12


def available_indexes(nproj: int, projection_type: int) -> np.ndarray:
    """ReconstructionParameters.getAvailableIndexes: even / odd indexes, at most nproj // 2 of them."""
    sel = []
    count = 0
    for i in range(nproj):
        if projection_type == EVEN_PROJECTIONS:
            take = i % 2 == 0
        elif projection_type == ODD_PROJECTIONS:
            take = i % 2 == 1
        else:
            take = True
        if take:
            count += 1
            if projection_type in (EVEN_PROJECTIONS, ODD_PROJECTIONS) and count > nproj // 2:
                take = False
                count -= 1
        if take:
            sel.append(i)
    return np.array(sel, np.int64)


def convert_to_frequency(x, size: int):
    """convertToFrequency (:699-701): signed frequency of index x in cycles per sample."""
    x = np.asarray(x, np.float64)
    return np.where(x <= (size >> 1), x, x - size) / size


def _shell_sums(fe, fo, widx, nbins):
    keep = widx < nbins
    idx = widx[keep]
    e = fe[keep]
    o = fo[keep]
    num = np.bincount(idx, weights=(e * np.conj(o)).real, minlength=nbins)
    den_e = np.bincount(idx, weights=np.abs(e) ** 2, minlength=nbins)
    den_o = np.bincount(idx, weights=np.abs(o) ** 2, minlength=nbins)
    err = np.bincount(idx, weights=np.abs(e - o), minlength=nbins)
    cnt = np.bincount(idx, minlength=nbins).astype(np.float64)
    return num, den_e, den_o, err, cnt


def _rows(num, den_e, den_o, err, cnt, width):
    nb = num.size
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.array([np.arange(nb) / width, num / np.sqrt(den_e * den_o), 2 / np.sqrt(cnt), err / cnt])


def _java_round(v):
    return np.floor(v + 0.5).astype(np.int64)


def fsc(even: np.ndarray, odd: np.ndarray) -> np.ndarray:
    """Fourier shell correlation of two (D, H, W) volumes: rows {frequency, FSC,
    2/sqrt(count), mean |E - O|} over W // 2 + 1 shells."""
    even = np.asarray(even, np.float32)
    odd = np.asarray(odd, np.float32)
    D, H, W = even.shape
    z = (np.arange(D) - D / 2.0) ** 2
    y = (np.arange(H) - H / 2.0) ** 2
    x = (np.arange(W) - W / 2.0) ** 2
    dist = np.sqrt(x[None, None, :] + (z[:, None, None] + y[None, :, None]))
    mask = np.where(dist < D, 1.0, np.where(dist < D + 20, (1 + np.cos((dist - D) * np.pi / 20)) * 0.5, 0.0))
    mask = mask.astype(np.float32)
    fe = np.fft.fftn((even * mask).astype(np.float64))
    fo = np.fft.fftn((odd * mask).astype(np.float64))
    fz = convert_to_frequency(np.arange(D), D) ** 2
    fy = convert_to_frequency(np.arange(H), H) ** 2
    fx = convert_to_frequency(np.arange(W), W) ** 2
    w = np.sqrt(fx[None, None, :] + fy[None, :, None] + fz[:, None, None])
    widx = _java_round(w * W)
    nb = W // 2 + 1
    return _rows(*_shell_sums(fe.ravel(), fo.ravel(), widx.ravel(), nb), W)


def frc(img1: np.ndarray, img2: np.ndarray) -> np.ndarray:
    """Fourier ring correlation of two (H, W) images (ResolutionEstimation.frc)."""
    a = np.asarray(img1, np.float32)
    b = np.asarray(img2, np.float32)
    H, W = a.shape
    y = (np.arange(H) - H / 2.0) ** 2
    x = (np.arange(W) - W / 2.0) ** 2
    dist = np.sqrt(x[None, :] + y[:, None])
    mask = np.where(dist < W, 1.0, np.where(dist < W + 20, (1 + np.cos((dist - W) * np.pi / 20)) * 0.5, 0.0))
    mask = mask.astype(np.float32)
    fe = np.fft.fft2((a * mask).astype(np.float64))
    fo = np.fft.fft2((b * mask).astype(np.float64))
    fy = convert_to_frequency(np.arange(H), H) ** 2
    fx = convert_to_frequency(np.arange(W), W) ** 2
    widx = _java_round(np.sqrt(fx[None, :] + fy[:, None]) * W)
    return _rows(*_shell_sums(fe.ravel(), fo.ravel(), widx.ravel(), W // 2 + 1), W)


def frc_slices(even: np.ndarray, odd: np.ndarray) -> np.ndarray:
    """ResolutionEstimation.frcSlices: (D, 4, W // 2 + 1); slice z holds the ring sums of
    slices 0..z (the reference never resets them)."""
    even = np.asarray(even, np.float32)
    odd = np.asarray(odd, np.float32)
    D, H, W = even.shape
    y = (np.arange(H) - H / 2.0) ** 2
    x = (np.arange(W) - W / 2.0) ** 2
    dist = np.sqrt(x[None, :] + y[:, None])
    mask = np.where(dist < W - 20, 1.0,
                    np.where(dist < W, (1 + np.cos((dist - W - 20) * np.pi / 20)) * 0.5, 0.0)).astype(np.float32)
    fy = convert_to_frequency(np.arange(H), H) ** 2
    fx = convert_to_frequency(np.arange(W), W) ** 2
    widx = _java_round(np.sqrt(fx[None, :] + fy[:, None]) * W).ravel()
    nb = W // 2 + 1
    acc = [np.zeros(nb) for _ in range(5)]
    out = np.zeros((D, 4, nb))
    for zi in range(D):
        fe = np.fft.fft2((even[zi] * mask).astype(np.float64)).ravel()
        fo = np.fft.fft2((odd[zi] * mask).astype(np.float64)).ravel()
        for a, s in zip(acc, _shell_sums(fe, fo, widx, nb)):
            a += s
        out[zi] = _rows(*acc, W)
    return out


class _FixedAlignment:
    """Alignment of a sub-series: each image keeps the final transform and Euler matrix it
    has in the full series (the reference reconstructs a half from the full series through
    getAvailableIndexes, so consecutive transforms of skipped images still compose)."""

    def __init__(self, transforms, eulers, tiltaxis=0.0):
        self._t = [tuple(map(float, t)) for t in transforms]
        self._e = [np.asarray(e, np.float64) for e in eulers]
        self.tiltaxis = float(tiltaxis)  # ts.getTiltAxis(), read by the WBP weighting

    def getTransform(self, index, combine=None):
        return self._t[index]

    def getEulerMatrix(self, index):
        return self._e[index]


def subseries(ts: TiltSeries, indexes) -> TiltSeries:
    """The tilt-series restricted to `indexes`, with their full-series geometry."""
    idx = np.asarray(indexes, np.int64)
    sub = TiltSeries(ts.pixels[idx], ts.tiltAngles[idx])
    sub.setNormalize(ts.isNormalized())
    sub.setFillType(ts.getFillType())
    T, E = ts.transforms(), ts.eulers()
    sub.alignment = _FixedAlignment(T[idx], E[idx], ts.getTiltAxis())
    if ts.stats is not None:
        sub.setStatistics(np.asarray(ts.statistics())[idx])
    return sub


def ssnr_rings(signal, th_signal, noise, th_noise, ring_width, acc):
    """ResolutionEstimation.addToVectors1D (:581-697) for one tilt: power spectra of the
    reprojection th and of the residual (exp - th) for the signal and the noise series,
    each pixel adding to the rings l in [max(0, ceil(|f| W - ringWidth)), floor(|f| W)).
    acc = [S_S, S_N, N_S, N_N, K] (length W each) is updated in place."""
    def clean(a):
        return np.nan_to_num(np.asarray(a, np.float32), nan=0.0)

    sig, th_s, noi, th_n = clean(signal), clean(th_signal), clean(noise), clean(th_noise)
    sig = sig - th_s
    noi = noi - th_n
    H, W = sig.shape
    ps = [np.abs(np.fft.fft2(x.astype(np.float64))) ** 2 for x in (th_s, sig, th_n, noi)]
    fy = convert_to_frequency(np.arange(H), H) ** 2
    fx = convert_to_frequency(np.arange(W), W) ** 2
    widx = (np.sqrt(fx[None, :] + fy[:, None]) * W).ravel()
    l0 = np.maximum(0, np.ceil(widx - ring_width)).astype(np.int64)
    lf = np.floor(widx).astype(np.int64)
    # each pixel adds to rings l0 .. lf - 1: a difference array over the ring index
    n = acc[0].size
    for arr, w in zip(acc, ps + [None]):
        d = np.zeros(n + 1)
        weight = np.ones(widx.size) if w is None else w.ravel()
        ok = lf > l0
        np.add.at(d, l0[ok], weight[ok])
        np.add.at(d, np.minimum(lf[ok], n), -weight[ok])
        arr += np.cumsum(d)[:n]
    return acc


def swap_quadrant_2d(data: np.ndarray, cx: int, cy: int) -> np.ndarray:
    """ResolutionEstimation.swapQuadrant2D (:709-721): row y moves to (y + cy) mod h and
    its halves [0, cx) and [cx, 2 cx) swap; for an odd width the last column stays 0."""
    h, w = data.shape
    out = np.zeros_like(data)
    rows = (np.arange(h) + cy) % h
    out[rows, cx:2 * cx] = data[:, :cx]
    out[rows, :cx] = data[:, cx:2 * cx]
    return out


def vssnr_image(signal, th_signal, noise, th_noise) -> np.ndarray:
    """The volumetric branch of ResolutionEstimation.addToVectors1D (:632-645) for one
    tilt: per frequency, 10 log10(max(ISSNR / alpha - 1, 0) + 1) with ISSNR the ratio of
    the reprojection's power to the residual's for the signal series and alpha the same
    for the noise series, as float, quadrant-swapped to put the origin at the centre."""
    def clean(a):
        return np.nan_to_num(np.asarray(a, np.float32), nan=0.0)

    th_s, th_n = clean(th_signal), clean(th_noise)
    res_s, res_n = clean(signal) - th_s, clean(noise) - th_n
    ps = [np.abs(np.fft.fft2(x.astype(np.float64))) ** 2 for x in (res_s, th_s, res_n, th_n)]
    with np.errstate(divide="ignore", invalid="ignore"):
        issnr = ps[1] / ps[0]
        alpha = ps[3] / ps[2]
        ssnr = np.maximum(issnr / alpha - 1.0, 0.0)  # NaN stays NaN, as Math.max
        img = (10.0 * np.log10(ssnr + 1.0)).astype(np.float32)
    h, w = img.shape
    return swap_quadrant_2d(img, w // 2, h // 2)


def ssnr_table(acc, pixel_size=1.0):
    """The SSNR output rows of ResolutionEstimation.SSNR (:206-265): index, frequency,
    corrected SSNR (dB), signal SNR, signal power and residual power (dB), and the same
    three for the noise series, up to the Nyquist ring."""
    S_S, S_N, N_S, N_N, K = (np.array(a, np.float64) for a in acc)
    n = S_S.size
    with np.errstate(divide="ignore", invalid="ignore"):
        s_snr = S_S / S_N
        n_snr = N_S / N_N
        S_S, S_N, N_S, N_N = S_S / K, S_N / K, N_S / K, N_N / K
        imgno = 1 + n  # the reference counts one per ring before writing the table
        rows = []
        for i in range(n):
            w = float(convert_to_frequency(i, n))
            if w < 0:
                break
            ss = s_snr[i] / n_snr[i]
            rows.append([i, w / pixel_size, 10 * np.log10(ss - 1) if ss > 1 else -1000.0, s_snr[i],
                         10 * np.log10(S_S[i] / imgno), 10 * np.log10(S_N[i] / imgno), n_snr[i],
                         10 * np.log10(N_S[i] / imgno), 10 * np.log10(N_N[i] / imgno)])
    return np.array(rows).T


class ResolutionEstimation:
    """ResolutionEstimation on the engine: generateFSCData reconstructs the even and odd
    halves with `params` (WBP, OS-SART / SIRT or TVM), fsc() compares them; SSNR()
    reconstructs the series and a Gaussian-noise series with the same geometry and
    compares each projection with its reprojection ring by ring."""

    def __init__(self, ts: TiltSeries, params: ReconstructionParameters, seed: int = 0):
        self.ts = ts
        self.params = params
        self.seed = seed
        self.recFSCeven = None
        self.recFSCodd = None
        self.recVSSNR = None

    def _reconstruct(self, ts: TiltSeries) -> np.ndarray:
        p = self.params
        rec = TomoReconstruction2(p.width, p.height, p.depth)
        proj = p.getProjector(ts, rec)
        try:
            if p.reconstructionType in (BP, WBP):
                rec.WBP(ts, proj, p)
            else:
                rec.OSSART(ts, proj, p, seed=self.seed)
            return rec.getVolume()
        finally:
            proj.close()

    def generateFSCData(self):
        n = self.ts.getImageStackSize()
        self.recFSCodd = self._reconstruct(subseries(self.ts, available_indexes(n, ODD_PROJECTIONS)))
        self.recFSCeven = self._reconstruct(subseries(self.ts, available_indexes(n, EVEN_PROJECTIONS)))

    def fsc(self) -> np.ndarray:
        self.generateFSCData()
        return fsc(self.recFSCeven, self.recFSCodd)

    def _reconstruct_and_reproject(self, ts: TiltSeries):
        """Reconstruction, each aligned projection and its reprojection."""
        p = self.params
        rec = TomoReconstruction2(p.width, p.height, p.depth)
        proj = p.getProjector(ts, rec)
        try:
            if p.reconstructionType in (BP, WBP):
                rec.WBP(ts, proj, p)
            else:
                rec.OSSART(ts, proj, p, seed=self.seed)
            n = ts.getImageStackSize()
            exp, th = [], []
            for i in range(n):
                proj.clearAllProjections()
                proj.addProjection(i)
                proj.project(0, p.height)
                th.append(proj.getProjection(0))
                exp.append(proj.getAlignedProjection(i))
            proj.clearAllProjections()
            return rec.getVolume(), exp, th
        finally:
            proj.close()

    def SSNR(self, ring_width: int = 4, pixel_size: float = 1.0, noise_seed: int = 12345,
             computeVSSNR: bool = False) -> np.ndarray:
        """ResolutionEstimation.SSNR (:167-273): the noise series is N(0, 1) per pixel from
        a seeded generator (the reference draws it with ImageJ's ImageProcessor.noise(1)).
        With computeVSSNR the per-tilt 2-D SSNR images form a new tilt-series (same tilt
        angles, no alignment) reconstructed with the same parameters: recVSSNR."""
        ts = self.ts
        self.recSignal, exp_s, th_s = self._reconstruct_and_reproject(ts)
        rng = np.random.Generator(np.random.PCG64(noise_seed))
        noise_pixels = rng.normal(0.0, 1.0, ts.pixels.shape).astype(np.float32)
        tsn = TiltSeries(noise_pixels, ts.tiltAngles)
        tsn.setNormalize(ts.isNormalized())
        tsn.setFillType(ts.getFillType())
        tsn.alignment = _FixedAlignment(ts.transforms(), ts.eulers(), ts.getTiltAxis())
        self.recNoise, exp_n, th_n = self._reconstruct_and_reproject(tsn)
        W = ts.getWidth()
        acc = [np.zeros(W) for _ in range(5)]
        for i in range(ts.getImageStackSize()):
            ssnr_rings(exp_s[i], th_s[i], exp_n[i], th_n[i], ring_width, acc)
        self.ssnr = ssnr_table(acc, pixel_size)
        if computeVSSNR:
            imgs = np.array([vssnr_image(exp_s[i], th_s[i], exp_n[i], th_n[i])
                             for i in range(ts.getImageStackSize())], np.float32)
            self.tsVSSNR = TiltSeries(imgs, ts.tiltAngles)
            self.recVSSNR = self._reconstruct(self.tsVSSNR)
        return self.ssnr

    def getVSSNR(self):
        return self.recVSSNR

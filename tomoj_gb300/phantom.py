"""Seeded synthetic inputs: ellipsoid phantoms, tilt schemes, per-tilt
misalignment transforms and detector noise.

The reference reconstructs experimental tilt-series; there is no public dataset
on this path, so every workload here is a seeded synthetic stand-in with the
shapes and value ranges of the benchmark configurations:
  * phantom: K ellipsoids, centres inside the volume, semi-axes U(0.05,0.25)*dim,
    random orientation, density U[0,1], overlaps add, zero background;
  * tilt angles: uniform, Saxton (TomoJ_Base/.../AnglesForTiltSeries.java:96-120)
    or dose-symmetric acquisition order;
  * per-tilt in-plane shift + rotation as java.awt.geom.AffineTransform flat
    matrices {m00, m10, m01, m11, m02, m12} (the form AffineAlignment stores);
  * Gaussian (sigma = fraction of max) or Poisson (electrons per pixel) noise.

Volumes are float32 (D, H, W): D slices of W x H, x fastest, as in
TomoReconstruction2.
"""
from __future__ import annotations

import math

import numpy as np


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def ellipsoid_phantom(W: int, H: int, D: int, n_ellipsoids: int, seed: int) -> np.ndarray:
    """Sum of `n_ellipsoids` random solid ellipsoids; float32 (D, H, W)."""
    g = rng(seed)
    vol = np.zeros((D, H, W), np.float32)
    dims = np.array([W, H, D], np.float64)
    zz, yy, xx = np.meshgrid(np.arange(D, dtype=np.float32), np.arange(H, dtype=np.float32),
                             np.arange(W, dtype=np.float32), indexing="ij")
    for _ in range(n_ellipsoids):
        axes = g.uniform(0.05, 0.25, 3) * dims
        centre = g.uniform(0.0, 1.0, 3) * (dims - 2 * axes) + axes
        centre = np.clip(centre, 0, dims - 1)
        a, b, c = g.uniform(0, 2 * np.pi, 3)
        ca, sa, cb, sb, cc, sc = math.cos(a), math.sin(a), math.cos(b), math.sin(b), math.cos(c), math.sin(c)
        Rz1 = np.array([[ca, -sa, 0], [sa, ca, 0], [0, 0, 1]])
        Ry = np.array([[cb, 0, sb], [0, 1, 0], [-sb, 0, cb]])
        Rz2 = np.array([[cc, -sc, 0], [sc, cc, 0], [0, 0, 1]])
        Rm = (Rz1 @ Ry @ Rz2).astype(np.float32)
        dens = np.float32(g.uniform(0.0, 1.0))
        r = float(np.max(axes)) + 1
        x0, x1 = int(max(0, centre[0] - r)), int(min(W, centre[0] + r + 1))
        y0, y1 = int(max(0, centre[1] - r)), int(min(H, centre[1] + r + 1))
        z0, z1 = int(max(0, centre[2] - r)), int(min(D, centre[2] + r + 1))
        if x0 >= x1 or y0 >= y1 or z0 >= z1:
            continue
        px = xx[z0:z1, y0:y1, x0:x1] - np.float32(centre[0])
        py = yy[z0:z1, y0:y1, x0:x1] - np.float32(centre[1])
        pz = zz[z0:z1, y0:y1, x0:x1] - np.float32(centre[2])
        u = (Rm[0, 0] * px + Rm[1, 0] * py + Rm[2, 0] * pz) / np.float32(axes[0])
        v = (Rm[0, 1] * px + Rm[1, 1] * py + Rm[2, 1] * pz) / np.float32(axes[1])
        w = (Rm[0, 2] * px + Rm[1, 2] * py + Rm[2, 2] * pz) / np.float32(axes[2])
        inside = (u * u + v * v + w * w) <= 1.0
        vol[z0:z1, y0:y1, x0:x1] += np.where(inside, dens, np.float32(0))
    return vol


def uniform_tilts(start: float, stop: float, step: float) -> np.ndarray:
    n = int(round((stop - start) / step)) + 1
    return np.array([start + i * step for i in range(n)], np.float64)


def saxton_tilts(max_angle: float, n: int) -> np.ndarray:
    """Symmetric Saxton scheme with n angles reaching about +/-max_angle.

    The ladder follows AnglesForTiltSeries (AnglesForTiltSeries.java:96-120):
    a_{k+1} = round(a_k + asin(sin(inc) cos(a_k)), 0.01 deg); the base increment
    `inc` is chosen so that (n-1)/2 steps land closest to max_angle."""
    half = (n - 1) // 2

    def ladder(inc):
        a, out = 0.0, [0.0]
        for _ in range(half):
            ang = a + math.degrees(math.asin(math.sin(math.radians(inc)) * math.cos(math.radians(a))))
            a = round(ang * 100) / 100.0
            out.append(a)
        return out

    lo, hi = 0.01, 45.0
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        if ladder(mid)[-1] < max_angle:
            lo = mid
        else:
            hi = mid
    pos = ladder(hi)
    angles = [-a for a in reversed(pos[1:])] + pos
    if len(angles) < n:
        angles.append(pos[-1] + (pos[-1] - pos[-2]))
    return np.array(angles[:n], np.float64)


def dose_symmetric_tilts(max_angle: float, n: int) -> np.ndarray:
    """Uniform angles in dose-symmetric acquisition order: 0, +d, -d, -2d, +2d, +3d, ..."""
    step = 2.0 * max_angle / (n - 1)
    out = [0.0]
    k, sign = 1, 1.0
    while len(out) < n:
        out.append(sign * k * step)
        if len(out) < n:
            out.append(-sign * k * step)
        sign = -sign
        k += 1
    return np.array(out[:n], np.float64)


def misalignment(n: int, seed: int, max_shift: float = 5.0, max_rot_deg: float = 1.0) -> np.ndarray:
    """Per-tilt AffineTransform {m00,m10,m01,m11,m02,m12}: rotation U(-r,r) deg then shift U(-s,s) px."""
    g = rng(seed)
    T = np.zeros((n, 6), np.float64)
    for i in range(n):
        phi = math.radians(g.uniform(-max_rot_deg, max_rot_deg))
        tx, ty = g.uniform(-max_shift, max_shift, 2)
        c, s = math.cos(phi), math.sin(phi)
        T[i] = (c, s, -s, c, tx, ty)
    return T


def unalign(ideal: np.ndarray, T) -> np.ndarray:
    """Build the measured image U from an ideal (aligned) one so that
    AffineAlignment.applyTransformOnImage(U, T) reproduces `ideal`:
    U(q) = ideal(T (q - c) + c), c = (w/2, h/2), bilinear, 0 outside."""
    ideal = np.asarray(ideal, np.float64)
    h, w = ideal.shape
    m00, m10, m01, m11, m02, m12 = [float(v) for v in T]
    cx, cy = w / 2.0, h / 2.0
    J, I = np.meshgrid(np.arange(h) - cy, np.arange(w) - cx, indexing="ij")
    xx = m00 * I + m01 * J + m02 + cx
    yy = m10 * I + m11 * J + m12 + cy
    x0 = np.floor(xx).astype(np.int64)
    y0 = np.floor(yy).astype(np.int64)
    fx, fy = xx - x0, yy - y0
    out = np.zeros((h, w))
    for dy, wy in ((0, 1 - fy), (1, fy)):
        for dx, wx in ((0, 1 - fx), (1, fx)):
            xi, yi = x0 + dx, y0 + dy
            ok = (xi >= 0) & (xi < w) & (yi >= 0) & (yi < h)
            v = np.where(ok, ideal[np.clip(yi, 0, h - 1), np.clip(xi, 0, w - 1)], 0.0)
            out += wx * wy * v
    return np.nan_to_num(out).astype(np.float32)


def add_gaussian_noise(series: np.ndarray, sigma_frac: float, seed: int) -> np.ndarray:
    g = rng(seed)
    finite = np.isfinite(series)
    mx = float(np.max(series[finite])) if finite.any() else 0.0
    noise = g.normal(0.0, sigma_frac * mx, series.shape).astype(np.float32)
    return np.where(finite, series + noise, series).astype(np.float32)


def add_poisson_noise(series: np.ndarray, electrons_per_px: float, seed: int) -> np.ndarray:
    """Scale so the mean finite value maps to `electrons_per_px`, sample, rescale."""
    g = rng(seed)
    finite = np.isfinite(series)
    s = np.where(finite, series, 0.0).astype(np.float64)
    lo = float(s[finite].min()) if finite.any() else 0.0
    shifted = s - lo
    mean = float(shifted[finite].mean()) if finite.any() else 1.0
    k = electrons_per_px / max(mean, 1e-12)
    counts = g.poisson(np.maximum(shifted * k, 0.0))
    out = counts / k + lo
    return np.where(finite, out, series).astype(np.float32)


def n_ellipsoids_for(W: int, H: int, D: int) -> int:
    """Ellipsoid count scaled with volume (20 at 256x64x256, 60 at 512x256x512)."""
    ref = 256 * 64 * 256
    k = 20 * (W * H * D / ref) ** (1.0 / 3.0) * 1.2
    return int(max(8, min(400, round(k))))

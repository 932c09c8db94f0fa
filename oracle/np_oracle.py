"""FP64 numpy twin of the CPU oracle.

TEST INFRASTRUCTURE ONLY (the reference for tests/ and bench.py's precision report).

Same algorithm and quirks as oracle/tomo_oracle.c (which follows the reference's
float/double operation order), but every value is stored and computed in
float64.  It serves two purposes:
  * an independent second implementation that pins the C restatement (the two
    must agree to float32 rounding), and
  * the "FP64 CPU oracle" against which reduced-precision results are scored.

Parity status: unpinned (no reference golden vectors exist for this path).
References are paths inside the TomoJ tree.
"""
from __future__ import annotations

import numpy as np

ACC = float(np.float32(1e-10))  # VoxelProjector3D.java:33, a float constant promoted to double


def euler(phi, theta, psi):
    """MatrixUtils.eulerAngles2Matrix (MatrixUtils.java:226-251)."""
    phi, theta, psi = np.deg2rad([phi, theta, psi])
    cphi, sphi, ct, st, cpsi, spsi = np.cos(phi), np.sin(phi), np.cos(theta), np.sin(theta), np.cos(psi), np.sin(psi)
    return np.array([[cpsi * ct * cphi - spsi * sphi, cpsi * ct * sphi + spsi * cphi, -cpsi * st],
                     [-spsi * ct * cphi - cpsi * sphi, -spsi * ct * sphi + cpsi * cphi, spsi * st],
                     [st * cphi, st * sphi, ct]])


def euler_tilt_y(theta):
    return euler(0.0, theta, -0.0)


def _get_pixel(vol, x, y, z):
    """TomoReconstruction2.getPixel(double,double,int) in FP64 (TomoReconstruction2.java:154-190)."""
    D, H, W = vol.shape
    xb = np.where(x < 0, 0, np.trunc(x)).astype(np.int64)
    yb = np.where(y < 0, 0, np.trunc(y)).astype(np.int64)
    raw = (xb == W - 1) | (yb == H - 1) | (z == D - 1)
    xf = np.where(x < 0, 0.0, x - xb)
    yf = np.where(y < 0, 0.0, y - yb)
    im = vol[z]
    xb1 = np.minimum(xb + 1, W - 1)
    yb1 = np.minimum(yb + 1, H - 1)
    v00 = im[yb, xb]
    v10 = im[yb, xb1]
    v01 = im[yb1, xb]
    v11 = im[yb1, xb1]
    lower = v00 + xf * (v10 - v00)
    val = lower + yf * ((v01 + xf * (v11 - v01)) - lower)
    return np.where(raw, v00, val)


def project(vol, g, R, y0=0, y1=None):
    """VoxelProjector3D.project + projectJosephPartial (VoxelProjector3D.java:333-376, 671-821)."""
    vol = np.asarray(vol, np.float64)
    D, H, W = vol.shape
    R = np.asarray(R, np.float64)
    w, h, s = g.w, g.h, g.scale
    proj = np.zeros((h, w))
    norm = np.zeros((h, w))
    offset = (h - H) // 2 if (h > H and s == 1) else 0
    start = int(np.floor((y0 + offset) * s + 0.5))
    if start >= h:
        return proj, norm
    icF = R[1, 0] / R[0, 0]
    zcF = R[1, 2] - R[1, 0] * R[0, 2] / R[0, 0]
    divY = R[1, 1] - R[1, 0] * R[0, 1] / R[0, 0]
    dirY = -(R[1, 2] - R[1, 0] * R[0, 2] / R[0, 0]) / (R[1, 1] - R[1, 0] * R[0, 1] / R[0, 0])
    dirX = (R[0, 1] * (-dirY) - R[0, 2]) / R[0, 0]
    ninc = np.sqrt(dirX * dirX + dirY * dirY + 1)
    vcx, vcy, vcz = g.vc
    jj, ii = np.meshgrid(np.arange(start, h), np.arange(w), indexing="ij")
    jc = (jj - g.pc[1]) / s
    ic = (ii - g.pc[0]) / s
    oldy = ((jc - icF * ic) - zcF * (-1 - vcz)) / divY
    oldx = (ic - R[0, 1] * oldy - R[0, 2] * (-1 - vcz)) / R[0, 0]
    ray = np.zeros(jj.shape)
    cnt = np.zeros(jj.shape)
    entered = np.zeros(jj.shape, bool)
    done = np.zeros(jj.shape, bool)
    for z in range(D):
        xc = oldx + dirX
        yc = oldy + dirY
        x = xc + vcx
        y = yc + vcy
        inside = (x + ACC >= 0) & (x < W) & (y + ACC >= 0) & (y < H) & ~done
        if inside.any():
            ray[inside] += _get_pixel(vol, x[inside], y[inside], z)
        cnt += inside
        leaving = ~inside & entered & ~done
        cnt += leaving
        done |= leaving
        entered |= inside
        oldx, oldy = xc, yc
    nrm = cnt * ninc
    p = np.where(cnt > 0, ray * ninc, np.nan)
    proj[start:] = p
    norm[start:] = np.where(cnt > 0, nrm, 0.0)
    if g.long_object:
        norm[:] = norm.max()
    return proj, norm


def difference(expv, th, norm, factor):
    """VoxelProjector3D.difference in FP64."""
    ok = ~np.isnan(expv) & ~np.isnan(th)
    with np.errstate(divide="ignore", invalid="ignore"):
        v = np.where(ok, (expv - th) / norm * factor, 0.0)
    return v, float(np.sum(v[ok] ** 2))


def _ij_interp(p, x, y):
    """ImageJ getInterpolatedValue (bilinear, edge-clamped) for 0<=x<w, 0<=y<h."""
    h, w = p.shape
    xb = np.floor(x).astype(np.int64)
    yb = np.floor(y).astype(np.int64)
    xf = np.maximum(x - xb, 0.0)
    yf = np.maximum(y - yb, 0.0)
    xb0 = np.clip(xb, 0, w - 1)
    yb0 = np.clip(yb, 0, h - 1)
    xb1 = np.clip(xb + 1, 0, w - 1)
    yb1 = np.clip(yb + 1, 0, h - 1)
    ll, lr, ur, ul = p[yb0, xb0], p[yb0, xb1], p[yb1, xb1], p[yb1, xb0]
    ua = ul + xf * (ur - ul)
    la = ll + xf * (lr - ll)
    return la + yf * (ua - la)


def backproject(vol, g, R, proj, y0=0, y1=None, positivity=None):
    """VoxelProjector3D.backProjectPartial over rows [y0,y1), in place, FP64 (VoxelProjector3D.java:221-308)."""
    D, H, W = vol.shape
    y1 = H if y1 is None else y1
    pos = g.positivity if positivity is None else positivity
    R = np.asarray(R, np.float64)
    proj = np.asarray(proj, np.float64)
    xs = np.arange(W) - g.vc[0]
    ys = np.arange(y0, y1) - g.vc[1]
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    for k in range(D):
        z = k - g.vc[2]
        xx = (X * R[0, 0] + Y * R[0, 1] + z * R[0, 2]) * g.scale + g.pc[2]
        yy = (X * R[1, 0] + Y * R[1, 1] + z * R[1, 2]) * g.scale + g.pc[3]
        ok = (xx >= 0) & (xx < g.w) & (yy >= 0) & (yy < g.h)
        v = np.zeros(xx.shape)
        v[ok] = _ij_interp(proj, xx[ok], yy[ok])
        add = ok & ~np.isnan(v)
        sl = vol[k, y0:y1]
        nv = sl + np.where(add, v, 0.0)
        nv = np.where(add & ~np.isfinite(nv), 0.0, nv)
        if pos:
            nv = np.where(add & (nv < 0), 0.0, nv)
        vol[k, y0:y1] = np.where(add, nv, sl)
    return vol


def align(un, T, normalize=False, mean=0.0, std=1.0, fill=2):
    """AffineAlignment.applyTransformOnImage in FP64 (AffineAlignment.java:136-259)."""
    un = np.asarray(un, np.float64)
    h, w = un.shape
    m00, m10, m01, m11, m02, m12 = [float(v) for v in T]
    if (m00, m10, m01, m11, m02, m12) == (1.0, 0.0, 0.0, 1.0, 0.0, 0.0):
        return (un - mean) / std if normalize else un.copy()
    det = m00 * m11 - m01 * m10
    i00, i10, i01, i11 = m11 / det, -m10 / det, -m01 / det, m00 / det
    i02, i12 = (m01 * m12 - m11 * m02) / det, (m10 * m02 - m00 * m12) / det
    cx, cy = w / 2.0, h / 2.0
    J, I = np.meshgrid(np.arange(h) - cy, np.arange(w) - cx, indexing="ij")
    xx = (i00 * I + i01 * J + i02) + cx
    yy = (i10 * I + i11 * J + i12) + cy
    ix = np.trunc(xx).astype(np.int64)
    iy = np.trunc(yy).astype(np.int64)
    dx, dy = xx - ix, yy - iy
    ok = (ix >= 0) & (ix < w) & (iy >= 0) & (iy < h)
    ixc, iyc = np.clip(ix, 0, w - 1), np.clip(iy, 0, h - 1)
    ix1, iy1 = np.clip(ix + 1, 0, w - 1), np.clip(iy + 1, 0, h - 1)
    edge = (ix == w - 1) | (iy == h - 1)
    f4 = dx * dy
    val = (un[iyc, ixc] * (1 - dx - dy + f4) + un[iyc, ix1] * (dx - f4) + un[iy1, ixc] * (dy - f4)
           + un[iy1, ix1] * f4)
    val = np.where(edge, un[iyc, ixc], val)
    if normalize:
        val = (val - mean) / std
    if fill == 1:
        outside = 0.0 if normalize else mean
    elif fill == 2:
        outside = np.nan
    else:
        outside = 0.0
    return np.where(ok, val, outside)


def weighting_mask(w, h, tilts, axes, diameter):
    """FFTWeighting.createWeightingMask (FFTWeighting.java:31-65) in FP64."""
    tilts = np.asarray(tilts, np.float64)
    axes = np.zeros_like(tilts) if axes is None else np.asarray(axes, np.float64)
    st = np.sin(np.deg2rad(tilts))
    cp, sp = np.cos(np.deg2rad(axes)), np.sin(np.deg2rad(axes))
    i = np.arange(w)
    j = np.arange(h)
    ci = np.where(i > w / 2.0, i - w, i).astype(np.float64)
    cj = np.where(j > h / 2.0, j - h, j).astype(np.float64)
    CJ, CI = np.meshgrid(cj, ci, indexing="ij")
    wt = np.zeros((h, w))
    for p in range(tilts.size):
        zj = (CI * st[p] * cp[p] + CJ * st[p] * sp[p]) / w
        v = diameter * np.pi * zj
        with np.errstate(invalid="ignore", divide="ignore"):
            wt += np.where(v == 0, 1.0, np.sin(v) / np.where(v == 0, 1.0, v))
    wt = np.where(wt < 0.005, 0.005, wt) * diameter
    return 1.0 / wt


def weighting_apply(img, mask):
    """FFTWeighting.weighting: 2-D FFT x mask, inverse, real part (FFTWeighting.java:87-112)."""
    F = np.fft.fft2(np.asarray(img, np.float64))
    return np.real(np.fft.ifft2(F * mask))


def tv_denoise(f, theta=25.0, g=1.0, dt=0.1, iterations=5):
    """TotalVariationDenoising_3D.denoise3D/updateP/updateU in FP64 (TotalVariationDenoising_3D.java:84-202).
    f has shape (D, H, W); returns the denoised volume."""
    f = np.asarray(f, np.float64)
    u = f.copy()
    px = np.zeros_like(f)
    py = np.zeros_like(f)
    pz = np.zeros_like(f)
    for _ in range(iterations):
        dux = np.zeros_like(u); dux[:, :, :-1] = u[:, :, 1:] - u[:, :, :-1]
        duy = np.zeros_like(u); duy[:, :-1, :] = u[:, 1:, :] - u[:, :-1, :]
        duz = np.zeros_like(u); duz[:-1] = u[1:] - u[:-1]
        dd = 1 + dt / theta / g * np.abs(np.sqrt(duy * duy + dux * dux + duz * duz))
        px = (px - dt / theta * dux) / dd
        py = (py - dt / theta * duy) / dd
        pz = (pz - dt / theta * duz) / dd
        div = np.empty_like(u)
        div[:, :, 1:-1] = px[:, :, 1:-1] - px[:, :, :-2]
        div[:, :, 0] = px[:, :, 0]
        div[:, :, -1] = -px[:, :, -1]
        if u.shape[2] == 1:
            div[:, :, 0] = px[:, :, 0]
        dy = np.empty_like(u)
        dy[:, 1:-1] = py[:, 1:-1] - py[:, :-2]
        dy[:, 0] = py[:, 0]
        if u.shape[1] > 1:
            dy[:, -1] = -py[:, -1]
        dz = np.empty_like(u)
        dz[1:-1] = pz[1:-1] - pz[:-2]
        dz[0] = pz[0]
        if u.shape[0] > 1:
            dz[-1] = -pz[-1]
        u = f - theta * (div + dy + dz)
    return u


def order_shuffle(eulers, first):
    """TomoReconstruction2.orderShuffleART with a fixed first index (TomoReconstruction2.java:735-781)."""
    n = len(eulers)
    Wr = [np.asarray(e, np.float64)[2] for e in eulers]
    todo = [True] * n
    out = []
    im = first
    while len(out) < n:
        if out:
            mini, omini = np.finfo(np.float64).max, -1
            for o in range(n):
                if todo[o]:
                    sp = abs(float(Wr[im][0] * Wr[o][0] + Wr[im][1] * Wr[o][1] + Wr[im][2] * Wr[o][2]))
                    if sp < mini:
                        mini, omini = sp, o
            im = omini
        if todo[im]:
            out.append(im)
            todo[im] = False
    return np.array(out, np.int32)


def ossart_iteration(vol, g, eulers, meas, order, relax, update, y0=0, y1=None):
    """osartIteration (TomoReconstruction2.java:636-733) in FP64; vol is float64 and updated in place."""
    n = len(order)
    upd = n if update == 0 else update
    factor = relax / upd
    som, errmin, errmax, imin, imax = 0.0, float(np.finfo(np.float32).max), 0.0, 0, 0
    batch = []
    for t in range(n):
        batch.append(int(order[t]))
        if len(batch) == upd or t == n - 1:
            diffs = []
            for e, p in enumerate(batch):
                th, nm = project(vol, g, eulers[p], y0, y1)
                d, err = difference(np.asarray(meas[p], np.float64), th, nm, factor)
                diffs.append(d)
                som += err
                if err > errmax:
                    errmax, imax = err, order[t - len(batch) + e + 1]
                elif err < errmin:
                    errmin, imin = err, order[t - len(batch) + e + 1]
            for e, p in enumerate(batch):
                backproject(vol, g, eulers[p], diffs[e], y0, y1)
            batch = []
    WH = g.W * g.H
    return np.array([np.sqrt(som / (n * WH)), np.sqrt(errmin / WH), imin, np.sqrt(errmax / WH), imax])

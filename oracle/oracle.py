"""ctypes front-end of the C oracle (oracle/tomo_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py to check the engine and as the CPU baseline, never by the engine.

Parity status: unpinned (the reference ships no golden vectors and cannot be
run without a JDK); see tomo_oracle.c's header.

Array conventions (TomoReconstruction2 / TiltSeries layouts):
  volume       float32 (D, H, W)  -- D slices of W x H, x fastest
  projections  float32 (N, h, w)
  euler        float64 (N, 3, 3)  row-major Euler matrices
  transforms   float64 (N, 6)     java.awt.geom.AffineTransform flat matrix
                                  {m00, m10, m01, m11, m02, m12}
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libtomo_oracle.so")
_lib = None

FILL_NONE, FILL_AVG, FILL_NAN = 0, 1, 2


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, no fused multiply-add)."""
    src = os.path.join(_HERE, "tomo_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "_build/libtomo_oracle.so"],
                       check=True)
    return _LIB_PATH


class _Geom(C.Structure):
    _fields_ = [("W", C.c_int), ("H", C.c_int), ("D", C.c_int), ("w", C.c_int), ("h", C.c_int),
                ("vc", C.c_double * 3), ("pc", C.c_double * 4), ("scale", C.c_double),
                ("positivity", C.c_int), ("long_object", C.c_int)]


@dataclass
class Geom:
    """Volume/projection geometry; centres default to TomoJ's ((n-1)/2) rule
    (TomoReconstruction2.java:63-66, TiltSeries.java:161-170)."""
    W: int
    H: int
    D: int
    w: int
    h: int
    vc: tuple = None
    pc: tuple = None
    scale: float = 1.0
    positivity: bool = False
    long_object: bool = False

    def __post_init__(self):
        if self.vc is None:
            self.vc = ((self.W - 1) / 2.0, (self.H - 1) / 2.0, (self.D - 1) / 2.0)
        if self.pc is None:
            self.pc = ((self.w - 1.0) / 2, (self.h - 1.0) / 2, (self.w - 1) / 2.0, (self.h - 1) / 2.0)

    def c(self) -> _Geom:
        g = _Geom()
        g.W, g.H, g.D, g.w, g.h = self.W, self.H, self.D, self.w, self.h
        g.vc = (C.c_double * 3)(*self.vc)
        g.pc = (C.c_double * 4)(*self.pc)
        g.scale = self.scale
        g.positivity = int(self.positivity)
        g.long_object = int(self.long_object)
        return g


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        f32, f64, i32 = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int)
        G = C.POINTER(_Geom)
        L.or_set_threads.argtypes = [C.c_int]
        L.or_get_threads.restype = C.c_int
        L.or_euler.argtypes = [C.c_double, C.c_double, C.c_double, f64]
        L.or_project.argtypes = [f32, G, f64, C.c_int, C.c_int, f32, f32]
        L.or_difference.argtypes = [f32, f32, f32, f32, C.c_int, C.c_double]
        L.or_difference.restype = C.c_double
        L.or_backproject.argtypes = [f32, G, f64, f32, C.c_int, C.c_int]
        L.or_align.argtypes = [f32, C.c_int, C.c_int, f64, C.c_int, C.c_double, C.c_double, C.c_int, f32]
        L.or_align.restype = C.c_int
        L.or_weighting_mask.argtypes = [C.c_int, C.c_int, C.c_int, f64, f64, C.c_double, f32]
        L.or_weighting_apply.argtypes = [f32, C.c_int, C.c_int, f32]
        L.or_tv_denoise.argtypes = [f32, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_int]
        L.or_order_shuffle.argtypes = [C.c_int, f64, C.c_int, i32]
        L.or_ossart_iteration.argtypes = [f32, G, f64, f32, C.c_int, i32, C.c_double, C.c_int, C.c_int,
                                          C.c_int, f64, f64]
        L.or_wbp.argtypes = [f32, G, f64, f32, C.c_int, f32, C.c_int, C.c_int]
        L.or_fista_step.argtypes = [f32, f32, C.c_size_t, C.c_double]
        L.or_fista_step.restype = C.c_double
        L.or_ossart_iteration_into.argtypes = [f32, f32, G, f64, f32, C.c_int, i32, C.c_double, C.c_int, C.c_int,
                                               C.c_int, f64]
        L.or_bayes_start.argtypes = [f32, f32, C.c_int, C.c_int, C.c_int, C.c_double]
        L.or_bayes_end.argtypes = [f32, f32, C.c_size_t, C.c_double, C.c_int]
        L.or_bgart_collapse.argtypes = [f32, C.c_size_t, C.c_double, C.c_int, C.c_double]
        L.or_bgart_collapse.restype = C.c_double
        L.or_bgart_median_cross.argtypes = [f32, C.c_int, C.c_int, C.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def euler(phi: float, theta: float, psi: float) -> np.ndarray:
    R = np.zeros(9, np.float64)
    lib().or_euler(phi, theta, psi, _p(R, C.c_double))
    return R.reshape(3, 3)


def euler_tilt_y(theta_deg: float) -> np.ndarray:
    """AffineAlignment.getEulerMatrix with a vertical tilt axis (ta = 0):
    eulerAngles2Matrix(0, theta, -0) (AffineAlignment.java:389-395)."""
    return euler(0.0, theta_deg, -0.0)


def _vol(v):
    assert v.dtype == np.float32 and v.flags.c_contiguous and v.ndim == 3
    return v


def project(vol, g: Geom, R, y0=0, y1=None):
    """VoxelProjector3D.project for one Euler matrix -> (proj, norm)."""
    _vol(vol)
    y1 = g.H if y1 is None else y1
    R = np.ascontiguousarray(R, np.float64).reshape(9)
    proj = np.zeros((g.h, g.w), np.float32)
    norm = np.zeros((g.h, g.w), np.float32)
    gc = g.c()
    lib().or_project(_p(vol, C.c_float), C.byref(gc), _p(R, C.c_double), y0, y1, _p(proj, C.c_float),
                     _p(norm, C.c_float))
    return proj, norm


def difference(expv, th, norm, factor):
    expv = np.ascontiguousarray(expv, np.float32)
    th = np.ascontiguousarray(th, np.float32)
    norm = np.ascontiguousarray(norm, np.float32)
    diff = np.zeros_like(expv)
    err = lib().or_difference(_p(expv, C.c_float), _p(th, C.c_float), _p(norm, C.c_float),
                              _p(diff, C.c_float), expv.size, float(factor))
    return diff, err


def backproject(vol, g: Geom, R, proj, y0=0, y1=None):
    """In-place backprojection of one projection into volume rows [y0, y1)."""
    _vol(vol)
    y1 = g.H if y1 is None else y1
    R = np.ascontiguousarray(R, np.float64).reshape(9)
    proj = np.ascontiguousarray(proj, np.float32)
    gc = g.c()
    lib().or_backproject(_p(vol, C.c_float), C.byref(gc), _p(R, C.c_double), _p(proj, C.c_float), y0, y1)
    return vol


def align(unaligned, T, normalize=False, mean=0.0, std=1.0, fill=FILL_NAN):
    un = np.ascontiguousarray(unaligned, np.float32)
    h, w = un.shape
    T = np.ascontiguousarray(T, np.float64).reshape(6)
    out = np.zeros_like(un)
    rc = lib().or_align(_p(un, C.c_float), w, h, _p(T, C.c_double), int(normalize), float(mean), float(std),
                        int(fill), _p(out, C.c_float))
    if rc != 0:
        raise ValueError("transform is not invertible")
    return out


def weighting_mask(w, h, tilts, axes, diameter):
    tilts = np.ascontiguousarray(tilts, np.float64)
    axes = np.ascontiguousarray(axes if axes is not None else np.zeros_like(tilts), np.float64)
    mask = np.zeros((h, w), np.float32)
    lib().or_weighting_mask(w, h, tilts.size, _p(tilts, C.c_double), _p(axes, C.c_double), float(diameter),
                            _p(mask, C.c_float))
    return mask


def ramp_mask(w, h, tilts_deg, hamming=False):
    """The engine's ramp / Hamming-ramp WBP filters (not in the reference), as a 2-D mask
    for weighting_apply: dtheta |k| / w per column frequency k (dtheta / (4 w) at k = 0),
    times 0.54 + 0.46 cos(2 pi k / w) for Hamming, dtheta the mean tilt spacing in
    radians; constant along the row frequency."""
    t = np.asarray(tilts_deg, np.float64)
    dth = (t.max() - t.min()) * (np.pi / 180.0) / (t.size - 1) if t.size > 1 else np.pi
    i = np.arange(w)
    ci = np.where(i > w / 2.0, i - w, i).astype(np.float64)
    m = np.where(ci == 0, dth / (4.0 * w), dth * np.abs(ci) / w)
    if hamming:
        m = m * (0.54 + 0.46 * np.cos(2.0 * np.pi * ci / w))
    return np.ascontiguousarray(np.broadcast_to(m.astype(np.float32), (h, w)))


def weighting_apply(img, mask):
    out = np.array(img, np.float32, copy=True, order="C")
    h, w = out.shape
    mask = np.ascontiguousarray(mask, np.float32)
    lib().or_weighting_apply(_p(out, C.c_float), w, h, _p(mask, C.c_float))
    return out


def tv_denoise(vol, theta=25.0, g=1.0, dt=0.1, iterations=5):
    _vol(vol)
    D, H, W = vol.shape
    lib().or_tv_denoise(_p(vol, C.c_float), W, H, D, theta, g, dt, iterations)
    return vol


def order_shuffle(eulers, first):
    e = np.ascontiguousarray(eulers, np.float64)
    n = e.shape[0]
    idx = np.zeros(n, np.int32)
    lib().or_order_shuffle(n, _p(e, C.c_double), int(first), _p(idx, C.c_int))
    return idx


def ossart_iteration(vol, g: Geom, eulers, meas, order, relax, update, y0=0, y1=None):
    """One OS-SART iteration in place; returns (err5, per-projection sum of squares)."""
    _vol(vol)
    y1 = g.H if y1 is None else y1
    e = np.ascontiguousarray(eulers, np.float64)
    meas = np.ascontiguousarray(meas, np.float32)
    order = np.ascontiguousarray(order, np.int32)
    n = e.shape[0]
    if order.shape != (n,) or meas.shape[0] != n:
        raise ValueError("order must list every projection once (use update_step for one update)")
    err5 = np.zeros(5, np.float64)
    errs = np.zeros(n, np.float64)
    gc = g.c()
    lib().or_ossart_iteration(_p(vol, C.c_float), C.byref(gc), _p(e, C.c_double), _p(meas, C.c_float), n,
                              _p(order, C.c_int), float(relax), int(update), y0, y1, _p(err5, C.c_double),
                              _p(errs, C.c_double))
    return err5, errs


def update_step(vol, g: Geom, eulers, meas, batch, factor, y0=0, y1=None):
    """One update of osartIteration (TomoReconstruction2.java:678-719): forward project and
    difference every projection of `batch` against the current volume, then backproject
    the differences in batch order.  Returns the per-projection sums of squares."""
    _vol(vol)
    errs = np.zeros(len(batch))
    diffs = []
    for k, p in enumerate(batch):
        th, nm = project(vol, g, eulers[p], y0, y1)
        d, errs[k] = difference(meas[p], th, nm, factor)
        diffs.append(d)
    for k, p in enumerate(batch):
        backproject(vol, g, eulers[p], diffs[k], y0, y1)
    return errs


def wbp(vol, g: Geom, eulers, meas, mask=None, y0=0, y1=None):
    """WBP with update 0: weight (optional) then backproject each projection in index order."""
    _vol(vol)
    y1 = g.H if y1 is None else y1
    e = np.ascontiguousarray(eulers, np.float64)
    m = np.array(meas, np.float32, copy=True, order="C")
    mk = None if mask is None else np.ascontiguousarray(mask, np.float32)
    gc = g.c()
    lib().or_wbp(_p(vol, C.c_float), C.byref(gc), _p(e, C.c_double), _p(m, C.c_float), e.shape[0],
                 None if mk is None else _p(mk, C.c_float), y0, y1)
    return vol


def ossart_iteration_dual(vol, g1: Geom, eul1, meas1, order1, g2: Geom, eul2, meas2, order2, relax, update):
    """TomoReconstruction2.osartIterationDual (TomoReconstruction2.java:1282-1428) on one
    volume: for t = 0, 2, ... while t < n1 - 1, series 1 then series 2 add two projections
    each (each inner loop stops when t + 1 reaches its series' length); one counter
    shared by both series triggers, at `update` or at a series' last index, the
    projection + difference of that series' pending projections and their
    backprojection (update_step).  `update` is used as given (0 gives factor = inf).
    Returns err5 over (n1 + n2) projections."""
    n1, n2 = len(order1), len(order2)
    factor = float(np.float32(relax / update)) if update else float(np.float32(np.inf))
    st = {"diff": 0, "som": 0.0, "min": float(np.finfo(np.float32).max), "max": 0.0, "imin": 0, "imax": 0}
    pend = {1: [], 2: []}

    def add(which, g, eul, meas, order, n, t, i):
        pend[which].append(int(order[t + i]))
        st["diff"] += 1
        if st["diff"] == update or t + i == n - 1:
            errs = update_step(vol, g, eul, meas, pend[which], factor)
            for e, v in enumerate(errs):
                st["som"] += v
                if v > st["max"]:
                    st["max"], st["imax"] = v, int(order[t + i - len(errs) + e + 1])
                elif v < st["min"]:
                    st["min"], st["imin"] = v, int(order[t + i - len(errs) + e + 1])
            pend[which] = []
            st["diff"] = 0

    for t in range(0, n1 - 1, 2):
        for i in range(2):
            if t + 1 >= n1:
                break
            add(1, g1, eul1, meas1, order1, n1, t, i)
        for i in range(2):
            if t + 1 >= n2:
                break
            add(2, g2, eul2, meas2, order2, n2, t, i)
    wh = g1.W * g1.H
    return np.array([np.sqrt(st["som"] / ((n1 + n2) * wh)), np.sqrt(st["min"] / wh), st["imin"],
                     np.sqrt(st["max"] / wh), st["imax"]])


def fista_step(rec, prev, t):
    _vol(rec)
    _vol(prev)
    return lib().or_fista_step(_p(rec, C.c_float), _p(prev, C.c_float), rec.size, float(t))


def bayesian_iteration(vol, g: Geom, eulers, meas, order, relax, update, lam, alpha, y0=0, y1=None):
    """One OS-SART iteration driven through BayesianVoxelProjector3D
    (TomoJ_AdvancedReconstruction/.../projectors/BayesianVoxelProjector3D.java): the
    distance volume starts as -lambda times the 27-point [1,-2,1]^3 stencil of the volume,
    every update's differences are backprojected into it (the volume itself is projected
    unchanged all iteration), and the end adds alpha times it to the volume (positivity
    after, when g.positivity).  Returns err5."""
    _vol(vol)
    y1 = g.H if y1 is None else y1
    D, H, W = vol.shape
    dist = np.zeros_like(vol)
    L = lib()
    L.or_bayes_start(_p(vol, C.c_float), _p(dist, C.c_float), W, H, D, float(lam))
    e = np.ascontiguousarray(eulers, np.float64)
    meas = np.ascontiguousarray(meas, np.float32)
    order = np.ascontiguousarray(order, np.int32)
    err5 = np.zeros(5, np.float64)
    gc = g.c()
    L.or_ossart_iteration_into(_p(vol, C.c_float), _p(dist, C.c_float), C.byref(gc), _p(e, C.c_double),
                               _p(meas, C.c_float), e.shape[0], _p(order, C.c_int), float(relax), int(update), y0,
                               y1, _p(err5, C.c_double))
    L.or_bayes_end(_p(vol, C.c_float), _p(dist, C.c_float), vol.size, float(alpha), int(g.positivity))
    return err5


def bgart_collapse(vol, k, dark_bg=True, bg_value=float("nan")):
    """BgARTVoxelProjector3D.collapseFilter in place; returns the background value."""
    _vol(vol)
    return lib().or_bgart_collapse(_p(vol, C.c_float), vol.size, float(k), int(bool(dark_bg)), float(bg_value))


def bgart_median_cross(vol):
    """BgARTVoxelProjector3D.medianFilter3Dcross in place."""
    _vol(vol)
    D, H, W = vol.shape
    lib().or_bgart_median_cross(_p(vol, C.c_float), W, H, D)
    return vol


def ossart(vol, g: Geom, eulers, meas, n_iter, relax, update, first=0, y0=0, y1=None, end_of_iteration=None):
    """OSSART driver (TomoReconstruction2.java:548-634) with a fixed first index.
    end_of_iteration(vol) is called after every iteration (TVM / FISTA hooks)."""
    errs = []
    order = order_shuffle(eulers, first)
    for _ in range(n_iter):
        e5, _ = ossart_iteration(vol, g, eulers, meas, order, relax, update, y0, y1)
        if end_of_iteration is not None:
            end_of_iteration(vol)
        errs.append(e5)
    return np.array(errs)

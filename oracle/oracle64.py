"""FP64 build of the C oracle (oracle/tomo_oracle.c compiled with float widened to double).

TEST INFRASTRUCTURE ONLY: the reference each reduced-precision result is measured
against (tests/ and the precision leg of bench.py), never used by the engine.

Same algorithm, operation order and decisions as oracle.py (VoxelProjector3D
projection / backprojection, TomoReconstruction2 OS-SART, TotalVariationDenoising_3D),
every value held in double.  Pinned against the numpy FP64 twin (np_oracle.py) in
tests/test_oracle.py.  Arrays are float64 with the layouts of oracle.py.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from oracle.oracle import Geom

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libtomo_oracle64.so")
_lib = None


class _Geom(C.Structure):
    _fields_ = [("W", C.c_int), ("H", C.c_int), ("D", C.c_int), ("w", C.c_int), ("h", C.c_int),
                ("vc", C.c_double * 3), ("pc", C.c_double * 4), ("scale", C.c_double),
                ("positivity", C.c_int), ("long_object", C.c_int)]


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "tomo_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "_build/libtomo_oracle64.so"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        f64, i32 = C.POINTER(C.c_double), C.POINTER(C.c_int)
        G = C.POINTER(_Geom)
        L.or_set_threads.argtypes = [C.c_int]
        L.or_ossart_iteration.argtypes = [f64, G, f64, f64, C.c_int, i32, C.c_double, C.c_int, C.c_int, C.c_int,
                                          f64, f64]
        L.or_tv_denoise.argtypes = [f64, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int]
        L.or_order_shuffle.argtypes = [C.c_int, f64, C.c_int, i32]
        _lib = L
    return _lib


def _c(g: Geom) -> _Geom:
    c = _Geom()
    c.W, c.H, c.D, c.w, c.h = g.W, g.H, g.D, g.w, g.h
    c.vc = (C.c_double * 3)(*g.vc)
    c.pc = (C.c_double * 4)(*g.pc)
    c.scale = g.scale
    c.positivity = int(g.positivity)
    c.long_object = int(g.long_object)
    return c


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def ossart_iteration(vol, g: Geom, eulers, meas, order, relax, update, y0=0, y1=None):
    """One OS-SART iteration in place on a float64 (D, H, W) volume; returns err5."""
    if vol.dtype != np.float64 or not vol.flags.c_contiguous:
        raise TypeError("vol must be C-contiguous float64 (D, H, W)")
    y1 = g.H if y1 is None else y1
    e = np.ascontiguousarray(eulers, np.float64)
    m = np.ascontiguousarray(meas, np.float64)
    o = np.ascontiguousarray(order, np.int32)
    n = e.shape[0]
    err5 = np.zeros(5)
    errs = np.zeros(n)
    gc = _c(g)
    lib().or_ossart_iteration(_p(vol, C.c_double), C.byref(gc), _p(e, C.c_double), _p(m, C.c_double), n,
                              _p(o, C.c_int), float(relax), int(update), int(y0), int(y1), _p(err5, C.c_double),
                              _p(errs, C.c_double))
    return err5


def tv_denoise(vol, theta=25.0, g=1.0, dt=0.1, iterations=5):
    if vol.dtype != np.float64 or not vol.flags.c_contiguous:
        raise TypeError("vol must be C-contiguous float64 (D, H, W)")
    D, H, W = vol.shape
    lib().or_tv_denoise(_p(vol, C.c_double), W, H, D, float(theta), float(g), float(dt), int(iterations))
    return vol


def row_slab_sirt(series_rows, eulers, W, D, orders, relax=1.0, tv_from=None, tv=(25.0, 1.0, 0.01, 5)):
    """SIRT on one volume row of a vertical-axis series in FP64.

    With the tilt axis vertical and whole-row centre offsets each volume row is an
    independent 2-D problem, and the sampler's last-row rule only touches the last row.
    The row is solved as a two-row volume (row 0: the row, row 1: its neighbour) so that
    row 0 takes the interior form; series_rows is (N, 2, w).  orders: one tilt order per
    iteration.  Returns row 0 of the result, (D, W) float64."""
    n = series_rows.shape[0]
    w = series_rows.shape[2]
    g = Geom(W, 2, D, w, 2)
    vol = np.zeros((D, 2, W), np.float64)
    for it, order in enumerate(orders):
        ossart_iteration(vol, g, eulers, series_rows, order, relax, 0)
        if tv_from is not None and it >= tv_from:
            tv_denoise(vol, *tv)
    return vol[:, 0, :].copy()

"""The autotuner (tomo_autotune): candidate kernel shapes are timed on the handle itself,
the handle's volume comes back unchanged, and a tuned handle reconstructs what an untuned
one does: every candidate computes the same values, up to the FP32 summation order when a
different tilt grouping changes the forward projector's depth split (<= 1e-6 relative L2)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from tests.cases import rel_l2, series_case
from tomoj_gb300 import _abi

pytestmark = pytest.mark.gpu


def _handle(lib, c, vol, precision=_abi.PREC_FP32):
    g = _abi.make_geom(c["W"], c["H"], c["D"], c["w"], c["h"], c["n"])
    p = _abi.make_params(precision=precision)
    h = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(g), C.byref(p), C.byref(h)))
    eul = np.ascontiguousarray(c["eul"], np.float64)
    series = np.ascontiguousarray(c["series"], np.float32)
    _abi.check(lib.tomo_load_series(h, series.ctypes.data, 0, _abi.ptr(eul, C.c_double), None, None))
    v = np.ascontiguousarray(vol, np.float32)
    _abi.check(lib.tomo_set_volume(h, v.ctypes.data, 0, 0, c["H"]))
    return h


def _volume(lib, h, c):
    out = np.empty((c["D"], c["H"], c["W"]), np.float32)
    _abi.check(lib.tomo_get_volume(h, out.ctypes.data, 0, 0, c["H"]))
    return out


@pytest.mark.parametrize("precision", [_abi.PREC_FP32, _abi.PREC_FP16])
def test_autotune_keeps_volume_and_results(engine, precision):
    c = series_case(W=256, H=16, D=96, n=21, seed=6)
    start = (np.random.default_rng(2).random((c["D"], c["H"], c["W"]), dtype=np.float32) * 0.1).astype(np.float32)
    ha = _handle(engine, c, start, precision)
    hb = _handle(engine, c, start, precision)
    try:
        before = _volume(engine, ha, c)
        _abi.check(engine.tomo_add_projection(ha, 3))  # cleared by the autotuner
        out = np.zeros(4)
        _abi.check(engine.tomo_autotune(ha, 7, 2, _abi.ptr(out, C.c_double)))
        assert engine.tomo_projection_count(ha) == 0
        assert np.array_equal(_volume(engine, ha, c).view(np.uint32), before.view(np.uint32))
        tpc, rows, fp_ms, bp_ms = out
        assert 0 <= tpc <= 16 and rows in (0, 1, 2) and fp_ms > 0 and bp_ms > 0, out
        for h in (ha, hb):
            _abi.check(engine.tomo_run_ossart(h, 2, 1.0, 7, 11, 0, c["H"], 1, None))
        assert rel_l2(_volume(engine, ha, c), _volume(engine, hb, c)) <= 1e-6
    finally:
        engine.tomo_destroy(ha)
        engine.tomo_destroy(hb)

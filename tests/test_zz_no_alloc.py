"""The no-allocation projection entry point against the handle-based one.

tomo_project_and_difference_noalloc serves callers that cannot call cudaMalloc
(a JVM that keeps all device memory in its own pool, a serving loop that must
not synchronise on allocation mid-request, code held to a fixed memory budget):
it runs the same forward projection + difference on the caller's device buffers
with its scratch in a static device array.  This test calls it twice in a row
through the C ABI (different tilts and factors, so the shared scratch is
reused) and checks proj, norm, diff and the residuals against
tomo_project_and_difference on the same inputs, for a square case, projections
taller than the volume (rows left at zero), more than 256 detector columns and
off-centre volume / projection centres.  It lives in a file collected
last and passes alone or after the other tests (the first call does the
per-device set-up)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from tests.cases import rel_l2, series_case
from tomoj_gb300 import _abi

pytestmark = pytest.mark.gpu


CASES = {
    # name: (series_case keywords, vol_center, proj_center, [(tilts, factor), (tilts, factor)])
    "square": (dict(W=64, H=12, D=48, n=21, misalign=True), None, None,
               [([3, 17, 0, 9], float(np.float32(1.0 / 7))), ([20, 5, 11], 0.25)]),
    # taller projections: rows below (h - H) / 2 are left at zero, the kernel starts at j0 > 0
    "tall": (dict(W=64, H=12, D=48, n=21, w=64, h=16), None, None,
             [([1, 8, 19], 0.5), ([0, 10, 2, 14, 6], float(np.float32(1.0 / 5)))]),
    # wider than 256 detector columns: two columns per thread, fewer tilts per CTA
    "wide": (dict(W=288, H=6, D=40, n=9, w=300, h=6), None, None, [([0, 4, 8], 1.0), ([7, 2], 0.125)]),
    # centres off the middle by whole rows (the projection row offset stays integral)
    "centres": (dict(W=64, H=12, D=48, n=21, misalign=True), (33.5, 6.5, 20.5), (30.0, 6.5, 31.5, 5.5),
                [([4, 12, 16], 0.3), ([9, 1], 0.7)]),
}


@pytest.mark.parametrize("name", list(CASES))
def test_noalloc_projection_matches_handle_path_twice(engine, name):
    torch = pytest.importorskip("torch")
    kw, vc, pc, calls = CASES[name]
    c = series_case(**kw)
    W, H, D, w, h, n = c["W"], c["H"], c["D"], c["w"], c["h"], c["n"]
    geom = _abi.make_geom(W, H, D, w, h, n, vol_center=vc, proj_center=pc)
    params = _abi.make_params(fill=_abi.FILL_NAN)
    hd = C.c_void_p()
    _abi.check(engine.tomo_create(C.byref(geom), C.byref(params), C.byref(hd)))
    try:
        eul = np.ascontiguousarray(c["eul"], np.float64)
        T6 = np.ascontiguousarray(c["T"], np.float64)
        series = np.ascontiguousarray(c["series"], np.float32)
        _abi.check(engine.tomo_load_series(hd, series.ctypes.data, 0, _abi.ptr(eul, C.c_double),
                                           _abi.ptr(T6, C.c_double), None))
        vol = np.ascontiguousarray(c["vol"] * np.float32(0.9))
        _abi.check(engine.tomo_set_volume(hd, vol.ctypes.data, 0, 0, H))
        dvol = C.c_void_p()
        _abi.check(engine.tomo_volume_device_ptr(hd, C.byref(dvol)))
        aligned = np.empty((n, h, w), np.float32)
        for i in range(n):
            _abi.check(engine.tomo_get_aligned(hd, i, _abi.ptr(aligned[i])))
        meas = torch.from_numpy(aligned).cuda()
        for tilts, factor in calls:
            T = len(tilts)
            # existing entry point
            _abi.check(engine.tomo_clear_projections(hd))
            for t in tilts:
                _abi.check(engine.tomo_add_projection(hd, t))
            err_ref = np.zeros(T)
            _abi.check(engine.tomo_project_and_difference(hd, factor, 0, H, _abi.ptr(err_ref, C.c_double)))
            ref = {}
            for nm, fn in (("proj", engine.tomo_get_projection), ("norm", engine.tomo_get_norm),
                           ("diff", engine.tomo_get_difference)):
                ref[nm] = np.empty((T, h, w), np.float32)
                for k in range(T):
                    _abi.check(fn(hd, k, _abi.ptr(ref[nm][k])))
            # no-allocation entry point on caller buffers (filled with garbage first: the
            # call must write every output pixel, including the rows it leaves at zero)
            outs = {k: torch.full((T, h, w), 7.0, dtype=torch.float32, device="cuda") for k in ("proj", "norm", "diff")}
            tl = np.ascontiguousarray(tilts, np.int32)
            err = np.zeros(T)
            torch.cuda.synchronize()
            _abi.check(engine.tomo_project_and_difference_noalloc(
                C.byref(geom), _abi.ptr(eul, C.c_double), _abi.ptr(tl, C.c_int32), T, factor, dvol,
                C.c_void_p(meas.data_ptr()), C.c_void_p(outs["proj"].data_ptr()),
                C.c_void_p(outs["norm"].data_ptr()), C.c_void_p(outs["diff"].data_ptr()),
                _abi.ptr(err, C.c_double), None))
            torch.cuda.synchronize()
            got = {k: v.cpu().numpy() for k, v in outs.items()}
            assert np.array_equal(np.isnan(got["proj"]), np.isnan(ref["proj"]))
            for k in ("proj", "norm", "diff"):
                assert rel_l2(got[k], ref[k]) <= 1e-5, (name, k, rel_l2(got[k], ref[k]))
            assert np.allclose(err, err_ref, rtol=1e-9), (name, err, err_ref)
    finally:
        engine.tomo_destroy(hd)


def test_noalloc_rejects_sizes_beyond_its_scratch(engine):
    geom = _abi.make_geom(64, 8, 32, 4096, 8, 3)
    eul = np.zeros((3, 9))
    tl = np.zeros(1, np.int32)
    err = np.zeros(1)
    dummy = C.c_void_p(16)
    rc = engine.tomo_project_and_difference_noalloc(C.byref(geom), _abi.ptr(eul, C.c_double), _abi.ptr(tl, C.c_int32),
                                                    1, 1.0, dummy, dummy, dummy, dummy, dummy,
                                                    _abi.ptr(err, C.c_double), None)
    assert rc == -1 and b"2048" in engine.tomo_last_error()
    # a volume row too wide for the forward projector's shared memory is refused up front
    geom = _abi.make_geom(30000, 8, 32, 1024, 8, 3)
    rc = engine.tomo_project_and_difference_noalloc(C.byref(geom), _abi.ptr(eul, C.c_double), _abi.ptr(tl, C.c_int32),
                                                    1, 1.0, dummy, dummy, dummy, dummy, dummy,
                                                    _abi.ptr(err, C.c_double), None)
    assert rc == -1 and b"width" in engine.tomo_last_error()

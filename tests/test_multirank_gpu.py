"""Y-slab sharding of one reconstruction over two ranks on the engine (the partitioning
of ReconstructionThreadManagerGPU.doGPURec, ReconstructionThreadManagerGPU.java:172-308):
two processes each reconstruct their row slab through the Projector surface of the C ABI
(two CUDA contexts on the one GPU of this run; no kernel waits on another rank), the
per-projection FP64 residuals of every update are summed over gloo (the only exchange),
and the gathered volume and the error summaries equal the single-process engine
reconstruction of the whole volume (to FP32 rounding: a slab's smaller grid may add a
ray's depth parts in another order)."""
from __future__ import annotations

import ctypes as C
import os
import socket

import numpy as np
import pytest

from tests.cases import rel_l2, series_case

pytestmark = pytest.mark.gpu


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _surface_iterations(lib, h, eul, n, rows, n_iter, update, reduce=None):
    """osartIteration through the surface calls; returns per-iteration error summaries'
    inputs (per-projection residual sums in update order, the order)."""
    from oracle import oracle as O
    from tomoj_gb300 import _abi
    upd = n if update == 0 else update
    factor = float(np.float32(1.0 / upd))
    out = []
    for it in range(n_iter):
        order = O.order_shuffle(eul, it % n)
        per = np.zeros(n)
        for s0 in range(0, n, upd):
            batch = order[s0:s0 + upd]
            _abi.check(lib.tomo_clear_projections(h))
            for t in batch:
                _abi.check(lib.tomo_add_projection(h, int(t)))
            err = np.zeros(len(batch))
            _abi.check(lib.tomo_project_and_difference(h, factor, 0, rows, _abi.ptr(err, C.c_double)))
            if reduce is not None:
                err = reduce(err)
            per[s0:s0 + len(batch)] = err
            _abi.check(lib.tomo_backproject(h, 0, rows))
        out.append((per, order))
    return out


def _handle(lib, W, H, D, w, h, n, series, eul, vc=None, pc=None):
    from tomoj_gb300 import _abi
    geom = _abi.make_geom(W, H, D, w, h, n, vol_center=vc, proj_center=pc)
    prm = _abi.make_params(fill=_abi.FILL_NAN)
    hd = C.c_void_p()
    _abi.check(lib.tomo_create(C.byref(geom), C.byref(prm), C.byref(hd)))
    s = np.ascontiguousarray(series, np.float32)
    e = np.ascontiguousarray(eul, np.float64)
    # the series is aligned already (on whole images, before cropping): identity transforms
    _abi.check(lib.tomo_load_series(hd, s.ctypes.data, 0, _abi.ptr(e, C.c_double), None, None))
    return hd


def _rank_main(rank, world, port, case, meas, n_iter, update, out_dir):
    import torch
    import torch.distributed as dist
    from tomoj_gb300 import _abi, slabs
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lib = _abi.load()
        W, H, D, w, h, n = case["W"], case["H"], case["D"], case["w"], case["h"], case["n"]
        sl = slabs.plan(W, H, D, w, h, world)[rank]
        hd = _handle(lib, W, sl.rows, D, w, sl.proj_rows, n, slabs.crop_series(meas, sl), case["eul"],
                     sl.vol_center, sl.proj_center)
        try:
            def reduce(err):
                t = torch.tensor(err, dtype=torch.float64)
                dist.all_reduce(t)
                return t.numpy()
            runs = _surface_iterations(lib, hd, case["eul"], n, sl.rows, n_iter, update, reduce)
            vol = np.empty((D, sl.rows, W), np.float32)
            _abi.check(lib.tomo_get_volume(hd, vol.ctypes.data, 0, 0, sl.rows))
        finally:
            lib.tomo_destroy(hd)
        np.save(os.path.join(out_dir, f"vol{rank}.npy"), vol[:, :sl.y1 - sl.y0, :])
        np.save(os.path.join(out_dir, f"err{rank}.npy"),
                np.array([slabs.error_summary(per, order, W, H) for per, order in runs]))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("update", [0, 3])
def test_two_rank_engine_slabs_equal_single_process(engine, tmp_path, update):
    import torch.multiprocessing as mp
    from oracle import oracle as O
    from tomoj_gb300 import slabs
    c = series_case(W=64, H=9, D=32, n=9, seed=15, misalign=True)
    meas = np.array([O.align(c["series"][i], c["T"][i]) for i in range(c["n"])], np.float32)
    n_iter = 2
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, c, meas, n_iter, update, str(tmp_path)))
             for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(180)
        assert p.exitcode == 0
    got = np.concatenate([np.load(tmp_path / f"vol{r}.npy") for r in range(2)], axis=1)
    e0, e1 = np.load(tmp_path / "err0.npy"), np.load(tmp_path / "err1.npy")
    assert np.array_equal(e0, e1)
    # the whole volume in this process, same surface loop
    hd = _handle(engine, c["W"], c["H"], c["D"], c["w"], c["h"], c["n"], meas, c["eul"])
    try:
        runs = _surface_iterations(engine, hd, c["eul"], c["n"], c["H"], n_iter, update)
        ref = np.empty((c["D"], c["H"], c["W"]), np.float32)
        engine.tomo_get_volume(hd, ref.ctypes.data, 0, 0, c["H"])
    finally:
        engine.tomo_destroy(hd)
    ref_err = np.array([slabs.error_summary(per, order, c["W"], c["H"]) for per, order in runs])
    assert got.shape == ref.shape
    assert rel_l2(got, ref) <= 1e-6, rel_l2(got, ref)
    assert np.allclose(e0[:, [0, 1, 3]], ref_err[:, [0, 1, 3]], rtol=1e-5)

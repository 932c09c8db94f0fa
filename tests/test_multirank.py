"""Y-slab sharding of one reconstruction over two ranks (gloo, CPU): each rank runs the
oracle on its slab, the per-projection FP64 residuals are all-reduced, and the
gathered volume and error summaries equal the single-rank reconstruction."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from tests.cases import series_case


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, case, n_iter, update, out_dir):
    import torch
    from oracle import oracle as O
    from tomoj_gb300 import slabs
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    W, H, D, w, h, n = case["W"], case["H"], case["D"], case["w"], case["h"], case["n"]
    sl = slabs.plan(W, H, D, w, h, world)[rank]
    meas = np.array([O.align(case["series"][i], case["T"][i]) for i in range(n)], np.float32)
    sub = slabs.crop_series(meas, sl)
    g = O.Geom(W, sl.rows, D, w, sl.proj_rows, vc=sl.vol_center, pc=sl.proj_center)
    vol = np.zeros((D, sl.rows, W), np.float32)
    upd = n if update == 0 else update
    errs = []
    for it in range(n_iter):
        order = O.order_shuffle(case["eul"], it % n)
        per = np.zeros(n)
        for s0 in range(0, n, upd):
            batch = order[s0:s0 + upd]
            # per-projection residual of this slab, summed over ranks (the only exchange)
            factor = float(np.float32(1.0 / upd))
            errs_slab = O.update_step(vol, g, case["eul"], sub, batch, factor)
            t = torch.tensor(errs_slab, dtype=torch.float64)
            dist.all_reduce(t)
            per[s0:s0 + len(batch)] = t.numpy()
        if vol.shape[1] > sl.y1 - sl.y0:
            vol[:, sl.y1 - sl.y0:, :] = 0.0  # the halo row's values are never used
        errs.append(slabs.error_summary(per, order, W, H))
    np.save(os.path.join(out_dir, f"vol{rank}.npy"), vol[:, :sl.y1 - sl.y0, :])
    np.save(os.path.join(out_dir, f"err{rank}.npy"), np.array(errs))
    dist.destroy_process_group()


@pytest.mark.parametrize("update", [0, 3])
def test_two_rank_slabs_equal_single_rank(oracle_lib, tmp_path, update):
    from oracle import oracle as O
    c = series_case(W=32, H=7, D=20, n=7, seed=5, misalign=True)
    n_iter = 2
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, c, n_iter, update, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = np.concatenate([np.load(tmp_path / f"vol{r}.npy") for r in range(2)], axis=1)
    e0, e1 = np.load(tmp_path / "err0.npy"), np.load(tmp_path / "err1.npy")
    assert np.array_equal(e0, e1)
    # single-rank reference with the same subset structure
    meas = np.array([O.align(c["series"][i], c["T"][i]) for i in range(c["n"])], np.float32)
    ref = np.zeros_like(c["vol"])
    upd = c["n"] if update == 0 else update
    ref_err = []
    from tomoj_gb300 import slabs
    for it in range(n_iter):
        order = O.order_shuffle(c["eul"], it % c["n"])
        per = np.zeros(c["n"])
        for s0 in range(0, c["n"], upd):
            batch = order[s0:s0 + upd]
            per[s0:s0 + len(batch)] = O.update_step(ref, c["g"], c["eul"], meas, batch, float(np.float32(1.0 / upd)))
        ref_err.append(slabs.error_summary(per, order, c["W"], c["H"]))
    assert np.array_equal(got, ref)
    assert np.allclose(e0, np.array(ref_err), rtol=1e-12)


def test_wbp_on_slabs_equals_full_wbp(oracle_lib):
    # WBP backprojects measurements directly: the slab keeps its halo row's real values
    # (a NaN halo would void the last row's bilinear reads)
    from oracle import oracle as O
    from tomoj_gb300 import slabs
    c = series_case(W=32, H=9, D=20, n=7, seed=8, misalign=False, noise=0.0)
    meas = np.array(c["series"], np.float32)
    ref = np.zeros_like(c["vol"])
    O.wbp(ref, c["g"], c["eul"], meas, None)
    got = []
    for sl in slabs.plan(c["W"], c["H"], c["D"], c["w"], c["h"], 3):
        g = O.Geom(c["W"], sl.rows, c["D"], c["w"], sl.proj_rows, vc=sl.vol_center, pc=sl.proj_center)
        v = np.zeros((c["D"], sl.rows, c["W"]), np.float32)
        O.wbp(v, g, c["eul"], slabs.crop_series(meas, sl, halo_nan=False), None)
        got.append(v[:, :sl.y1 - sl.y0, :])
    assert np.array_equal(np.concatenate(got, axis=1), ref)

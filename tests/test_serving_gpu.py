"""Serving on the GPU: requests that arrive while others run are admitted and advance in
the shared batch, and every request's volume is the same as when it runs alone."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from tomoj_gb300 import _abi
from tomoj_gb300.serving import OSSART, SIRT, TVM, WBP, EngineAdapter, Server, summarize, synthetic_requests

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [_abi.PREC_FP32, _abi.PREC_FP16])
def test_each_result_is_the_same_alone_and_in_the_mix(engine, precision):
    """Three lanes (bounds between the sizes drawn) on prioritised streams, WBP on its worker."""
    reqs = synthetic_requests(6, seed=5, rate=200.0, sizes=(64, 96), thick=(24, 40), tilts=(21, 31),
                              mix=((WBP, 0.2), (SIRT, 0.3), (OSSART, 0.3), (TVM, 0.2)), iters=(2, 5),
                              keep_volume=True, precision=precision)
    reqs[0].kind, reqs[1].kind, reqs[2].kind = SIRT, OSSART, TVM
    reqs[1].update = 4
    for r in reqs[:3]:
        r.n_iter = max(r.n_iter, 2)
    eng = EngineAdapter()
    try:
        res = Server(eng, max_active=8, lane_bounds=(3e6, 6e6)).run(reqs)
        assert len({r.lane for r in res if r.kind != WBP}) >= 2
        s = summarize(res)
        assert s["requests"] == 6
        for r, q in zip(res, reqs):
            hd = eng.create(q)
            try:
                if q.kind == WBP:
                    eng.run_wbp(hd, q)
                else:
                    upd = 0 if q.kind in (SIRT, TVM) else q.update
                    _abi.check(eng.lib.tomo_run_ossart(hd, q.n_iter, q.relax, upd, q.seed, 0, q.H, 1, None))
                alone = eng.read_volume(hd, q)
            finally:
                eng.destroy(hd)
            assert np.array_equal(r.volume, alone), (q.rid, q.kind)
    finally:
        eng.close()

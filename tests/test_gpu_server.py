"""The continuous-batching server: solves submitted while others run are
admitted as slots free up, overlap on the device, and each result is bit for
bit the result of the same solve run alone through vacgpu_step."""
import time

import numpy as np
import pytest

from vac_gb300 import abi, inistate
from vac_gb300.engine import Engine, Server

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def _req(i):
    if i % 3 == 2:
        s = inistate.random_modes(16 + 4 * i, seed=i)
        p = inistate.params_for(s, limiter="woodward", precision=abi.PREC_MIXED)
    else:
        s = inistate.random_modes(40 + 16 * i, seed=i, ndim=2)
        p = inistate.params_for(s, limiter="minmod", precision=abi.PREC_MIXED)
    return p, s.x, s.w, 10 + 7 * i


def test_results_alone_equal_results_in_the_mix(gpu_lib):
    reqs = [_req(i) for i in range(7)]
    srv = Server(hbm_budget_bytes=2e9, max_active=4, steps_per_chunk=8)
    ids = []
    for i, (p, x, w, n) in enumerate(reqs):
        ids.append(srv.submit(p, x, w, n))
        if i == 3:
            time.sleep(0.05)  # later arrivals join a running mix
    results = [srv.result(rid, wait=120.0) for rid in ids]
    st = srv.stats()
    srv.close()
    assert st["done"] == len(reqs) and st["peak_active"] >= 2
    for (p, x, w, n), r in zip(reqs, results):
        assert r is not None
        e = Engine(p, x, w)
        e.step(n)
        state, t, it, tts = r
        assert it == n and t == e.t and tts > 0
        assert np.array_equal(bits(state), bits(e.state()))


def test_budget_admits_one_at_a_time(gpu_lib):
    reqs = [_req(i) for i in range(3)]
    srv = Server(hbm_budget_bytes=1.0, max_active=8, steps_per_chunk=4)
    ids = [srv.submit(p, x, w, n) for (p, x, w, n) in reqs]
    for rid in ids:
        assert srv.result(rid, wait=120.0, fetch=False) is not None
    assert srv.stats()["peak_active"] == 1
    srv.close()

"""Batched grids: every grid of a batch (persistent sweep kernels over all
grids' tiles in one CUDA graph, or, for 2-D grids, all steps of a call in
one cooperative launch) gives bit for bit the state, t and it of the same
grid advanced alone by vacgpu_step in the same precision, and stays within
the mixed tolerance of the FP64 oracle."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from vac_gb300 import abi, inistate
from vac_gb300.engine import Batch, Engine

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def test_batch_matches_single_grid_runs(gpu_lib):
    grids = inistate.riemann_batch(n=6, seed=3, lo=20, hi=90)
    b = Batch(grids)
    b.step(7)
    b.step(7)  # second call replays the captured graph
    for i, (p, x, w) in enumerate(grids):
        e = Engine(p, x, w)
        e.step(14)
        t, it, dt, fin = b.status(i)
        assert (it, t) == (e.it, e.t), (i, it, e.it, t, e.t)
        assert np.array_equal(bits(b.state(i)), bits(e.state())), i


def test_batch_mhd3d_and_tuner(gpu_lib):
    snaps = [inistate.random_modes(n, seed=i) for i, n in enumerate([12, 20, 33])]
    grids = [(inistate.params_for(s, limiter="woodward", precision=abi.PREC_MIXED), s.x, s.w)
             for s in snaps]
    b = Batch(grids)
    ctas, order, rows, one, ms = b.tune()
    assert ctas > 0 and order in (0, 1) and rows == 0 and not one and len(ms) == 6
    b.step(5)
    for i, (p, x, w) in enumerate(grids):
        e = Engine(p, x, w)
        e.step(5)
        assert np.array_equal(bits(b.state(i)), bits(e.state())), i
        o = Oracle(inistate.params_for(snaps[i], limiter="woodward"), x, w)
        o.step(5)
        ref, got = o.state(), b.state(i)
        for iw in range(p.nw):
            rel = np.abs(got[iw] - ref[iw]).sum() / np.abs(ref[iw]).sum()
            assert rel <= 1e-5, (i, iw, rel)


def test_batch_mhd2d_general_and_tuned_rows(gpu_lib):
    """2-D MHD grids of different sizes on the warp-marching line sweep, one
    of them with reflecting walls, so the batch runs the sweep's general
    form while the periodic grids alone run its fast form: the same bits.
    The tuner picks the rows per work item: 16, or a guided list whose
    items shrink toward its end (chunking does not change any
    arithmetic)."""
    from tests.test_gpu_fused import reflecting
    snaps = [inistate.orszag_tang(n) for n in (40, 75, 130)]
    grids = []
    for i, s in enumerate(snaps):
        p = inistate.params_for(s, limiter="woodward", precision=abi.PREC_MIXED)
        if i == 1:
            reflecting(p, 2)
        grids.append((p, s.x, s.w))
    b = Batch(grids)
    ctas, order, rows, one, ms = b.tune()
    assert rows in (16, -32, -16) and len(ms) == 24
    b.step(6)
    for i, (p, x, w) in enumerate(grids):
        e = Engine(p, x, w)
        e.step(6)
        assert np.array_equal(bits(b.state(i)), bits(e.state())), i


@pytest.mark.parametrize("form", ["graph", "one_launch"])
@pytest.mark.parametrize("case", ["hd_outflow", "mhd_periodic", "mhd_reflecting"])
def test_batch_line_sweep_forms(gpu_lib, monkeypatch, form, case):
    """Both forms of a 2-D line-sweep batch, forced through VACGPU_ONELAUNCH:
    the graph of launches per step, and all steps of a call in one
    cooperative launch with grid-wide barriers between the phases.  Each
    gives the bits, t and it of the grids advanced alone, over two calls,
    and with a tstop that the grids reach at different steps (grids that
    are done sit out the remaining steps of the launch), and over the call
    after it, which steps grids at different parities of it."""
    monkeypatch.setenv("VACGPU_ONELAUNCH", "1" if form == "one_launch" else "0")
    if case == "hd_outflow":
        grids = inistate.riemann_batch(n=5, seed=7, lo=24, hi=140)
    else:
        from tests.test_gpu_fused import reflecting
        grids = []
        for k, n in enumerate((36, 64, 100)):
            s = inistate.orszag_tang(n)
            p = inistate.params_for(s, limiter="woodward", precision=abi.PREC_MIXED)
            if case == "mhd_reflecting" and k == 1:
                reflecting(p, 2)  # the whole batch runs the general form
            grids.append((p, s.x, s.w))
    b = Batch(grids)
    ctas, order, rows, one, ms = b.tune()
    assert bool(one) == (form == "one_launch") and ctas > 0
    b.step(3)
    b.step(4)
    assert (b.tune()[3] in (1, 2)) == (form == "one_launch")
    for i, (p, x, w) in enumerate(grids):
        e = Engine(p, x, w)
        e.step(7)
        t, it, dt, fin = b.status(i)
        assert (it, t) == (e.it, e.t), (i, it, e.it, t, e.t)
        assert np.array_equal(bits(b.state(i)), bits(e.state())), i
    # a stop time that the grids reach at different steps, of both parities
    for k in (4, 5, 3, 6):
        e0 = Engine(*grids[0])
        e0.step(k)
        tstop = e0.t
        singles = [Engine(*g) for g in grids]
        for e in singles:
            e.step(9, tstop)
        if len({e.it % 2 for e in singles}) > 1:
            break
    else:
        pytest.fail("no stop time leaves the grids at different parities of it")
    b2 = Batch(grids)
    b2.step(9, tstop)
    its = set()
    for i, e in enumerate(singles):
        t, it, dt, fin = b2.status(i)
        its.add(it % 2)
        assert (it, t) == (e.it, e.t), (i, it, e.it, t, e.t)
        assert np.array_equal(bits(b2.state(i)), bits(e.state())), i
    # the grids stopped at different parities of it; the next call steps each
    # with the sweep order of its own it ('xyyx')
    assert its == {0, 1}
    b2.step(5)
    for i, e in enumerate(singles):
        e.step(5)
        t, it, dt, fin = b2.status(i)
        assert (it, t) == (e.it, e.t), (i, it, e.it, t, e.t)
        assert np.array_equal(bits(b2.state(i)), bits(e.state())), i


def test_batch3d_refuses_mixed_parities(gpu_lib):
    """A 3-D batch whose grids a stop time left at different parities of it
    ('xyyx': each grid's next step starts with the sweep its own it
    selects) refuses the next call instead of stepping some grids in the
    wrong order."""
    snaps = [inistate.random_modes(n, seed=i) for i, n in enumerate([12, 20, 33])]
    grids = [(inistate.params_for(s, limiter="woodward", precision=abi.PREC_MIXED), s.x, s.w)
             for s in snaps]
    for k in (4, 5, 3, 6):
        e0 = Engine(*grids[0])
        e0.step(k)
        singles = [Engine(*g) for g in grids]
        for e in singles:
            e.step(9, e0.t)
        if len({e.it % 2 for e in singles}) > 1:
            break
    else:
        pytest.fail("no stop time leaves the grids at different parities of it")
    b = Batch(grids)
    b.step(9, e0.t)
    with pytest.raises(RuntimeError, match="parities"):
        b.step(2)

"""Asynchronous snapshots (vacgpu_snapshot_begin / vacgpu_snapshot_wait):
the state VAC's timetosave event would write (src/vac.t:56-58,631-661),
copied off the device while later steps run.  A snapshot equals the state
downloaded at the same point bit for bit, in both precisions and both
slots, and the steps that run while it is in flight are unchanged."""
import numpy as np
import pytest

from vac_gb300 import abi, inistate


def _bits(a):
    return a.view(np.uint64)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [abi.PREC_FP64, abi.PREC_MIXED])
def test_snapshot_equals_download_and_overlaps_steps(gpu_lib, prec):
    from vac_gb300.engine import Engine
    s = inistate.random_modes(24, seed=5, p0=0.5)
    p = inistate.params_for(s, limiter="woodward", precision=prec)
    ref = Engine(p, s.x, s.w)
    ref.step(3)
    w3 = ref.state()
    ref.step(4)
    w7 = ref.state()
    ref.step(2)
    w9 = ref.state()
    e = Engine(p, s.x, s.w)
    e.step(3)
    e.snapshot_begin(0)
    e.step(4)                    # runs while slot 0 is in flight
    e.snapshot_begin(1)
    e.step(2)
    assert np.array_equal(_bits(e.snapshot_wait(1)), _bits(w7))
    assert np.array_equal(_bits(e.snapshot_wait(0)), _bits(w3))
    assert np.array_equal(_bits(e.state()), _bits(w9))
    assert (e.it, e.t) == (ref.it, ref.t)
    # a slot is reusable after its wait
    e.snapshot_begin(0)
    assert np.array_equal(_bits(e.snapshot_wait(0)), _bits(w9))


@pytest.mark.gpu
def test_snapshot_slot_errors(gpu_lib):
    from vac_gb300.engine import Engine
    s = inistate.orszag_tang(16)
    e = Engine(inistate.params_for(s), s.x, s.w)
    with pytest.raises(RuntimeError, match="no snapshot in flight"):
        e.snapshot_wait(1)
    with pytest.raises(RuntimeError, match="slot must be 0 or 1"):
        e.snapshot_begin(2)
    e.snapshot_begin(0)
    with pytest.raises(RuntimeError, match="still in flight"):
        e.snapshot_begin(0)
    e.step(2)
    e.snapshot_wait(0)

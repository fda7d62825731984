"""The kernels' device waits are bounded: a TMA copy that never completes
an mbarrier phase, or a CTA of the one-launch batched step that never
reaches a grid-wide barrier, makes the wait give up after its limit and
report a fault, which the host reads, instead of hanging the GPU.

The failure is made without a fault: vacgpu_test_bounded_waits waits on an
mbarrier phase that nothing completes and runs a cooperative launch in
which one CTA skips the barrier, each with a limit of about 2^22 cycles.
Afterwards the context is still usable: a grid steps to the same bits as
on a fresh engine."""
import ctypes as C

import numpy as np
import pytest

from vac_gb300 import abi, inistate
from vac_gb300.engine import Engine

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def test_bounded_waits_give_up_and_report(gpu_lib):
    s = inistate.orszag_tang(48)
    p = inistate.params_for(s, limiter="woodward", precision=abi.PREC_MIXED)
    before = Engine(p, s.x, s.w)
    before.step(3)
    m, g = C.c_int(-1), C.c_int(-1)
    gpu_lib.vacgpu_test_bounded_waits.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
    assert gpu_lib.vacgpu_test_bounded_waits(C.byref(m), C.byref(g)) == 0
    assert (m.value, g.value) == (1, 1)
    after = Engine(p, s.x, s.w)
    after.step(3)
    assert (after.it, after.t) == (before.it, before.t)
    assert np.array_equal(bits(after.state()), bits(before.state()))

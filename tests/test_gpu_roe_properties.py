"""Size-independent properties of the TVD-MUSCL/Roe corrector ('tvdmu') at
sizes beyond the oracle's: the flux form conserves the volume sums without
the Powell source (FP64 to double rounding, mixed to FP32 rounding), and a
uniform state stays bit for bit uniform (every jump is zero, so every
dissipative flux is)."""
import numpy as np
import pytest

from vac_gb300 import abi, inistate
from vac_gb300.engine import Engine

pytestmark = pytest.mark.gpu


def _params(s, precision):
    p = inistate.params_for(s, limiter="woodward", precision=precision)
    p.typefull = abi.TVDMU
    p.divbfix = 0
    return p


@pytest.mark.parametrize("precision,n,tol", [(abi.PREC_MIXED, 192, 2e-7),
                                             (abi.PREC_FP64, 128, 1e-13)],
                         ids=["mixed-192", "fp64-128"])
def test_tvdmu_conserves_volume_sums(precision, n, tol):
    s = inistate.random_modes(n, seed=0)
    e = Engine(_params(s, precision), s.x, s.w)
    m0 = e.sums()
    e.step(4)
    m1 = e.sums()
    e.close()
    scale = np.abs(s.w).reshape(s.w.shape[0], -1).mean(axis=1)
    assert np.all(np.abs(m1 - m0) <= tol * np.maximum(scale, 1e-3)), (m1 - m0) / scale


@pytest.mark.parametrize("precision", [abi.PREC_MIXED, abi.PREC_FP64],
                         ids=["mixed", "fp64"])
def test_tvdmu_uniform_state_is_preserved_exactly(precision):
    n = 96
    s = inistate.random_modes(n, seed=0)
    w = s.w.copy()
    for iw in range(w.shape[0]):
        w[iw] = w[iw].mean()
    p = _params(s, precision)
    p.divbfix = 1
    e = Engine(p, s.x, w)
    e.step(4)
    out = e.state()
    e.close()
    for iw in range(w.shape[0]):
        assert np.all(out[iw] == out[iw].flat[0]), iw
        ref = np.float32(w[iw].flat[0]) if precision == abi.PREC_MIXED else w[iw].flat[0]
        assert abs(out[iw].flat[0] - ref) <= 1e-7 * abs(w[iw].flat[0]) + 1e-30, iw

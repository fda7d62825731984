"""Host-side helpers of bench.py (CPU): the served stream's device-side
initial-state generator follows vac_gb300.inistate.random_modes draw for
draw (the same seeded modes, amplitudes and phases) and differs from the
NumPy evaluation by rounding only; the error and physicality summaries."""
import numpy as np
import pytest

import bench
from vac_gb300 import inistate


@pytest.mark.parametrize("n,nd,seed", [(8, 3, 3), (12, 2, 7), (6, 3, 101)])
def test_random_modes_dev_matches_numpy(n, nd, seed):
    pytest.importorskip("torch")
    x, w = bench.random_modes_dev(n, seed, nd, "cpu")
    s = inistate.random_modes(n, seed=seed, ndim=nd)
    assert np.array_equal(x, s.x)
    assert w.shape == s.w.shape
    assert np.allclose(w, s.w, rtol=1e-12, atol=1e-13)


def test_errors_and_physical():
    a = np.ones((2, 4, 4))
    b = a.copy()
    b[1, 0, 0] = 1.5
    l1, linf = bench._errors(b, a)
    assert l1 == [0.0, 0.5 / 16] and linf == [0.0, 0.5]
    s = inistate.random_modes(6, seed=1)
    ph = bench._physical(s.w, 5.0 / 3.0, True)
    assert abs(ph["min_p"] - 0.05) < 1e-12 and ph["min_rho"] > 0.79

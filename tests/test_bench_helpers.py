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


@pytest.mark.parametrize("n,nd", [(6, 2), (5, 3)])
def test_random_modes_dev_packed_layout(n, nd):
    """The served stream's requests drawn straight into the C ABI's packed
    layout (each component in Fortran order, permuted on the device) are the
    unpacked draw run through the binding's own packing, and the server's
    submit takes them as they are."""
    pytest.importorskip("torch")
    from vac_gb300.engine import pack_mesh
    x, w = bench.random_modes_dev(n, 3, nd, "cpu")
    xf, wf = bench.random_modes_dev(n, 3, nd, "cpu", packed=True)
    assert xf.ndim == 1 and wf.ndim == 1
    assert np.array_equal(pack_mesh(x), xf)
    assert np.array_equal(pack_mesh(w), wf)


def test_served_requests_are_seeded():
    """The served stream (kind, side, steps, seed) is the same on every run:
    half 2-D sides in [128, 2048], half 3-D sides in [64, 256], 20..500
    steps."""
    class A:
        served = 200
    r1, r2 = bench._served_requests(A), bench._served_requests(A)
    assert r1 == r2 and len(r1) == 200
    for nd, n, steps, seed in r1:
        assert (nd == 2 and 128 <= n <= 2048) or (nd == 3 and 64 <= n <= 256)
        assert 20 <= steps <= 500

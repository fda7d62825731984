"""Algebraic identities the mixed-precision kernels rely on, checked in
float64 on random states (no GPU).

* The fused sweep takes the thermal pressure of a face's mean state
  M = (L+R)/2 from the two face-state pressures (physics_mixed.cuh,
  cmax_mean):
      p(M) = (pL+pR)/2 + (g-1) (|rhoR mL - rhoL mR|^2 / (4 rhoL rhoR (rhoL+rhoR))
                                + |BL-BR|^2 / 8).
* The mixed Roe average forms the fast/slow speeds without cancellation
  (roe.cuh, average_mhd_f32): cf^2-cs^2 = sqrt((a2-b2)^2 + 4 a2 bt2) and
  cs^2 = a2 ca2 / cf^2, equal to the reference's
  cs^2 = ((a2+b2) - sqrt((a2+b2)^2 - 4 a2 ca2)) / 2 and cf^2 = a2+b2-cs^2
  (src/vacphys.mhdroe.t:57-70).
"""
import numpy as np
import pytest

GAMMA = 5.0 / 3.0


def pthermal(w, ndir, mhd):
    rho, m, e = w[0], w[1:1 + ndir], w[1 + ndir]
    p = e - 0.5 * (m * m).sum(axis=0) / rho
    if mhd:
        b = w[2 + ndir:2 + 2 * ndir]
        p = p - 0.5 * (b * b).sum(axis=0)
    return (GAMMA - 1.0) * p


def random_states(rng, n, ndir, mhd):
    rho = rng.uniform(0.1, 3.0, n)
    v = rng.normal(0.0, 1.0, (ndir, n))
    p = rng.uniform(0.01, 2.0, n)
    w = [rho, *(rho * v)]
    kin = 0.5 * rho * (v * v).sum(axis=0)
    if mhd:
        b = rng.normal(0.0, 2.0, (ndir, n))
        e = p / (GAMMA - 1.0) + kin + 0.5 * (b * b).sum(axis=0)
        w += [e, *b]
    else:
        w += [p / (GAMMA - 1.0) + kin]
    return np.array(w)


@pytest.mark.parametrize("ndir,mhd", [(1, False), (2, False), (3, False),
                                      (2, True), (3, True)])
def test_mean_state_pressure_identity(ndir, mhd):
    rng = np.random.default_rng(7 + ndir + 10 * mhd)
    L = random_states(rng, 4096, ndir, mhd)
    R = random_states(rng, 4096, ndir, mhd)
    M = 0.5 * (L + R)
    pL, pR = pthermal(L, ndir, mhd), pthermal(R, ndir, mhd)
    t = R[0] * L[1:1 + ndir] - L[0] * R[1:1 + ndir]
    corr = (t * t).sum(axis=0) / (4.0 * L[0] * R[0] * (L[0] + R[0]))
    if mhd:
        db = L[2 + ndir:] - R[2 + ndir:]
        corr = corr + 0.125 * (db * db).sum(axis=0)
    assert (corr >= 0).all()
    lhs = pthermal(M, ndir, mhd)
    rhs = 0.5 * (pL + pR) + (GAMMA - 1.0) * corr
    scale = np.abs(M[1 + ndir]) * (GAMMA - 1.0)  # the energy scale
    assert np.max(np.abs(lhs - rhs) / scale) < 1e-13


def test_cancellation_free_fast_slow_speeds():
    rng = np.random.default_rng(11)
    n = 4096
    a2 = 10.0 ** rng.uniform(-3, 1, n)
    ca2 = 10.0 ** rng.uniform(-3, 1, n)
    bt2 = 10.0 ** rng.uniform(-3, 1, n)
    b2 = ca2 + bt2
    s = a2 + b2
    root = np.sqrt(s * s - 4.0 * a2 * ca2)
    cf2_ref, cs2_ref = 0.5 * (s + root), 0.5 * (s - root)
    dr = np.sqrt((a2 - b2) ** 2 + 4.0 * a2 * bt2)
    cf2 = 0.5 * (a2 + b2 + dr)
    cs2 = a2 * ca2 / cf2
    assert np.allclose(dr, root, rtol=1e-12, atol=0)
    assert np.allclose(cf2, cf2_ref, rtol=1e-13, atol=0)
    # the reference's difference form loses digits where cs^2 << cf^2;
    # compare against it only to its own rounding level
    assert np.all(np.abs(cs2 - cs2_ref) <= 1e-12 * cf2_ref)

"""The fused single-kernel sweep of the mixed path (TMA-fed z-marching
tiles): against the FP64 oracle within the mixed tolerance, and against the
split predictor/corrector kernels of the same precision, on periodic,
outflow ('cont') and reflecting ('symm'/'asymm') boundaries and on grids that
are not multiples of the 32x8 tile."""
import os

import numpy as np
import pytest

from oracle.oracle import Oracle
from vac_gb300 import abi, inistate
from vac_gb300.engine import Engine

pytestmark = pytest.mark.gpu

MIXED_REL_L1 = 1e-5     # mixed path vs FP64 oracle, per variable
FUSED_VS_SPLIT = 1e-6   # fused vs split FP32 kernels (different rounding only)


def rel_l1(a, b):
    return [float(np.abs(a[i] - b[i]).sum() / max(np.abs(b[i]).sum(), 1e-300))
            for i in range(a.shape[0])]


def reflecting(p, ndim):
    """symm walls, asymm for the normal momentum (and normal B)."""
    for d in range(ndim):
        for side in (0, 1):
            for iw in range(p.nw):
                p.typeB[2 * d + side][iw] = abi.BC_SYMM
            p.typeB[2 * d + side][1 + d] = abi.BC_ASYMM
            if p.physics == abi.PHYS_MHD:
                p.typeB[2 * d + side][p.ndir + 2 + d] = abi.BC_ASYMM


def _blast(n):
    s = inistate.blast_3d(n)
    return s


CASES = [
    ("rm3-periodic-40", lambda: inistate.random_modes(40, seed=4), "woodward", "periodic", 12, None),
    ("blast3-cont-36", lambda: _blast(36), "woodward", "cont", 10, None),
    ("rm3-reflect-33", lambda: inistate.random_modes(33, seed=5), "minmod", "symm", 8,
     lambda p: reflecting(p, 3)),
    ("hd2-cont-70x50", lambda: _hd(70, 50), "minmod", "cont", 20, None),
    ("ot2-periodic-64", lambda: inistate.orszag_tang(64), "minmod", "periodic", 30, None),
    ("ot2-reflect-45", lambda: inistate.orszag_tang(45), "woodward", "symm", 15,
     lambda p: reflecting(p, 2)),
]


def _hd(nx, ny):
    s = inistate.riemann_2d(8, 11)
    x = inistate.domain_grid((nx, ny), (0.0, 0.0), (1.0, 1.0))
    X, Y = x
    left = X + 0.3 * Y < 0.6
    rho = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    w = inistate.conserve_hd(rho, [np.where(left, 0.2, -0.1), np.zeros_like(X)], p, 1.4)
    s.x, s.w, s.nx = x, w, (nx, ny)
    return s


@pytest.mark.parametrize("name,mk,lim,bc,n,tweak", CASES, ids=[c[0] for c in CASES])
def test_fused_against_oracle_and_split(gpu_lib, monkeypatch, name, mk, lim, bc, n, tweak):
    s = mk()
    p64 = inistate.params_for(s, limiter=lim, bc=bc)
    pm = inistate.params_for(s, limiter=lim, bc=bc, precision=abi.PREC_MIXED)
    if tweak:
        tweak(p64)
        tweak(pm)
    o = Oracle(p64, s.x, s.w)
    o.step(n)
    ref = o.state()
    monkeypatch.setenv("VACGPU_FUSED", "1")
    ef = Engine(pm, s.x, s.w)
    ef.step(n)
    wf = ef.state()
    st = ef.kernel_stats()
    assert st["sweep"][0] > 0, "fused kernel did not run"
    monkeypatch.setenv("VACGPU_FUSED", "0")
    es = Engine(pm, s.x, s.w)
    es.step(n)
    ws = es.state()
    assert es.kernel_stats()["sweep"][0] == 0
    assert max(rel_l1(wf, ref)) <= MIXED_REL_L1, rel_l1(wf, ref)
    assert max(rel_l1(wf, ws)) <= FUSED_VS_SPLIT, rel_l1(wf, ws)


def test_z_chunk_tuning_is_invisible(monkeypatch):
    """At 128^3 the first step call tunes the fused sweep's z chunk from a
    snapshot of the state; the run must be bit-identical to one with the
    chunk pinned (VACGPU_NZC), in state, t and it."""
    s = inistate.random_modes(128, seed=5)
    p = inistate.params_for(s, limiter="woodward", precision=abi.PREC_MIXED)
    tuned = Engine(p, s.x, s.w)
    tuned.step(4)
    monkeypatch.setenv("VACGPU_NZC", "32")
    pinned = Engine(p, s.x, s.w)
    pinned.step(4)
    assert (tuned.it, tuned.t) == (pinned.it, pinned.t)
    assert np.array_equal(tuned.state().view(np.uint64), pinned.state().view(np.uint64))


def test_full_size_conservation_and_symmetry():
    """The benchmark's workload at its full size (256^3 random-mode MHD,
    woodward, periodic, mixed, fused sweeps): without the Powell source the
    flux form conserves mass, momentum, energy and B (volume sums, FP64,
    relative to their scale); and a state mirrored in x evolves into the
    mirror image (m_x and B_x change sign) to FP32 rounding."""
    n = 256
    s = inistate.random_modes(n, seed=0)
    p = inistate.params_for(s, limiter="woodward", precision=abi.PREC_MIXED)
    p.divbfix = 0
    e = Engine(p, s.x, s.w)
    m0 = e.sums()
    e.step(6)
    m1 = e.sums()
    scale = np.abs(s.w).reshape(s.w.shape[0], -1).mean(axis=1)
    assert np.all(np.abs(m1 - m0) <= 2e-7 * np.maximum(scale, 1e-3)), (m1 - m0) / scale
    a = e.state()
    e.close()
    # mirror x -> -x about the box centre: cell i <-> n-1-i
    w = s.w[:, ::-1].copy()
    w[1] = -w[1]
    w[5] = -w[5]
    em = Engine(p, s.x, w)
    em.step(6)
    b = em.state()[:, ::-1]
    em.close()
    b[1] = -b[1]
    b[5] = -b[5]
    rel = [float(np.abs(a[i] - b[i]).sum() / np.abs(a[i]).sum()) for i in range(a.shape[0])]
    assert max(rel) <= 1e-5, rel


def test_full_size_uniform_state_is_preserved_exactly():
    """A uniform state at 256^3 stays bit for bit uniform: identical face
    fluxes cancel exactly and div B is zero."""
    n = 256
    s = inistate.random_modes(n, seed=0)
    w = s.w.copy()
    for iw in range(w.shape[0]):
        w[iw] = w[iw].mean()
    p = inistate.params_for(s, limiter="woodward", precision=abi.PREC_MIXED)
    e = Engine(p, s.x, w)
    e.step(4)
    out = e.state()
    e.close()
    for iw in range(w.shape[0]):
        assert np.all(out[iw] == out[iw].flat[0])
        assert abs(out[iw].flat[0] - np.float32(w[iw].flat[0])) <= 1e-7 * abs(w[iw].flat[0]) + 1e-30


GRAVITY_CASES = [
    ("hd2-gravity-cont", lambda: inistate.riemann_2d(48, 5), "woodward", "cont", 12, [0.0, -0.5]),
    ("ot2-gravity-periodic", lambda: inistate.orszag_tang(40), "minmod", "periodic", 10,
     [0.3, -0.2]),
    ("rm3-gravity-periodic", lambda: inistate.random_modes(20, seed=6), "woodward", "periodic", 6,
     [0.2, 0.0, -0.3]),
]


@pytest.mark.parametrize("name,mk,lim,bc,n,grav", GRAVITY_CASES, ids=[c[0] for c in GRAVITY_CASES])
def test_fused_with_gravity(gpu_lib, monkeypatch, name, mk, lim, bc, n, grav):
    """The fused sweeps' general form (the gravity source of vacusr.gravity.t
    in the predictor and the corrector) against the oracle and the split
    kernels."""
    s = mk()
    p64 = inistate.params_for(s, limiter=lim, bc=bc)
    pm = inistate.params_for(s, limiter=lim, bc=bc, precision=abi.PREC_MIXED)
    o = Oracle(p64, s.x, s.w)
    o.register_source(abi.SRC_GRAVITY, grav)
    o.step(n)
    ref = o.state()
    out = {}
    for fz in ("1", "0"):
        monkeypatch.setenv("VACGPU_FUSED", fz)
        e = Engine(pm, s.x, s.w)
        e.register_source(abi.SRC_GRAVITY, grav)
        e.step(n)
        out[fz] = e.state()
        assert (e.kernel_stats()["sweep"][0] > 0) == (fz == "1")
    assert max(rel_l1(out["1"], ref)) <= MIXED_REL_L1, rel_l1(out["1"], ref)
    assert max(rel_l1(out["1"], out["0"])) <= FUSED_VS_SPLIT, rel_l1(out["1"], out["0"])


def _ot_shape(nx, ny):
    """Orszag-Tang's fields on an nx x ny periodic box (uneven shapes)."""
    x = inistate.domain_grid((nx, ny), (0.0, 0.0), (2 * np.pi, 2 * np.pi))
    X, Y = x
    g = 5.0 / 3.0
    rho = np.full_like(X, g * g)
    v = [-np.sin(Y), np.sin(X)]
    b = [-np.sin(Y), np.sin(2 * X)]
    w = inistate.conserve_mhd(rho, v, np.full_like(X, g), b, g)
    return inistate._snap(x, w, g, True, 2, "Orszag-Tang fields %dx%d" % (nx, ny))


LINE2_SHAPES = [
    ("mhd-61x33-periodic", lambda: _ot_shape(61, 33), "woodward", "periodic", 10, None),
    ("mhd-124x9-periodic", lambda: _ot_shape(124, 9), "minmod", "periodic", 10, None),
    ("mhd-6x70-reflect", lambda: _ot_shape(6, 70), "minmod", "symm", 8,
     lambda p: reflecting(p, 2)),
    ("mhd-129x65-reflect", lambda: _ot_shape(129, 65), "woodward", "symm", 6,
     lambda p: reflecting(p, 2)),
    ("hd-67x131-cont", lambda: _hd(67, 131), "woodward", "cont", 12, None),
    ("hd-128x4-cont", lambda: _hd(128, 4), "minmod", "cont", 12, None),
]


@pytest.mark.parametrize("name,mk,lim,bc,n,tweak", LINE2_SHAPES, ids=[c[0] for c in LINE2_SHAPES])
def test_line_sweep_shapes(gpu_lib, monkeypatch, name, mk, lim, bc, n, tweak):
    """The 2-D line sweep on shapes that cut its 60- and 64-column strips
    and 32-row chunks unevenly (one strip, partly filled strips, fewer rows
    than a chunk, several chunks), against the oracle and the split kernels."""
    test_fused_against_oracle_and_split(gpu_lib, monkeypatch, name, mk, lim, bc, n, tweak)

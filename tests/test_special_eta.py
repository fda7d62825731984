"""specialeta (src/vacphys.mhdres.t, eqpar(eta_) < 0): the resistivity is a
field from a registered hook, evaluated before each resistive source (from
that source's state) and before the first step's diffusion dt limit.  The
test hook (tests/hooks/eta.*) depends on x and on the current J_3; it is
written once for the oracle (host C) and once for the engine (CUDA)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from oracle.oracle import Oracle
from vac_gb300 import abi, inistate

HOOKS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hooks")
BUILD = os.path.join(HOOKS, "_build")


def _host_hook():
    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(BUILD, "libeta_host.so")
    src = os.path.join(HOOKS, "eta.c")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                        "-o", so, src], check=True)
    L = C.CDLL(so)
    return L, C.cast(L.eta_host, C.c_void_p).value


def _device_hook():
    from vac_gb300 import build
    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(BUILD, "libeta_dev.so")
    src = os.path.join(HOOKS, "eta.cu")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run([build.nvcc(), build.ARCH, "-O3", "-fmad=false",
                        "-Xcompiler", "-fPIC", "-shared", "-o", so, src], check=True)
    L = C.CDLL(so)
    return L, C.cast(L.eta_dev, C.c_void_p).value


def _eta_field(compact=0):
    def tweak(p):
        p.eqpar[1] = -1.0
        p.compactres = compact
    return tweak


def test_oracle_eta_field_sets_the_diffusion_dt():
    """First step: dt = min over idim of dtdiffpar/(1e-99 + max eta/dx^2),
    with eta from the hook formula and J_3 = dBy/dx - dBx/dy (central
    differences) of the initial state, when that limit is the smallest."""
    Lh, fn = _host_hook()
    s = inistate.orszag_tang(24)
    p = inistate.params_for(s)
    _eta_field()(p)
    p.dtdiffpar = 0.01  # make the diffusion limit bind
    o = Oracle(p, s.x, s.w, eta=(fn, None))
    o.step(1)
    w = s.w
    dx = s.x[0][1, 0] - s.x[0][0, 0]
    dy = s.x[1][0, 1] - s.x[1][0, 0]
    bx, by = w[4], w[5]
    j3 = (0.5 * (np.roll(by, -1, 0) - np.roll(by, 1, 0)) / dx
          - 0.5 * (np.roll(bx, -1, 1) - np.roll(bx, 1, 1)) / dy)
    eta = 0.005 * (1.0 + s.x[0] ** 2) + 0.001 * (j3 * j3)
    want = min(p.dtdiffpar / (1e-99 + (eta / dx ** 2).max()),
               p.dtdiffpar / (1e-99 + (eta / dy ** 2).max()))
    assert abs(o.dt - want) <= 1e-12 * want


ETA_CASES = [
    ("ot-eta-curl", lambda: inistate.orszag_tang(32), 8, _eta_field(0)),
    ("ot-eta-compact", lambda: inistate.orszag_tang(32), 8, _eta_field(1)),
    ("rm3-eta-curl", lambda: inistate.random_modes(12, seed=7), 4, _eta_field(0)),
    ("rm25-eta-compact", lambda: inistate.random_modes(16, seed=2, ndim=2, ndir=3), 6,
     _eta_field(1)),
    ("ot-eta-dtdiff", lambda: inistate.orszag_tang(24), 6,
     lambda p: (_eta_field(0)(p), setattr(p, "dtdiffpar", 0.01))),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,mk,n,tweak", ETA_CASES, ids=[c[0] for c in ETA_CASES])
def test_gpu_eta_field_bit_exact(gpu_lib, name, mk, n, tweak):
    from vac_gb300.engine import Engine
    Lh, hfn = _host_hook()
    Ld, dfn = _device_hook()
    s = mk()
    p = inistate.params_for(s, limiter="woodward")
    tweak(p)
    o = Oracle(p, s.x, s.w, eta=(hfn, None))
    e = Engine(p, s.x, s.w, eta=(dfn, None))
    o.step(n)
    e.step(n)
    assert e.it == o.it and e.t == o.t, (e.t, o.t)
    a, b = e.state(), o.state()
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), np.abs(a - b).max()


@pytest.mark.gpu
@pytest.mark.parametrize("compact", [0, 1])
def test_gpu_eta_field_mixed_within_tolerance(gpu_lib, compact):
    from vac_gb300.engine import Engine
    Lh, hfn = _host_hook()
    Ld, dfn = _device_hook()
    s = inistate.orszag_tang(64)
    p64 = inistate.params_for(s)
    pm = inistate.params_for(s, precision=abi.PREC_MIXED)
    _eta_field(compact)(p64)
    _eta_field(compact)(pm)
    o = Oracle(p64, s.x, s.w, eta=(hfn, None))
    e = Engine(pm, s.x, s.w, eta=(dfn, None))
    o.step(30)
    e.step(30)
    a, b = e.state(), o.state()
    for iw in range(a.shape[0]):
        rel = np.abs(a[iw] - b[iw]).sum() / np.abs(b[iw]).sum()
        assert rel <= 1e-5, (iw, rel)


@pytest.mark.gpu
def test_gpu_eta_field_needs_a_hook(gpu_lib):
    from vac_gb300.engine import Engine
    s = inistate.orszag_tang(16)
    p = inistate.params_for(s)
    _eta_field()(p)
    with pytest.raises(RuntimeError, match="specialeta"):
        Engine(p, s.x, s.w)

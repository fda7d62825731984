"""specialsource and getdt_special (src/vac.t:66,592; user routines
src/vacnul.specialsource.t:9-71) as registered hooks: the user's source
terms are added in every addsource2 call -- after the Hancock predictor
(wCT = the state, qtC = t) and after the corrector (wCT = the predictor
output, qtC = t+dt/2) -- before the physics sources, and the user's dt limit
enters every step's dt choice.  The test hook (tests/hooks/source.*) pushes
along x_1 with a force that depends on x_1 and on qtC, does the matching
work on e, damps m_2, and limits dt by max |m_1|/rho; it is written once for
the oracle (host C) and once for the engine (CUDA)."""
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
    so = os.path.join(BUILD, "libsource_host.so")
    src = os.path.join(HOOKS, "source.c")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                        "-o", so, src], check=True)
    L = C.CDLL(so)
    return L, C.cast(L.src_host, C.c_void_p).value, C.cast(L.dt_host, C.c_void_p).value


def _device_hook():
    from vac_gb300 import build
    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(BUILD, "libsource_dev.so")
    src = os.path.join(HOOKS, "source.cu")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run([build.nvcc(), build.ARCH, "-O3", "-fmad=false",
                        "-Xcompiler", "-fPIC", "-shared", "-o", so, src], check=True)
    L = C.CDLL(so)
    return L, C.cast(L.src_dev, C.c_void_p).value, C.cast(L.dt_dev, C.c_void_p).value


def _e_index(p):
    return 1 + p.ndir


def test_oracle_source_on_a_uniform_state():
    """A uniform periodic HD state: the fluxes conserve the total m_1, so
    after one step it grew by the source alone, dt*sum(rho*f(x_1, t+dt/2))
    to O(dt^2) (each split sweep adds qdt = dt/2 with qtC = t+dt/2 in its
    corrector; the density the corrector sees differs from the initial one
    by dt^2 terms).  Taking qtC = t instead would be off by dt/2 relative."""
    Lh, sfn, _ = _host_hook()
    s = inistate.riemann_2d(16, 3)
    w = s.w.copy()
    for iw in range(w.shape[0]):
        w[iw] = w[iw].mean()
    p = inistate.params_for(s, bc="periodic")
    o = Oracle(p, s.x, w, source=(sfn, None, _e_index(p)))
    o.step(1)
    dt = o.dt
    got = o.state()
    f = 0.02 * (0.5 + 0.1 * s.x[0]) * (1.0 + dt / 2)
    gain = got[1].sum() - w[1].sum()
    want = dt * (w[0] * f).sum()
    assert abs(gain - want) <= 1e-6 * abs(want), (gain, want, dt)
    # the same with qtC = t is told apart
    want_t = dt * (w[0] * 0.02 * (0.5 + 0.1 * s.x[0])).sum()
    assert abs(gain - want_t) > 100 * abs(gain - want)


def test_oracle_getdt_special_binds():
    """With the dt hook, the first step's dt is min(CFL dt, 0.05/(0.001 +
    max |m_1|/rho)); the Orszag-Tang state has max |v_1| = 1."""
    Lh, sfn, dfn = _host_hook()
    s = inistate.orszag_tang(24)
    p = inistate.params_for(s)
    o0 = Oracle(p, s.x, s.w)
    o0.step(1)
    o = Oracle(p, s.x, s.w, source=(None, dfn, _e_index(p)))
    o.step(1)
    lim = 0.05 / (0.001 + np.abs(s.w[1] / s.w[0]).max())
    assert lim < o0.dt
    assert o.dt == lim


SOURCE_CASES = [
    ("ot-tvdlf", lambda: inistate.orszag_tang(32), "minmod", "periodic", 8, None),
    ("rm3-woodward", lambda: inistate.random_modes(12, seed=7, p0=0.5), "woodward",
     "periodic", 5, None),
    ("sod-hd-cont", lambda: inistate.sod_1d(64), "woodward", "cont", 12, None),
    ("ot-tvdlf1", lambda: inistate.orszag_tang(24), "minmod", "periodic", 6,
     lambda p: setattr(p, "typefull", abi.TVDLF1)),
    ("ot-tvdmu-roe", lambda: inistate.orszag_tang(24), "woodward", "periodic", 6,
     lambda p: setattr(p, "typefull", abi.TVDMU)),
    ("ot-unsplit", lambda: inistate.orszag_tang(24), "minmod", "periodic", 6,
     lambda p: (setattr(p, "dimsplit", 0), setattr(p, "typelimited", abi.LIMITED_PREVIOUS))),
]


@pytest.mark.gpu
@pytest.mark.parametrize("dt_hook", [False, True])
@pytest.mark.parametrize("name,mk,lim,bc,n,tweak", SOURCE_CASES, ids=[c[0] for c in SOURCE_CASES])
def test_gpu_source_hook_bit_exact(gpu_lib, name, mk, lim, bc, n, tweak, dt_hook):
    from vac_gb300.engine import Engine
    Lh, hs, hd = _host_hook()
    Ld, ds, dd = _device_hook()
    s = mk()
    p = inistate.params_for(s, limiter=lim, bc=bc)
    if tweak:
        tweak(p)
    o = Oracle(p, s.x, s.w, source=(hs, hd if dt_hook else None, _e_index(p)))
    e = Engine(p, s.x, s.w, source=(ds, dd if dt_hook else None, None))
    o.step(n)
    e.step(n)
    assert e.it == o.it and e.t == o.t, (e.t, o.t)
    a, b = e.state(), o.state()
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), np.abs(a - b).max()


@pytest.mark.gpu
def test_gpu_source_hook_mixed_within_tolerance(gpu_lib):
    """The mixed path with the hooks (the split kernels; the hook adds its
    source to the FP32 state in double) against the FP64 oracle."""
    from vac_gb300.engine import Engine
    Lh, hs, hd = _host_hook()
    Ld, ds, dd = _device_hook()
    s = inistate.random_modes(32, seed=3, p0=0.5)
    p64 = inistate.params_for(s, limiter="woodward")
    pm = inistate.params_for(s, limiter="woodward", precision=abi.PREC_MIXED)
    o = Oracle(p64, s.x, s.w, source=(hs, hd, _e_index(p64)))
    e = Engine(pm, s.x, s.w, source=(ds, dd, None))
    o.step(10)
    e.step(10)
    a, b = e.state(), o.state()
    assert e.it == o.it and abs(e.t - o.t) <= 1e-6 * o.t
    for iw in range(a.shape[0]):
        rel = np.abs(a[iw] - b[iw]).sum() / np.abs(b[iw]).sum()
        assert rel <= 1e-5, (iw, rel)


@pytest.mark.gpu
def test_gpu_source_hook_in_graphs_and_replaced(gpu_lib):
    """Steps replayed from CUDA graphs call the hook's captured kernels: a
    run split into calls of 1, 3 and 4 steps equals one call of 8; and
    removing the hook restores the source-free run."""
    from vac_gb300.engine import Engine, lib, _ck
    Ld, ds, dd = _device_hook()
    s = inistate.orszag_tang(32)
    p = inistate.params_for(s)
    e1 = Engine(p, s.x, s.w, source=(ds, dd, None))
    e1.step(8)
    e2 = Engine(p, s.x, s.w, source=(ds, dd, None))
    for k in (1, 3, 4):
        e2.step(k)
    assert np.array_equal(e1.state().view(np.uint64), e2.state().view(np.uint64))
    e3 = Engine(p, s.x, s.w, source=(ds, dd, None))
    _ck(lib().vacgpu_register_source_fn(e3.h, None, None, None), "vacgpu_register_source_fn")
    e3.step(8)
    e4 = Engine(p, s.x, s.w)
    e4.step(8)
    assert np.array_equal(e3.state().view(np.uint64), e4.state().view(np.uint64))

"""specialbound (src/vacgrid.t:355-371): typeB='special' faces filled by a
registered hook, region by region after the region's other variables, at
getboundary's time qt (t, t+dt/2, t+dt).  The test hook (tests/hooks/) is a
time-dependent inflow mixed with the edge value, written once for the
oracle (host C) and once for the engine (CUDA)."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from oracle.oracle import Oracle, lib as oracle_lib
from vac_gb300 import abi, inistate

HOOKS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hooks")
BUILD = os.path.join(HOOKS, "_build")


def _host_hook():
    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(BUILD, "libinflow_host.so")
    src = os.path.join(HOOKS, "inflow.c")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                        "-o", so, src], check=True)
    L = C.CDLL(so)
    return L, C.cast(L.inflow_bound_host, C.c_void_p).value


def _device_hook():
    from vac_gb300 import build
    os.makedirs(BUILD, exist_ok=True)
    so = os.path.join(BUILD, "libinflow_dev.so")
    src = os.path.join(HOOKS, "inflow.cu")
    if not os.path.exists(so) or os.path.getmtime(so) < os.path.getmtime(src):
        subprocess.run([build.nvcc(), build.ARCH, "-O3", "-fmad=false",
                        "-Xcompiler", "-fPIC", "-shared", "-o", so, src], check=True)
    L = C.CDLL(so)
    return L, C.cast(L.inflow_bound, C.c_void_p).value


def _special(faces, ivars=None):
    """typeB='special' on the given regions (0-based iB) for the variables
    ivars (all if None), 'cont' elsewhere on those faces' dimension."""
    def tweak(p):
        for iB in faces:
            for iw in range(p.nw):
                if ivars is None or iw in ivars:
                    p.typeB[iB][iw] = abi.BC_SPECIAL
    return tweak


def test_oracle_special_faces_follow_the_hook():
    """The oracle's ghost cells on a special face hold the hook's formula
    at qt = t + dt after a step (the corrector's fill is the last)."""
    Lh, fn = _host_hook()
    s = inistate.riemann_2d(16, 3)
    p = inistate.params_for(s, bc="cont")
    _special([0])(p)
    o = Oracle(p, s.x, s.w, bound=(fn, None))
    o.step(3)
    n = oracle_lib().vo_ncells_full(o.h)
    full = np.empty(n * p.nw)
    oracle_lib().vo_get_state_full(o.h, full.ctypes.data_as(C.POINTER(C.c_double)))
    nG = (p.nx[0] + 4, p.nx[1] + 4)
    w = full.reshape(p.nw, nG[1], nG[0])  # [iw][gy][gx]
    xfull = np.empty(n)
    oracle_lib().vo_get_x(o.h, 0, xfull.ctypes.data_as(C.POINTER(C.c_double)))
    x = xfull.reshape(nG[1], nG[0])
    qt = o.t  # after the step: t of the last fill = t_old + dt = o.t
    for iw in range(p.nw):
        for gx in (0, 1):
            want = 0.5 * (w[iw][:, 2] + (1.0 + 0.1 * iw) * (1.0 + 0.1 * qt)) + 0.01 * x[:, gx]
            np.testing.assert_allclose(w[iw][:, gx], want, rtol=1e-14, atol=1e-14)
    assert np.isfinite(o.state()).all()


SPECIAL_CASES = [
    ("hd-special-xlo", lambda: inistate.riemann_2d(32, 3), "cont", 10, _special([0])),
    ("ot-special-rho-e-xhi", lambda: inistate.orszag_tang(24), "cont", 8,
     _special([1], ivars=[0, 3])),
    ("rm3-special-zlo", lambda: inistate.random_modes(12, seed=2), "periodic", 3,
     lambda p: (_special([4, 5])(p))),
    ("hd-special-tvdmu", lambda: inistate.riemann_2d(32, 5), "cont", 8,
     lambda p: (_special([2])(p), setattr(p, "typefull", abi.TVDMU))),
]


@pytest.mark.gpu
@pytest.mark.parametrize("name,mk,bc,n,tweak", SPECIAL_CASES, ids=[c[0] for c in SPECIAL_CASES])
def test_gpu_special_bound_bit_exact(gpu_lib, name, mk, bc, n, tweak):
    from vac_gb300.engine import Engine
    Lh, hfn = _host_hook()
    Ld, dfn = _device_hook()
    s = mk()
    p = inistate.params_for(s, bc=bc)
    tweak(p)
    o = Oracle(p, s.x, s.w, bound=(hfn, None))
    e = Engine(p, s.x, s.w, bound=(dfn, None))
    o.step(n)
    e.step(n)
    assert e.it == o.it and e.t == o.t
    a, b = e.state(), o.state()
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), np.abs(a - b).max()


@pytest.mark.gpu
def test_gpu_special_bound_mixed_within_tolerance(gpu_lib):
    from vac_gb300.engine import Engine
    Lh, hfn = _host_hook()
    Ld, dfn = _device_hook()
    s = inistate.riemann_2d(64, 3)
    p64 = inistate.params_for(s, bc="cont")
    pm = inistate.params_for(s, bc="cont", precision=abi.PREC_MIXED)
    _special([0, 3])(p64)
    _special([0, 3])(pm)
    o = Oracle(p64, s.x, s.w, bound=(hfn, None))
    e = Engine(pm, s.x, s.w, bound=(dfn, None))
    o.step(30)
    e.step(30)
    a, b = e.state(), o.state()
    for iw in range(a.shape[0]):
        rel = np.abs(a[iw] - b[iw]).sum() / np.abs(b[iw]).sum()
        assert rel <= 1e-5, (iw, rel)


@pytest.mark.gpu
def test_gpu_special_bound_needs_a_hook(gpu_lib):
    from vac_gb300.engine import Engine
    s = inistate.riemann_2d(16, 3)
    p = inistate.params_for(s, bc="cont")
    _special([0])(p)
    with pytest.raises(RuntimeError, match="Special boundary is not defined"):
        Engine(p, s.x, s.w)

"""vacgpu_sweep_noalloc: the allocation-free sweep entry point.

Callers that cannot call cudaMalloc -- hosts recording the engine into their
own CUDA graph or stream capture, hosts that own all device memory through
their own pool, latency-bound loops where an allocation would synchronise the
device -- advance a grid with vacgpu_sweep_noalloc on device arrays they own;
the library keeps the predictor's intermediate state in a fixed static device
array instead of allocating.  These tests drive it through the C ABI on
device buffers allocated by the test (torch) and check two full time steps
(2 * ndim sweep calls in a row, all sharing the static scratch) against
vacgpu_step, bit for bit, the FP64 tolerance of every other FP64 test: 1-D,
2-D and 3-D grids, MHD and HD, tvdlf and tvdlf1, limiter bases 'original'
and 'predictor', periodic, cont, symm and asymm faces.  This file is
collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from oracle.oracle import Oracle
from vac_gb300 import abi, inistate
from vac_gb300.engine import Engine, lib, last_error

pytestmark = pytest.mark.gpu


def _hd_walls():
    """2-D HD Riemann problem in a box: symm faces, the normal momentum
    asymm (reflecting walls)."""
    s = inistate.riemann_2d(40, 3)
    p = inistate.params_for(s, limiter="woodward", bc="symm")
    for ib in range(4):
        p.typeB[ib][1 + ib // 2] = abi.BC_ASYMM
    return s, p


def _case(name):
    if name == "ot2d":
        s = inistate.orszag_tang(64)
        return s, inistate.params_for(s)
    if name == "rm3d":
        s = inistate.random_modes(16, seed=2, p0=0.5)
        return s, inistate.params_for(s, limiter="woodward")
    if name == "sod1d-cont":
        s = inistate.sod_1d(64)
        return s, inistate.params_for(s, limiter="woodward", bc="cont")
    if name == "ot2d-tvdlf1":
        s = inistate.orszag_tang(48)
        p = inistate.params_for(s)
        p.typefull = abi.TVDLF1
        return s, p
    if name == "ot2d-predictor":
        s = inistate.orszag_tang(48)
        p = inistate.params_for(s, limiter="vanleer")
        p.typelimited = abi.LIMITED_PREDICTOR
        return s, p
    if name == "hd2d-walls":
        return _hd_walls()
    raise KeyError(name)


CASES = ["ot2d", "rm3d", "sod1d-cont", "ot2d-tvdlf1", "ot2d-predictor", "hd2d-walls"]


def _mesh_of(full, nw, nx):
    nG = tuple(n + 4 for n in nx)
    n = int(np.prod(nG))
    sl = tuple(slice(2, -2) for _ in nx)
    return np.stack([full[i * n:(i + 1) * n].reshape(nG, order="F")[sl]
                     for i in range(nw)])


def _dx_lines(o, nx):
    """dx of gridsetup1 along each dimension over the ghost-extended range."""
    nG = tuple(n + 4 for n in nx)
    out = []
    for d in range(len(nx)):
        full = o.dx_full(d).reshape(nG, order="F")
        idx = tuple(slice(None) if k == d else 2 for k in range(len(nx)))
        out.append(np.ascontiguousarray(full[idx]))
    return out


@pytest.mark.parametrize("name", CASES)
def test_noalloc_sweeps_match_vacgpu_step(gpu_lib, name):
    import torch
    s, p = _case(name)
    p.smallp = 1.0e-6  # given explicitly: both paths then clip alike
    nx = tuple(s.w.shape[1:])
    ndim = len(nx)
    eng = Engine(p, s.x, s.w)
    eng.step(1)
    dt1, w_step1 = eng.dt, eng.state()
    eng.step(1)
    dt2, w_step2 = eng.dt, eng.state()
    eng.close()

    # the initial state with its ghost cells filled by getboundary, and dx
    o = Oracle(p, s.x, s.w)
    full = np.empty(lib_full_cells(o), dtype=np.float64)
    from oracle.oracle import lib as olib, _dp
    olib().vo_get_state_full(o.h, _dp(full))
    dev = torch.device("cuda")
    dx = [torch.from_numpy(a).to(dev) for a in _dx_lines(o, nx)]
    dxp = [C.c_void_p(dx[d].data_ptr()) if d < ndim else None for d in range(3)]
    wa = torch.from_numpy(full).to(dev)
    wb = torch.empty_like(wa)
    cm = torch.zeros(3, dtype=torch.float64, device=dev)
    L = lib()

    def sweep(src, dst, dt, idim):
        rc = L.vacgpu_sweep_noalloc(C.byref(p), C.c_void_p(src.data_ptr()),
                                    C.c_void_p(dst.data_ptr()), dxp[0], dxp[1], dxp[2],
                                    dt, idim, C.c_void_p(cm[idim:].data_ptr()), None)
        assert rc == 0, last_error()

    def step(dt, order):
        src, dst = wa, wb
        for d in order:
            sweep(src, dst, dt, d)
            src, dst = dst, src
        torch.cuda.synchronize()
        return src

    # step 1 (it=0, even): sweeps 0..ndim-1; step 2 (odd, xyyx): reversed
    cur = step(dt1, range(ndim))
    got1 = _mesh_of(cur.cpu().numpy(), p.nw, nx)
    assert np.array_equal(got1.view(np.uint64), w_step1.view(np.uint64))
    # the corrector CFL maxima give the next dt exactly as getdt_courant does
    c = cm.cpu().numpy()
    assert min(p.courantpar / c[d] for d in range(ndim)) == dt2
    if cur is not wa:
        wa.copy_(cur)
    cur = step(dt2, range(ndim - 1, -1, -1))
    got2 = _mesh_of(cur.cpu().numpy(), p.nw, nx)
    assert np.array_equal(got2.view(np.uint64), w_step2.view(np.uint64))


def lib_full_cells(o):
    from oracle.oracle import lib as olib
    return int(olib().vo_ncells_full(o.h)) * o.nw


@pytest.mark.parametrize("nx", [(1024, 1024), (2**31 - 1, 2), (70000, 70000, 70000)])
def test_noalloc_rejects_oversized_grid(gpu_lib, nx):
    s = inistate.orszag_tang(16) if len(nx) == 2 else inistate.random_modes(4, seed=0)
    p = inistate.params_for(s)
    p.smallp = 1.0e-6
    for d, n in enumerate(nx):
        p.nx[d] = n  # with ghosts far above the 262144-cell limit
    rc = lib().vacgpu_sweep_noalloc(C.byref(p), C.c_void_p(16), C.c_void_p(16),
                                    C.c_void_p(16), C.c_void_p(16), C.c_void_p(16), 0.1, 0,
                                    None, None)
    assert rc != 0 and "VACGPU_NOALLOC_MAX_GCELLS" in last_error()

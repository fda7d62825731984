"""vacgpu_sweep_noalloc: the allocation-free sweep entry point.

Callers that cannot call cudaMalloc -- hosts recording the engine into their
own CUDA graph or stream capture, hosts that own all device memory through
their own pool, latency-bound loops where an allocation would synchronise the
device -- advance a grid with vacgpu_sweep_noalloc on device arrays they own;
the library keeps the predictor's intermediate state in a fixed static device
array instead of allocating.  This test drives it through the C ABI on device
buffers allocated by the test (torch) and checks two full time steps (four
sweep calls in a row) against vacgpu_step, bit for bit, the FP64 tolerance of
every other FP64 test.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from oracle.oracle import Oracle
from vac_gb300 import abi, inistate
from vac_gb300.engine import Engine, lib, last_error

pytestmark = pytest.mark.gpu


def _full_grid_periodic(wm):
    """Mesh state (nw, n1, n2) -> VAC full-grid layout w(ixG^T,nw) with
    periodic ghost cells, flattened column-major per variable."""
    return np.concatenate([np.pad(wm[iw], 2, mode="wrap").ravel(order="F")
                           for iw in range(wm.shape[0])])


def _mesh_of(full, nw, nx):
    nG = tuple(n + 4 for n in nx)
    n = int(np.prod(nG))
    return np.stack([full[i * n:(i + 1) * n].reshape(nG, order="F")[2:-2, 2:-2]
                     for i in range(nw)])


def test_noalloc_sweeps_match_vacgpu_step(gpu_lib):
    import torch
    n = 64
    s = inistate.orszag_tang(n)
    p = inistate.params_for(s)
    p.smallp = 1.0e-6  # given explicitly: both paths then clip alike
    eng = Engine(p, s.x, s.w)
    eng.step(1)
    dt1, w_step1 = eng.dt, eng.state()
    eng.step(1)
    dt2, w_step2 = eng.dt, eng.state()

    o = Oracle(p, s.x, s.w)  # dx of gridsetup1 over the ghost-extended range
    nG = (n + 4, n + 4)
    dxa = [o.dx_full(0).reshape(nG[1], nG[0])[2, :].copy(),
           o.dx_full(1).reshape(nG[1], nG[0])[:, 2].copy()]
    dev = torch.device("cuda")
    dx = [torch.from_numpy(a).to(dev) for a in dxa]
    wa = torch.from_numpy(_full_grid_periodic(s.w)).to(dev)
    wb = torch.empty_like(wa)
    cm = torch.zeros(2, dtype=torch.float64, device=dev)
    L = lib()

    def sweep(src, dst, dt, idim):
        rc = L.vacgpu_sweep_noalloc(C.byref(p), C.c_void_p(src.data_ptr()),
                                    C.c_void_p(dst.data_ptr()),
                                    C.c_void_p(dx[0].data_ptr()),
                                    C.c_void_p(dx[1].data_ptr()), None, dt,
                                    idim, C.c_void_p(cm[idim:].data_ptr()), None)
        assert rc == 0, last_error()

    # step 1 (it=0, even): sweeps x then y
    sweep(wa, wb, dt1, 0)
    sweep(wb, wa, dt1, 1)
    torch.cuda.synchronize()
    got1 = _mesh_of(wa.cpu().numpy(), p.nw, (n, n))
    assert np.array_equal(got1.view(np.uint64), w_step1.view(np.uint64))
    # the corrector CFL maxima give the next dt exactly as getdt_courant does
    c = cm.cpu().numpy()
    assert min(p.courantpar / c[0], p.courantpar / c[1]) == dt2
    # step 2 (it=1, odd, xyyx): sweeps y then x, reusing the same scratch
    sweep(wa, wb, dt2, 1)
    sweep(wb, wa, dt2, 0)
    torch.cuda.synchronize()
    got2 = _mesh_of(wa.cpu().numpy(), p.nw, (n, n))
    assert np.array_equal(got2.view(np.uint64), w_step2.view(np.uint64))


def test_noalloc_rejects_oversized_grid(gpu_lib):
    s = inistate.orszag_tang(16)
    p = inistate.params_for(s)
    p.smallp = 1.0e-6
    p.nx[0] = p.nx[1] = 1024  # 1028^2 cells with ghosts > 262144
    rc = lib().vacgpu_sweep_noalloc(C.byref(p), C.c_void_p(16), C.c_void_p(16),
                                    C.c_void_p(16), C.c_void_p(16), None, 0.1, 0,
                                    None, None)
    assert rc != 0 and "VACGPU_NOALLOC_MAX_GCELLS" in last_error()

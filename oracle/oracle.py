"""ctypes binding of the FP64 CPU oracle (``oracle/vac_oracle.c``).

Test infrastructure only: the parity tests, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` use it as the checker.  The product
never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from vac_gb300.abi import VacParams

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libvacoracle.so")

_lib = None


def build():
    """Compile the oracle (make, gcc -O2 -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        dp = C.POINTER(C.c_double)
        L.vo_create.restype = vp
        L.vo_create.argtypes = [C.POINTER(VacParams)]
        L.vo_destroy.argtypes = [vp]
        L.vo_set_grid.argtypes = [vp, dp]
        L.vo_set_state.argtypes = [vp, dp, C.c_int, C.c_double]
        L.vo_get_state.argtypes = [vp, dp]
        L.vo_get_state_full.argtypes = [vp, dp]
        L.vo_step.restype = C.c_int
        L.vo_step.argtypes = [vp, C.c_int, C.c_double, C.POINTER(C.c_int)]
        L.vo_t.restype = C.c_double
        L.vo_t.argtypes = [vp]
        L.vo_it.restype = C.c_int
        L.vo_it.argtypes = [vp]
        L.vo_dt.restype = C.c_double
        L.vo_dt.argtypes = [vp]
        L.vo_smallp.restype = C.c_double
        L.vo_smallp.argtypes = [vp]
        L.vo_smallrho.restype = C.c_double
        L.vo_smallrho.argtypes = [vp]
        L.vo_volume.restype = C.c_double
        L.vo_volume.argtypes = [vp]
        L.vo_nerror.argtypes = [vp, C.POINTER(C.c_int)]
        L.vo_ncells_full.restype = C.c_long
        L.vo_ncells_full.argtypes = [vp]
        L.vo_get_dx.argtypes = [vp, C.c_int, dp]
        L.vo_get_x.argtypes = [vp, C.c_int, dp]
        L.vo_sums.argtypes = [vp, dp]
        L.vo_register_source.argtypes = [vp, C.c_int, dp, C.c_int]
        L.vo_register_bound.argtypes = [vp, vp, vp]
        L.vo_register_eta.argtypes = [vp, vp, vp]
        L.vo_register_source_fn.argtypes = [vp, vp, vp, vp]
        L.vo_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """One VAC run on the CPU.  ``x``: mesh coordinates (ndim, *nx) in C
    order of the numpy array whose Fortran layout is VAC's x(ixM^S,1:ndim);
    ``w``: (nw, *nx) likewise.  Arrays are passed as VAC column-major
    blocks: x[d] is stored with ix1 fastest."""

    def __init__(self, params, x, w, it=0, t=0.0, bound=None, eta=None, source=None):
        """bound: (function pointer, user pointer) of a specialbound hook
        with vo_register_bound's signature, installed before the first
        ghost fill; eta: likewise a specialeta hook (vo_register_eta);
        source: (specialsource, getdt_special, user) of
        vo_register_source_fn (either function pointer may be None)."""
        L = lib()
        self.p = params
        self.h = L.vo_create(C.byref(params))
        if not self.h:
            raise RuntimeError(L.vo_last_error().decode())
        if bound:
            L.vo_register_bound(self.h, bound[0], bound[1])
        if eta:
            L.vo_register_eta(self.h, eta[0], eta[1])
        if source:
            L.vo_register_source_fn(self.h, source[0], source[1], source[2])
        self.nx = tuple(params.nx[d] for d in range(params.ndim))
        self.nw = params.nw
        xf = np.ascontiguousarray(pack_mesh(x), dtype=np.float64)
        L.vo_set_grid(self.h, _dp(xf))
        wf = np.ascontiguousarray(pack_mesh(w), dtype=np.float64)
        L.vo_set_state(self.h, _dp(wf), it, t)

    def __del__(self):
        if getattr(self, "h", None):
            lib().vo_destroy(self.h)
            self.h = None

    def register_source(self, sid, par):
        a = np.ascontiguousarray(par, dtype=np.float64)
        lib().vo_register_source(self.h, sid, _dp(a), len(a))

    def step(self, maxsteps, tstop=1e300):
        fin = C.c_int(0)
        n = lib().vo_step(self.h, maxsteps, tstop, C.byref(fin))
        return n, bool(fin.value)

    def state(self):
        out = np.empty(self.nw * int(np.prod(self.nx)), dtype=np.float64)
        lib().vo_get_state(self.h, _dp(out))
        return unpack_mesh(out, self.nw, self.nx)

    def sums(self):
        out = np.empty(self.nw, dtype=np.float64)
        lib().vo_sums(self.h, _dp(out))
        return out

    def dx_full(self, idim):
        n = lib().vo_ncells_full(self.h)
        out = np.empty(n, dtype=np.float64)
        lib().vo_get_dx(self.h, idim, _dp(out))
        return out

    def nerror(self):
        a = (C.c_int * 4)()
        lib().vo_nerror(self.h, a)
        return list(a)

    @property
    def t(self):
        return lib().vo_t(self.h)

    @property
    def it(self):
        return lib().vo_it(self.h)

    @property
    def dt(self):
        return lib().vo_dt(self.h)

    @property
    def smallp(self):
        return lib().vo_smallp(self.h)

    @property
    def smallrho(self):
        return lib().vo_smallrho(self.h)

    @property
    def volume(self):
        return lib().vo_volume(self.h)


def pack_mesh(a):
    """(nv, n1, n2, n3) numpy array -> VAC column-major blocks, one per
    variable, ix1 fastest."""
    a = np.asarray(a)
    return np.concatenate([np.asarray(a[i]).ravel(order="F")
                           for i in range(a.shape[0])])


def unpack_mesh(flat, nv, nx):
    n = int(np.prod(nx))
    return np.stack([flat[i * n:(i + 1) * n].reshape(nx, order="F")
                     for i in range(nv)])

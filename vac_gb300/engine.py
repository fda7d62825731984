"""Python binding of the C ABI (``include/vacgpu.h``) through ctypes.

This is how the tests, the benchmark and Python hosts drive the engine; it
mirrors the sequence VAC's driver performs (readfileini -> gridsetup1 ->
time loop -> savefile).  The shared library must have been built
(``vac_gb300.build.build()``); there is no fallback path.
"""
import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "lib", "libvacgpu.so")

SYMBOLS = [
    "vacgpu_default_params", "vacgpu_create", "vacgpu_set_grid",
    "vacgpu_upload", "vacgpu_download", "vacgpu_step", "vacgpu_sums",
    "vacgpu_error_counts", "vacgpu_register_source", "vacgpu_destroy",
    "vacgpu_last_error", "vacgpu_version", "vacgpu_set_stream",
    "vacgpu_timing", "vacgpu_kernel_stats", "vacgpu_sweep_noalloc",
    "vacgpu_batch_create", "vacgpu_batch_set_grid", "vacgpu_batch_upload",
    "vacgpu_batch_download", "vacgpu_batch_step", "vacgpu_batch_status",
    "vacgpu_batch_tune", "vacgpu_batch_destroy", "vacgpu_server_create",
    "vacgpu_server_submit", "vacgpu_server_result", "vacgpu_server_timing",
    "vacgpu_server_stats", "vacgpu_server_destroy", "vacgpu_measure_fp64_peak",
    "vacgpu_register_source_fn", "vacgpu_snapshot_begin", "vacgpu_snapshot_wait",
    "vacgpu_snapshot_data", "vacgpu_test_bounded_waits",
]

K_PREDICT, K_CORRECT, K_SWEEP, K_GHOST, K_DT, K_CONTROL, K_NCLASS = range(7)
K_NAMES = ["predict", "correct", "sweep", "ghost", "dt", "control"]

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(
                "libvacgpu.so is not built (%s); run "
                "python -c 'import __graft_entry__ as g; g.build()'" % LIB)
        L = C.CDLL(LIB)
        vp = C.c_void_p
        dp = C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        L.vacgpu_default_params.argtypes = [C.POINTER(abi.VacParams), C.c_int,
                                            C.c_int, C.c_int, ip]
        L.vacgpu_create.argtypes = [C.POINTER(abi.VacParams), C.POINTER(vp)]
        L.vacgpu_set_grid.argtypes = [vp, dp]
        L.vacgpu_upload.argtypes = [vp, dp, C.c_int, C.c_double]
        L.vacgpu_download.argtypes = [vp, dp]
        L.vacgpu_step.argtypes = [vp, C.c_int, C.c_double, dp, ip, dp, ip]
        L.vacgpu_sums.argtypes = [vp, dp]
        L.vacgpu_error_counts.argtypes = [vp, ip]
        L.vacgpu_register_source.argtypes = [vp, C.c_int, dp, C.c_int]
        L.vacgpu_register_bound.argtypes = [vp, vp, vp]
        L.vacgpu_register_eta.argtypes = [vp, vp, vp]
        L.vacgpu_register_source_fn.argtypes = [vp, vp, vp, vp]
        L.vacgpu_snapshot_begin.argtypes = [vp, C.c_int]
        L.vacgpu_snapshot_wait.argtypes = [vp, C.c_int, vp]
        L.vacgpu_snapshot_data.argtypes = [vp, C.c_int]
        L.vacgpu_snapshot_data.restype = C.POINTER(C.c_double)
        L.vacgpu_destroy.argtypes = [vp]
        L.vacgpu_destroy.restype = None
        L.vacgpu_last_error.argtypes = [C.c_char_p, C.c_int]
        L.vacgpu_version.restype = C.c_char_p
        L.vacgpu_set_stream.argtypes = [vp, vp]
        L.vacgpu_timing.argtypes = [vp, C.c_int]
        L.vacgpu_kernel_stats.argtypes = [vp, C.c_int, C.POINTER(C.c_longlong), dp]
        L.vacgpu_sweep_noalloc.argtypes = [C.POINTER(abi.VacParams), vp, vp, vp,
                                           vp, vp, C.c_double, C.c_int, vp, vp]
        L.vacgpu_batch_create.argtypes = [C.POINTER(abi.VacParams), C.c_int, C.POINTER(vp)]
        L.vacgpu_batch_set_grid.argtypes = [vp, C.c_int, dp]
        L.vacgpu_batch_upload.argtypes = [vp, C.c_int, dp, C.c_int, C.c_double]
        L.vacgpu_batch_download.argtypes = [vp, C.c_int, dp]
        L.vacgpu_batch_step.argtypes = [vp, C.c_int, C.c_double]
        L.vacgpu_batch_status.argtypes = [vp, C.c_int, dp, ip, dp, ip]
        L.vacgpu_batch_tune.argtypes = [vp, ip, ip, ip, ip, dp]
        L.vacgpu_batch_destroy.argtypes = [vp]
        L.vacgpu_batch_destroy.restype = None
        L.vacgpu_server_create.argtypes = [C.c_double, C.c_int, C.c_int, C.POINTER(vp)]
        L.vacgpu_server_submit.argtypes = [vp, C.POINTER(abi.VacParams), dp, dp, C.c_int,
                                           C.POINTER(C.c_longlong)]
        L.vacgpu_server_result.argtypes = [vp, C.c_longlong, C.c_double, dp, dp, ip, dp]
        L.vacgpu_server_timing.argtypes = [vp, C.c_longlong, dp, dp]
        L.vacgpu_server_stats.argtypes = [vp, ip, ip, ip, ip, dp, dp]
        L.vacgpu_measure_fp64_peak.argtypes = [dp, vp]
        L.vacgpu_server_destroy.argtypes = [vp]
        L.vacgpu_server_destroy.restype = None
        _lib = L
    return _lib


def last_error():
    buf = C.create_string_buffer(1024)
    lib().vacgpu_last_error(buf, 1024)
    return buf.value.decode()


def _ck(rc, what):
    if rc != 0:
        raise RuntimeError("%s: %s" % (what, last_error()))


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def pack_mesh(a):
    a = np.asarray(a)
    return np.concatenate([np.asarray(a[i]).ravel(order="F")
                           for i in range(a.shape[0])])


class Engine:
    """One grid advanced on the GPU.  ``x``: (ndim, n1, ...) mesh
    coordinates, ``w``: (nw, n1, ...) conservative state, both indexed like
    VAC's x(ix^D,idim) and w(ix^D,iw)."""

    def __init__(self, params, x, w, it=0, t=0.0, bound=None, eta=None, source=None):
        """bound: (function pointer, user pointer) of a vacgpu_bound_fn
        specialbound hook, installed before the first ghost fill; eta:
        likewise a vacgpu_eta_fn specialeta hook; source: (specialsource
        function pointer or None, getdt_special function pointer or None,
        user pointer) of vacgpu_register_source_fn."""
        L = lib()
        self.p = params
        h = C.c_void_p()
        _ck(L.vacgpu_create(C.byref(params), C.byref(h)), "vacgpu_create")
        self.h = h
        if bound:
            _ck(L.vacgpu_register_bound(self.h, C.c_void_p(bound[0]),
                                        C.c_void_p(bound[1])),
                "vacgpu_register_bound")
        if eta:
            _ck(L.vacgpu_register_eta(self.h, C.c_void_p(eta[0]), C.c_void_p(eta[1])),
                "vacgpu_register_eta")
        if source:
            _ck(L.vacgpu_register_source_fn(self.h, C.c_void_p(source[0]),
                                            C.c_void_p(source[1]), C.c_void_p(source[2])),
                "vacgpu_register_source_fn")
        self.nw = params.nw
        self.nx = tuple(params.nx[d] for d in range(params.ndim))
        xf = np.ascontiguousarray(pack_mesh(x), dtype=np.float64)
        _ck(L.vacgpu_set_grid(self.h, _dp(xf)), "vacgpu_set_grid")
        self.upload(w, it, t)

    def upload(self, w, it=0, t=0.0):
        wf = np.ascontiguousarray(pack_mesh(w), dtype=np.float64)
        _ck(lib().vacgpu_upload(self.h, _dp(wf), it, t), "vacgpu_upload")

    def upload_flat(self, wflat, it=0, t=0.0):
        """Upload a VAC-ordered flat FP64 host buffer (e.g. pinned memory)."""
        _ck(lib().vacgpu_upload(self.h, C.cast(wflat, C.POINTER(C.c_double)),
                                it, t), "vacgpu_upload")

    def download_flat(self, out_ptr):
        _ck(lib().vacgpu_download(self.h, C.cast(out_ptr, C.POINTER(C.c_double))),
            "vacgpu_download")

    def register_source(self, sid, par):
        a = np.ascontiguousarray(par, dtype=np.float64)
        _ck(lib().vacgpu_register_source(self.h, sid, _dp(a), len(a)),
            "vacgpu_register_source")

    def step(self, maxsteps, tstop=1e300):
        t = C.c_double()
        it = C.c_int()
        dt = C.c_double()
        fin = C.c_int()
        _ck(lib().vacgpu_step(self.h, maxsteps, tstop, C.byref(t), C.byref(it),
                              C.byref(dt), C.byref(fin)), "vacgpu_step")
        self.t, self.it, self.dt = t.value, it.value, dt.value
        return bool(fin.value)

    def state(self):
        n = int(np.prod(self.nx))
        out = np.empty(self.nw * n, dtype=np.float64)
        _ck(lib().vacgpu_download(self.h, _dp(out)), "vacgpu_download")
        return np.stack([out[i * n:(i + 1) * n].reshape(self.nx, order="F")
                         for i in range(self.nw)])

    def snapshot_begin(self, slot=0):
        """Start an asynchronous copy of the current state into `slot`."""
        _ck(lib().vacgpu_snapshot_begin(self.h, slot), "vacgpu_snapshot_begin")

    def snapshot_wait(self, slot=0, out_ptr=None):
        """Wait for the snapshot in `slot`; return it as (nw, *nx), or write
        it to the VAC-ordered flat FP64 host buffer at out_ptr."""
        if out_ptr is not None:
            _ck(lib().vacgpu_snapshot_wait(self.h, slot, C.c_void_p(out_ptr)),
                "vacgpu_snapshot_wait")
            return None
        n = int(np.prod(self.nx))
        out = np.empty(self.nw * n, dtype=np.float64)
        _ck(lib().vacgpu_snapshot_wait(self.h, slot, C.c_void_p(out.ctypes.data)),
            "vacgpu_snapshot_wait")
        return np.stack([out[i * n:(i + 1) * n].reshape(self.nx, order="F")
                         for i in range(self.nw)])

    def snapshot_view(self, slot=0):
        """Wait for the snapshot in `slot` and return the library's
        page-locked copy in place: a list of nw arrays of shape nx (views, no
        host copy; valid until the next snapshot_begin on the slot)."""
        _ck(lib().vacgpu_snapshot_wait(self.h, slot, None), "vacgpu_snapshot_wait")
        ptr = lib().vacgpu_snapshot_data(self.h, slot)
        if not ptr:
            raise RuntimeError("vacgpu_snapshot_data: %s" % last_error())
        n = int(np.prod(self.nx))
        flat = np.ctypeslib.as_array(ptr, shape=(self.nw * n,))
        return [flat[i * n:(i + 1) * n].reshape(self.nx, order="F") for i in range(self.nw)]

    def sums(self):
        out = np.empty(self.nw, dtype=np.float64)
        _ck(lib().vacgpu_sums(self.h, _dp(out)), "vacgpu_sums")
        return out

    def nerror(self):
        a = (C.c_int * 4)()
        _ck(lib().vacgpu_error_counts(self.h, a), "vacgpu_error_counts")
        return list(a)

    def set_stream(self, stream_ptr):
        """Run on a caller-owned cudaStream_t (int handle, e.g.
        torch.cuda.Stream().cuda_stream); None returns to the own stream."""
        _ck(lib().vacgpu_set_stream(self.h, C.c_void_p(stream_ptr or 0)),
            "vacgpu_set_stream")

    def timing(self, enable):
        _ck(lib().vacgpu_timing(self.h, 1 if enable else 0), "vacgpu_timing")

    def kernel_stats(self):
        """{class name: (launches, device ms)}"""
        out = {}
        for k, name in enumerate(K_NAMES):
            n = C.c_longlong()
            ms = C.c_double()
            _ck(lib().vacgpu_kernel_stats(self.h, k, C.byref(n), C.byref(ms)),
                "vacgpu_kernel_stats")
            out[name] = (n.value, ms.value)
        return out

    def close(self):
        if getattr(self, "h", None):
            lib().vacgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many grids advanced together (vacgpu_batch_*): ``snaps`` is a list of
    (params, x, w) for each grid."""

    def __init__(self, grids):
        L = lib()
        n = len(grids)
        arr = (abi.VacParams * n)(*[g[0] for g in grids])
        h = C.c_void_p()
        _ck(L.vacgpu_batch_create(arr, n, C.byref(h)), "vacgpu_batch_create")
        self.h = h
        self.n = n
        self.meta = [(g[0].nw, tuple(g[0].nx[d] for d in range(g[0].ndim))) for g in grids]
        for i, (p, x, w) in enumerate(grids):
            xf = np.ascontiguousarray(pack_mesh(x), dtype=np.float64)
            _ck(L.vacgpu_batch_set_grid(self.h, i, _dp(xf)), "vacgpu_batch_set_grid")
            wf = np.ascontiguousarray(pack_mesh(w), dtype=np.float64)
            _ck(L.vacgpu_batch_upload(self.h, i, _dp(wf), 0, 0.0), "vacgpu_batch_upload")

    def step(self, nsteps, tstop=1e300):
        _ck(lib().vacgpu_batch_step(self.h, nsteps, tstop), "vacgpu_batch_step")

    def tune(self):
        """(persistent CTAs, work-list order, rows per item of the 2-D line
        sweep or 0, one cooperative launch for all steps (0 no, 1 yes, 2 yes
        and captured in a CUDA graph by a step call), trial times in ms of
        the candidates tried)."""
        c, o, r, one = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        ms = (C.c_double * 24)()
        _ck(lib().vacgpu_batch_tune(self.h, C.byref(c), C.byref(o), C.byref(r),
                                    C.byref(one), ms), "vacgpu_batch_tune")
        return c.value, o.value, r.value, one.value, [m for m in ms if m > 0]

    def status(self, i):
        t, it, dt, fin = C.c_double(), C.c_int(), C.c_double(), C.c_int()
        _ck(lib().vacgpu_batch_status(self.h, i, C.byref(t), C.byref(it), C.byref(dt),
                                      C.byref(fin)), "vacgpu_batch_status")
        return t.value, it.value, dt.value, bool(fin.value)

    def state(self, i):
        nw, nx = self.meta[i]
        n = int(np.prod(nx))
        out = np.empty(nw * n, dtype=np.float64)
        _ck(lib().vacgpu_batch_download(self.h, i, _dp(out)), "vacgpu_batch_download")
        return np.stack([out[k * n:(k + 1) * n].reshape(nx, order="F") for k in range(nw)])

    def close(self):
        if getattr(self, "h", None):
            lib().vacgpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def measure_fp64_peak(stream_ptr=None):
    """FP64-pipe throughput of the current GPU, FLOP/s (2 x DFMA/s)."""
    v = C.c_double()
    _ck(lib().vacgpu_measure_fp64_peak(C.byref(v), stream_ptr), "vacgpu_measure_fp64_peak")
    return v.value


class Server:
    """Continuous-batching solve server (vacgpu_server_*)."""

    def __init__(self, hbm_budget_bytes=150e9, max_active=16, steps_per_chunk=16):
        h = C.c_void_p()
        _ck(lib().vacgpu_server_create(float(hbm_budget_bytes), max_active,
                                       steps_per_chunk, C.byref(h)), "vacgpu_server_create")
        self.h = h
        self.meta = {}

    def submit(self, params, x, w, nsteps):
        """Queue a solve of nsteps steps; x, w as for Engine, or already
        flat in the C ABI's packed layout (each component in Fortran
        order).  Returns the request id."""
        x, w = np.asarray(x), np.asarray(w)
        xf = np.ascontiguousarray(x if x.ndim == 1 else pack_mesh(x), dtype=np.float64)
        wf = np.ascontiguousarray(w if w.ndim == 1 else pack_mesh(w), dtype=np.float64)
        rid = C.c_longlong()
        _ck(lib().vacgpu_server_submit(self.h, C.byref(params), _dp(xf), _dp(wf),
                                       nsteps, C.byref(rid)), "vacgpu_server_submit")
        self.meta[rid.value] = (params.nw, tuple(params.nx[d] for d in range(params.ndim)))
        return rid.value

    def result(self, rid, wait=0.0, fetch=True):
        """None if not finished, else (state or None, t, it, seconds to solution)."""
        nw, nx = self.meta[rid]
        n = int(np.prod(nx))
        out = np.empty(nw * n, dtype=np.float64) if fetch else None
        t, it, tts = C.c_double(), C.c_int(), C.c_double()
        rc = lib().vacgpu_server_result(self.h, rid, wait, _dp(out) if fetch else None,
                                        C.byref(t), C.byref(it), C.byref(tts))
        if rc == 1:
            return None
        _ck(rc, "vacgpu_server_result")
        st = None
        if fetch:
            st = np.stack([out[k * n:(k + 1) * n].reshape(nx, order="F") for k in range(nw)])
        return st, t.value, it.value, tts.value

    def timing(self, rid):
        """(queue seconds, service seconds) of a finished solve, else None."""
        q, sv = C.c_double(), C.c_double()
        rc = lib().vacgpu_server_timing(self.h, rid, C.byref(q), C.byref(sv))
        if rc == 1:
            return None
        _ck(rc, "vacgpu_server_timing")
        return q.value, sv.value

    def stats(self):
        q, a, d, pk = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        cu, span = C.c_double(), C.c_double()
        _ck(lib().vacgpu_server_stats(self.h, C.byref(q), C.byref(a), C.byref(d),
                                      C.byref(pk), C.byref(cu), C.byref(span)),
            "vacgpu_server_stats")
        return {"queued": q.value, "active": a.value, "done": d.value,
                "peak_active": pk.value, "cell_updates": cu.value, "span_s": span.value}

    def close(self):
        if getattr(self, "h", None):
            lib().vacgpu_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

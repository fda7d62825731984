"""VAC data files: binary/ASCII ``.ini``/``.out`` snapshots and ``.log`` rows.

Binary files are Fortran sequential unformatted records with 4-byte
little-endian record markers, exactly as ``savefileout_bin`` writes and
``readfileini_bin`` reads them (src/vacio.t:682-755, :1008-1047):

    record 1  fileheadout            character*79
    record 2  it t ndim neqpar nw    int32 float64 int32 int32 int32
    record 3  nx(1:ndim)             int32 * ndim
    record 4  eqpar(1:neqpar)        float64 * neqpar
    record 5  varnames               character*79
    record 6  x(ixM^S,1:ndim)        float64, column-major, one block per dim
    record 6+iw  w(ixM^S,iw)         float64, column-major

A file may hold several snapshots back to back; ``read`` returns the last
one unless ``snapshot`` is given (snapshotini semantics).
"""
import struct
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Snapshot:
    header: str
    it: int
    t: float
    ndim: int
    eqpar: np.ndarray
    varnames: str
    x: np.ndarray          # (ndim, n1[, n2[, n3]]) indexed like x(ix^D, idim)
    w: np.ndarray          # (nw,   n1[, n2[, n3]])
    nx: tuple = field(default=())

    @property
    def nw(self):
        return self.w.shape[0]


def _rec(buf, pos, endian="<"):
    (n,) = struct.unpack_from(endian + "i", buf, pos)
    data = buf[pos + 4:pos + 4 + n]
    (n2,) = struct.unpack_from(endian + "i", buf, pos + 4 + n)
    if n2 != n:
        raise ValueError("corrupt Fortran record at byte %d" % pos)
    return data, pos + 8 + n


def _pad79(s):
    s = s[:79]
    return s + " " * (79 - len(s))


def detect_type(path):
    """typefileini='auto' detection (src/vacio.t:534-570)."""
    with open(path, "rb") as f:
        head = f.read(91)
    if len(head) >= 4 and all(b != 0 for b in head[:4]):
        return "ascii"
    if len(head) >= 91 and head[88] == 0 and head[89] == 0 and (
            head[87] == 24 or head[90] == 24):
        return "binary"
    return "special"


def read(path, snapshot=0):
    kind = detect_type(path)
    if kind == "ascii":
        return read_ascii(path, snapshot)
    if kind != "binary":
        raise ValueError("%s: not a VAC binary or ascii file" % path)
    buf = open(path, "rb").read()
    endian = "<" if buf[87] == 24 else ">"
    pos, snaps = 0, []
    while pos < len(buf):
        h, pos = _rec(buf, pos, endian)
        r, pos = _rec(buf, pos, endian)
        it, t, ndim, neqpar, nw = struct.unpack(endian + "idiii", r)
        r, pos = _rec(buf, pos, endian)
        nx = struct.unpack(endian + "%di" % abs(ndim), r)
        r, pos = _rec(buf, pos, endian)
        eqpar = np.frombuffer(r, dtype=endian + "f8").copy()
        vn, pos = _rec(buf, pos, endian)
        ncell = int(np.prod(nx))
        r, pos = _rec(buf, pos, endian)
        xs = np.frombuffer(r, dtype=endian + "f8")
        if xs.size != ncell * abs(ndim):
            raise ValueError("x record size mismatch")
        x = np.stack([xs[d * ncell:(d + 1) * ncell].reshape(nx, order="F")
                      for d in range(abs(ndim))])
        ws = []
        for _ in range(nw):
            r, pos = _rec(buf, pos, endian)
            a = np.frombuffer(r, dtype=endian + "f8")
            if a.size != ncell:
                raise ValueError("w record size mismatch")
            ws.append(a.reshape(nx, order="F"))
        snaps.append(Snapshot(h.decode("latin-1").rstrip(), it, t, ndim, eqpar,
                              vn.decode("latin-1").rstrip(),
                              x.astype(np.float64),
                              np.stack(ws).astype(np.float64), tuple(nx)))
        if snapshot and len(snaps) == snapshot:
            break
    if not snaps:
        raise ValueError("%s: empty file" % path)
    return snaps[-1]


def _wrec(f, payload):
    f.write(struct.pack("<i", len(payload)))
    f.write(payload)
    f.write(struct.pack("<i", len(payload)))


def write(path, snap, append=False):
    """savefileout_bin (src/vacio.t:1008-1047)."""
    nx = snap.w.shape[1:]
    with open(path, "ab" if append else "wb") as f:
        _wrec(f, _pad79(snap.header).encode("latin-1"))
        _wrec(f, struct.pack("<idiii", snap.it, snap.t, snap.ndim,
                             len(snap.eqpar), snap.w.shape[0]))
        _wrec(f, struct.pack("<%di" % len(nx), *nx))
        _wrec(f, np.asarray(snap.eqpar, dtype="<f8").tobytes())
        _wrec(f, _pad79(snap.varnames).encode("latin-1"))
        _wrec(f, b"".join(np.asarray(snap.x[d], dtype="<f8").tobytes(order="F")
                          for d in range(snap.x.shape[0])))
        for iw in range(snap.w.shape[0]):
            _wrec(f, np.asarray(snap.w[iw], dtype="<f8").tobytes(order="F"))


def read_ascii(path, snapshot=0):
    """readfileini_asc (src/vacio.t:594-679): header, it t ndim neqpar nw,
    nx, eqpar, varnames, then one line per cell: x(1:ndim) w(1:nw)."""
    lines = open(path).read().split("\n")
    pos, snaps = 0, []
    while pos < len(lines) and lines[pos].strip():
        head = lines[pos]
        it, t, ndim, neqpar, nw = lines[pos + 1].split()
        it, t, ndim, neqpar, nw = int(it), float(t), int(ndim), int(neqpar), int(nw)
        nx = tuple(int(v) for v in lines[pos + 2].split())
        eq = np.array([float(v) for v in lines[pos + 3].split()])
        vn = lines[pos + 4]
        ncell = int(np.prod(nx))
        vals = np.array([[float(v) for v in ln.split()]
                         for ln in lines[pos + 5:pos + 5 + ncell]])
        x = np.stack([vals[:, d].reshape(nx, order="F") for d in range(abs(ndim))])
        w = np.stack([vals[:, abs(ndim) + iw].reshape(nx, order="F")
                      for iw in range(nw)])
        snaps.append(Snapshot(head.rstrip(), it, t, ndim, eq, vn.rstrip(), x, w, nx))
        pos += 5 + ncell
        if snapshot and len(snaps) == snapshot:
            break
    return snaps[-1]


def write_ascii(path, snap):
    """savefileout_asc (src/vacio.t:964-1005); 1pe18.10 data columns and
    |w|<=5e-16 written as 0."""
    nx = snap.w.shape[1:]
    with open(path, "w") as f:
        f.write(_pad79(snap.header).rstrip() + "\n")
        f.write("%7d%13.5E%3d%3d%3d\n" % (snap.it, snap.t, snap.ndim,
                                          len(snap.eqpar), snap.w.shape[0]))
        f.write("".join("%4d" % n for n in nx) + "\n")
        f.write("".join("%13.5E" % v for v in snap.eqpar) + "\n")
        f.write(snap.varnames + "\n")
        xs = [snap.x[d].ravel(order="F") for d in range(snap.x.shape[0])]
        ws = [snap.w[iw].ravel(order="F") for iw in range(snap.w.shape[0])]
        for i in range(int(np.prod(nx))):
            row = [a[i] for a in xs] + [a[i] if abs(a[i]) > 5.0e-16 else 0.0
                                        for a in ws]
            f.write("".join("%18.10E" % v for v in row) + "\n")


def log_line(it, t, dt, wmean):
    """One savefilelog_default row, format (i7,100(1pe13.5))."""
    return "%7d" % it + "".join("%13.5E" % v for v in [t, dt] + list(wmean))

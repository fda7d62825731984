"""Generate the golden fixtures: one small run per case of the benchmark
recipes and scheme variants, stored in VAC's own binary snapshot format.

For each case this writes ``<name>.ini`` (the seeded initial state, what
VAC's ``readfileini`` reads, src/vacio.t:534-755) and ``<name>.out`` (the
FP64 CPU oracle's state after ``nsteps`` steps, ``it`` and ``t`` in its
header, as ``savefileout_bin`` writes it, src/vacio.t:1008-1047), and
records the par settings and a SHA-256 of every output in ``cases.json``;
``<name>.par`` is the same case as a VAC par file, so that the Fortran
build of the reference (or the drop-in host program) runs it unchanged.

The fixtures freeze the oracle's results: the tests replay each ``.ini``
through the C oracle, the NumPy restatement and the FP64 GPU path and
require the ``.out`` bit for bit.  The initial states are stored rather
than regenerated because they go through libm's sin/cos, which may differ
in the last bit between machines; the step itself uses only IEEE
+ - * / and sqrt.  The reference ships no golden vectors of its own, so
these pin the restatement against drift, not against the Fortran binary.

Run from the repository root:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.oracle import Oracle  # noqa: E402
from vac_gb300 import abi, inistate, vacfile  # noqa: E402
from vac_gb300.vacfile import Snapshot  # noqa: E402


def hd_from_mhd(snap):
    """The gas part of an MHD snapshot as an HD one (e minus B^2/2)."""
    ndir = inistate.snap_ndir(snap)
    w = snap.w
    bb = sum(w[ndir + 2 + c] ** 2 for c in range(ndir))
    hd = np.concatenate([w[:ndir + 1], (w[ndir + 1] - 0.5 * bb)[None]])
    head = snap.header.replace("_mhd", "_hd")
    return Snapshot(head, 0, 0.0, snap.ndim, snap.eqpar[:1], "", snap.x, hd, snap.nx)


# name, initial state, limiter, boundary, steps, par settings beyond the
# path's defaults (field -> value; list values set array fields from 0)
CASES = [
    # Orszag-Tang (the 2-D FP64 plain-method recipe, 24^2 instead of 200^2)
    ("ot24-minmod", lambda: inistate.orszag_tang(24), "minmod", "periodic", 20, {}),
    # 3-D random modes, low beta (the 256^3 recipe at 10^3)
    ("rm10-woodward", lambda: inistate.random_modes(10, seed=11), "woodward", "periodic", 4, {}),
    # 2-D gamma-law hydro Riemann problem with outflow faces (the batched recipe)
    ("hd-riemann32-cont", lambda: inistate.riemann_2d(32, 7), "minmod", "cont", 15, {}),
    # 3-D MHD blast with outflow faces (the 512^3 recipe at 12^3)
    ("blast12-woodward", lambda: inistate.blast_3d(12), "woodward", "cont", 4, {}),
    # scheme variants
    ("ot20-unsplit-previous", lambda: inistate.orszag_tang(20), "vanleer", "periodic", 6,
     {"dimsplit": 0, "typelimited": abi.LIMITED_PREVIOUS}),
    ("ot20-tvdlf1", lambda: inistate.orszag_tang(20), "minmod", "periodic", 6,
     {"typefull": abi.TVDLF1}),
    ("ot20-resistive", lambda: inistate.orszag_tang(20), "superbee", "periodic", 6,
     {"eqpar": [5.0 / 3.0, 0.01]}),
    ("ot20-tvdmu-roe", lambda: inistate.orszag_tang(20), "woodward", "periodic", 8,
     {"typefull": abi.TVDMU}),
    ("sod100-tvdmu-harten", lambda: inistate.sod_1d(100), "minmod", "cont", 30,
     {"typefull": abi.TVDMU, "typeentropy": [abi.ENTROPY_NAMES["harten"]] * 3,
      "entropycoef": [0.1] * 3}),
    ("hd3-tvdmu1", lambda: hd_from_mhd(inistate.random_modes(8, seed=5, p0=0.5)), "albada",
     "periodic", 4, {"typefull": abi.TVDMU1}),
]


def apply_settings(p, settings):
    for k, v in settings.items():
        if isinstance(v, list):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(p, k, v)


def params(snap, case):
    """vacgpu_params of a case (shared with the tests)."""
    p = inistate.params_for(snap, limiter=case["limiter"], bc=case["bc"])
    apply_settings(p, case["settings"])
    return p


LIMITER = {v: k for k, v in abi.LIMITER_NAMES.items()}
TYPEFULL = {v: k for k, v in abi.TYPEFULL_NAMES.items()}
ENTROPY = {v: k for k, v in abi.ENTROPY_NAMES.items()}
LIMITED = {abi.LIMITED_ORIGINAL: "original", abi.LIMITED_PREVIOUS: "previous",
           abi.LIMITED_PREDICTOR: "predictor"}


def par_file(name, snap, case):
    """A VAC par file (namelists read by src/vacio.t:25-118) that runs the
    case from ``<name>.ini``: ``vac < <name>.par`` with the Fortran build
    or ``vacgb < <name>.par`` writes ``<name>.run.out`` whose last snapshot
    is the case's ``.out``."""
    p = params(snap, case)
    nw, nb = p.nw, 2 * p.ndim
    tf = lambda b: "T" if b else "F"
    lines = [" &testlist /",
             " &filelist",
             "        filenameini='%s.ini'" % name,
             "        filename='%s.log','%s.run.out'" % (name, name),
             " /",
             " &savelist",
             "        ditsave=%d,%d" % (case["nsteps"], case["nsteps"]),
             " /",
             " &stoplist",
             "        itmax=%d" % case["nsteps"],
             " /",
             " &methodlist",
             "        typefull=%d*'%s'" % (nw, TYPEFULL[p.typefull]),
             "        typelimiter=%d*'%s'" % (nw, LIMITER[p.typelimiter[0]]),
             "        typelimited='%s'" % LIMITED[p.typelimited],
             "        dimsplit=%s" % tf(p.dimsplit)]
    if p.typefull in (abi.TVDMU, abi.TVDMU1) and "typeentropy" in case["settings"]:
        lines.append("        typeentropy=%d*'%s'" % (nw, ENTROPY[p.typeentropy[0]]))
        lines.append("        entropycoef=%d*%r" % (nw, p.entropycoef[0]))
    lines += [" /",
              " &boundlist",
              "        typeB=%d*'%s'" % (nw * nb, case["bc"]),
              " /",
              " &paramlist",
              "        courantpar=%r" % p.courantpar,
              "        dtpar=%r" % p.dtpar,
              " /"]
    return "\n".join(lines) + "\n"


def sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def main():
    index = {}
    for name, mk, lim, bc, nsteps, settings in CASES:
        s = mk()
        case = {"limiter": lim, "bc": bc, "nsteps": nsteps, "settings": settings}
        if "eqpar" in settings:
            # eqpar travels in the .ini header, as in VAC's own files
            s.eqpar = np.asarray(settings["eqpar"], dtype=np.float64)
        ini = os.path.join(HERE, name + ".ini")
        vacfile.write(ini, s)
        s0 = vacfile.read(ini)
        o = Oracle(params(s0, case), s0.x, s0.w)
        o.step(nsteps)
        out = Snapshot(s0.header, o.it, o.t, s0.ndim, s0.eqpar, s0.varnames, s0.x,
                       o.state(), s0.nx)
        outp = os.path.join(HERE, name + ".out")
        vacfile.write(outp, out)
        with open(os.path.join(HERE, name + ".par"), "w") as f:
            f.write(par_file(name, s0, case))
        case.update(it=int(o.it), t=float(o.t).hex(), nerror=list(map(int, o.nerror())),
                    sha256_ini=sha(ini), sha256_out=sha(outp))
        index[name] = case
        print(name, o.it, o.t)
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(index, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()

"""Golden fixtures (tests/golden): seeded initial states and the FP64
oracle's results after a fixed number of steps, stored in VAC's binary
snapshot format (src/vacio.t:534-755 reads them, :1008-1047 writes them).

CPU: the fixture files are intact, and the C oracle and the NumPy
restatement reproduce every ``.out`` bit for bit from its ``.ini`` (with
``it``, ``t`` and the error counters).  GPU: the FP64 path through the C
ABI reproduces the same bits.  Regenerate with tests/golden/make_golden.py
only when the oracle's arithmetic is meant to change."""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

from oracle.oracle import Oracle
from oracle.vac_numpy import NumpyVac
from vac_gb300 import vacfile

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
from make_golden import params  # noqa: E402

with open(os.path.join(GOLDEN, "cases.json")) as _f:
    CASES = json.load(_f)
NAMES = sorted(CASES)


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def load(name):
    case = CASES[name]
    ini = vacfile.read(os.path.join(GOLDEN, name + ".ini"))
    out = vacfile.read(os.path.join(GOLDEN, name + ".out"))
    return case, ini, out


def check(run, case, out):
    assert run.it == case["it"] == out.it
    assert run.t == float.fromhex(case["t"]) == out.t
    a = run.state()
    bad = np.count_nonzero(bits(a) != bits(out.w))
    assert bad == 0, "%d of %d values differ, max |diff| %g" % (
        bad, a.size, np.abs(a - out.w).max())


def test_fixture_files_intact():
    assert len(NAMES) >= 10
    for name in NAMES:
        for ext in ("ini", "out"):
            with open(os.path.join(GOLDEN, name + "." + ext), "rb") as f:
                assert hashlib.sha256(f.read()).hexdigest() == CASES[name]["sha256_" + ext], name


def test_fixture_states_are_not_trivial():
    """Every case evolves: the final state differs from the initial one in
    every variable that the step moves."""
    for name in NAMES:
        case, ini, out = load(name)
        assert out.it == case["nsteps"] and out.t > 0.0
        assert np.abs(out.w[0] - ini.w[0]).max() > 1e-6, name


@pytest.mark.parametrize("name", NAMES)
def test_c_oracle_reproduces_fixture(name):
    case, ini, out = load(name)
    o = Oracle(params(ini, case), ini.x, ini.w)
    o.step(case["nsteps"])
    check(o, case, out)
    assert o.nerror() == case["nerror"]


@pytest.mark.parametrize("name", NAMES)
def test_numpy_restatement_reproduces_fixture(name):
    case, ini, out = load(name)
    nv = NumpyVac(params(ini, case), ini.x, ini.w)
    nv.step(case["nsteps"])
    check(nv, case, out)


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_fp64_reproduces_fixture(gpu_lib, name):
    from vac_gb300.engine import Engine
    case, ini, out = load(name)
    e = Engine(params(ini, case), ini.x, ini.w)
    e.step(case["nsteps"])
    check(e, case, out)
    assert e.nerror() == case["nerror"]


@pytest.mark.parametrize("name", NAMES)
def test_par_file_states_the_case(name):
    """Each case's VAC par file, read by the drop-in host program's namelist
    parser (``vacgb --dump-params``, no GPU), gives the case's parameters."""
    import subprocess
    from vac_gb300 import abi, build
    build.build()
    case, ini, _ = load(name)
    with open(os.path.join(GOLDEN, name + ".par")) as f:
        par = f.read()
    d = json.loads(subprocess.run([build.VACGB, "--dump-params"], cwd=GOLDEN, input=par,
                                  capture_output=True, text=True, check=True).stdout)
    p = params(ini, case)
    nw = p.nw
    for k in ("ndim", "ndir", "physics", "nw", "typefull", "typelimited", "dimsplit",
              "typedimsplit", "divbfix", "courantpar", "dtpar", "useprimitive", "smallfix"):
        assert d[k] == getattr(p, k), k
    assert d["nx"][:p.ndim] == list(p.nx)[:p.ndim]
    assert d["gamma"] == p.eqpar[0] and d["itmax"] == case["nsteps"]
    assert d["typelimiter"] == list(p.typelimiter)[:nw]
    assert d["typeB"] == [list(p.typeB[ib])[:nw] for ib in range(2 * p.ndim)]
    if p.typefull in (abi.TVDMU, abi.TVDMU1):
        assert d["typeentropy"] == list(p.typeentropy)[:nw]
        assert d["entropycoef"] == list(p.entropycoef)[:nw]
    assert d["filenames"] == [name + ".log", name + ".run.out"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_host_program_runs_par_file(gpu_lib, name, tmp_path):
    """The drop-in host program run the way VAC is run (``vacgb < <case>.par``
    beside ``<case>.ini``) writes a ``.run.out`` whose last snapshot is the
    fixture, bit for bit."""
    import shutil
    import subprocess
    from vac_gb300 import build
    case, _, out = load(name)
    for ext in ("ini", "par"):
        shutil.copy(os.path.join(GOLDEN, name + "." + ext), tmp_path)
    with open(tmp_path / (name + ".par")) as f:
        r = subprocess.run([build.VACGB], cwd=tmp_path, input=f.read(),
                           capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    got = vacfile.read(str(tmp_path / (name + ".run.out")))
    assert got.it == out.it and got.t == out.t
    assert np.array_equal(bits(got.w), bits(out.w))

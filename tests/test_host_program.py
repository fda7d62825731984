"""vacgb, the drop-in host program: VAC par files (namelists with repeat
counts, subscripts, comments, &end) and .ini files in, .out snapshots and
.log rows out, exactly where VAC's timetosave puts them."""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle.oracle import Oracle
from vac_gb300 import abi, inistate, vacfile

PAR = """ &testlist /
 &filelist
        filenameini='ot.ini'                ! initial file
        filename='ot.log','ot.out'
 /
 &savelist
        ditsave=5,10
 /
 &stoplist
        itmax=20
 /
 &methodlist
        typefull=   6*'tvdlf'
        typelimiter=6*'woodward'
        typelimiter(2)='minmod'
        dimsplit=T
        smallpcoeff=1.D-6
 &end
 &boundlist
        typeB=6*'periodic',6*'periodic',
              12*'periodic'
        typeB(1,3)='periodic'
 /
 &paramlist
        courantpar=0.8D0
 /
"""


@pytest.fixture(scope="module")
def vacgb():
    from vac_gb300 import build
    build.build()
    return build.VACGB


def _setup(tmp_path, n=32):
    s = inistate.orszag_tang(n)
    vacfile.write(str(tmp_path / "ot.ini"), s)
    (tmp_path / "ot.par").write_text(PAR)
    return s


def test_par_parsing(vacgb, tmp_path):
    _setup(tmp_path)
    out = subprocess.run([vacgb, "--dump-params"], cwd=tmp_path, capture_output=True,
                         text=True, input=PAR, check=True).stdout
    d = json.loads(out)
    assert (d["ndim"], d["ndir"], d["physics"], d["nw"]) == (2, 2, abi.PHYS_MHD, 6)
    assert d["typelimiter"] == [1, 0, 1, 1, 1, 1]
    assert d["typeB"] == [[1] * 6] * 4
    assert d["ditsave"] == [5, 10] and d["itmax"] == 20
    assert d["filenames"] == ["ot.log", "ot.out"]
    assert abs(d["gamma"] - 5.0 / 3.0) < 1e-15


@pytest.mark.gpu
def test_run_writes_vac_outputs(vacgb, tmp_path):
    s = _setup(tmp_path)
    r = subprocess.run([vacgb], cwd=tmp_path, capture_output=True, text=True,
                       input=PAR)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Finish Advance" in r.stdout
    p = inistate.params_for(s, limiter="woodward")
    p.typelimiter[1] = abi.LIM_MINMOD
    o = Oracle(p, s.x, s.w)
    for snap, it in ((1, 10), (2, 20)):
        got = vacfile.read(str(tmp_path / "ot.out"), snapshot=snap)
        o.step(it - o.it)
        assert got.it == it and got.t == o.t
        assert np.array_equal(got.w.view(np.uint64), o.state().view(np.uint64))
    rows = [ln.split() for ln in open(tmp_path / "ot.log").read().splitlines()[2:]]
    assert [int(r[0]) for r in rows] == [5, 10, 15, 20]
    np.testing.assert_allclose([float(v) for v in rows[-1][3:]], o.sums(), rtol=1e-5,
                               atol=1e-12)  # momentum means are round-off sized


def test_par_parsing_smallfix(vacgb, tmp_path):
    """keeppositive settings of &methodlist reach the parameter block."""
    _setup(tmp_path)
    par = PAR.replace("smallpcoeff=1.D-6", "smallpcoeff=1.D-6\n        smallfix=T\n"
                      "        useprimitive=T\n"
                      "        smallp=0.25\n        smallrho=0.5D0\n"
                      "        smallrhocoeff=1.D-4\n        vacuumrho=1.D-3")
    out = subprocess.run([vacgb, "--dump-params"], cwd=tmp_path, capture_output=True,
                         text=True, input=par, check=True).stdout
    d = json.loads(out)
    assert d["smallfix"] == 1 and d["smallp"] == 0.25 and d["smallrho"] == 0.5
    assert d["smallrhocoeff"] == 1e-4 and d["vacuumrho"] == 1e-3
    assert d["useprimitive"] == 1
    d0 = json.loads(subprocess.run([vacgb, "--dump-params"], cwd=tmp_path,
                                   capture_output=True, text=True, input=PAR,
                                   check=True).stdout)
    assert (d0["smallfix"], d0["smallrho"], d0["vacuumrho"]) == (0, -1.0, -1.0)


def test_par_parsing_tvdmu(vacgb, tmp_path):
    """typefull='tvdmu' with per-wave typeentropy/entropycoef and divbwave
    (&methodlist, src/vacio.t:35,80); physini's default entropycoef are the
    single precision literals 0.2 and 0.4 (src/vacphys.mhd0.t:18-28)."""
    _setup(tmp_path)
    par = PAR.replace("typefull=   6*'tvdlf'", "typefull=   6*'tvdmu'\n"
                      "        typeentropy=4*'harten',2*'nul'\n"
                      "        typeentropy(6)='powell'\n"
                      "        entropycoef(5)=0.3D0\n        divbwave=F")
    d = json.loads(subprocess.run([vacgb, "--dump-params"], cwd=tmp_path,
                                  capture_output=True, text=True, input=par,
                                  check=True).stdout)
    assert d["typefull"] == abi.TVDMU and d["divbwave"] == 0
    assert d["typeentropy"] == [abi.ENTROPY_HARTEN] * 4 + [abi.ENTROPY_NUL, abi.ENTROPY_POWELL]
    f02 = float(np.float32(0.2))
    assert d["entropycoef"] == [f02] * 4 + [0.3, -1.0]
    d0 = json.loads(subprocess.run([vacgb, "--dump-params"], cwd=tmp_path,
                                   capture_output=True, text=True, input=PAR,
                                   check=True).stdout)
    assert d0["typeentropy"] == [0] * 6 and d0["divbwave"] == 1
    assert d0["entropycoef"] == [abi.default_entropycoef(abi.PHYS_MHD, il) for il in range(6)]


@pytest.mark.gpu
def test_run_tvdmu_writes_vac_outputs(vacgb, tmp_path):
    """The host program on the TVD-MUSCL/Roe path: .out snapshots bit-equal
    to the oracle."""
    s = _setup(tmp_path)
    par = PAR.replace("typefull=   6*'tvdlf'", "typefull=   6*'tvdmu'")
    r = subprocess.run([vacgb], cwd=tmp_path, capture_output=True, text=True, input=par)
    assert r.returncode == 0, r.stdout + r.stderr
    p = inistate.params_for(s, limiter="woodward")
    p.typelimiter[1] = abi.LIM_MINMOD
    p.typefull = abi.TVDMU
    o = Oracle(p, s.x, s.w)
    for snap, it in ((1, 10), (2, 20)):
        got = vacfile.read(str(tmp_path / "ot.out"), snapshot=snap)
        o.step(it - o.it)
        assert got.it == it and got.t == o.t
        assert np.array_equal(got.w.view(np.uint64), o.state().view(np.uint64))


@pytest.mark.gpu
def test_run_special_bound_hook(vacgb, tmp_path):
    """typeB='special' through the host program: the specialbound hook
    comes from VACGB_SPECIALBOUND=lib.so:symbol; results equal the oracle
    with the host twin of the hook."""
    from tests.test_special_bound import _device_hook, _host_hook
    s = _setup(tmp_path)
    par = PAR.replace("typeB=6*'periodic',6*'periodic',", "typeB=6*'special',6*'cont',")
    Ld, _ = _device_hook()
    env = dict(os.environ, VACGB_SPECIALBOUND=Ld._name + ":inflow_bound")
    r = subprocess.run([vacgb], cwd=tmp_path, capture_output=True, text=True, input=par,
                       env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    Lh, hfn = _host_hook()
    p = inistate.params_for(s, limiter="woodward")
    p.typelimiter[1] = abi.LIM_MINMOD
    for iw in range(p.nw):
        p.typeB[0][iw] = abi.BC_SPECIAL
        p.typeB[1][iw] = abi.BC_CONT
    o = Oracle(p, s.x, s.w, bound=(hfn, None))
    got = vacfile.read(str(tmp_path / "ot.out"), snapshot=2)
    o.step(20)
    assert got.it == 20 and got.t == o.t
    assert np.array_equal(got.w.view(np.uint64), o.state().view(np.uint64))
    r2 = subprocess.run([vacgb], cwd=tmp_path, capture_output=True, text=True, input=par,
                        env={k: v for k, v in os.environ.items() if k != "VACGB_SPECIALBOUND"})
    assert r2.returncode != 0 and "Special boundary is not defined" in r2.stdout + r2.stderr


@pytest.mark.gpu
def test_run_special_source_hook(vacgb, tmp_path):
    """The user's specialsource and getdt_special through the host program
    (VACGB_SPECIALSOURCE=lib.so:source:getdt); results equal the oracle with
    the host twins of the hooks."""
    from tests.test_special_source import _device_hook, _host_hook
    s = _setup(tmp_path)
    Ld, _, _ = _device_hook()
    env = dict(os.environ, VACGB_SPECIALSOURCE=Ld._name + ":src_dev:dt_dev")
    r = subprocess.run([vacgb], cwd=tmp_path, capture_output=True, text=True, input=PAR,
                       env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    Lh, hs, hd = _host_hook()
    p = inistate.params_for(s, limiter="woodward")
    p.typelimiter[1] = abi.LIM_MINMOD
    o = Oracle(p, s.x, s.w, source=(hs, hd, 1 + p.ndir))
    for snap, it in ((1, 10), (2, 20)):
        got = vacfile.read(str(tmp_path / "ot.out"), snapshot=snap)
        o.step(it - o.it)
        assert got.it == it and got.t == o.t
        assert np.array_equal(got.w.view(np.uint64), o.state().view(np.uint64))
    bad = dict(os.environ, VACGB_SPECIALSOURCE=Ld._name + ":no_such_symbol")
    r2 = subprocess.run([vacgb], cwd=tmp_path, capture_output=True, text=True, input=PAR,
                        env=bad)
    assert r2.returncode != 0 and "no symbol no_such_symbol" in r2.stdout + r2.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_async_saves_match_synchronous_saves(vacgb, tmp_path, precision):
    """Snapshots written by the writer thread while the run continues give
    the same .out and .log files, byte for byte, as a download and write
    before the run continues (VACGB_SYNC_SAVE=1); a snapshot every step."""
    par = PAR.replace("ditsave=5,10", "ditsave=1,1").replace("itmax=20", "itmax=12")
    outs = {}
    for mode in ("async", "sync"):
        d = tmp_path / mode
        d.mkdir()
        _setup(d)
        env = dict(os.environ)
        env.pop("VACGB_SYNC_SAVE", None)
        if mode == "sync":
            env["VACGB_SYNC_SAVE"] = "1"
        r = subprocess.run([vacgb, "--precision=" + precision], cwd=d, capture_output=True,
                           text=True, input=par, env=env)
        assert r.returncode == 0, r.stdout + r.stderr
        outs[mode] = ((d / "ot.out").read_bytes(), (d / "ot.log").read_bytes())
    assert outs["async"] == outs["sync"]
    last = vacfile.read(str(tmp_path / "async" / "ot.out"))  # the last snapshot
    assert last.it == 12

"""The drop-in host program's namelist reader on seeded random VAC par
files: repeat counts (n*'x'), subscripted assignments (typeB(iw,iB)=...,
with or without blanks inside the subscript, on their own line or after
other values), Fortran logicals (T, .false., .TRUE.) and reals with D
exponents, trailing comments.  ``vacgb --dump-params`` (no GPU) must give
back the parameters the file states (src/vacio.t:25-118 reads the same
namelists)."""
import json
import subprocess

import numpy as np
import pytest

from vac_gb300 import abi, inistate, vacfile

BCS = ["cont", "periodic", "symm", "asymm", "fixed", "fixed1", "cont1", "grad1", "symm0"]
LIMS = ["minmod", "woodward", "superbee", "vanleer", "albada"]
SCHEMES = ["tvdlf", "tvdlf1", "tvdmu", "tvdmu1"]
ENTS = ["nul", "harten", "powell", "ratio", "yee"]
REALS = [("0.8", 0.8), ("8.D-1", 0.8), ("8.0d-1", 0.8), ("0.75E0", 0.75), (".6", 0.6),
         ("5d-1", 0.5), ("0.45D0", 0.45)]
TRUE = ["T", ".true.", ".TRUE.", ".t."]
FALSE = ["F", ".false.", ".FALSE.", ".f."]

INIS = [("ot", lambda: inistate.orszag_tang(8)),
        ("rm3", lambda: inistate.random_modes(6, seed=1)),
        ("hd2", lambda: inistate.riemann_2d(8, 1)),
        ("sod", lambda: inistate.sod_1d(16))]


@pytest.fixture(scope="module")
def setup(tmp_path_factory):
    from vac_gb300 import build
    build.build()
    d = tmp_path_factory.mktemp("par")
    nws = {}
    for name, mk in INIS:
        s = mk()
        vacfile.write(str(d / (name + ".ini")), s)
        nws[name] = (s.w.shape[0], s.ndim)
    return build.VACGB, d, nws


def runs(vals):
    """n*'x' run-length form of a list of names."""
    out, k = [], 0
    while k < len(vals):
        m = k
        while m < len(vals) and vals[m] == vals[k]:
            m += 1
        out.append("%d*'%s'" % (m - k, vals[k]) if m - k > 1 else "'%s'" % vals[k])
        k = m
    return out


def sub(rng, *idx):
    sep = [",", ", ", " , "][rng.integers(3)]
    pad = ["", " "][rng.integers(2)]
    return "(" + pad + sep.join(str(i) for i in idx) + pad + ")"


def make_par(rng, ini, nw, ndim):
    """A random par file and the parameters it states."""
    exp = {}
    lim = [LIMS[rng.integers(5)] for _ in range(nw)]
    over = {int(rng.integers(nw)): LIMS[rng.integers(5)] for _ in range(rng.integers(3))}
    scheme = SCHEMES[rng.integers(4)]
    split = bool(rng.integers(2))
    nb = 2 * ndim
    tb = [[BCS[rng.integers(len(BCS))] for _ in range(nw)] for _ in range(nb)]
    bover = {}
    for _ in range(rng.integers(4)):
        bover[(int(rng.integers(nw)), int(rng.integers(nb)))] = BCS[rng.integers(len(BCS))]
    cr, cval = REALS[rng.integers(len(REALS))]
    L = [" &testlist /", " &filelist", "    filenameini='%s.ini'   ! initial state" % ini, " /",
         " &methodlist",
         "    typefull= %d*'%s'" % (nw, scheme),
         "    typelimiter= " + ", ".join(runs(lim))]
    for iw, l in over.items():
        L.append("    typelimiter%s = '%s'" % (sub(rng, iw + 1), l))
        lim[iw] = l
    L.append("    dimsplit=%s" % (TRUE if split else FALSE)[rng.integers(4)])
    tl = ["original", "previous", "predictor", None][rng.integers(4)]
    if tl:
        L.append("    typelimited='%s'" % tl)
    ent = None
    if scheme.startswith("tvdmu"):
        ent = [ENTS[rng.integers(5)] for _ in range(nw)]
        L.append("    typeentropy=" + ",".join(runs(ent)) + "  ! per wave")
    L.append(" /")
    flat = [tb[ib][iw] for ib in range(nb) for iw in range(nw)]
    items = runs(flat)
    bl = " &boundlist typeB= " + ", ".join(items)
    for (iw, ib), b in bover.items():
        bl += [" ", ", ", "\n    "][rng.integers(3)] + "typeB%s='%s'" % (sub(rng, iw + 1, ib + 1), b)
        tb[ib][iw] = b
    L += [bl, " /", " &paramlist courantpar=%s, dtpar=-1d0 /" % cr,
          " &stoplist itmax=%d /" % rng.integers(1, 500)]
    exp.update(typelimiter=[LIMS.index(l) for l in lim], typefull=SCHEMES.index(scheme),
               dimsplit=int(split), typeB=[[BCS.index(b) for b in row] for row in tb],
               courantpar=cval)
    if not split:
        exp["typelimited"] = (abi.LIMITED_PREDICTOR if tl == "predictor"
                              else abi.LIMITED_PREVIOUS)
    elif tl:
        exp["typelimited"] = ["original", "previous", "predictor"].index(tl)
    else:
        exp["typelimited"] = abi.LIMITED_ORIGINAL
    if ent:
        exp["typeentropy"] = [ENTS.index(e) for e in ent]
    return "\n".join(L) + "\n", exp


@pytest.mark.parametrize("k", range(40))
def test_random_par_files_read_back(setup, k):
    vacgb, d, nws = setup
    rng = np.random.default_rng(700 + k)
    ini = INIS[k % len(INIS)][0]
    nw, ndim = nws[ini]
    par, exp = make_par(rng, ini, nw, ndim)
    r = subprocess.run([vacgb, "--dump-params"], cwd=d, input=par, capture_output=True,
                       text=True)
    assert r.returncode == 0, par + r.stderr
    got = json.loads(r.stdout)
    for key, val in exp.items():
        assert got[key] == val, (key, par)


ARRAYS = """ &filelist filenameini='ot.ini'
   filename(2)='b.out'
   filename(1)='a.log' /
 &savelist ditsave(1)=10
   ditsave(2)=20
   dtsave(2)=0.5d0, itsave(2,1)=7 /
 &methodlist typefull=6*'tvdmu' typefull(2)='tvdmu'
   eqpar(1)=1.4d0
   eqpar(2)=0.01
   typeentropy=3*'harten' typeentropy(4)='yee', entropycoef(2)=0.3 /
"""


def test_array_assignments_accumulate(setup):
    """Several assignments to elements of one array all take effect, in
    file order (filename, eqpar, typefull, dtsave, ditsave, itsave,
    typeentropy, entropycoef)."""
    vacgb, d, _ = setup
    got = json.loads(subprocess.run([vacgb, "--dump-params"], cwd=d, input=ARRAYS,
                                    capture_output=True, text=True, check=True).stdout)
    assert got["filenames"] == ["a.log", "b.out"]
    assert got["ditsave"] == [10, 20] and got["dtsave"] == [1e99, 0.5]
    assert got["itsave1"] == [10000000, 7]
    assert got["eqpar"] == [1.4, 0.01] and got["typefull"] == abi.TVDMU
    assert got["typeentropy"] == [abi.ENTROPY_HARTEN] * 3 + [abi.ENTROPY_YEE, 0, 0]
    assert got["entropycoef"][1] == 0.3


@pytest.mark.parametrize("bad", ["typeB(7,1)='cont'", "typeB(0,1)='cont'",
                                 "typeB(1,5)='cont'", "typeB(25)='cont'",
                                 "typeB(1,1,1)='cont'", "typelimiter(0)='minmod'",
                                 "typelimiter(7)='minmod'", "typelimiter(1,1)='minmod'",
                                 "eqpar(5)=1.0", "dtsave(3)=1.0", "ditsave(3)=5",
                                 "tsave(1,3)=1.0", "itsave(101,1)=5", "tsave(201)=1.0"])
def test_subscript_out_of_range_is_an_error(setup, bad):
    vacgb, d, _ = setup
    grp = "boundlist" if bad.startswith("typeB") else "methodlist"
    par = " &filelist filenameini='ot.ini' /\n &%s %s /\n" % (grp, bad)
    r = subprocess.run([vacgb, "--dump-params"], cwd=d, input=par, capture_output=True,
                       text=True)
    assert r.returncode != 0 and "subscript out of range" in (r.stdout + r.stderr)


@pytest.mark.parametrize("cut,msg", [(-8, "Error in ReadFileIni"), (200, "Error in ReadFileIni"),
                                     ("eqpar", "wrong size of the eqpar"),
                                     ("ndir", "ndir outside"), ("nw", "Incompatible number")])
def test_damaged_ini_is_an_error(setup, tmp_path, cut, msg):
    """A truncated binary .ini, or one whose records disagree with its
    header, stops the program with a message instead of being read."""
    vacgb, d, _ = setup
    raw = (d / "ot.ini").read_bytes()
    if cut == "eqpar":
        s = vacfile.read(str(d / "ot.ini"))
        vacfile.write(str(tmp_path / "bad.ini"), s)
        raw = bytearray((tmp_path / "bad.ini").read_bytes())
        # neqpar in the it,t,ndim,neqpar,nw record (after the 79-byte header record)
        raw[4 + 79 + 4 + 4 + 16:4 + 79 + 4 + 4 + 20] = (3).to_bytes(4, "little")
        raw = bytes(raw)
    elif cut in ("ndir", "nw"):
        # a header whose ndir digit asks for 9 vector components, with a
        # file that holds the 20 variables they would need; or an honest
        # 2-D header over 20 variables
        import numpy as np
        s = vacfile.read(str(d / "ot.ini"))
        s.w = np.concatenate([s.w] * 4)[:20].copy()
        s.header = "damaged_mhd29" if cut == "ndir" else "damaged_mhd22"
        vacfile.write(str(tmp_path / "bad.ini"), s)
        raw = (tmp_path / "bad.ini").read_bytes()
    else:
        raw = raw[:cut]
    (tmp_path / "bad.ini").write_bytes(raw)
    r = subprocess.run([vacgb, "--dump-params"], cwd=tmp_path, capture_output=True, text=True,
                       input=" &filelist filenameini='bad.ini' /\n")
    assert r.returncode != 0 and msg in (r.stdout + r.stderr), r.stdout + r.stderr


def test_ascii_ini_header_is_read(setup, tmp_path):
    """An ASCII .ini (typefileini='auto' detects it, src/vacio.t:534-570)
    gives the same grid and equation parameters as the binary one."""
    vacgb, d, _ = setup
    s = vacfile.read(str(d / "rm3.ini"))
    vacfile.write_ascii(str(tmp_path / "a.ini"), s)
    # this host writes binary .out files only; with an ASCII .ini VAC's
    # typefileout would default to ASCII
    par = " &filelist filenameini='%s' typefileout='binary' /\n"
    out = []
    for path in (str(tmp_path / "a.ini"), str(d / "rm3.ini")):
        out.append(json.loads(subprocess.run([vacgb, "--dump-params"], cwd=tmp_path,
                                             input=par % path, capture_output=True, text=True,
                                             check=True).stdout))
    for key in ("ndim", "ndir", "physics", "nw", "nx"):
        assert out[0][key] == out[1][key], key
    # the ASCII file keeps 6 significant digits
    assert abs(out[0]["gamma"] - out[1]["gamma"]) <= 1e-5 * out[1]["gamma"]

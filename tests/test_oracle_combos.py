"""The two restatements of the reference against each other on seeded
random combinations of the path's switches: physics (MHD, HD), 2-D and
3-D, every limiter, every boundary type, every scheme (tvdlf, tvdlf1,
tvdmu, tvdmu1), sweep order (xyyx, xy, unsplit) and limiter base
('original', 'previous', 'predictor').  The C oracle and the NumPy
restatement must agree bit for bit (state, t, it) on each combination."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from oracle.vac_numpy import NumpyVac
from vac_gb300 import abi, inistate
from vac_gb300.vacfile import Snapshot

LIMITERS = ["minmod", "woodward", "superbee", "vanleer", "albada"]
# 'reflect': symm for every variable, asymm for the momentum normal to the
# face (a reflecting wall; asymm on every variable would make the ghost
# density negative)
BOUNDS = ["periodic", "cont", "symm", "reflect", "cont1", "grad1", "fixed", "fixed1", "symm0"]
SCHEMES = [abi.TVDLF, abi.TVDLF1, abi.TVDMU, abi.TVDMU1]
SPLITS = ["xyyx", "xy", "unsplit"]
LIMITED = [abi.LIMITED_ORIGINAL, abi.LIMITED_PREVIOUS, abi.LIMITED_PREDICTOR]


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def hd_from_mhd(snap):
    ndir = inistate.snap_ndir(snap)
    w = snap.w
    bb = sum(w[ndir + 2 + c] ** 2 for c in range(ndir))
    hd = np.concatenate([w[:ndir + 1], (w[ndir + 1] - 0.5 * bb)[None]])
    return Snapshot(snap.header.replace("_mhd", "_hd"), 0, 0.0, snap.ndim, snap.eqpar[:1], "",
                    snap.x, hd, snap.nx)


def combo(k):
    """The k-th seeded combination: (label, snapshot, params, steps)."""
    rng = np.random.default_rng(1000 + k)
    mhd = bool(rng.integers(2))
    ndim = int(rng.choice([2, 3]))
    n = int(rng.integers(10, 19)) if ndim == 2 else int(rng.integers(6, 10))
    s = inistate.random_modes(n, seed=k, ndim=ndim, p0=0.05 if mhd else 0.5)
    if not mhd:
        s = hd_from_mhd(s)
    lim = LIMITERS[rng.integers(len(LIMITERS))]
    bc = BOUNDS[rng.integers(len(BOUNDS))]
    p = inistate.params_for(s, limiter=lim, bc="symm" if bc == "reflect" else bc)
    if bc == "reflect":
        for d in range(ndim):
            for upper in (0, 1):
                p.typeB[2 * d + upper][1 + d] = abi.BC_NAMES["asymm"]
    p.typefull = SCHEMES[rng.integers(len(SCHEMES))]
    split = SPLITS[rng.integers(len(SPLITS))]
    if split == "unsplit":
        p.dimsplit = 0
        p.typelimited = abi.LIMITED_PREVIOUS
    else:
        p.typedimsplit = abi.SPLIT_XY if split == "xy" else abi.SPLIT_XYYX
        p.typelimited = LIMITED[rng.integers(len(LIMITED))]
    steps = int(rng.integers(3, 6))
    label = "%s%dd-n%d-%s-%s-%s-%s-%s" % (
        "mhd" if mhd else "hd", ndim, n, lim, bc,
        {abi.TVDLF: "tvdlf", abi.TVDLF1: "tvdlf1", abi.TVDMU: "tvdmu",
         abi.TVDMU1: "tvdmu1"}[p.typefull], split,
        {abi.LIMITED_ORIGINAL: "orig", abi.LIMITED_PREVIOUS: "prev",
         abi.LIMITED_PREDICTOR: "pred"}[p.typelimited])
    return label, s, p, steps


NCOMBO = 32

# a run that overflows would compare overflows, not arithmetic
pytestmark = pytest.mark.filterwarnings("error::RuntimeWarning")


@pytest.mark.parametrize("k", range(NCOMBO), ids=[combo(k)[0] for k in range(NCOMBO)])
def test_c_oracle_matches_numpy_on_random_switches(k):
    _, s, p, steps = combo(k)
    o = Oracle(p, s.x, s.w)
    nv = NumpyVac(p, s.x, s.w)
    o.step(steps)
    nv.step(steps)
    assert o.it == nv.it == steps and o.t == nv.t
    a, b = o.state(), nv.state()
    bad = np.count_nonzero(bits(a) != bits(b))
    assert bad == 0, "%d of %d values differ, max |diff| %g" % (
        bad, a.size, np.abs(a - b).max())


def test_combinations_cover_every_switch():
    labels = [combo(k)[0] for k in range(NCOMBO)]
    for group in (LIMITERS, BOUNDS, ["tvdlf-", "tvdlf1", "tvdmu-", "tvdmu1"], SPLITS,
                  ["orig", "prev", "pred"], ["mhd2d", "mhd3d", "hd2d", "hd3d"]):
        for item in group:
            assert any(item in lab for lab in labels), item


HD_ENTROPY = ["nul", "harten", "powell", "yee"]        # 'ratio' has no HD speeds
MHD_ENTROPY = ["nul", "harten", "powell", "ratio", "yee"]


def extras(k):
    """The k-th seeded combination of the source terms and side switches on
    top of a base combination: resistivity (curl or compact form), the
    gravity hook, a stretched grid, divbfix off, smallfix, useprimitive,
    Courant number and one entropy fix for every Roe wave."""
    label, s, p, steps = combo(NCOMBO + k)
    rng = np.random.default_rng(5000 + k)
    mhd = p.physics == abi.PHYS_MHD
    tags = []
    if rng.random() < 0.4:
        s = inistate.stretched(s, amp=float(rng.uniform(0.05, 0.2)))
        tags.append("stretched")
    if mhd and rng.random() < 0.5:
        p.eqpar[1] = float(rng.choice([0.002, 0.01, 0.03]))
        p.compactres = int(rng.integers(2))
        tags.append("eta%g%s" % (p.eqpar[1], "c" if p.compactres else ""))
    if mhd and rng.random() < 0.25:
        p.divbfix = 0
        tags.append("nodivb")
    grav = None
    if rng.random() < 0.5:
        grav = [float(g) for g in rng.uniform(-0.2, 0.2, size=s.ndim)]
        tags.append("grav")
    if rng.random() < 0.3:
        p.smallfix = 1
        p.smallp = float(rng.uniform(0.01, 0.04))
        tags.append("smallfix")
    if p.dimsplit and p.typelimited == abi.LIMITED_ORIGINAL and rng.random() < 0.4:
        p.useprimitive = 1
        tags.append("useprim")
    # Courant numbers up to 0.7 and periodic, outflow or reflecting faces:
    # on these small random grids the Roe dissipation runs away within a
    # few steps at Courant 0.86 with superbee and Harten's fix, with the
    # extrapolating faces (the reference warns that extrapolation "can be
    # numericly unstable", src/vacgrid.t:276) and with 'symm0' on every
    # variable -- in both restatements alike, which would compare
    # overflows rather than arithmetic
    p.courantpar = float(rng.uniform(0.3, 0.7))
    bc = ["periodic", "cont", "reflect"][rng.integers(3)]
    abi.set_all_bc(p, abi.BC_NAMES["symm" if bc == "reflect" else bc])
    if bc == "reflect":
        for d in range(s.ndim):
            for upper in (0, 1):
                p.typeB[2 * d + upper][1 + d] = abi.BC_NAMES["asymm"]
    parts = label.split("-")
    parts[3] = bc
    label = "-".join(parts)
    if p.typefull in (abi.TVDMU, abi.TVDMU1):
        ent = (MHD_ENTROPY if mhd else HD_ENTROPY)[rng.integers(5 if mhd else 4)]
        for il in range(p.nw):
            p.typeentropy[il] = abi.ENTROPY_NAMES[ent]
            p.entropycoef[il] = float(rng.uniform(0.05, 0.4))
        tags.append("ent-" + ent)
    return label + "+" + "+".join(tags or ["plain"]), s, p, steps, grav


NEXTRA = 32


@pytest.mark.parametrize("k", range(NEXTRA), ids=[extras(k)[0] for k in range(NEXTRA)])
def test_c_oracle_matches_numpy_on_random_sources(k):
    _, s, p, steps, grav = extras(k)
    o = Oracle(p, s.x, s.w)
    nv = NumpyVac(p, s.x, s.w)
    if grav is not None:
        o.register_source(abi.SRC_GRAVITY, grav)
        nv.src_id, nv.src_par = abi.SRC_GRAVITY, grav
    o.step(steps)
    nv.step(steps)
    assert o.it == nv.it == steps and o.t == nv.t
    a, b = o.state(), nv.state()
    bad = np.count_nonzero(bits(a) != bits(b))
    assert bad == 0, "%d of %d values differ, max |diff| %g" % (
        bad, a.size, np.abs(a - b).max())
    assert o.nerror() == getattr(nv, "nerror", o.nerror())


def test_source_combinations_cover_every_switch():
    labels = [extras(k)[0] for k in range(NEXTRA)]
    for item in ("stretched", "+eta", "c+", "nodivb", "grav", "smallfix", "useprim",
                 "-periodic-", "-cont-", "-reflect-", "tvdlf-", "tvdmu-", "mhd3d", "hd3d"):
        assert any(item in lab for lab in labels), item
    for ent in MHD_ENTROPY:
        assert any("ent-" + ent in lab for lab in labels), ent

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

"""The FP64 CPU oracle: the C restatement against the independent NumPy
restatement (bit for bit), the committed golden fixtures, and the
reference-independent properties of the scheme (conservation, free-stream
preservation, symmetry)."""
import numpy as np
import pytest

from oracle.oracle import Oracle
from oracle.vac_numpy import NumpyVac
from vac_gb300 import abi, inistate


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


CASES = [
    ("ot-minmod", lambda: inistate.orszag_tang(24), "minmod", "periodic", 8, None),
    ("ot-woodward", lambda: inistate.orszag_tang(20), "woodward", "periodic", 6, None),
    ("rm3-woodward", lambda: inistate.random_modes(10, seed=1), "woodward", "periodic", 3, None),
    ("hd-riemann-cont", lambda: inistate.riemann_2d(24, 3), "minmod", "cont", 8, None),
    ("ot-superbee-cont", lambda: inistate.orszag_tang(16), "superbee", "cont", 4, None),
    ("ot-vanleer-symm", lambda: inistate.orszag_tang(16), "vanleer", "symm", 4, None),
    ("ot-albada", lambda: inistate.orszag_tang(16), "albada", "periodic", 4, None),
    ("ot-unsplit", lambda: inistate.orszag_tang(16), "minmod", "periodic", 4,
     lambda p: (setattr(p, "dimsplit", 0), setattr(p, "typelimited", abi.LIMITED_PREVIOUS))),
    ("rm3-xy", lambda: inistate.random_modes(8, seed=2), "minmod", "periodic", 3,
     lambda p: setattr(p, "typedimsplit", abi.SPLIT_XY)),
    ("ot-tvdlf1", lambda: inistate.orszag_tang(16), "minmod", "periodic", 4,
     lambda p: setattr(p, "typefull", abi.TVDLF1)),
]


def smallfix(**kw):
    """Tweak: smallfix=T with the given smallp/smallrho/vacuumrho."""
    def tweak(p):
        p.smallfix = 1
        for k, v in kw.items():
            setattr(p, k, v)
    return tweak


# keeppositive branches: density floor and pressure repair (HD, MHD),
# vacuum state (HD, MHD 3-D), automatic smallp/smallrho
SMALLFIX_CASES = [
    ("hd-smallfix-floor", lambda: inistate.riemann_2d(24, 3), "minmod", "cont", 6,
     smallfix(smallp=0.3, smallrho=0.3)),
    ("hd-smallfix-vacuum", lambda: inistate.riemann_2d(24, 5), "minmod", "cont", 6,
     smallfix(smallp=0.2, smallrho=0.3, vacuumrho=0.05)),
    ("ot-smallfix", lambda: inistate.orszag_tang(16), "woodward", "periodic", 5,
     smallfix(smallp=1.6)),
    ("rm3-smallfix-vacuum", lambda: inistate.random_modes(8, seed=3), "minmod", "periodic", 3,
     smallfix(smallp=0.049, smallrho=0.9, vacuumrho=0.1)),
    ("hd-smallfix-auto", lambda: inistate.riemann_2d(20, 7), "minmod", "cont", 6,
     smallfix()),
]
def bcs(*per_face):
    """Tweak: typeB per face (x-lo, x-hi, y-lo, y-hi[, z-lo, z-hi]) for all
    variables; a face entry may be a dict {iw: type} over a default."""
    def tweak(p):
        for iB, spec in enumerate(per_face):
            if isinstance(spec, dict):
                dflt = spec.get("*", abi.BC_CONT)
                for iw in range(p.nw):
                    p.typeB[iB][iw] = spec.get(iw, dflt)
            else:
                for iw in range(p.nw):
                    p.typeB[iB][iw] = spec
    return tweak


B = abi
BC_CASES = [
    ("hd-fixed-cont1", lambda: inistate.riemann_2d(20, 8), "minmod", "cont", 6,
     bcs(B.BC_FIXED, B.BC_CONT1, B.BC_CONT1, B.BC_FIXED)),
    ("hd-fixed1-grad1", lambda: inistate.riemann_2d(20, 9), "minmod", "cont", 6,
     bcs(B.BC_FIXED1, B.BC_GRAD1, B.BC_GRAD1, B.BC_FIXED1)),
    ("ot-symm0-walls", lambda: inistate.orszag_tang(16), "woodward", "cont", 5,
     bcs({"*": B.BC_SYMM0, 1: B.BC_ASYMM, 4: B.BC_ASYMM}, {"*": B.BC_SYMM0, 1: B.BC_ASYMM, 4: B.BC_ASYMM},
         B.BC_PERIODIC, B.BC_PERIODIC)),
    ("rm3-mixed-bcs", lambda: inistate.random_modes(8, seed=6), "minmod", "cont", 3,
     bcs(B.BC_GRAD1, B.BC_FIXED, B.BC_SYMM0, B.BC_CONT1, B.BC_PERIODIC, B.BC_PERIODIC)),
]

def resistive(eta, compact=0):
    def tweak(p):
        p.eqpar[1] = eta
        p.compactres = compact
    return tweak


RES_CASES = [
    ("ot-resistive", lambda: inistate.orszag_tang(16), "woodward", "periodic", 5,
     resistive(0.01)),
    ("ot-resistive-compact", lambda: inistate.orszag_tang(16), "minmod", "periodic", 5,
     resistive(0.01, 1)),
    ("rm3-resistive", lambda: inistate.random_modes(8, seed=7), "minmod", "periodic", 3,
     resistive(0.002)),
    ("ot-resistive-dtdiff", lambda: inistate.orszag_tang(16), "minmod", "periodic", 4,
     resistive(1.0)),
]

CASES = CASES + SMALLFIX_CASES + BC_CASES + RES_CASES + [
    # reconstruction in primitive variables (useprimitive=T)
    ("ot-useprimitive", lambda: inistate.orszag_tang(16), "woodward", "periodic", 5,
     lambda p: setattr(p, "useprimitive", 1)),
    ("hd-useprimitive-cont", lambda: inistate.riemann_2d(20, 4), "minmod", "cont", 6,
     lambda p: setattr(p, "useprimitive", 1)),
    ("rm3-useprimitive-smallfix", lambda: inistate.random_modes(8, seed=4), "minmod",
     "periodic", 3, lambda p: (setattr(p, "useprimitive", 1), smallfix(smallp=0.049)(p))),
]


@pytest.mark.parametrize("name,mk,lim,bc,nsteps,tweak", CASES, ids=[c[0] for c in CASES])
def test_c_oracle_matches_numpy_restatement(name, mk, lim, bc, nsteps, tweak):
    s = mk()
    p = inistate.params_for(s, limiter=lim, bc=bc)
    if tweak:
        tweak(p)
    o = Oracle(p, s.x, s.w)
    nv = NumpyVac(p, s.x, s.w)
    o.step(nsteps)
    nv.step(nsteps)
    assert np.array_equal(bits(o.state()), bits(nv.state()))
    assert o.t == nv.t and o.it == nv.it


def test_periodic_conserves_mass_and_energy_without_powell():
    s = inistate.orszag_tang(32)
    p = inistate.params_for(s)
    p.divbfix = 0
    o = Oracle(p, s.x, s.w)
    m0 = o.sums()
    o.step(20)
    m1 = o.sums()
    # addflux is conservative: every sum changes only by round-off
    assert np.all(np.abs(m1 - m0) <= 1e-12 * np.abs(m0).max())


def test_uniform_state_is_preserved():
    s = inistate.orszag_tang(16)
    w = s.w.copy()
    for iw in range(w.shape[0]):
        w[iw] = w[iw].mean()
    p = inistate.params_for(s)
    o = Oracle(p, s.x, w)
    o.step(5)
    out = o.state()
    for iw in range(w.shape[0]):
        assert np.allclose(out[iw], w[iw], rtol=1e-13, atol=1e-13)


def test_itmax_and_tstop_semantics():
    s = inistate.orszag_tang(16)
    p = inistate.params_for(s)
    p.itmax = 5
    o = Oracle(p, s.x, s.w)
    n, fin = o.step(100)
    assert (n, fin, o.it) == (5, True, 5)
    # stopping at a save time and resuming gives the same trajectory
    o1 = Oracle(inistate.params_for(s), s.x, s.w)
    o2 = Oracle(inistate.params_for(s), s.x, s.w)
    o1.step(6)
    n, fin = o2.step(100, tstop=0.3)
    assert not fin and o2.t >= 0.3
    o2.step(6 - n)
    assert np.array_equal(bits(o1.state()), bits(o2.state()))


def test_smallfix_counts_and_floors():
    """keeppositive fires: nerror(toosmallp_) and nerror(toosmallr_) count
    the getboundary calls that found small values; afterwards the mesh
    holds no density below smallrho and no pressure below smallp."""
    s = inistate.riemann_2d(24, 3)
    p = inistate.params_for(s, bc="cont")
    smallfix(smallp=0.3, smallrho=0.3)(p)
    o = Oracle(p, s.x, s.w)
    o.step(3)
    ne = o.nerror()
    assert ne[0] >= 1 and ne[1] >= 1
    w = o.state()
    assert w[0].min() >= 0.3
    gm1 = p.eqpar[0] - 1
    pth = gm1 * (w[3] - 0.5 * (w[1] ** 2 + w[2] ** 2) / w[0])
    assert pth.min() >= 0.3 * (1 - 1e-12)

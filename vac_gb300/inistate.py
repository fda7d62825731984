"""Seeded initial states for the TVDLF workloads, written as VAC snapshots.

VAC builds its initial files with ``vacini`` (src/vacini.t:6-228).  These
generators reproduce its ``domain`` grid semantics (ini_grid with
coord=.false., src/vacini.t:231-290) and its ``conserve`` conversion
(src/vacphys0.t.mhd:5-28, src/vacphys0.t.hd:5-25); the physical states are
the synthetic workloads this engine is measured on:

* ``orszag_tang``    2-D ideal MHD vortex, periodic [0,2pi]^2 (the
                     Orszag-Tang state of Man/inipar.html with gamma=5/3)
* ``random_modes``   3-D (or 2-D) ideal MHD, 8 random Fourier modes each in
                     rho, v and a divergence-free B, low beta, periodic
* ``riemann_2d``     2-D gamma-law HD two-state problem split along a
                     random line (outflow boundaries)
* ``blast_3d``       3-D MHD blast wave in a uniform oblique field
* ``sod_1d``         1-D gamma-law HD shock tube (Sod's states)
"""
import numpy as np

from . import abi
from .vacfile import Snapshot


def domain_grid(nx, xmin, xmax):
    """Cell centres of vacini's 'domain' action: dx=(xmax-xmin)/nx, the
    centres run from xmin+dx/2 to xmax-dx/2 by linear interpolation
    ((ix-ixmin)*xmax'+(ixmax-ix)*xmin')/(ixmax-ixmin)."""
    axes = []
    for n, a, b in zip(nx, xmin, xmax):
        d = (b - a) / n
        hi, lo = b - d / 2, a + d / 2
        ix = np.arange(n, dtype=np.float64)
        axes.append(((ix - 0) * hi + ((n - 1) - ix) * lo) / (n - 1))
    grids = np.meshgrid(*axes, indexing="ij")
    return np.stack(grids)


def conserve_mhd(rho, v, p, b, gamma):
    """conserve, src/vacphys0.t.mhd:5-28."""
    v2 = sum(vc * vc for vc in v)
    b2 = sum(bc * bc for bc in b)
    e = p / (gamma - 1) + 0.5 * (rho * v2 + b2)
    return np.stack([rho] + [rho * vc for vc in v] + [e] + list(b))


def conserve_hd(rho, v, p, gamma):
    """conserve, src/vacphys0.t.hd:5-25."""
    v2 = sum(vc * vc for vc in v)
    e = p / (gamma - 1) + 0.5 * rho * v2
    return np.stack([rho] + [rho * vc for vc in v] + [e])


MHD_NAMES = {2: "rho m1 m2 e b1 b2", 3: "rho m1 m2 m3 e b1 b2 b3"}
HD_NAMES = {1: "rho m1 e", 2: "rho m1 m2 e", 3: "rho m1 m2 m3 e"}


def _snap(x, w, gamma, mhd, ndim, header, ndir=None):
    """A snapshot whose header ends in VAC's physics tag _mhdDC / _hdDC
    (D = ndim, C = ndir)."""
    ndir = ndim if ndir is None else ndir
    names = (MHD_NAMES if mhd else HD_NAMES)[ndir]
    eq = np.array([gamma, 0.0]) if mhd else np.array([gamma])
    return Snapshot(header + ("_mhd%d%d" % (ndim, ndir) if mhd else
                              "_hd%d%d" % (ndim, ndir)),
                    0, 0.0, ndim, eq, names + " gamma" + (" eta" if mhd else ""),
                    x, w, tuple(w.shape[1:]))


def snap_ndir(snap):
    """ndir from the physics tag at the end of the header (ndim if none)."""
    tag = snap.header.rstrip()[-2:]
    if tag.isdigit() and int(tag[0]) == snap.ndim:
        return int(tag[1])
    return snap.ndim


def orszag_tang(n=200, gamma=5.0 / 3.0):
    """rho=gamma^2, p=gamma, v=(-sin y, sin x), B=(-sin y, sin 2x) on the
    periodic [0,2pi]^2 box."""
    x = domain_grid((n, n), (0.0, 0.0), (2 * np.pi, 2 * np.pi))
    X, Y = x
    rho = np.full_like(X, gamma * gamma)
    p = np.full_like(X, gamma)
    w = conserve_mhd(rho, [-np.sin(Y), np.sin(X)], p,
                     [-np.sin(Y), np.sin(2 * X)], gamma)
    return _snap(x, w, gamma, True, 2, "Orszag-Tang vortex")


def _modes(rng, nmodes, ndim, kmax=4):
    ks = []
    while len(ks) < nmodes:
        k = rng.integers(-kmax, kmax + 1, size=3)
        if ndim == 2:
            k[2] = 0
        n2 = int((k * k).sum())
        if 0 < n2 <= kmax * kmax:
            ks.append(k)
    return np.array(ks, dtype=np.float64)


def _phase_fields(x, ks, phis):
    """cos(2 pi k.x + phi) for each mode, built from separable complex
    exponentials."""
    ndim = x.shape[0]
    out = []
    for k, ph in zip(ks, phis):
        z = np.exp(1j * ph)
        for d in range(ndim):
            z = z * np.exp(2j * np.pi * k[d] * x[d])
        out.append(z.real)
    return out


def random_modes(n=256, seed=0, gamma=5.0 / 3.0, ndim=3, nmodes=8,
                 rho_amp=0.2, v_rms=0.3, b_rms=0.1, p0=0.05, ndir=None):
    """rho=1+sum a_k cos(2pi k.x+phi_k) with sum|a_k|=rho_amp; v from random
    vector modes scaled to rms v_rms; B=(1,0,0)+sum a_k (e_k x k)cos(..)
    (divergence free) scaled to rms b_rms; uniform p=p0.  Unit periodic box;
    0<|k|<=4 (k_z=0 in 2-D).  ndir=3 with ndim=2 keeps the z components
    of v and B (2.5-D)."""
    ndir = ndim if ndir is None else ndir
    rng = np.random.default_rng(seed)
    nx = (n,) * ndim
    x = domain_grid(nx, (0.0,) * ndim, (1.0,) * ndim)
    shape = x.shape[1:]
    ks = _modes(rng, nmodes, ndim)
    a = rng.uniform(0.5, 1.0, nmodes)
    a *= rho_amp / a.sum()
    cs = _phase_fields(x, ks, rng.uniform(0, 2 * np.pi, nmodes))
    rho = np.ones(shape)
    for ak, c in zip(a, cs):
        rho += ak * c
    # velocity: random directions per mode
    ks = _modes(rng, nmodes, ndim)
    dirs = rng.normal(size=(nmodes, 3))
    if ndir == 2:
        dirs[:, 2] = 0.0
    cs = _phase_fields(x, ks, rng.uniform(0, 2 * np.pi, nmodes))
    v = [np.zeros(shape) for _ in range(ndir)]
    for dvec, c in zip(dirs, cs):
        for d in range(ndir):
            v[d] += dvec[d] * c
    vr = np.sqrt(np.mean(sum(vc * vc for vc in v)))
    v = [vc * (v_rms / vr) for vc in v]
    # magnetic field: (e x k) cos(2 pi k.x + phi) is divergence free
    ks = _modes(rng, nmodes, ndim)
    es = rng.normal(size=(nmodes, 3))
    cs = _phase_fields(x, ks, rng.uniform(0, 2 * np.pi, nmodes))
    bp = [np.zeros(shape) for _ in range(ndir)]
    for k, e, c in zip(ks, es, cs):
        pol = np.cross(e, k)
        for d in range(ndir):
            bp[d] += pol[d] * c
    br = np.sqrt(np.mean(sum(bc * bc for bc in bp)))
    b = [bc * (b_rms / br) for bc in bp]
    b[0] = b[0] + 1.0
    p = np.full(shape, p0)
    w = conserve_mhd(rho, v, p, b, gamma)
    return _snap(x, w, gamma, True, ndim, "random-mode MHD seed=%d" % seed,
                 ndir=ndir)


def riemann_2d(side, seed, gamma=1.4):
    """Two-state gamma-law problem on [0,1]^2 split by a line through a
    random point at a random angle; each side rho,p~U[0.1,1],
    v = random direction * U[0,0.5]."""
    rng = np.random.default_rng(seed)
    x = domain_grid((side, side), (0.0, 0.0), (1.0, 1.0))
    X, Y = x
    px, py = rng.uniform(0.2, 0.8, 2)
    ang = rng.uniform(0, np.pi)
    left = (X - px) * np.sin(ang) - (Y - py) * np.cos(ang) < 0
    st = []
    for _ in range(2):
        r, p = rng.uniform(0.1, 1.0, 2)
        th = rng.uniform(0, 2 * np.pi)
        sp = rng.uniform(0, 0.5)
        st.append((r, p, sp * np.cos(th), sp * np.sin(th)))
    rho = np.where(left, st[0][0], st[1][0])
    p = np.where(left, st[0][1], st[1][1])
    v = [np.where(left, st[0][2], st[1][2]), np.where(left, st[0][3], st[1][3])]
    w = conserve_hd(rho, v, p, gamma)
    return _snap(x, w, gamma, False, 2, "Riemann 2D seed=%d" % seed)


def blast_3d(n=512, gamma=5.0 / 3.0, r0=0.1, pin=10.0, pout=0.1):
    """rho=1, v=0, B=(1,1,0)/sqrt2, p=pout+(pin-pout)*S(r) with
    S=(1-tanh((r-r0)/dx))/2 on [-0.5,0.5]^3."""
    x = domain_grid((n,) * 3, (-0.5,) * 3, (0.5,) * 3)
    r = np.sqrt(x[0] ** 2 + x[1] ** 2 + x[2] ** 2)
    dxc = 1.0 / n
    S = 0.5 * (1.0 - np.tanh((r - r0) / dxc))
    p = pout + (pin - pout) * S
    rho = np.ones_like(r)
    z = np.zeros_like(r)
    b0 = 1.0 / np.sqrt(2.0)
    w = conserve_mhd(rho, [z, z, z], p, [z + b0, z + b0, z], gamma)
    return _snap(x, w, gamma, True, 3, "MHD blast 3D")


def stretched(snap, amp=0.15):
    """The snapshot's state on a smoothly non-uniform grid: along each axis
    the cell centres move as x -> x + amp L/(2 pi) sin(2 pi (x - x0)/L) over
    the box [x0, x0+L) (monotonic for amp < 1), so that dx, the face widths
    and dvolume vary from cell to cell (gridsetup1 derives them from the
    centres, src/vacgrid.t:457-593)."""
    x = np.array(snap.x, dtype=np.float64, copy=True)
    for d in range(snap.ndim):
        c = x[d]
        n = c.shape[d]
        lo, hi = c.min(), c.max()
        length = (hi - lo) * n / (n - 1)
        x0 = lo - 0.5 * length / n
        x[d] = c + amp * length / (2.0 * np.pi) * np.sin(2.0 * np.pi * (c - x0) / length)
    return Snapshot(snap.header, snap.it, snap.t, snap.ndim, snap.eqpar,
                    snap.varnames, x, snap.w, snap.nx)


def sod_1d(n=100, gamma=1.4):
    """Sod's shock tube on [0,1]: (rho,p)=(1,1) left of x=0.5, (0.125,0.1)
    right, at rest."""
    x = domain_grid((n,), (0.0,), (1.0,))
    left = x[0] < 0.5
    rho = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    w = conserve_hd(rho, [np.zeros_like(rho)], p, gamma)
    return _snap(x, w, gamma, False, 1, "Sod shock tube")


def params_for(snap, limiter="minmod", bc="periodic", precision=abi.PREC_FP64):
    """vacgpu_params for a snapshot with the path's par settings
    (typefull=nw*'tvdlf', twostep, dimsplit xyyx, divbfix, sourceunsplit,
    courantpar=0.8, dtpar=-1)."""
    mhd = "mhd" in snap.header
    ndim = snap.ndim
    nx = snap.w.shape[1:]
    p = abi.default_params(ndim, snap_ndir(snap), abi.PHYS_MHD if mhd else abi.PHYS_HD,
                           list(nx), gamma=float(snap.eqpar[0]))
    abi.set_all_limiters(p, abi.LIMITER_NAMES[limiter])
    abi.set_all_bc(p, abi.BC_NAMES[bc])
    p.precision = precision
    return p


def batch_sides(n=64, seed=0, lo=64, hi=1024):
    """Grid sides drawn log-uniformly in [lo, hi] (seeded)."""
    rng = np.random.default_rng(seed)
    return [int(round(np.exp(v))) for v in rng.uniform(np.log(lo), np.log(hi), n)]


def riemann_batch(n=64, seed=0, lo=64, hi=1024, precision=abi.PREC_MIXED):
    """The batched workload: n two-state gamma=1.4 problems on square grids
    with log-uniform sides, outflow ('cont') boundaries, minmod."""
    grids = []
    for i, side in enumerate(batch_sides(n, seed, lo, hi)):
        s = riemann_2d(side, seed * 1000 + i)
        p = params_for(s, limiter="minmod", bc="cont", precision=precision)
        grids.append((p, s.x, s.w))
    return grids

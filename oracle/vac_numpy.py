"""Second, independent restatement of VAC's explicit TVDLF/Hancock step in
NumPy whole-array form.  TEST INFRASTRUCTURE ONLY.

Each Fortran array statement of the reference becomes one NumPy slice
expression over the same index range, evaluated in the same left-to-right
order (IEEE double elementwise, no contraction), so it must agree bit for bit
with the C restatement in ``vac_oracle.c``; ``tests/test_oracle.py`` checks
that.  Only small grids are meant to run through it.

Arrays carry ghost cells: shape (nw, nG1, nG2, nG3) with nG=nx+4 in a used
dimension and 1 otherwise; the mesh is [2, nG-3].
"""
import numpy as np

from vac_gb300 import abi

HALF, ONE, TWO, ZERO, QUARTER = 0.5, 1.0, 2.0, 0.0, 0.25
SMALLDOUBLE, BIGDOUBLE = 1.0e-99, 1.0e99


def _fmax(a, b):
    """Fortran MAX(a,b) as the select a>b ? a : b (the C oracle's fmax2)."""
    return np.where(a > b, a, b)


def _fmin(a, b):
    return np.where(a < b, a, b)


class Box:
    def __init__(self, lo, hi):
        self.lo, self.hi = list(lo), list(hi)

    def sl(self, d=None, s=0):
        out = []
        for k in range(3):
            a, b = self.lo[k], self.hi[k]
            if k == d:
                a, b = a + s, b + s
            out.append(slice(a, b + 1))
        return tuple(out)

    def shifted(self, d, s):
        b = Box(self.lo, self.hi)
        b.lo[d] += s
        b.hi[d] += s
        return b


class NumpyVac:
    def __init__(self, p, x, w, it=0, t=0.0):
        self.p = p
        self.ndim, self.ndir, self.nw = p.ndim, p.ndir, p.nw
        self.mhd = p.physics == abi.PHYS_MHD
        self.gamma = p.eqpar[0]
        self.e_ = 1 + self.ndir
        self.b0 = self.e_
        self.nG = [p.nx[d] + 4 if d < self.ndim else 1 for d in range(3)]
        self.ixG = Box([0, 0, 0], [n - 1 for n in self.nG])
        self.ixM = Box([2 if d < self.ndim else 0 for d in range(3)],
                       [self.nG[d] - 3 if d < self.ndim else 0 for d in range(3)])
        self.smallp = p.smallp
        self.smallrho = p.smallrho
        self.fixB = {}
        self.initialized = False
        self.nstep = 1 if p.typefull in (abi.TVDLF1, abi.TVDMU1) else 2
        self.courantpar = p.courantpar
        self.dtpar = p.dtpar
        if self.dtpar > 0 and p.slowsteps != 1:
            self.courantpar = -1.0
        self.dtcourant = [BIGDOUBLE] * 3
        self.nerror = [0] * 4
        self.dt = 0.0
        self.dtold = 0.0
        self._grid(np.asarray(x, dtype=np.float64))
        self.w = np.zeros([self.nw] + self.nG)
        self.w[(slice(None),) + self.ixM.sl()] = np.asarray(w).reshape(
            [self.nw] + [p.nx[d] if d < self.ndim else 1 for d in range(3)])
        self.it, self.itmin, self.t = it, it, t
        self.getboundary(self.w)

    # ------------------------------------------------------------- grid
    def _grid(self, xm):
        """gridsetup1, src/vacgrid.t:457-593."""
        nd = self.ndim
        nQ = [self.nG[d] + 2 if d < nd else 1 for d in range(3)]
        q0 = [1 if d < nd else 0 for d in range(3)]
        qx = np.zeros([nd] + nQ)
        msl = tuple(slice(self.ixM.lo[d] + q0[d], self.ixM.hi[d] + q0[d] + 1)
                    for d in range(3))
        qx[(slice(None),) + msl] = xm.reshape([nd] + [self.p.nx[d] if d < nd else 1
                                                      for d in range(3)])
        for idim in range(nd):
            for upper in (True, False):
                if upper:
                    lo, hi = self.ixM.hi[idim] + 1 + q0[idim], nQ[idim] - 1
                    ixe, ixf = lo - 1, lo - 2
                else:
                    lo, hi = 0, self.ixM.lo[idim] - 1 + q0[idim]
                    ixe, ixf = hi + 1, hi + 2
                for jd in range(nd):
                    for ix in range(lo, hi + 1):
                        c = abs(ixe - ix)
                        a = [slice(None)] * 3
                        e = [slice(None)] * 3
                        f = [slice(None)] * 3
                        a[idim], e[idim], f[idim] = ix, ixe, ixf
                        qx[(jd,) + tuple(a)] = ((1 + c) * qx[(jd,) + tuple(e)]
                                                - c * qx[(jd,) + tuple(f)])
        gsl = tuple(slice(q0[d], q0[d] + self.nG[d]) for d in range(3))
        self.dx = np.zeros([3] + self.nG)
        for idim in range(nd):
            j = list(gsl)
            h = list(gsl)
            j[idim] = slice(gsl[idim].start + 1, gsl[idim].stop + 1)
            h[idim] = slice(gsl[idim].start - 1, gsl[idim].stop - 1)
            self.dx[idim] = HALF * (qx[(idim,) + tuple(j)] - qx[(idim,) + tuple(h)])
        dv = self.dx[0].copy()
        for idim in range(1, nd):
            dv = dv * self.dx[idim]
        self.dvolume = dv
        acc = 0.0
        for v in self.dvolume[self.ixM.sl()].ravel(order="F"):
            acc = acc + v
        self.volume = acc

    # ------------------------------------------------------------ physics
    def sq_sum(self, w, i0, sl):
        acc = w[(i0 + 1,) + sl] * w[(i0 + 1,) + sl]
        for c in range(2, self.ndir + 1):
            acc = acc + w[(i0 + c,) + sl] * w[(i0 + c,) + sl]
        return acc

    def getptotal(self, w, b):
        sl = b.sl()
        g = self.gamma
        p = (ONE - HALF * g) * self.sq_sum(w, self.b0, sl)
        p = p + (g - ONE) * w[(self.e_,) + sl]
        p = p - HALF * (g - ONE) * self.sq_sum(w, 0, sl) / w[(0,) + sl]
        return p

    def getpthermal(self, w, b, clipping=True):
        sl = b.sl()
        g = self.gamma
        if self.mhd:
            p = self.sq_sum(w, 0, sl) / w[(0,) + sl]
            for c in range(1, self.ndir + 1):
                bc = w[(self.b0 + c,) + sl]
                p = p + bc * bc
            p = (g - 1) * (w[(self.e_,) + sl] - HALF * p)
        else:
            p = (g - 1) * (w[(self.e_,) + sl] - HALF * self.sq_sum(w, 0, sl) / w[(0,) + sl])
        if self.smallp < ZERO:
            self.smallp = p.min() * self.p.smallpcoeff
            if self.mhd and self.smallp < ZERO:
                self.smallp = p.max() * self.p.smallpcoeff
        if clipping:
            p = np.where(p >= self.smallp, p, self.smallp)
        return p

    def getcmax(self, w, b, idim, cache):
        sl = b.sl()
        rho = w[(0,) + sl]
        m = w[(1 + idim,) + sl]
        if self.mhd:
            if "cs2" not in cache:
                cs2 = self.gamma * self.getpthermal(w, b) / rho
                cache["cs2"] = cs2
                cache["cf2"] = self.sq_sum(w, self.b0, sl) / rho + cs2
            cs2, cf2 = cache["cs2"], cache["cf2"]
            bi = w[(self.b0 + 1 + idim,) + sl]
            return (np.sqrt(HALF * (cf2 + np.sqrt(cf2 * cf2 - 4 * cs2 * (bi * bi) / rho)))
                    + np.abs(m / rho))
        if "cs" not in cache:
            cache["cs"] = np.sqrt(self.gamma * self.getpthermal(w, b) / rho)
        return cache["cs"] + np.abs(m / rho)

    def getflux(self, w, b, iw, idim):
        sl = b.sl()
        rho = w[(0,) + sl]
        nd = self.ndir
        if self.mhd:
            if iw == 0:
                return np.zeros_like(rho), True
            if 1 <= iw <= nd:
                bk = w[(self.b0 + iw,) + sl]
                bi = w[(self.b0 + 1 + idim,) + sl]
                if iw == idim + 1:
                    return self.getptotal(w, b) - bk * bi, True
                return -bk * bi, True
            if iw == self.e_:
                pt = self.getptotal(w, b)
                bm = w[(self.b0 + 1,) + sl] * w[(1,) + sl]
                for c in range(2, nd + 1):
                    bm = bm + w[(self.b0 + c,) + sl] * w[(c,) + sl]
                return (w[(1 + idim,) + sl] * pt - w[(self.b0 + 1 + idim,) + sl] * bm) / rho, True
            k = iw - self.b0
            if k == idim + 1:
                return np.zeros_like(rho), False
            return -w[(k,) + sl] / rho * w[(self.b0 + 1 + idim,) + sl], True
        if iw == 1 + idim:
            return self.getpthermal(w, b), True
        if iw == self.e_:
            return w[(1 + idim,) + sl] / rho * self.getpthermal(w, b), True
        return np.zeros_like(rho), True

    # ------------------------------------------------------------ limiter
    def dwlimiter2(self, dwC, ixC, iw, idim):
        ixO = Box(ixC.lo, ixC.hi)
        ixO.lo[idim] += 1
        a = dwC[ixO.sl()]
        bb = dwC[ixO.sl(idim, -1)]
        s = np.copysign(ONE, a)
        lim = self.p.typelimiter[iw]
        if lim == abi.LIM_MINMOD:
            r = s * np.maximum(ZERO, np.minimum(np.abs(a), s * bb))
        elif lim == abi.LIM_WOODWARD:
            r = 2 * s * np.maximum(ZERO, np.minimum(np.minimum(np.abs(a), s * bb),
                                                    s * 0.25 * (bb + a)))
        elif lim == abi.LIM_SUPERBEE:
            r = s * np.maximum(np.maximum(ZERO, np.minimum(2 * np.abs(a), s * bb)),
                               np.minimum(np.abs(a), 2 * s * bb))
        elif lim == abi.LIM_VANLEER:
            r = 2 * np.maximum(bb * a, 0.0) / (a + bb + 1.0e-12)
        else:
            r = (bb * (a * a + 1.0e-12) + a * (bb * bb + 1.0e-12)) / (a * a + bb * bb + 2.0e-12)
        ldw = np.zeros(self.nG)
        ldw[ixO.sl()] = r
        return ldw

    def primitive(self, b, w):
        """src/vacphys0.t.mhd:31-52, src/vacphys0.t.hd:30-51 (in place)."""
        sl = b.sl()
        w[(self.e_,) + sl] = self.getpthermal(w, b, clipping=True)
        for c in range(1, self.ndir + 1):
            w[(c,) + sl] = w[(c,) + sl] / w[(0,) + sl]

    def conserve(self, b, w):
        """src/vacphys0.t.mhd:5-27, src/vacphys0.t.hd:5-26 (in place)."""
        sl = b.sl()
        g = self.gamma
        rho = w[(0,) + sl]
        vv = self.sq_sum(w, 0, sl)
        if self.mhd:
            w[(self.e_,) + sl] = (w[(self.e_,) + sl] / (g - 1)
                                  + HALF * (rho * vv + self.sq_sum(w, self.b0, sl)))
        else:
            w[(self.e_,) + sl] = w[(self.e_,) + sl] / (g - 1) + HALF * rho * vv
        for c in range(1, self.ndir + 1):
            w[(c,) + sl] = rho * w[(c,) + sl]

    def upwindLR(self, ixL, ixR, idim, w, wLC, wRC):
        """src/vactvdlf.t:302-367; with useprimitive the base w (over
        ixG) and the face states are limited in primitive variables and
        converted back in place."""
        if self.p.useprimitive:
            self.primitive(self.ixG, w)
            self.primitive(ixL, wLC)
            self.primitive(ixR, wRC)
        ixC = Box(ixL.lo, ixR.shifted(idim, 1).hi)
        ixC.lo[idim] = ixL.lo[idim] - 1
        for iw in range(self.nw):
            dwC = np.zeros(self.nG)
            dwC[ixC.sl()] = w[(iw,) + ixC.sl(idim, 1)] - w[(iw,) + ixC.sl()]
            ldw = self.dwlimiter2(dwC, ixC, iw, idim)
            wRC[(iw,) + ixR.sl()] = wRC[(iw,) + ixR.sl()] - HALF * ldw[ixR.sl(idim, 1)]
            wLC[(iw,) + ixL.sl()] = wLC[(iw,) + ixL.sl()] + HALF * ldw[ixL.sl()]
        if self.p.useprimitive:
            self.conserve(self.ixG, w)
            self.conserve(ixL, wLC)
            self.conserve(ixR, wRC)

    # ------------------------------------------------------- grid helpers
    def addflux(self, qdt, ixO, iw, idim, fR, ixR, fL, ixL, wnew):
        """src/vacgrid.t:596-741 (slab); qdt<0 adds a dissipative flux."""
        self.setnoflux(iw, idim, ixO, fR, ixR, fL, ixL)
        if qdt < ZERO:
            wnew[(iw,) + ixO.sl()] = (wnew[(iw,) + ixO.sl()]
                                      + (fR[ixR.sl()] - fL[ixL.sl()])
                                      / self.dvolume[ixO.sl()])
            return
        wnew[(iw,) + ixO.sl()] = (wnew[(iw,) + ixO.sl()]
                                  - qdt / self.dx[(idim,) + ixO.sl()]
                                  * (fR[ixR.sl()] - fL[ixL.sl()]))

    def addsource2(self, qdt, ixO, wCT, wnew):
        sl = ixO.sl()
        if getattr(self, "src_id", 0) == abi.SRC_GRAVITY:
            for iw in range(self.nw):
                if 1 <= iw <= self.ndim:
                    g = self.src_par[iw - 1]
                    if abs(g) > SMALLDOUBLE:
                        wnew[(iw,) + sl] = wnew[(iw,) + sl] + qdt * g * wCT[(0,) + sl]
                elif iw == self.e_:
                    for d in range(1, self.ndim + 1):
                        g = self.src_par[d - 1]
                        if abs(g) > SMALLDOUBLE:
                            wnew[(iw,) + sl] = wnew[(iw,) + sl] + qdt * g * wCT[(d,) + sl]
        if self.mhd and abs(self.p.eqpar[1]) > SMALLDOUBLE:
            if self.p.compactres:
                self.addsource_res1(qdt, ixO, wCT, wnew)
            else:
                self.addsource_res2(qdt, ixO, wCT, wnew)
        if self.mhd and self.p.divbfix:
            divb = np.zeros(self.nG)[sl]
            for idim in range(self.ndim):
                q = wCT[self.b0 + 1 + idim]
                g = HALF * (q[ixO.sl(idim, 1)] - q[ixO.sl(idim, -1)]) / self.dx[(idim,) + sl]
                divb = divb + g
            divb = qdt * divb
            rho = wCT[(0,) + sl]
            for iw in range(self.nw):
                if 1 <= iw <= self.ndir:
                    wnew[(iw,) + sl] = wnew[(iw,) + sl] - wCT[(self.b0 + iw,) + sl] * divb
                elif self.b0 < iw <= self.b0 + self.ndir:
                    wnew[(iw,) + sl] = (wnew[(iw,) + sl]
                                        - wCT[(iw - self.b0,) + sl] / rho * divb)
                elif iw == self.e_:
                    mb = wCT[(1,) + sl] * wCT[(self.b0 + 1,) + sl]
                    for c in range(2, self.ndir + 1):
                        mb = mb + wCT[(c,) + sl] * wCT[(self.b0 + c,) + sl]
                    wnew[(iw,) + sl] = wnew[(iw,) + sl] - mb / rho * divb

    @staticmethod
    def lvc(i, j, k):
        if i == j or j == k or i == k:
            return 0
        return 1 if (i, j, k) in ((1, 2, 3), (2, 3, 1), (3, 1, 2)) else -1

    def grad(self, q, b, idim):
        """slab gradient, src/vacgrid.t:816-823, on box b (full arrays)"""
        out = np.zeros(self.nG)
        out[b.sl()] = HALF * (q[b.sl(idim, 1)] - q[b.sl(idim, -1)]) / self.dx[(idim,) + b.sl()]
        return out

    def getcurrent(self, w, b):
        """src/vacphys.mhdres.t:48-93: J = curl B on b; (idirmin, J)."""
        idirmin0 = 7 - 2 * self.ndir
        idirmin = 4
        cur = {i: np.zeros(self.nG) for i in range(idirmin0, 4)}
        for idir in range(idirmin0, 4):
            for jdir in range(1, self.ndim + 1):
                for kdir in range(1, self.ndir + 1):
                    l = self.lvc(idir, jdir, kdir)
                    if not l:
                        continue
                    g = self.grad(w[self.b0 + kdir], b, jdir - 1)
                    c = cur[idir]
                    c[b.sl()] = c[b.sl()] + g[b.sl()] if l == 1 else c[b.sl()] - g[b.sl()]
                    idirmin = min(idirmin, idir)
        return idirmin, cur

    def addsource_res2(self, qdt, ixO, w, wnew):
        """src/vacphys.mhdres.t:236-315, constant eta"""
        ix = Box(ixO.lo, ixO.hi)
        for d in range(self.ndim):
            ix.lo[d] -= 1
            ix.hi[d] += 1
        idirmin, cur = self.getcurrent(w, ix)
        eta = self.p.eqpar[1]
        sl = ixO.sl()
        for iw in range(self.nw):
            if self.b0 < iw <= self.b0 + self.ndir:
                idir = iw - self.b0
                for jdir in range(1, self.ndim + 1):
                    for kdir in range(idirmin, 4):
                        l = self.lvc(idir, jdir, kdir)
                        if not l:
                            continue
                        tmp = np.zeros(self.nG)
                        tmp[ix.sl()] = cur[kdir][ix.sl()] * eta * qdt
                        g = self.grad(tmp, ixO, jdir - 1)[sl]
                        wnew[(iw,) + sl] = wnew[(iw,) + sl] - g if l == 1 else wnew[(iw,) + sl] + g
            elif iw == self.e_:
                for idir in range(1, self.ndim + 1):
                    for jdir in range(1, self.ndir + 1):
                        for kdir in range(idirmin, 4):
                            l = self.lvc(idir, jdir, kdir)
                            if not l:
                                continue
                            tmp = np.zeros(self.nG)
                            tmp[ix.sl()] = (w[(self.b0 + jdir,) + ix.sl()] * cur[kdir][ix.sl()]
                                            * eta * qdt)
                            g = self.grad(tmp, ixO, idir - 1)[sl]
                            wnew[(iw,) + sl] = (wnew[(iw,) + sl] + g if l == 1
                                                else wnew[(iw,) + sl] - g)

    def addsource_res1(self, qdt, ixO, w, wnew):
        """src/vacphys.mhdres.t:96-233, constant eta"""
        idirmin, cur = self.getcurrent(w, ixO)
        eta = self.p.eqpar[1]
        sl = ixO.sl()
        for idir in range(1, self.ndir + 1):
            q = w[self.b0 + idir]
            tmp = np.zeros(self.nG)[sl]
            for idim in range(self.ndim):
                dx = self.dx[(idim,) + sl]
                tmp = tmp + (q[ixO.sl(idim, 1)] - 2 * q[sl] + q[ixO.sl(idim, -1)]) / (dx * dx)
            tmp = tmp * eta
            for iw in range(self.nw):
                if iw == self.b0 + idir:
                    wnew[(iw,) + sl] = wnew[(iw,) + sl] + qdt * tmp
                elif iw == self.e_:
                    wnew[(iw,) + sl] = wnew[(iw,) + sl] + qdt * tmp * q[sl]
        jj = np.zeros(self.nG)[sl]
        for idir in range(idirmin, 4):
            jj = jj + cur[idir][sl] * cur[idir][sl]
        wnew[(self.e_,) + sl] = wnew[(self.e_,) + sl] + qdt * eta * jj

    def keeppositive(self, w):
        """smallfix: src/vacphys.t.mhd:9-53, src/vacphys.t.hd:176-219,
        src/vacproc.positive.t:2-34 (density floor or vacuum state, then e
        from max(p, smallp) in every mesh cell when any p < max(0, smallp))."""
        sl = self.ixM.sl()
        g = self.gamma
        rho = w[(0,) + sl]
        if self.p.vacuumrho < ZERO:
            if self.smallrho == -ONE:
                self.smallrho = rho.min() * self.p.smallrhocoeff
            if (rho < max(ZERO, self.smallrho)).any():
                self.nerror[1] += 1
                if self.smallrho > ZERO:
                    w[(0,) + sl] = np.where(rho > self.smallrho, rho, self.smallrho)
        else:
            vac = rho < self.smallrho
            for c in range(1, self.ndir + 1):
                w[(c,) + sl][vac] = ZERO
            w[(0,) + sl][vac] = self.p.vacuumrho
            if self.mhd:
                e = self.smallp / (g - ONE) + HALF * self.sq_sum(w, self.b0, sl)
            else:
                e = np.full(rho.shape, self.smallp / (g - ONE))
            w[(self.e_,) + sl][vac] = e[vac]
        p = self.getpthermal(w, self.ixM, clipping=False)
        if (p < max(ZERO, self.smallp)).any():
            self.nerror[0] += 1
            if self.smallp > ZERO:
                a = np.where(p > self.smallp, p, self.smallp) / (g - 1)
                mm = self.sq_sum(w, 0, sl)
                rho = w[(0,) + sl]
                if self.mhd:
                    w[(self.e_,) + sl] = a + HALF * (mm / rho + self.sq_sum(w, self.b0, sl))
                else:
                    w[(self.e_,) + sl] = a + HALF / rho * mm

    def region(self, iB):
        idim, upper = iB // 2, iB % 2
        r = Box(self.ixG.lo, self.ixG.hi)
        if upper:
            r.lo[idim] = self.ixM.hi[idim] + 1
        else:
            r.hi[idim] = self.ixM.lo[idim] - 1
        return r

    def getboundary(self, w):
        """src/vacgrid.t:195-413: regions in iB order over the full extent
        of the other dimensions; fixed/fixed1/grad1 store their ghost
        values (grad1: minus the edge) at the first call."""
        if self.p.smallfix:
            self.keeppositive(w)
        fixed_types = (abi.BC_FIXED, abi.BC_FIXED1, abi.BC_GRAD1)
        for iB in range(2 * self.ndim):
            idim, upper = iB // 2, iB % 2
            r = self.region(iB)
            ixe = r.lo[idim] - 1 if upper else r.hi[idim] + 1
            ixf = ixe - 1 if upper else ixe + 1
            for iw in range(self.nw):
                typ = self.p.typeB[iB][iw]
                if typ == abi.BC_PERIODIC:
                    n = self.nG[idim] - 4
                    w[(iw,) + r.sl()] = w[(iw,) + r.sl(idim, -n if upper else n)]
                    continue
                for k in range(r.lo[idim], r.hi[idim] + 1):
                    row = Box(r.lo, r.hi)
                    row.lo[idim] = row.hi[idim] = k
                    if typ in fixed_types and self.initialized:
                        fb = self.fixB[(iB, iw)][row.sl()]
                        if typ == abi.BC_GRAD1:
                            w[(iw,) + row.sl()] = fb + w[(iw,) + row.sl(idim, ixe - k)]
                        else:
                            w[(iw,) + row.sl()] = fb
                    elif typ in (abi.BC_CONT, abi.BC_FIXED):
                        w[(iw,) + row.sl()] = w[(iw,) + row.sl(idim, ixe - k)]
                    elif typ in (abi.BC_CONT1, abi.BC_FIXED1, abi.BC_GRAD1):
                        dk = abs(k - ixe)
                        w[(iw,) + row.sl()] = ((dk + 1) * w[(iw,) + row.sl(idim, ixe - k)]
                                               - dk * w[(iw,) + row.sl(idim, ixf - k)])
                    else:
                        ixm = (2 * r.lo[idim] - 1 if upper else 2 * r.hi[idim] + 1) - k
                        w[(iw,) + row.sl()] = w[(iw,) + row.sl(idim, ixm - k)]
                if typ == abi.BC_ASYMM:
                    w[(iw,) + r.sl()] = -w[(iw,) + r.sl()]
        if not self.initialized:
            self.initialized = True
            for iB in range(2 * self.ndim):
                idim, upper = iB // 2, iB % 2
                r = self.region(iB)
                ixe = r.lo[idim] - 1 if upper else r.hi[idim] + 1
                for iw in range(self.nw):
                    typ = self.p.typeB[iB][iw]
                    if typ not in fixed_types:
                        continue
                    fb = np.zeros(self.nG)
                    for k in range(r.lo[idim], r.hi[idim] + 1):
                        row = Box(r.lo, r.hi)
                        row.lo[idim] = row.hi[idim] = k
                        if typ == abi.BC_GRAD1:
                            fb[row.sl()] = w[(iw,) + row.sl()] - w[(iw,) + row.sl(idim, ixe - k)]
                        else:
                            fb[row.sl()] = w[(iw,) + row.sl()]
                    self.fixB[(iB, iw)] = fb

    def setnoflux(self, iw, idim, ixO, fR, ixR, fL, ixL):
        """src/vacgrid.t:416-454: zero flux through a 'symm0' face."""
        for upper in (0, 1):
            iB = 2 * idim + upper
            if self.p.typeB[iB][iw] != abi.BC_SYMM0:
                continue
            face = self.region(iB)
            if upper:
                ixe = face.lo[idim] - 1 + ixR.lo[idim] - ixO.lo[idim]
                face.lo[idim] = face.hi[idim] = ixe
                fR[face.sl()] = ZERO
            else:
                ixe = face.hi[idim] + 1 + ixL.lo[idim] - ixO.lo[idim]
                face.lo[idim] = face.hi[idim] = ixe
                fL[face.sl()] = ZERO


    # --------------------------------------------------------- Roe solver
    def roe_dirs(self, idim):
        """idir, jdir of src/vacphys.mhdroe.t:97 (0-based)."""
        nd = self.ndir
        i1 = idim + 1
        d1 = i1 + 1 - nd * (i1 // nd)
        j1 = d1 + 1 - nd * (d1 // nd)
        return d1 - 1, j1 - 1

    def roe_average(self, wL, wR, ixC, idim):
        """Roe state at the faces ixC: src/vacphys.mhdroe.t:4-127 (MHD,
        arithmetic means), src/vacphys.hdroe.t:4-45 (HD, sqrt(rho) weights).
        Returns a dict of face arrays."""
        sl = ixC.sl()
        g, nd, e, b0 = self.gamma, self.ndir, self.e_, self.b0
        rL, rR = wL[(0,) + sl], wR[(0,) + sl]
        R = {}
        if self.mhd:
            rho = HALF * (rL + rR)
            v = {c: HALF * (wL[(c,) + sl] / rL + wR[(c,) + sl] / rR)
                 for c in range(1, nd + 1)}
            B = {c: HALF * (wL[(b0 + c,) + sl] + wR[(b0 + c,) + sl])
                 for c in range(1, nd + 1)}
            pL = self.getpthermal(wL, ixC)
            pR = self.getpthermal(wR, ixC)
            p = HALF * (pL + pR)
            if self.p.useprimitive:
                dp = pR - pL
            else:
                s1 = s2 = s3 = None
                for c in range(1, nd + 1):
                    t1 = v[c] * (wR[(c,) + sl] - wL[(c,) + sl])
                    s1 = t1 if c == 1 else s1 + t1
                    s2 = v[c] * v[c] if c == 1 else s2 + v[c] * v[c]
                    bR, bL = wR[(b0 + c,) + sl], wL[(b0 + c,) + sl]
                    s3 = bR * bR - bL * bL if c == 1 else s3 + bR * bR - bL * bL
                dp = (g - 1) * (wR[(e,) + sl] - wL[(e,) + sl] - s1
                                + HALF * s2 * (rR - rL) - HALF * s3)
            R["rhodv"] = (wR[(1 + idim,) + sl] - wL[(1 + idim,) + sl]
                          - v[1 + idim] * (rR - rL))
            cs2 = g * p / rho
            bb = B[1] * B[1]
            for c in range(2, nd + 1):
                bb = bb + B[c] * B[c]
            cf = bb / rho + cs2
            bi = B[1 + idim]
            cs = _fmax(ZERO, HALF * (cf - np.sqrt(cf * cf - 4.0 * cs2 * (bi * bi) / rho)))
            cf = cf - cs
            af = (cs2 - cs) / (cf - cs)
            af = _fmin(ONE, _fmax(af, ZERO))
            R["as"] = np.sqrt(ONE - af)
            R["af"] = np.sqrt(af)
            R["cf"] = np.sqrt(cf)
            R["cs"] = np.sqrt(cs)
            R["cs2"], R["dp"], R["v"] = cs2, dp, v
            R["sr"] = np.sqrt(rho)
            B[1 + idim] = np.where(np.abs(bi) < SMALLDOUBLE, SMALLDOUBLE, bi)
            idir, jdir = self.roe_dirs(idim)
            if nd == 2:
                B[1 + idir] = np.where(B[1 + idir] >= ZERO, ONE, -ONE)
            else:
                bI, bJ = B[1 + idir], B[1 + jdir]
                t = np.sqrt(bI * bI + bJ * bJ)
                big = t > SMALLDOUBLE
                B[1 + idir] = np.where(big, bI / t, np.sqrt(HALF))
                B[1 + jdir] = np.where(big, bJ / t, np.sqrt(HALF))
            R["B"] = B
        else:
            t = np.sqrt(rL)
            t2 = np.sqrt(rR)
            R["rho"] = t * t2
            t = t / t2
            R["v"] = {c: (wL[(c,) + sl] / rL * t + wR[(c,) + sl] / rR) / (1 + t)
                      for c in range(1, nd + 1)}
            hL = (self.getpthermal(wL, ixC) + wL[(e,) + sl]) / rL
            hR = (self.getpthermal(wR, ixC) + wR[(e,) + sl]) / rR
            R["h"] = (hL * t + hR) / (1 + t)
        return R

    def roe_wave(self, R, wL, wR, ixC, il, idim):
        """Eigenvalue a, jump L(il)*dw and the entropy-fix bound smalla of
        wave il: src/vacphys.mhdroe.t:130-281, src/vacphys.hdroe.t:48-141,
        entropyfix src/vactvd.t:422-451."""
        sl = ixC.sl()
        g, nd, b0 = self.gamma, self.ndir, self.b0
        rL, rR = wL[(0,) + sl], wR[(0,) + sl]
        v = R["v"]
        vi = v[1 + idim]
        te = self.p.typeentropy[il]
        lr = te in (abi.ENTROPY_HARTEN, abi.ENTROPY_POWELL, abi.ENTROPY_RATIO)
        aL = aR = smalla = None
        if self.mhd:
            idir, jdir = self.roe_dirs(idim)
            B, sr = R["B"], R["sr"]
            bi, bI, bJ = B[1 + idim], B[1 + idir], B[1 + jdir]
            dvI = wR[(1 + idir,) + sl] / rR - wL[(1 + idir,) + sl] / rL
            dvJ = wR[(1 + jdir,) + sl] / rR - wL[(1 + jdir,) + sl] / rL
            dbI = wR[(b0 + 1 + idir,) + sl] - wL[(b0 + 1 + idir,) + sl]
            dbJ = wR[(b0 + 1 + jdir,) + sl] - wL[(b0 + 1 + jdir,) + sl]
            cf, cs, af, as_, cs2 = R["cf"], R["cs"], R["af"], R["as"], R["cs2"]
            dp, rhodv = R["dp"], R["rhodv"]
            if il == 0:
                bdv = bI * dvI
                if nd == 3:
                    bdv = bdv + bJ * dvJ
                R["bdv"] = bdv * np.copysign(sr * sr, bi)
                bdb = bI * dbI
                if nd == 3:
                    bdb = bdb + bJ * dbJ
                R["bdb"] = bdb * np.sqrt(cs2) * sr
            if il == 6:
                R["bdv"] = (bJ * dvI - bI * dvJ) * HALF * (sr * sr)
                R["bdb"] = (bJ * dbI - bI * dbJ) * HALF * np.copysign(sr, bi)
            bdv, bdb = R["bdv"], R["bdb"]
            if il == 0:
                a = vi + cf
                jump = HALF / cs2 * (af * (+cf * rhodv + dp) + as_ * (-cs * bdv + bdb))
            elif il == 1:
                a = vi - cf
                jump = HALF / cs2 * (af * (-cf * rhodv + dp) + as_ * (+cs * bdv + bdb))
            elif il == 2:
                a = vi + cs
                jump = HALF / cs2 * (as_ * (+cs * rhodv + dp) + af * (+cf * bdv - bdb))
            elif il == 3:
                a = vi - cs
                jump = HALF / cs2 * (as_ * (-cs * rhodv + dp) + af * (-cf * bdv - bdb))
            elif il == 4:
                a = vi
                jump = rR - rL - dp / cs2
            elif il == 5:
                if self.p.divbwave:
                    a = vi
                    jump = wR[(b0 + 1 + idim,) + sl] - wL[(b0 + 1 + idim,) + sl]
                else:
                    a = np.zeros_like(vi)
                    jump = np.zeros_like(vi)
            elif il == 6:
                a = vi + np.abs(bi) / sr
                jump = +bdv - bdb
            else:
                a = vi - np.abs(bi) / sr
                jump = -bdv - bdb
            if lr:
                aL = wL[(1 + idim,) + sl] / rL
                aR = wR[(1 + idim,) + sl] / rR
                bLi = wL[(b0 + 1 + idim,) + sl]
                bRi = wR[(b0 + 1 + idim,) + sl]
                if il == 0:
                    c2L = g * self.getpthermal(wL, ixC) / rL
                    c2R = g * self.getpthermal(wR, ixC) / rR
                    ccL = c2L + self.sq_sum(wL, b0, sl) / rL
                    ccR = c2R + self.sq_sum(wR, b0, sl) / rR
                    R["ccL"], R["ccR"] = ccL, ccR
                    R["dL"] = np.sqrt(ccL * ccL - 4 * c2L * (bLi * bLi) / rL)
                    R["dR"] = np.sqrt(ccR * ccR - 4 * c2R * (bRi * bRi) / rR)
                if il in (0, 1, 2, 3):
                    sg = ONE if il in (0, 2) else -ONE
                    dsg = ONE if il in (0, 1) else -ONE
                    ccL, ccR, dL, dR = R["ccL"], R["ccR"], R["dL"], R["dR"]
                    qL = np.sqrt(HALF * (ccL + dL)) if dsg > 0 else np.sqrt(HALF * (ccL - dL))
                    qR = np.sqrt(HALF * (ccR + dR)) if dsg > 0 else np.sqrt(HALF * (ccR - dR))
                    aL = aL + qL if sg > 0 else aL - qL
                    aR = aR + qR if sg > 0 else aR - qR
                elif il in (6, 7):
                    if il == 6:
                        R["caL"] = np.abs(bLi) / np.sqrt(rL)
                        R["caR"] = np.abs(bRi) / np.sqrt(rR)
                    aL = aL + R["caL"] if il == 6 else aL - R["caL"]
                    aR = aR + R["caR"] if il == 6 else aR - R["caR"]
        else:
            rho = R["rho"]
            if il == 0:
                vv = v[1] * v[1]
                for c in range(2, nd + 1):
                    vv = vv + v[c] * v[c]
                c2 = (g - 1) * (R["h"] - HALF * vv)
                c2 = _fmax(g * self.smallp / rho, c2)
                pL = self.getpthermal(wL, ixC)
                pR = self.getpthermal(wR, ixC)
                R["dpc"] = (pR - pL) / c2
                R["c"] = np.sqrt(c2)
                R["dvc"] = (wR[(1 + idim,) + sl] / rR - wL[(1 + idim,) + sl] / rL) / R["c"]
            c, dpc, dvc = R["c"], R["dpc"], R["dvc"]
            if il == 0:
                a = vi + c
                jump = HALF * (dpc + rho * dvc)
            elif il == 1:
                a = vi - c
                jump = HALF * (dpc - rho * dvc)
            elif il == 2:
                a = vi
                jump = -dpc + rR - rL
            else:
                idir = il - 3
                if idir >= idim:
                    idir += 1
                a = vi
                jump = rho * (wR[(1 + idir,) + sl] / rR - wL[(1 + idir,) + sl] / rL)
            if te in (abi.ENTROPY_HARTEN, abi.ENTROPY_POWELL):
                uL = wL[(1 + idim,) + sl] / rL
                uR = wR[(1 + idim,) + sl] / rR
                if il in (0, 1):
                    sL = np.sqrt(g * self.getpthermal(wL, ixC) / rL)
                    sR = np.sqrt(g * self.getpthermal(wR, ixC) / rR)
                    aL = uL + sL if il == 0 else uL - sL
                    aR = uR + sR if il == 0 else uR - sR
                else:
                    aL, aR = uL, uR
        if te == abi.ENTROPY_YEE:
            smalla = np.full_like(a, self.p.entropycoef[il])
        elif te == abi.ENTROPY_HARTEN:
            smalla = _fmax(_fmax(ZERO, a - aL), aR - a)
        elif te == abi.ENTROPY_POWELL:
            smalla = _fmax(ZERO, TWO * (aR - aL))
        elif te == abi.ENTROPY_RATIO:
            a = np.where((aL < ZERO) & (aR > ZERO), a - 2 * aR * aL / (aR - aL), a)
        return a, jump, smalla

    def roe_rtimes(self, R, q, iw, il, idim):
        """R(iw,il)*q: src/vacphys.mhdroe.t:284-449, src/vacphys.hdroe.t:144-215."""
        g, nd, e, b0 = self.gamma, self.ndir, self.e_, self.b0
        v = R["v"]
        vi = v[1 + idim]
        z = np.zeros_like(q)
        if self.mhd:
            idir, jdir = self.roe_dirs(idim)
            B, sr = R["B"], R["sr"]
            bi, bI, bJ = B[1 + idim], B[1 + idir], B[1 + jdir]
            cf, cs, af, as_, cs2 = R["cf"], R["cs"], R["af"], R["as"], R["cs2"]
            sgn = np.copysign(ONE, bi)
            if iw == 0:
                return [q * af, q * af, q * as_, q * as_, q, z, z, z][il]
            if iw == e:
                vv = v[1] * v[1]
                for c in range(2, nd + 1):
                    vv = vv + v[c] * v[c]
                v2a2 = HALF * vv + (2 - g) / (g - 1) * cs2
                if il < 6:
                    bv = bI * v[1 + idir]
                    if nd == 3:
                        bv = bv + bJ * v[1 + jdir]
                    bv = bv * sgn
                else:
                    bv = bJ * v[1 + idir] - bI * v[1 + jdir]
                if il == 0:
                    return q * (-as_ * cs * bv + af * (v2a2 + cf * (cf + vi)))
                if il == 1:
                    return q * (+as_ * cs * bv + af * (v2a2 + cf * (cf - vi)))
                if il == 2:
                    return q * (+af * cf * bv + as_ * (v2a2 + cs * (cs + vi)))
                if il == 3:
                    return q * (-af * cf * bv + as_ * (v2a2 + cs * (cs - vi)))
                if il == 4:
                    return q * HALF * vv
                if il == 5:
                    return q * bi if self.p.divbwave else z
                return +q * bv if il == 6 else -q * bv
            if iw <= nd:
                vw = v[iw]
                if iw == 1 + idim:
                    return [q * af * (vw + cf), q * af * (vw - cf), q * as_ * (vw + cs),
                            q * as_ * (vw - cs), q * vw, z, z, z][il]
                bw = B[iw]
                isI = iw == 1 + idir
                if il == 0:
                    return q * (af * vw - as_ * cs * bw * sgn)
                if il == 1:
                    return q * (af * vw + as_ * cs * bw * sgn)
                if il == 2:
                    return q * (as_ * vw + af * cf * bw * sgn)
                if il == 3:
                    return q * (as_ * vw - af * cf * bw * sgn)
                if il == 4:
                    return q * vw
                if il == 5:
                    return z
                if il == 6:
                    return +q * bJ if isI else -q * bI
                return -q * bJ if isI else +q * bI
            k = iw - b0
            if k == 1 + idim:
                return q if (il == 5 and self.p.divbwave) else z
            bw = B[k]
            if il in (0, 1):
                return +q * as_ * np.sqrt(cs2) * bw / sr
            if il in (2, 3):
                return -q * af * np.sqrt(cs2) * bw / sr
            if il in (4, 5):
                return z
            ss = np.copysign(sr, bi)
            if k == 1 + idir:
                return -q * bJ / ss
            return +q * bI / ss
        c, h = R["c"], R["h"]
        shear = il >= 3
        idir = -1
        if shear:
            idir = il - 3
            if idir >= idim:
                idir += 1
        if iw == 0:
            return z if shear else q
        if iw == e:
            if il == 0:
                return q * (h + vi * c)
            if il == 1:
                return q * (h - vi * c)
            if il == 2:
                vv = v[1] * v[1]
                for k in range(2, nd + 1):
                    vv = vv + v[k] * v[k]
                return q * HALF * vv
            return q * v[1 + idir]
        if iw == 1 + idim:
            return [q * (vi + c), q * (vi - c), q * vi][il] if il < 3 else z
        if shear:
            return q if iw == 1 + idir else z
        return q * v[iw]

    def tvdlimit2(self, qdt, ixC, ixO, idim, wL, wR, wnew):
        """src/vactvd.t:86-206 with getphi's TVD-MUSCL branch (:227-243)."""
        sl = ixC.sl()
        hxO = ixO.shifted(idim, -1)
        R = self.roe_average(wL, wR, ixC, idim)
        norm_dx = self.dx[(idim,) + sl] + self.dx[(idim,) + ixC.sl(idim, 1)]
        for il in range(self.nw):
            a, jump, smalla = self.roe_wave(R, wL, wR, ixC, il, idim)
            te = self.p.typeentropy[il]
            a = a * qdt * TWO / norm_dx
            if te in (abi.ENTROPY_HARTEN, abi.ENTROPY_POWELL):
                smalla = smalla * qdt * TWO / norm_dx
            if il in (0, 1) and self.courantpar > ZERO and self.istep == self.nstep:
                cm = np.abs(a).max()
                if cm > ONE:
                    self.nerror[2] += 1
                if cm > SMALLDOUBLE:
                    self.dtcourant[idim] = min(self.dtcourant[idim],
                                               qdt * self.courantpar / cm)
            if te in (abi.ENTROPY_NUL, abi.ENTROPY_RATIO):
                phi = np.abs(a) * jump
            else:
                phi = np.where(np.abs(a) >= smalla, np.abs(a) * jump,
                               HALF * (smalla + a * a / smalla) * jump)
            for iw in range(self.nw):
                F = np.zeros(self.nG)
                F[sl] = self.roe_rtimes(R, phi, iw, il, idim) * QUARTER * (
                    self.dvolume[ixC.sl(idim, 1)] + self.dvolume[sl])
                self.addflux(-ONE, ixO, iw, idim, F, ixO, F, hxO, wnew)

    # ------------------------------------------------------------ schemes
    def hancock(self, qdt, ixO, d0, d1, wCT, wnew):
        for idim in range(d0, d1 + 1):
            hxO = ixO.shifted(idim, -1)
            wLC = np.zeros_like(wCT)
            wRC = np.zeros_like(wCT)
            wRC[(slice(None),) + hxO.sl()] = wCT[(slice(None),) + ixO.sl()]
            wLC[(slice(None),) + ixO.sl()] = wCT[(slice(None),) + ixO.sl()]
            self.upwindLR(ixO, hxO, idim, wCT, wLC, wRC)
            vR = np.zeros(self.nG)
            vL = np.zeros(self.nG)
            vR[hxO.sl()] = wRC[(1 + idim,) + hxO.sl()] / wRC[(0,) + hxO.sl()]
            vL[ixO.sl()] = wLC[(1 + idim,) + ixO.sl()] / wLC[(0,) + ixO.sl()]
            for iw in range(self.nw):
                fR = np.zeros(self.nG)
                fL = np.zeros(self.nG)
                fR[hxO.sl()], tr = self.getflux(wRC, hxO, iw, idim)
                fL[ixO.sl()], tr = self.getflux(wLC, ixO, iw, idim)
                if tr:
                    fR[hxO.sl()] = fR[hxO.sl()] + vR[hxO.sl()] * wRC[(iw,) + hxO.sl()]
                    fL[ixO.sl()] = fL[ixO.sl()] + vL[ixO.sl()] * wLC[(iw,) + ixO.sl()]
                self.addflux(qdt, ixO, iw, idim, fL, ixO, fR, hxO, wnew)
        if self.p.sourceunsplit:
            self.addsource2(qdt * (d1 - d0 + ONE) / self.ndim, ixO, wCT, wnew)

    def tvdmusclf(self, qdt, ixO, d0, d1, wCT, wnew):
        for idim in range(d0, d1 + 1):
            hxO = ixO.shifted(idim, -1)
            ixC = Box(ixO.lo, ixO.hi)
            ixC.lo[idim] = hxO.lo[idim]
            wLC = np.zeros_like(wCT)
            wRC = np.zeros_like(wCT)
            wRC[(slice(None),) + ixC.sl()] = wCT[(slice(None),) + ixC.sl(idim, 1)]
            wLC[(slice(None),) + ixC.sl()] = wCT[(slice(None),) + ixC.sl()]
            tf = self.p.typefull
            lf = tf in (abi.TVDLF, abi.TVDLF1)
            if tf not in (abi.TVDLF1, abi.TVDMU1):
                base = {abi.LIMITED_PREVIOUS: self.wold,
                        abi.LIMITED_PREDICTOR: wCT}.get(self.p.typelimited, wnew)
                self.upwindLR(ixC, ixC, idim, base, wLC, wRC)
            A = (slice(None),) + ixC.sl()
            if lf:
                wLC[A] = HALF * (wLC[A] + wRC[A])
                cmax = np.zeros(self.nG)
                cmax[ixC.sl()] = self.getcmax(wLC, ixC, idim, {})
                if self.courantpar > ZERO and self.istep == self.nstep:
                    q = cmax[ixC.sl()] * TWO / (self.dx[(idim,) + ixC.sl()]
                                                + self.dx[(idim,) + ixC.sl(idim, 1)])
                    cm = q.max()
                    if qdt * cm > ONE:
                        self.nerror[2] += 1
                    if cm > SMALLDOUBLE:
                        self.dtcourant[idim] = min(self.dtcourant[idim], self.courantpar / cm)
                wLC[A] = 2 * wLC[A] - wRC[A]
            vL = wLC[(1 + idim,) + ixC.sl()] / wLC[(0,) + ixC.sl()]
            vR = wRC[(1 + idim,) + ixC.sl()] / wRC[(0,) + ixC.sl()]
            for iw in range(self.nw):
                fL, tr = self.getflux(wLC, ixC, iw, idim)
                fR, tr = self.getflux(wRC, ixC, iw, idim)
                if tr:
                    fL = fL + vL * wLC[(iw,) + ixC.sl()]
                    fR = fR + vR * wRC[(iw,) + ixC.sl()]
                fL = HALF * (fL + fR)
                if lf:
                    fR = -cmax[ixC.sl()] * HALF * (wRC[(iw,) + ixC.sl()] - wLC[(iw,) + ixC.sl()])
                    fL = fL + fR
                F = np.zeros(self.nG)
                F[ixC.sl()] = fL
                self.addflux(qdt, ixO, iw, idim, F, ixO, F, hxO, wnew)
            if not lf:
                with np.errstate(all="ignore"):
                    self.tvdlimit2(qdt, ixC, ixO, idim, wLC, wRC, wnew)
        if self.p.sourceunsplit:
            self.addsource2(qdt * (d1 - d0 + ONE) / self.ndim, ixO, wCT, wnew)

    def advect(self, d0, d1):
        w1 = self.w.copy()
        if self.p.typefull in (abi.TVDLF1, abi.TVDMU1):  # typepred1='nul': onestep
            self.istep = 1
            self.tvdmusclf(self.dt, self.ixM, d0, d1, w1, self.w)
            self.getboundary(self.w)
            return
        self.istep = 1
        self.hancock(self.dt / 2, self.ixM, d0, d1, self.w, w1)
        self.getboundary(w1)
        self.istep = 2
        self.tvdmusclf(self.dt, self.ixM, d0, d1, w1, self.w)
        self.getboundary(self.w)

    def getdt_courant(self):
        self.dt = BIGDOUBLE
        cm = ZERO
        cache = {}
        for idim in range(self.ndim):
            if self.dtcourant[idim] < BIGDOUBLE:
                self.dt = min(self.dt, self.dtcourant[idim])
            else:
                c = self.getcmax(self.w, self.ixM, idim, cache)
                cm = max(cm, (c / self.dx[(idim,) + self.ixM.sl()]).max())
        self.dtcourant = [BIGDOUBLE] * 3
        if cm > SMALLDOUBLE:
            self.dt = min(self.dt, self.courantpar / cm)

    def step(self, nsteps):
        for _ in range(nsteps):
            if self.dtpar > ZERO:
                self.dt = self.dtpar
            else:
                if self.courantpar > ZERO:
                    self.getdt_courant()
                if self.mhd and self.p.eqpar[1] != ZERO:
                    # getdt_res, src/vacphys.mhdres.t:5-45
                    m = min(self.dx[(d,) + self.ixM.sl()].min() for d in range(self.ndim))
                    self.dt = min(self.dt, self.p.dtdiffpar * (m * m) / self.p.eqpar[1])
            p = self.p
            if self.it >= p.itmax or self.t >= p.tmax or self.dt < p.dtmin:
                return True
            if p.tmaxexact:
                self.dt = min(self.dt, p.tmax - self.t + SMALLDOUBLE)
            self.wold = self.w.copy()
            if p.dimsplit:
                order = (range(self.ndim) if (self.it // 2) * 2 == self.it
                         or p.typedimsplit == abi.SPLIT_XY
                         else range(self.ndim - 1, -1, -1))
                for d in order:
                    self.advect(d, d)
            else:
                self.advect(0, self.ndim - 1)
            self.it += 1
            self.t = self.t + self.dt
        return False

    def state(self):
        return self.w[(slice(None),) + self.ixM.sl()].reshape(
            [self.nw] + [self.p.nx[d] for d in range(self.ndim)])

/*
 * vac_oracle.c - CPU FP64 restatement of VAC 4.52's explicit TVDLF/Hancock
 * time step.  TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and
 * the CPU-baseline leg of the benchmark use it as the checker.  Nothing in the
 * product links it.
 *
 * PARITY STATUS: unpinned.  The reference is Fortran 90 and no Fortran
 * compiler exists where this project builds or runs, and the reference ships
 * no golden vectors or fixtures.  This file therefore restates the
 * reference's algorithm statement by statement from its sources (file:line
 * cited at every routine), keeping each Fortran array statement as one loop
 * over the same index range with the same expression shape, so that each
 * element sees the same IEEE operations in the same order.  It is
 * cross-checked bit for bit against an independent NumPy whole-array
 * restatement (oracle/vac_numpy.py) on committed fixtures.
 *
 * Build with -O2 -ffp-contract=off (no FMA contraction), no -ffast-math.
 *
 * Layout: like VAC, w(ixG1,ixG2,ixG3,nw) column-major with ix1 fastest and
 * dixB=2 ghost layers in every used dimension; indices here are 0-based, the
 * mesh is [2, nG-3] in a used dimension.  Unused dimensions have extent 1.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/vacgpu.h"

#define ZERO 0.0
#define ONE 1.0
#define TWO 2.0
#define HALF 0.5
#define SMALLDOUBLE 1.0e-99
#define BIGDOUBLE 1.0e+99

typedef struct {
  int lo[3], hi[3];
} box;

typedef struct vo_state {
  vacgpu_params p;
  int ndim, ndir, nw, mhd;
  int nG[3];
  long N;
  long st[3];
  box ixG, ixM;
  /* variable indices (src/vacpar.t.mhd:9-26, src/vacpar.t.hd:9-26) */
  int rho_, m0_, e_, b0_;
  double *x, *dx, *dvolume;
  double volume;
  double *w, *w1, *wold;
  double *wLC, *wRC, *fLC, *fRC, *vLC, *vRC, *cmaxC, *ldw, *dwC, *tmp,
      *tmp2, *divb, *csound2, *cfast2, *pp;
  double* cur[3];    /* current density components (resistive MHD) */
  double* wroe;      /* Roe average (tvdmu) */
  double* roe[22];   /* tvdlimit2 / Roe solver work arrays (ROE_* below) */
  double dtcourant[3];
  double dt, t, dtold, dtpar, courantpar, dtgrav;
  int it, itmin;
  double smallp;
  double smallrho;   /* keeppositive_rho: -1 until set from min(rho) */
  /* fixed/fixed1/grad1 ghost values (grad1: minus the edge), stored by the
   * first getboundary call (src/vacgrid.t:373-409); full-size arrays per
   * boundary region, only the region's cells used */
  double* fixB[VACGPU_MAXB];
  int initialized;
  int nerror[4];
  int istep, nstep;
  int src_id;
  double src_par[VACGPU_MAXSRCPAR];
  /* specialbound hook: fills variable iw of region iB (box lo..hi) */
  void (*bound_fn)(void* user, double* w, const int* lo, const int* hi,
                   const long* st, long N, const double* x, int iw, int iB,
                   double qt);
  void* bound_user;
  /* specialeta hook (eqpar(eta_) < 0): eta, and gradeta for the compact
   * form, on box lo..hi from w and the current J (components idirmin..3) */
  void (*eta_fn)(void* user, const double* w, const double* const* cur,
                 double* eta, double* const* gradeta, const int* lo,
                 const int* hi, const long* st, long N,
                 const double* const* x, int idirmin, double t);
  void* eta_user;
  /* specialsource hook (src/vacnul.specialsource.t:9-47): w += qdt*S(wCT)
   * on box lo..hi, wCT at time qtC, w at qt; and getdt_special
   * (src/vacnul.specialsource.t:50-71): the user's dt limit from w */
  void (*src_fn)(void* user, double qdt, double qtC, const double* wCT,
                 double qt, double* w, const int* lo, const int* hi,
                 const long* st, long N, const double* const* x);
  double (*dtsp_fn)(void* user, const double* w, const int* lo, const int* hi,
                    const long* st, long N, const double* const* x);
  void* src_user;
  double qtc;         /* qtC of the advect1 call in progress */
  double* eta;        /* eta(ixG^T) of the common block */
  double* gradeta[3];
} vo_state;

/* ------------------------------------------------------------------ boxes */

static long IDX(const vo_state* s, int i1, int i2, int i3) {
  return (long)i1 + s->st[1] * i2 + s->st[2] * i3;
}

/* Elementwise array statement over a box.  Every use is a pure elementwise
 * update (no element reads a value another element of the same statement
 * writes), so the rows may run on several threads without changing a bit. */
#define FORBOX(b, ix)                                            \
  _Pragma("omp parallel for collapse(2) schedule(static)")       \
  for (int i3_ = (b).lo[2]; i3_ <= (b).hi[2]; i3_++)             \
    for (int i2_ = (b).lo[1]; i2_ <= (b).hi[1]; i2_++)           \
      for (long ix = IDX(s, (b).lo[0], i2_, i3_),                \
                ixend_ = IDX(s, (b).hi[0], i2_, i3_);            \
           ix <= ixend_; ix++)

/* Sequential loop over a box (reductions: min/max/sum in column order). */
#define FORBOX_SEQ(b, ix)                                        \
  for (int i3_ = (b).lo[2]; i3_ <= (b).hi[2]; i3_++)             \
    for (int i2_ = (b).lo[1]; i2_ <= (b).hi[1]; i2_++)           \
      for (long ix = IDX(s, (b).lo[0], i2_, i3_),                \
                ixend_ = IDX(s, (b).hi[0], i2_, i3_);            \
           ix <= ixend_; ix++)

static box shift(box b, int idim, int d) {
  b.lo[idim] += d;
  b.hi[idim] += d;
  return b;
}

#define W(a, iw) ((a) + (long)(iw)*s->N)

/* ------------------------------------------------------------ physics MHD */

/* getptotal, src/vacphys0.t.mhd:225-257 (ptot = (1-g/2)B^2+(g-1)e-(g-1)/2
 * m^2/rho), unclipped */
static void getptotal(vo_state* s, const double* w, box b, double* p) {
  const double gamma = s->p.eqpar[0];
  if (s->mhd) {
    FORBOX(b, ix) {
      double bb = 0.0;
      for (int c = 1; c <= s->ndir; c++) {
        double bc = W(w, s->b0_ + c)[ix];
        bb = (c == 1) ? bc * bc : bb + bc * bc;
      }
      p[ix] = (ONE - HALF * gamma) * bb;
    }
    FORBOX(b, ix) { p[ix] = p[ix] + (gamma - ONE) * W(w, s->e_)[ix]; }
    FORBOX(b, ix) {
      double mm = 0.0;
      for (int c = 1; c <= s->ndir; c++) {
        double mc = W(w, s->m0_ + c)[ix];
        mm = (c == 1) ? mc * mc : mm + mc * mc;
      }
      p[ix] = p[ix] - HALF * (gamma - ONE) * mm / W(w, s->rho_)[ix];
    }
  }
}

/* smallp initialisation inside getpthermal (src/vacphys0.t.mhd:202-217,
 * src/vacphys0.t.hd:123-126) */
static void init_smallp(vo_state* s, const double* p, box b) {
  if (s->smallp < ZERO) {
    double mn = BIGDOUBLE, mx = -BIGDOUBLE;
    int first = 1;
    FORBOX_SEQ(b, ix) {
      if (first) { mn = p[ix]; mx = p[ix]; first = 0; }
      if (p[ix] < mn) mn = p[ix];
      if (p[ix] > mx) mx = p[ix];
    }
    s->smallp = mn * s->p.smallpcoeff;
    if (s->mhd && s->smallp < ZERO) s->smallp = mx * s->p.smallpcoeff;
  }
}

/* getpthermal, src/vacphys0.t.mhd:165-222 and src/vacphys0.t.hd:103-134 */
static void getpthermal(vo_state* s, int clipping, const double* w, box b,
                        double* p) {
  const double gamma = s->p.eqpar[0];
  if (s->mhd) {
    FORBOX(b, ix) {
      double mm = 0.0;
      for (int c = 1; c <= s->ndir; c++) {
        double mc = W(w, s->m0_ + c)[ix];
        mm = (c == 1) ? mc * mc : mm + mc * mc;
      }
      p[ix] = mm / W(w, s->rho_)[ix];
    }
    FORBOX(b, ix) {
      double q = p[ix];
      for (int c = 1; c <= s->ndir; c++) {
        double bc = W(w, s->b0_ + c)[ix];
        q = q + bc * bc;
      }
      p[ix] = q;
    }
    FORBOX(b, ix) {
      p[ix] = (gamma - 1) * (W(w, s->e_)[ix] - HALF * p[ix]);
    }
  } else {
    FORBOX(b, ix) {
      double mm = 0.0;
      for (int c = 1; c <= s->ndir; c++) {
        double mc = W(w, s->m0_ + c)[ix];
        mm = (c == 1) ? mc * mc : mm + mc * mc;
      }
      p[ix] = (gamma - 1) *
              (W(w, s->e_)[ix] - HALF * mm / W(w, s->rho_)[ix]);
    }
  }
  init_smallp(s, p, b);
  if (clipping) {
    FORBOX(b, ix) {
      if (!(p[ix] >= s->smallp)) p[ix] = s->smallp;
    }
  }
}

/* getcsound2, src/vacphys0.t.mhd:140-162: csound2 = gamma*p/rho, p clipped */
static void getcsound2(vo_state* s, const double* w, box b, double* cs2) {
  getpthermal(s, 1, w, b, cs2);
  const double gamma = s->p.eqpar[0];
  FORBOX(b, ix) { cs2[ix] = gamma * cs2[ix] / W(w, s->rho_)[ix]; }
}

/* getcmax, src/vacphys0.t.mhd:79-116 (MHD fast speed) and
 * src/vacphys0.t.hd:72-100 (HD sound speed).  new_cmax semantics: the
 * direction independent part is recomputed when *new_cmax is set. */
static void getcmax(vo_state* s, int* new_cmax, const double* w, box b,
                    int idim, double* cmax) {
  const double gamma = s->p.eqpar[0];
  if (s->mhd) {
    if (*new_cmax) {
      *new_cmax = 0;
      getcsound2(s, w, b, s->csound2);
      FORBOX(b, ix) {
        double bb = 0.0;
        for (int c = 1; c <= s->ndir; c++) {
          double bc = W(w, s->b0_ + c)[ix];
          bb = (c == 1) ? bc * bc : bb + bc * bc;
        }
        s->cfast2[ix] = bb / W(w, s->rho_)[ix] + s->csound2[ix];
      }
    }
    const double* bi = W(w, s->b0_ + idim + 1);
    const double* mi = W(w, s->m0_ + idim + 1);
    const double* rho = W(w, s->rho_);
    FORBOX(b, ix) {
      double cf2 = s->cfast2[ix];
      cmax[ix] = sqrt(HALF * (cf2 + sqrt(cf2 * cf2 - 4 * s->csound2[ix] *
                                                          (bi[ix] * bi[ix]) /
                                                          rho[ix]))) +
                 fabs(mi[ix] / rho[ix]);
    }
  } else {
    if (*new_cmax) {
      *new_cmax = 0;
      getpthermal(s, 1, w, b, s->csound2);
      FORBOX(b, ix) {
        s->csound2[ix] = sqrt(gamma * s->csound2[ix] / W(w, s->rho_)[ix]);
      }
    }
    const double* mi = W(w, s->m0_ + idim + 1);
    const double* rho = W(w, s->rho_);
    FORBOX(b, ix) { cmax[ix] = s->csound2[ix] + fabs(mi[ix] / rho[ix]); }
  }
}

/* getv, src/vacphys0.t.mhd:57-75: v = m_idim/rho */
static void getv(vo_state* s, const double* w, box b, int idim, double* v) {
  FORBOX(b, ix) { v[ix] = W(w, s->m0_ + idim + 1)[ix] / W(w, s->rho_)[ix]; }
}

/* getflux, src/vacphys.mhd0.t:149-205 (MHD) and src/vacphys.t.hd:49-75 (HD)
 * Returns the transport flag. */
static int getflux(vo_state* s, const double* w, box b, int iw, int idim,
                   double* f) {
  const double* rho = W(w, s->rho_);
  if (s->mhd) {
    if (iw == s->rho_) {
      FORBOX(b, ix) f[ix] = ZERO;
      return 1;
    }
    if (iw > s->m0_ && iw <= s->m0_ + s->ndir) {
      int k = iw - s->m0_;
      const double* bk = W(w, s->b0_ + k);
      const double* bi = W(w, s->b0_ + idim + 1);
      if (k == idim + 1) {
        getptotal(s, w, b, f);
        FORBOX(b, ix) f[ix] = f[ix] - bk[ix] * bi[ix];
      } else {
        FORBOX(b, ix) f[ix] = -bk[ix] * bi[ix];
      }
      return 1;
    }
    if (iw == s->e_) {
      getptotal(s, w, b, f);
      const double* mi = W(w, s->m0_ + idim + 1);
      const double* bi = W(w, s->b0_ + idim + 1);
      FORBOX(b, ix) {
        double bm = 0.0;
        for (int c = 1; c <= s->ndir; c++) {
          double t = W(w, s->b0_ + c)[ix] * W(w, s->m0_ + c)[ix];
          bm = (c == 1) ? t : bm + t;
        }
        f[ix] = (mi[ix] * f[ix] - bi[ix] * bm) / rho[ix];
      }
      return 1;
    }
    /* b_k */
    int k = iw - s->b0_;
    if (k == idim + 1) {
      FORBOX(b, ix) f[ix] = ZERO;
      return 0;
    }
    const double* mk = W(w, s->m0_ + k);
    const double* bi = W(w, s->b0_ + idim + 1);
    FORBOX(b, ix) f[ix] = -mk[ix] / rho[ix] * bi[ix];
    return 1;
  } else {
    if (iw == s->m0_ + idim + 1) {
      getpthermal(s, 1, w, b, f);
    } else if (iw == s->e_) {
      getpthermal(s, 1, w, b, f);
      const double* mi = W(w, s->m0_ + idim + 1);
      FORBOX(b, ix) f[ix] = mi[ix] / rho[ix] * f[ix];
    } else {
      FORBOX(b, ix) f[ix] = ZERO;
    }
    return 1;
  }
}

/* ---------------------------------------------------------------- limiter */

static double sgn(double a) { return copysign(ONE, a); }
static double fmax2(double a, double b) { return a > b ? a : b; }
static double fmin2(double a, double b) { return a < b ? a : b; }

/* dwlimiter2, src/vacgrid.t:938-996: ldw(ixO) from dwC(ixO), dwC(hxO) with
 * ixO = ixC contracted by one at the low end in idim. */
static void dwlimiter2(vo_state* s, const double* dwC, box ixC, int iw,
                       int idim, double* ldw) {
  box ixO = ixC;
  ixO.lo[idim] += 1;
  long sh = s->st[idim];
  double* tmp = s->tmp;
  FORBOX(ixO, ix) tmp[ix] = sgn(dwC[ix]);
  const double qsmall = 1.0e-12, qsmall2 = 2.0e-12;
  switch (s->p.typelimiter[iw]) {
    case VACGPU_LIM_MINMOD:
      FORBOX(ixO, ix) {
        ldw[ix] = tmp[ix] * fmax2(ZERO, fmin2(fabs(dwC[ix]), tmp[ix] * dwC[ix - sh]));
      }
      break;
    case VACGPU_LIM_WOODWARD:
      FORBOX(ixO, ix) {
        double m = fmin2(fmin2(fabs(dwC[ix]), tmp[ix] * dwC[ix - sh]),
                         tmp[ix] * 0.25 * (dwC[ix - sh] + dwC[ix]));
        ldw[ix] = 2 * tmp[ix] * fmax2(ZERO, m);
      }
      break;
    case VACGPU_LIM_SUPERBEE:
      FORBOX(ixO, ix) {
        double a = fmin2(2 * fabs(dwC[ix]), tmp[ix] * dwC[ix - sh]);
        double c = fmin2(fabs(dwC[ix]), 2 * tmp[ix] * dwC[ix - sh]);
        ldw[ix] = tmp[ix] * fmax2(fmax2(ZERO, a), c);
      }
      break;
    case VACGPU_LIM_VANLEER:
      FORBOX(ixO, ix) {
        ldw[ix] = 2 * fmax2(dwC[ix - sh] * dwC[ix], 0.0) /
                  (dwC[ix] + dwC[ix - sh] + qsmall);
      }
      break;
    case VACGPU_LIM_ALBADA:
      FORBOX(ixO, ix) {
        double a = dwC[ix], b = dwC[ix - sh];
        ldw[ix] = (b * (a * a + qsmall) + a * (b * b + qsmall)) /
                  (a * a + b * b + qsmall2);
      }
      break;
  }
}

/* primitive, src/vacphys0.t.mhd:31-52 and src/vacphys0.t.hd:30-51: the
 * clipped thermal pressure into e_, v = m/rho */
static void primitive(vo_state* s, box b, double* w) {
  getpthermal(s, 1, w, b, s->pp);
  FORBOX(b, ix) W(w, s->e_)[ix] = s->pp[ix];
  for (int c = 1; c <= s->ndir; c++) {
    double* m = W(w, s->m0_ + c);
    FORBOX(b, ix) m[ix] = m[ix] / W(w, s->rho_)[ix];
  }
}

/* conserve, src/vacphys0.t.mhd:5-27 and src/vacphys0.t.hd:5-26 */
static void conserve(vo_state* s, box b, double* w) {
  const double gamma = s->p.eqpar[0];
  FORBOX(b, ix) {
    double vv = 0.0;
    for (int c = 1; c <= s->ndir; c++) {
      double vc = W(w, s->m0_ + c)[ix];
      vv = (c == 1) ? vc * vc : vv + vc * vc;
    }
    const double rho = W(w, s->rho_)[ix];
    double* e = W(w, s->e_);
    if (s->mhd) {
      double bb = 0.0;
      for (int c = 1; c <= s->ndir; c++) {
        double bc = W(w, s->b0_ + c)[ix];
        bb = (c == 1) ? bc * bc : bb + bc * bc;
      }
      e[ix] = e[ix] / (gamma - 1) + HALF * (rho * vv + bb);
    } else {
      e[ix] = e[ix] / (gamma - 1) + HALF * rho * vv;
    }
  }
  for (int c = 1; c <= s->ndir; c++) {
    double* m = W(w, s->m0_ + c);
    FORBOX(b, ix) m[ix] = W(w, s->rho_)[ix] * m[ix];
  }
}

/* upwindLR, src/vactvdlf.t:302-367 (musclomega<=1):
 * wRC(ixR) -= ldw(jxR)/2, wLC(ixL) += ldw(ixL)/2.  With useprimitive the
 * base w (over ixG) and the face states are limited in primitive
 * variables and converted back in place (:325-330,357-362), so w leaves
 * round-tripped. */
static void upwindLR(vo_state* s, box ixL, box ixR, int idim, double* w,
                     double* wLC, double* wRC) {
  if (s->p.useprimitive) {
    primitive(s, s->ixG, w);
    primitive(s, ixL, wLC);
    primitive(s, ixR, wRC);
  }
  box jxR = shift(ixR, idim, 1);
  box ixC = jxR;
  ixC.lo[idim] = ixL.lo[idim] - 1;
  for (int d = 0; d < 3; d++)
    if (d != idim) {
      ixC.lo[d] = ixL.lo[d];
      ixC.hi[d] = jxR.hi[d];
    }
  long sh = s->st[idim];
  for (int iw = 0; iw < s->nw; iw++) {
    const double* wi = W(w, iw);
    FORBOX(ixC, ix) s->dwC[ix] = wi[ix + sh] - wi[ix];
    dwlimiter2(s, s->dwC, ixC, iw, idim, s->ldw);
    double* r = W(wRC, iw);
    double* l = W(wLC, iw);
    FORBOX(ixR, ix) r[ix] = r[ix] - HALF * s->ldw[ix + sh];
    FORBOX(ixL, ix) l[ix] = l[ix] + HALF * s->ldw[ix];
  }
  if (s->p.useprimitive) {
    conserve(s, s->ixG, w);
    conserve(s, ixL, wLC);
    conserve(s, ixR, wRC);
  }
}

/* -------------------------------------------------------------- grid/flux */

static box region(vo_state* s, int iB);
/* setnoflux, src/vacgrid.t:416-454 (called from addflux, :639-640): a
 * variable with 'symm0' at a face of idim has zero flux through that face:
 * fR at the last mesh layer (upper face), fL at the layer before the first
 * (lower face); fR/fL are indexed as addflux's fRC(ixR)/fLC(ixL). */
static void setnoflux(vo_state* s, int iw, int idim, box ixO, double* fR,
                      box ixR, double* fL, box ixL) {
  for (int upper = 0; upper < 2; upper++) {
    const int iB = 2 * idim + upper;
    if (s->p.typeB[iB][iw] != VACGPU_BC_SYMM0) continue;
    box r = region(s, iB);
    box face = r;
    if (upper) {
      /* fRC(ixe) with ixe = ixBmin-1+ixRmin-ixmin */
      const int ixe = r.lo[idim] - 1 + ixR.lo[idim] - ixO.lo[idim];
      face.lo[idim] = face.hi[idim] = ixe;
      FORBOX(face, ix) fR[ix] = ZERO;
    } else {
      const int ixe = r.hi[idim] + 1 + ixL.lo[idim] - ixO.lo[idim];
      face.lo[idim] = face.hi[idim] = ixe;
      FORBOX(face, ix) fL[ix] = ZERO;
    }
  }
}

/* addflux, src/vacgrid.t:596-741, Cartesian slab branch (:669-678), after
 * setnoflux (:639-640):
 * wnew(ix) -= qdt/dx(ix,idim)*(fRC(ixR)-fLC(ixL)); for qdt<0 (dissipative
 * flux, :707-717) wnew(ix) += (fRC(ixR)-fLC(ixL))/dvolume(ix) */
static void addflux(vo_state* s, double qdt, box ixO, int iw, int idim,
                    double* fR, box ixR, double* fL, box ixL, double* wnew) {
  setnoflux(s, iw, idim, ixO, fR, ixR, fL, ixL);
  long oR = IDX(s, ixR.lo[0], ixR.lo[1], ixR.lo[2]) -
            IDX(s, ixO.lo[0], ixO.lo[1], ixO.lo[2]);
  long oL = IDX(s, ixL.lo[0], ixL.lo[1], ixL.lo[2]) -
            IDX(s, ixO.lo[0], ixO.lo[1], ixO.lo[2]);
  double* wn = W(wnew, iw);
  if (qdt < ZERO) {
    const double* dv = s->dvolume;
    FORBOX(ixO, ix) { wn[ix] = wn[ix] + (fR[ix + oR] - fL[ix + oL]) / dv[ix]; }
    return;
  }
  const double* dx = W(s->dx, idim);
  FORBOX(ixO, ix) { wn[ix] = wn[ix] - qdt / dx[ix] * (fR[ix + oR] - fL[ix + oL]); }
}

/* gradient, src/vacgrid.t:775-837, slab branch (:816-823) */
static void gradient(vo_state* s, const double* q, box ixO, int idir,
                     double* gradq) {
  long sh = s->st[idir];
  const double* dx = W(s->dx, idir);
  FORBOX(ixO, ix) gradq[ix] = HALF * (q[ix + sh] - q[ix - sh]) / dx[ix];
}

/* getdivb, src/vacphys.mhd0.t:106-146 (second order) */
static void getdivb(vo_state* s, const double* w, box ixO, double* divb) {
  FORBOX(ixO, ix) divb[ix] = ZERO;
  for (int idim = 0; idim < s->ndim; idim++) {
    gradient(s, W(w, s->b0_ + idim + 1), ixO, idim, s->tmp2);
    FORBOX(ixO, ix) divb[ix] = divb[ix] + s->tmp2[ix];
  }
}

/* addsource_divb, src/vacphys.mhd0.t:246-280 (Powell source) */
static void addsource_divb(vo_state* s, double qdt, box ixO, const double* w,
                           double* wnew) {
  double* divb = s->divb;
  getdivb(s, w, ixO, divb);
  FORBOX(ixO, ix) divb[ix] = qdt * divb[ix];
  const double* rho = W(w, s->rho_);
  for (int iw = 0; iw < s->nw; iw++) {
    double* wn = W(wnew, iw);
    if (iw > s->m0_ && iw <= s->m0_ + s->ndir) {
      const double* bk = W(w, s->b0_ + (iw - s->m0_));
      FORBOX(ixO, ix) wn[ix] = wn[ix] - bk[ix] * divb[ix];
    } else if (iw > s->b0_ && iw <= s->b0_ + s->ndir) {
      const double* mk = W(w, s->m0_ + (iw - s->b0_));
      FORBOX(ixO, ix) wn[ix] = wn[ix] - mk[ix] / rho[ix] * divb[ix];
    } else if (iw == s->e_) {
      FORBOX(ixO, ix) {
        double mb = 0.0;
        for (int c = 1; c <= s->ndir; c++) {
          double t = W(w, s->m0_ + c)[ix] * W(w, s->b0_ + c)[ix];
          mb = (c == 1) ? t : mb + t;
        }
        wn[ix] = wn[ix] - mb / rho[ix] * divb[ix];
      }
    }
  }
}

/* addsource_grav, vacusr.gravity.t:24-75 (uniform gravity as specialsource) */
static void addsource_grav(vo_state* s, double qdt, box ixO, const double* w,
                           double* wnew) {
  for (int iw = 0; iw < s->nw; iw++) {
    if (iw > s->m0_ && iw <= s->m0_ + s->ndim) {
      int idim = iw - s->m0_;
      double g = s->src_par[idim - 1];
      if (fabs(g) > SMALLDOUBLE) {
        double* wn = W(wnew, iw);
        const double* rho = W(w, s->rho_);
        FORBOX(ixO, ix) wn[ix] = wn[ix] + qdt * g * rho[ix];
      }
    } else if (iw == s->e_) {
      for (int idim = 1; idim <= s->ndim; idim++) {
        double g = s->src_par[idim - 1];
        if (fabs(g) > SMALLDOUBLE) {
          double* wn = W(wnew, iw);
          const double* m = W(w, s->m0_ + idim);
          FORBOX(ixO, ix) wn[ix] = wn[ix] + qdt * g * m[ix];
        }
      }
    }
  }
}

/* Levi-Civita symbol lvc(i,j,k), 1-based indices */
static int lvc(int i, int j, int k) {
  if (i == j || j == k || i == k) return 0;
  return ((i == 1 && j == 2) || (i == 2 && j == 3) || (i == 3 && j == 1)) ? 1 : -1;
}

/* getcurrent, src/vacphys.mhdres.t:48-93: J_i = eps_ijk d_j B_k on ix with
 * the slab gradient; components idirmin0=7-2*ndir..3; returns idirmin */
static int getcurrent(vo_state* s, const double* w, box ix) {
  const int idirmin0 = 7 - 2 * s->ndir;
  int idirmin = 4;
  for (int idir = idirmin0; idir <= 3; idir++) FORBOX(ix, i) s->cur[idir - 1][i] = ZERO;
  for (int idir = idirmin0; idir <= 3; idir++)
    for (int jdir = 1; jdir <= s->ndim; jdir++)
      for (int kdir = 1; kdir <= s->ndir; kdir++) {
        const int l = lvc(idir, jdir, kdir);
        if (!l) continue;
        gradient(s, W(w, s->b0_ + kdir), ix, jdir - 1, s->tmp2);
        double* c = s->cur[idir - 1];
        if (l == 1)
          FORBOX(ix, i) c[i] = c[i] + s->tmp2[i];
        else
          FORBOX(ix, i) c[i] = c[i] - s->tmp2[i];
        if (idir < idirmin) idirmin = idir;
      }
  return idirmin;
}

/* specialeta (src/vacphys.mhdres.t:26-30,127-129,271-273): the user's
 * eta(ix) -- and gradeta for the compact form -- on box ix from w and the
 * current of getcurrent, at the time-loop t */
static void special_eta(vo_state* s, const double* w, box ix, int idirmin) {
  if (!s->eta_fn) return;
  const double* cur[3] = {s->cur[0], s->cur[1], s->cur[2]};
  const double* x[3] = {W(s->x, 0), W(s->x, s->ndim > 1 ? 1 : 0),
                        W(s->x, s->ndim > 2 ? 2 : 0)};
  double* g[3] = {s->gradeta[0], s->gradeta[1], s->gradeta[2]};
  s->eta_fn(s->eta_user, w, cur, s->eta, g, ix.lo, ix.hi, s->st, s->N, x,
            idirmin, s->t);
}

/* addsource_res2, src/vacphys.mhdres.t:236-315 (curl form, compactres=F):
 * B_i -= eps_ijk d_j (eta J_k) qdt, e += eps_ijk d_i (B_j eta J_k qdt);
 * eta = eqpar(eta_) > 0 or the specialeta field */
static void addsource_res2(vo_state* s, double qdt, box ixO, const double* w,
                           double* wnew) {
  box ix = ixO;
  for (int d = 0; d < s->ndim; d++) {
    ix.lo[d]--;
    ix.hi[d]++;
  }
  const int idirmin = getcurrent(s, w, ix);
  const double eta = s->p.eqpar[1];
  const int field = eta < ZERO;
  if (field) special_eta(s, w, ix, idirmin);
  const double* ef = s->eta;
  for (int iw = 0; iw < s->nw; iw++) {
    double* wn = W(wnew, iw);
    if (iw > s->b0_ && iw <= s->b0_ + s->ndir) {
      const int idir = iw - s->b0_;
      for (int jdir = 1; jdir <= s->ndim; jdir++)
        for (int kdir = idirmin; kdir <= 3; kdir++) {
          const int l = lvc(idir, jdir, kdir);
          if (!l) continue;
          const double* c = s->cur[kdir - 1];
          if (field)
            FORBOX(ix, i) s->tmp[i] = c[i] * ef[i] * qdt;
          else
            FORBOX(ix, i) s->tmp[i] = c[i] * eta * qdt;
          gradient(s, s->tmp, ixO, jdir - 1, s->tmp2);
          if (l == 1)
            FORBOX(ixO, i) wn[i] = wn[i] - s->tmp2[i];
          else
            FORBOX(ixO, i) wn[i] = wn[i] + s->tmp2[i];
        }
    } else if (iw == s->e_) {
      for (int idir = 1; idir <= s->ndim; idir++)
        for (int jdir = 1; jdir <= s->ndir; jdir++)
          for (int kdir = idirmin; kdir <= 3; kdir++) {
            const int l = lvc(idir, jdir, kdir);
            if (!l) continue;
            const double* c = s->cur[kdir - 1];
            const double* bj = W(w, s->b0_ + jdir);
            if (field)
              FORBOX(ix, i) s->tmp[i] = bj[i] * c[i] * ef[i] * qdt;
            else
              FORBOX(ix, i) s->tmp[i] = bj[i] * c[i] * eta * qdt;
            gradient(s, s->tmp, ixO, idir - 1, s->tmp2);
            if (l == 1)
              FORBOX(ixO, i) wn[i] = wn[i] + s->tmp2[i];
            else
              FORBOX(ixO, i) wn[i] = wn[i] - s->tmp2[i];
          }
    }
  }
}

/* addsource_res1, src/vacphys.mhdres.t:96-233 (compact form, compactres=T):
 * B_i += qdt (eta lap(B_i) - [grad(eta) x J]_i), e += the same times B_i for
 * each i, then e += qdt eta J^2 (the gradeta terms for the specialeta
 * field only) */
static void addsource_res1(vo_state* s, double qdt, box ixO, const double* w,
                           double* wnew) {
  const int idirmin = getcurrent(s, w, ixO);
  const double eta = s->p.eqpar[1];
  const int field = eta < ZERO;
  if (field) special_eta(s, w, ixO, idirmin);
  const double* ef = s->eta;
  double* tmp = s->tmp;
  for (int idir = 1; idir <= s->ndir; idir++) {
    FORBOX(ixO, i) tmp[i] = ZERO;
    const double* q = W(w, s->b0_ + idir);
    for (int idim = 0; idim < s->ndim; idim++) {
      const long sh = s->st[idim];
      const double* dx = W(s->dx, idim);
      FORBOX(ixO, i) tmp[i] = tmp[i] + (q[i + sh] - 2 * q[i] + q[i - sh]) / (dx[i] * dx[i]);
    }
    if (field) {
      FORBOX(ixO, i) tmp[i] = tmp[i] * ef[i];
      for (int jdir = 1; jdir <= s->ndim; jdir++)
        for (int kdir = idirmin; kdir <= 3; kdir++) {
          const int l = lvc(idir, jdir, kdir);
          if (!l) continue;
          const double* ge = s->gradeta[jdir - 1];
          const double* c = s->cur[kdir - 1];
          if (l == 1)
            FORBOX(ixO, i) tmp[i] = tmp[i] - ge[i] * c[i];
          else
            FORBOX(ixO, i) tmp[i] = tmp[i] + ge[i] * c[i];
        }
    } else {
      FORBOX(ixO, i) tmp[i] = tmp[i] * eta;
    }
    for (int iw = 0; iw < s->nw; iw++) {
      double* wn = W(wnew, iw);
      if (iw == s->b0_ + idir)
        FORBOX(ixO, i) wn[i] = wn[i] + qdt * tmp[i];
      else if (iw == s->e_)
        FORBOX(ixO, i) wn[i] = wn[i] + qdt * tmp[i] * q[i];
    }
  }
  double* e = W(wnew, s->e_);
  FORBOX(ixO, i) {
    double jj = ZERO;
    for (int idir = idirmin; idir <= 3; idir++) jj = jj + s->cur[idir - 1][i] * s->cur[idir - 1][i];
    e[i] = e[i] + qdt * (field ? ef[i] : eta) * jj;
  }
}

/* addsource2, src/vac.t:575-605: specialsource then addsource (resistive
 * terms, src/vacphys.mhd0.t:223-230, then Powell) */
static void addsource2(vo_state* s, double qdt, box ixO, const double* wCT,
                       double* w) {
  if (s->src_fn) {
    const double* x[3] = {W(s->x, 0), W(s->x, s->ndim > 1 ? 1 : 0),
                          W(s->x, s->ndim > 2 ? 2 : 0)};
    s->src_fn(s->src_user, qdt, s->qtc, wCT, s->t, w, ixO.lo, ixO.hi, s->st, s->N, x);
  } else if (s->src_id == VACGPU_SRC_GRAVITY) {
    addsource_grav(s, qdt, ixO, wCT, w);
  }
  if (s->mhd && fabs(s->p.eqpar[1]) > SMALLDOUBLE) {
    if (s->p.compactres)
      addsource_res1(s, qdt, ixO, wCT, w);
    else
      addsource_res2(s, qdt, ixO, wCT, w);
  }
  if (s->mhd && s->p.divbfix) addsource_divb(s, qdt, ixO, wCT, w);
}

/* keeppositive (smallfix=T), src/vacphys.t.mhd:9-53 and src/vacphys.t.hd:
 * 176-219, with keeppositive_rho, src/vacproc.positive.t:2-34: on the mesh,
 * density floor (or vacuum state), then, if any unclipped pressure is below
 * max(0,smallp), e recomputed from max(p,smallp) in every mesh cell.
 * nerror(toosmallp_=1), nerror(toosmallr_=2) count calls that found any. */
static void keeppositive(vo_state* s, double* w) {
  const box b = s->ixM;
  const double gamma = s->p.eqpar[0];
  double* rho = W(w, s->rho_);
  double* e = W(w, s->e_);
  if (s->p.vacuumrho < ZERO) {
    if (s->smallrho == -ONE) {
      double mn = ZERO;
      int first = 1;
      FORBOX_SEQ(b, ix) {
        if (first || rho[ix] < mn) mn = rho[ix];
        first = 0;
      }
      s->smallrho = mn * s->p.smallrhocoeff;
    }
    const double lim = fmax2(ZERO, s->smallrho);
    int toosmallr = 0;
    FORBOX_SEQ(b, ix) {
      if (rho[ix] < lim) toosmallr = 1;
    }
    if (toosmallr) {
      s->nerror[1]++;
      if (s->smallrho > ZERO) FORBOX(b, ix) { rho[ix] = fmax2(rho[ix], s->smallrho); }
    }
  } else {
    FORBOX(b, ix) {
      if (rho[ix] < s->smallrho) {
        for (int c = 1; c <= s->ndir; c++) W(w, s->m0_ + c)[ix] = ZERO;
        rho[ix] = s->p.vacuumrho;
        if (s->mhd) {
          double bb = 0.0;
          for (int c = 1; c <= s->ndir; c++) {
            double bc = W(w, s->b0_ + c)[ix];
            bb = (c == 1) ? bc * bc : bb + bc * bc;
          }
          e[ix] = s->smallp / (gamma - ONE) + HALF * bb;
        } else {
          e[ix] = s->smallp / (gamma - ONE);
        }
      }
    }
  }
  getpthermal(s, 0, w, b, s->tmp);
  const double plim = fmax2(ZERO, s->smallp);
  int toosmallp = 0;
  FORBOX_SEQ(b, ix) {
    if (s->tmp[ix] < plim) toosmallp = 1;
  }
  if (toosmallp) {
    s->nerror[0]++;
    if (s->smallp > ZERO) {
      FORBOX(b, ix) {
        double mm = 0.0;
        for (int c = 1; c <= s->ndir; c++) {
          double mc = W(w, s->m0_ + c)[ix];
          mm = (c == 1) ? mc * mc : mm + mc * mc;
        }
        const double a = fmax2(s->tmp[ix], s->smallp) / (gamma - 1);
        if (s->mhd) {
          double bb = 0.0;
          for (int c = 1; c <= s->ndir; c++) {
            double bc = W(w, s->b0_ + c)[ix];
            bb = (c == 1) ? bc * bc : bb + bc * bc;
          }
          e[ix] = a + HALF * (mm / rho[ix] + bb);
        } else {
          e[ix] = a + HALF / rho[ix] * mm;
        }
      }
    }
  }
}

/* ghost region iB (boundsetup defaults, src/vacgrid.t:53-69): the two
 * ghost layers of idim over the full ghost box in the other dimensions */
static box region(vo_state* s, int iB) {
  const int idim = iB / 2, upper = iB % 2;
  box r = s->ixG;
  if (upper) {
    r.lo[idim] = s->ixM.hi[idim] + 1;
    r.hi[idim] = s->ixG.hi[idim];
  } else {
    r.lo[idim] = s->ixG.lo[idim];
    r.hi[idim] = s->ixM.lo[idim] - 1;
  }
  return r;
}

/* getboundary, src/vacgrid.t:195-413 with the default regions of boundsetup
 * (src/vacgrid.t:53-69) and periodic pairing (:121-135); keeppositive first
 * when smallfix (:213).  Regions are filled in iB order, each over the full
 * extent of the other dimensions; a region's 'special' variables go to the
 * specialbound hook after its other variables (:355-371), with the fill's
 * time qt. */
static void getboundary(vo_state* s, double* w, double qt) {
  if (s->p.smallfix) keeppositive(s, w);
  for (int iB = 0; iB < 2 * s->ndim; iB++) {
    const int idim = iB / 2, upper = iB % 2;
    const box r = region(s, iB);
    long sh = s->st[idim];
    /* edge (ixe) and inner edge (ixf) mesh layers */
    const int ixe = upper ? r.lo[idim] - 1 : r.hi[idim] + 1;
    const int ixf = upper ? ixe - 1 : ixe + 1;
    for (int iw = 0; iw < s->nw; iw++) {
      double* a = W(w, iw);
      int type = s->p.typeB[iB][iw];
      const int fixedtype = type == VACGPU_BC_FIXED || type == VACGPU_BC_FIXED1 ||
                            type == VACGPU_BC_GRAD1;
      if (type == VACGPU_BC_SPECIAL) {
        continue;
      } else if (fixedtype && s->initialized) {
        /* restore the stored values, grad1 on top of the current edge */
        const double* fb = W(s->fixB[iB], iw);
        for (int k = r.lo[idim]; k <= r.hi[idim]; k++) {
          box row = r;
          row.lo[idim] = row.hi[idim] = k;
          long off = (long)(ixe - k) * sh;
          if (type == VACGPU_BC_GRAD1)
            FORBOX(row, ix) a[ix] = fb[ix] + a[ix + off];
          else
            FORBOX(row, ix) a[ix] = fb[ix];
        }
      } else if (type == VACGPU_BC_CONT || type == VACGPU_BC_FIXED) {
        for (int k = r.lo[idim]; k <= r.hi[idim]; k++) {
          box row = r;
          row.lo[idim] = row.hi[idim] = k;
          long off = (long)(ixe - k) * sh;
          FORBOX(row, ix) a[ix] = a[ix + off];
        }
      } else if (type == VACGPU_BC_CONT1 || type == VACGPU_BC_FIXED1 ||
                 type == VACGPU_BC_GRAD1) {
        /* first order extrapolation, (|ix-ixe|+1)*w(ixe)-|ix-ixe|*w(ixf) */
        for (int k = r.lo[idim]; k <= r.hi[idim]; k++) {
          box row = r;
          row.lo[idim] = row.hi[idim] = k;
          const int dk = abs(k - ixe);
          long oe = (long)(ixe - k) * sh, of = (long)(ixf - k) * sh;
          FORBOX(row, ix) a[ix] = (dk + 1) * a[ix + oe] - dk * a[ix + of];
        }
      } else if (type == VACGPU_BC_PERIODIC) {
        long off = (long)(upper ? -(s->nG[idim] - 4) : (s->nG[idim] - 4)) * sh;
        FORBOX(r, ix) a[ix] = a[ix + off];
      } else {
        /* symm, symm0, asymm */
        int ixm = upper ? 2 * r.lo[idim] - 1 : 2 * r.hi[idim] + 1;
        for (int k = r.lo[idim]; k <= r.hi[idim]; k++) {
          box row = r;
          row.lo[idim] = row.hi[idim] = k;
          long off = (long)((ixm - k) - k) * sh;
          FORBOX(row, ix) a[ix] = a[ix + off];
        }
        if (type == VACGPU_BC_ASYMM) FORBOX(r, ix) a[ix] = -a[ix];
      }
    }
    for (int iw = 0; iw < s->nw; iw++)
      if (s->p.typeB[iB][iw] == VACGPU_BC_SPECIAL && s->bound_fn)
        s->bound_fn(s->bound_user, w, r.lo, r.hi, s->st, s->N,
                    W(s->x, idim), iw, iB, qt);
  }
  if (!s->initialized) {
    /* fixed boundaries store their values, grad1 its differences */
    s->initialized = 1;
    for (int iB = 0; iB < 2 * s->ndim; iB++) {
      const int idim = iB / 2, upper = iB % 2;
      const box r = region(s, iB);
      long sh = s->st[idim];
      const int ixe = upper ? r.lo[idim] - 1 : r.hi[idim] + 1;
      for (int iw = 0; iw < s->nw; iw++) {
        int type = s->p.typeB[iB][iw];
        if (type != VACGPU_BC_FIXED && type != VACGPU_BC_FIXED1 && type != VACGPU_BC_GRAD1)
          continue;
        if (!s->fixB[iB]) s->fixB[iB] = calloc(s->N * s->nw, sizeof(double));
        double* fb = W(s->fixB[iB], iw);
        const double* a = W(w, iw);
        for (int k = r.lo[idim]; k <= r.hi[idim]; k++) {
          box row = r;
          row.lo[idim] = row.hi[idim] = k;
          long off = (long)(ixe - k) * sh;
          if (type == VACGPU_BC_GRAD1)
            FORBOX(row, ix) fb[ix] = a[ix] - a[ix + off];
          else
            FORBOX(row, ix) fb[ix] = a[ix];
        }
      }
    }
  }
}


/* ------------------------------------------------------------ Roe solver */
/* Work arrays of tvdlimit2 and the Roe solvers (allocated for tvdmu). */
enum {
  ROE_CF, ROE_CS, ROE_AF, ROE_AS, ROE_CS2, ROE_DP, ROE_RHODV, ROE_BDV,
  ROE_BDB, ROE_AL, ROE_AR, ROE_CS2L, ROE_CS2R, ROE_CC2L, ROE_CC2R, ROE_A,
  ROE_SMALLA, ROE_JUMP, ROE_PHI, ROE_RPHI, ROE_T1, ROE_T2, NROE
};
#define QUARTER 0.25

/* Fortran SIGN(a,b): |a| with the sign of b */
static double fsign(double a, double b) { return copysign(fabs(a), b); }

/* idir, jdir of the MHD Roe solver (idir=idim+1-ndir*(idim/ndir), 1-based,
 * src/vacphys.mhdroe.t:97,145-146), returned 0-based */
static void roe_dirs(const vo_state* s, int idim, int* idir, int* jdir) {
  const int nd = s->ndir;
  const int i1 = idim + 1;
  const int d1 = i1 + 1 - nd * (i1 / nd);
  const int j1 = d1 + 1 - nd * (d1 / nd);
  *idir = d1 - 1;
  *jdir = j1 - 1;
}

/* average, src/vacphys.mhdroe.t:4-127: arithmetic means of rho, v, B, p;
 * dp, rho*dv_idim, the sound, fast and slow speeds and their weights; then
 * rho -> sqrt(rho), B_idir,B_jdir -> beta_idir,beta_jdir. */
static void average_mhd(vo_state* s, const double* wL, const double* wR,
                        box b, int idim, double* wroe) {
  double** R = s->roe;
  const double gamma = s->p.eqpar[0];
  const int nd = s->ndir;
  const double *rL = W(wL, s->rho_), *rR = W(wR, s->rho_);
  double* rr = W(wroe, s->rho_);
  FORBOX(b, ix) rr[ix] = HALF * (rL[ix] + rR[ix]);
  for (int c = 1; c <= nd; c++) {
    const double *mL = W(wL, s->m0_ + c), *mR = W(wR, s->m0_ + c);
    const double *bL = W(wL, s->b0_ + c), *bR = W(wR, s->b0_ + c);
    double *vr = W(wroe, s->m0_ + c), *br = W(wroe, s->b0_ + c);
    FORBOX(b, ix) vr[ix] = HALF * (mL[ix] / rL[ix] + mR[ix] / rR[ix]);
    FORBOX(b, ix) br[ix] = HALF * (bL[ix] + bR[ix]);
  }
  double *pL = R[ROE_AF], *pR = R[ROE_AS];
  getpthermal(s, 1, wL, b, pL);
  getpthermal(s, 1, wR, b, pR);
  double* pr = W(wroe, s->e_);
  FORBOX(b, ix) pr[ix] = HALF * (pL[ix] + pR[ix]);
  double* dp = R[ROE_DP];
  if (s->p.useprimitive) {
    FORBOX(b, ix) dp[ix] = pR[ix] - pL[ix];
  } else {
    const double *eL = W(wL, s->e_), *eR = W(wR, s->e_);
    FORBOX(b, ix) {
      double s1 = 0.0, s2 = 0.0, s3 = 0.0;
      for (int c = 1; c <= nd; c++) {
        const double v = W(wroe, s->m0_ + c)[ix];
        const double dm = W(wR, s->m0_ + c)[ix] - W(wL, s->m0_ + c)[ix];
        const double bR = W(wR, s->b0_ + c)[ix], bL = W(wL, s->b0_ + c)[ix];
        s1 = (c == 1) ? v * dm : s1 + v * dm;
        s2 = (c == 1) ? v * v : s2 + v * v;
        s3 = (c == 1) ? bR * bR - bL * bL : s3 + bR * bR - bL * bL;
      }
      dp[ix] = (gamma - 1) * (eR[ix] - eL[ix] - s1 +
                              HALF * s2 * (rR[ix] - rL[ix]) - HALF * s3);
    }
  }
  {
    const double *mL = W(wL, s->m0_ + idim + 1), *mR = W(wR, s->m0_ + idim + 1);
    const double* vr = W(wroe, s->m0_ + idim + 1);
    double* rhodv = R[ROE_RHODV];
    FORBOX(b, ix) rhodv[ix] = mR[ix] - mL[ix] - vr[ix] * (rR[ix] - rL[ix]);
  }
  double *cs2 = R[ROE_CS2], *cf = R[ROE_CF], *cs = R[ROE_CS];
  double *af = R[ROE_AF], *as = R[ROE_AS];
  FORBOX(b, ix) cs2[ix] = gamma * pr[ix] / rr[ix];
  FORBOX(b, ix) {
    double bb = 0.0;
    for (int c = 1; c <= nd; c++) {
      const double bc = W(wroe, s->b0_ + c)[ix];
      bb = (c == 1) ? bc * bc : bb + bc * bc;
    }
    cf[ix] = bb / rr[ix] + cs2[ix];
  }
  const double* bi = W(wroe, s->b0_ + idim + 1);
  FORBOX(b, ix) {
    cs[ix] = fmax2(ZERO, HALF * (cf[ix] - sqrt(cf[ix] * cf[ix] -
                                               4.0 * cs2[ix] *
                                                   (bi[ix] * bi[ix]) /
                                                   rr[ix])));
  }
  FORBOX(b, ix) cf[ix] = cf[ix] - cs[ix];
  FORBOX(b, ix) af[ix] = (cs2[ix] - cs[ix]) / (cf[ix] - cs[ix]);
  FORBOX(b, ix) af[ix] = fmin2(ONE, fmax2(af[ix], ZERO));
  FORBOX(b, ix) as[ix] = sqrt(ONE - af[ix]);
  FORBOX(b, ix) af[ix] = sqrt(af[ix]);
  FORBOX(b, ix) cf[ix] = sqrt(cf[ix]);
  FORBOX(b, ix) cs[ix] = sqrt(cs[ix]);
  FORBOX(b, ix) rr[ix] = sqrt(rr[ix]);
  double* bw = W(wroe, s->b0_ + idim + 1);
  FORBOX(b, ix) if (fabs(bw[ix]) < SMALLDOUBLE) bw[ix] = SMALLDOUBLE;
  int idir, jdir;
  roe_dirs(s, idim, &idir, &jdir);
  double* bI = W(wroe, s->b0_ + idir + 1);
  if (nd == 2) {
    FORBOX(b, ix) bI[ix] = bI[ix] >= ZERO ? ONE : -ONE;
  } else {
    double* bJ = W(wroe, s->b0_ + jdir + 1);
    double* t = R[ROE_T1];
    FORBOX(b, ix) t[ix] = sqrt(bI[ix] * bI[ix] + bJ[ix] * bJ[ix]);
    FORBOX(b, ix) {
      if (t[ix] > SMALLDOUBLE) {
        bI[ix] = bI[ix] / t[ix];
        bJ[ix] = bJ[ix] / t[ix];
      } else {
        bI[ix] = sqrt(HALF);
        bJ[ix] = sqrt(HALF);
      }
    }
  }
}

/* average, src/vacphys.hdroe.t:4-45: sqrt(rho) weighted Roe average;
 * rho -> sqrt(rhoL*rhoR), m -> v, e -> enthalpy h. */
static void average_hd(vo_state* s, const double* wL, const double* wR, box b,
                       double* wroe) {
  double** R = s->roe;
  double *t = R[ROE_T1], *t2 = R[ROE_T2];
  const double *rL = W(wL, s->rho_), *rR = W(wR, s->rho_);
  double* rr = W(wroe, s->rho_);
  FORBOX(b, ix) t[ix] = sqrt(rL[ix]);
  FORBOX(b, ix) t2[ix] = sqrt(rR[ix]);
  FORBOX(b, ix) rr[ix] = t[ix] * t2[ix];
  FORBOX(b, ix) t[ix] = t[ix] / t2[ix];
  for (int c = 1; c <= s->ndir; c++) {
    const double *mL = W(wL, s->m0_ + c), *mR = W(wR, s->m0_ + c);
    double* vr = W(wroe, s->m0_ + c);
    FORBOX(b, ix) vr[ix] = (mL[ix] / rL[ix] * t[ix] + mR[ix] / rR[ix]) / (1 + t[ix]);
  }
  double* h = W(wroe, s->e_);
  getpthermal(s, 1, wL, b, t2);
  FORBOX(b, ix) h[ix] = (t2[ix] + W(wL, s->e_)[ix]) / rL[ix];
  getpthermal(s, 1, wR, b, t2);
  FORBOX(b, ix) t2[ix] = (t2[ix] + W(wR, s->e_)[ix]) / rR[ix];
  FORBOX(b, ix) h[ix] = (h[ix] * t[ix] + t2[ix]) / (1 + t[ix]);
}

/* entropyfix, src/vactvd.t:422-451 */
static void entropyfix(vo_state* s, box b, int il, const double* aL,
                       const double* aR, double* a, double* smalla) {
  switch (s->p.typeentropy[il]) {
    case VACGPU_ENTROPY_HARTEN:
      FORBOX(b, ix) smalla[ix] = fmax2(fmax2(ZERO, a[ix] - aL[ix]), aR[ix] - a[ix]);
      break;
    case VACGPU_ENTROPY_POWELL:
      FORBOX(b, ix) smalla[ix] = fmax2(ZERO, TWO * (aR[ix] - aL[ix]));
      break;
    case VACGPU_ENTROPY_RATIO:
      FORBOX(b, ix) {
        if (aL[ix] < ZERO && aR[ix] > ZERO)
          a[ix] = a[ix] - 2 * aR[ix] * aL[ix] / (aR[ix] - aL[ix]);
      }
      break;
    default:
      break;
  }
}

/* geteigenjump, src/vacphys.mhdroe.t:130-281: eigenvalue a, jump L*dw and
 * the entropy-fix bound of wave il (0-based: fastRW, fastLW, slowRW, slowLW,
 * entroW, diverW, alfvRW, alfvLW). */
static void geteigenjump_mhd(vo_state* s, const double* wL, const double* wR,
                             const double* wroe, box b, int il, int idim) {
  double** R = s->roe;
  const int nd = s->ndir;
  int idir, jdir;
  roe_dirs(s, idim, &idir, &jdir);
  const double *rL = W(wL, s->rho_), *rR = W(wR, s->rho_);
  const double* sr = W(wroe, s->rho_);
  const double* bi = W(wroe, s->b0_ + idim + 1);
  const double* bI = W(wroe, s->b0_ + idir + 1);
  const double* bJ = W(wroe, s->b0_ + jdir + 1);
  const double *mLI = W(wL, s->m0_ + idir + 1), *mRI = W(wR, s->m0_ + idir + 1);
  const double *mLJ = W(wL, s->m0_ + jdir + 1), *mRJ = W(wR, s->m0_ + jdir + 1);
  const double *bLI = W(wL, s->b0_ + idir + 1), *bRI = W(wR, s->b0_ + idir + 1);
  const double *bLJ = W(wL, s->b0_ + jdir + 1), *bRJ = W(wR, s->b0_ + jdir + 1);
  double *bdv = R[ROE_BDV], *bdb = R[ROE_BDB];
  const double *cf = R[ROE_CF], *cs = R[ROE_CS], *af = R[ROE_AF],
               *as = R[ROE_AS], *cs2 = R[ROE_CS2], *dp = R[ROE_DP],
               *rhodv = R[ROE_RHODV];
  if (il == 0) {
    FORBOX(b, ix) bdv[ix] = bI[ix] * (mRI[ix] / rR[ix] - mLI[ix] / rL[ix]);
    if (nd == 3)
      FORBOX(b, ix) bdv[ix] = bdv[ix] + bJ[ix] * (mRJ[ix] / rR[ix] - mLJ[ix] / rL[ix]);
    FORBOX(b, ix) bdv[ix] = bdv[ix] * fsign(sr[ix] * sr[ix], bi[ix]);
    FORBOX(b, ix) bdb[ix] = bI[ix] * (bRI[ix] - bLI[ix]);
    if (nd == 3) FORBOX(b, ix) bdb[ix] = bdb[ix] + bJ[ix] * (bRJ[ix] - bLJ[ix]);
    FORBOX(b, ix) bdb[ix] = bdb[ix] * sqrt(cs2[ix]) * sr[ix];
  }
  if (il == 6) {
    FORBOX(b, ix) {
      bdv[ix] = bJ[ix] * (mRI[ix] / rR[ix] - mLI[ix] / rL[ix]) -
                bI[ix] * (mRJ[ix] / rR[ix] - mLJ[ix] / rL[ix]);
    }
    FORBOX(b, ix) bdb[ix] = bJ[ix] * (bRI[ix] - bLI[ix]) - bI[ix] * (bRJ[ix] - bLJ[ix]);
    FORBOX(b, ix) bdv[ix] = bdv[ix] * HALF * (sr[ix] * sr[ix]);
    FORBOX(b, ix) bdb[ix] = bdb[ix] * HALF * fsign(sr[ix], bi[ix]);
  }
  const double* v = W(wroe, s->m0_ + idim + 1);
  double *a = R[ROE_A], *jump = R[ROE_JUMP];
  switch (il) {
    case 0:
      FORBOX(b, ix) a[ix] = v[ix] + cf[ix];
      FORBOX(b, ix) {
        jump[ix] = HALF / cs2[ix] *
                   (af[ix] * (+cf[ix] * rhodv[ix] + dp[ix]) +
                    as[ix] * (-cs[ix] * bdv[ix] + bdb[ix]));
      }
      break;
    case 1:
      FORBOX(b, ix) a[ix] = v[ix] - cf[ix];
      FORBOX(b, ix) {
        jump[ix] = HALF / cs2[ix] *
                   (af[ix] * (-cf[ix] * rhodv[ix] + dp[ix]) +
                    as[ix] * (+cs[ix] * bdv[ix] + bdb[ix]));
      }
      break;
    case 2:
      FORBOX(b, ix) a[ix] = v[ix] + cs[ix];
      FORBOX(b, ix) {
        jump[ix] = HALF / cs2[ix] *
                   (as[ix] * (+cs[ix] * rhodv[ix] + dp[ix]) +
                    af[ix] * (+cf[ix] * bdv[ix] - bdb[ix]));
      }
      break;
    case 3:
      FORBOX(b, ix) a[ix] = v[ix] - cs[ix];
      FORBOX(b, ix) {
        jump[ix] = HALF / cs2[ix] *
                   (as[ix] * (-cs[ix] * rhodv[ix] + dp[ix]) +
                    af[ix] * (-cf[ix] * bdv[ix] - bdb[ix]));
      }
      break;
    case 4:
      FORBOX(b, ix) a[ix] = v[ix];
      FORBOX(b, ix) jump[ix] = rR[ix] - rL[ix] - dp[ix] / cs2[ix];
      break;
    case 5:
      if (s->p.divbwave) {
        const double *bLi = W(wL, s->b0_ + idim + 1), *bRi = W(wR, s->b0_ + idim + 1);
        FORBOX(b, ix) a[ix] = v[ix];
        FORBOX(b, ix) jump[ix] = bRi[ix] - bLi[ix];
      } else {
        FORBOX(b, ix) a[ix] = ZERO;
        FORBOX(b, ix) jump[ix] = ZERO;
      }
      break;
    case 6:
      FORBOX(b, ix) a[ix] = v[ix] + fabs(bi[ix]) / sr[ix];
      FORBOX(b, ix) jump[ix] = +bdv[ix] - bdb[ix];
      break;
    case 7:
      FORBOX(b, ix) a[ix] = v[ix] - fabs(bi[ix]) / sr[ix];
      FORBOX(b, ix) jump[ix] = -bdv[ix] - bdb[ix];
      break;
  }
  const int te = s->p.typeentropy[il];
  double *aL = R[ROE_AL], *aR = R[ROE_AR], *smalla = R[ROE_SMALLA];
  if (te == VACGPU_ENTROPY_YEE) {
    const double c = s->p.entropycoef[il];
    FORBOX(b, ix) smalla[ix] = c;
  } else if (te == VACGPU_ENTROPY_HARTEN || te == VACGPU_ENTROPY_POWELL ||
             te == VACGPU_ENTROPY_RATIO) {
    const double *mLi = W(wL, s->m0_ + idim + 1), *mRi = W(wR, s->m0_ + idim + 1);
    const double *bLi = W(wL, s->b0_ + idim + 1), *bRi = W(wR, s->b0_ + idim + 1);
    double *cs2L = R[ROE_CS2L], *cs2R = R[ROE_CS2R];
    double *ccL = R[ROE_CC2L], *ccR = R[ROE_CC2R];
    FORBOX(b, ix) aL[ix] = mLi[ix] / rL[ix];
    FORBOX(b, ix) aR[ix] = mRi[ix] / rR[ix];
    switch (il) {
      case 0:
        getcsound2(s, wL, b, cs2L);
        getcsound2(s, wR, b, cs2R);
        FORBOX(b, ix) {
          double bb = 0.0;
          for (int c = 1; c <= nd; c++) {
            const double bc = W(wL, s->b0_ + c)[ix];
            bb = (c == 1) ? bc * bc : bb + bc * bc;
          }
          ccL[ix] = cs2L[ix] + bb / rL[ix];
        }
        FORBOX(b, ix) {
          double bb = 0.0;
          for (int c = 1; c <= nd; c++) {
            const double bc = W(wR, s->b0_ + c)[ix];
            bb = (c == 1) ? bc * bc : bb + bc * bc;
          }
          ccR[ix] = cs2R[ix] + bb / rR[ix];
        }
        FORBOX(b, ix) {
          cs2L[ix] = sqrt(ccL[ix] * ccL[ix] -
                          4 * cs2L[ix] * (bLi[ix] * bLi[ix]) / rL[ix]);
        }
        FORBOX(b, ix) {
          cs2R[ix] = sqrt(ccR[ix] * ccR[ix] -
                          4 * cs2R[ix] * (bRi[ix] * bRi[ix]) / rR[ix]);
        }
        FORBOX(b, ix) aL[ix] = aL[ix] + sqrt(HALF * (ccL[ix] + cs2L[ix]));
        FORBOX(b, ix) aR[ix] = aR[ix] + sqrt(HALF * (ccR[ix] + cs2R[ix]));
        break;
      case 1:
        FORBOX(b, ix) aL[ix] = aL[ix] - sqrt(HALF * (ccL[ix] + cs2L[ix]));
        FORBOX(b, ix) aR[ix] = aR[ix] - sqrt(HALF * (ccR[ix] + cs2R[ix]));
        break;
      case 2:
        FORBOX(b, ix) aL[ix] = aL[ix] + sqrt(HALF * (ccL[ix] - cs2L[ix]));
        FORBOX(b, ix) aR[ix] = aR[ix] + sqrt(HALF * (ccR[ix] - cs2R[ix]));
        break;
      case 3:
        FORBOX(b, ix) aL[ix] = aL[ix] - sqrt(HALF * (ccL[ix] - cs2L[ix]));
        FORBOX(b, ix) aR[ix] = aR[ix] - sqrt(HALF * (ccR[ix] - cs2R[ix]));
        break;
      case 6:
        FORBOX(b, ix) ccL[ix] = fabs(bLi[ix]) / sqrt(rL[ix]);
        FORBOX(b, ix) ccR[ix] = fabs(bRi[ix]) / sqrt(rR[ix]);
        FORBOX(b, ix) aL[ix] = aL[ix] + ccL[ix];
        FORBOX(b, ix) aR[ix] = aR[ix] + ccR[ix];
        break;
      case 7:
        FORBOX(b, ix) aL[ix] = aL[ix] - ccL[ix];
        FORBOX(b, ix) aR[ix] = aR[ix] - ccR[ix];
        break;
      default:
        break;
    }
  }
  entropyfix(s, b, il, aL, aR, a, smalla);
}

/* geteigenjump, src/vacphys.hdroe.t:48-141 (0-based il: soundRW, soundLW,
 * entropW, then the shear waves) */
static void geteigenjump_hd(vo_state* s, const double* wL, const double* wR,
                            const double* wroe, box b, int il, int idim) {
  double** R = s->roe;
  const double gamma = s->p.eqpar[0];
  const double *rL = W(wL, s->rho_), *rR = W(wR, s->rho_);
  const double* rr = W(wroe, s->rho_);
  const double* v = W(wroe, s->m0_ + idim + 1);
  const double *mLi = W(wL, s->m0_ + idim + 1), *mRi = W(wR, s->m0_ + idim + 1);
  double *c = R[ROE_CS], *dpc = R[ROE_DP], *dvc = R[ROE_RHODV];
  double *t = R[ROE_T1], *t2 = R[ROE_T2];
  if (il == 0) {
    const double* h = W(wroe, s->e_);
    FORBOX(b, ix) {
      double vv = 0.0;
      for (int k = 1; k <= s->ndir; k++) {
        const double vk = W(wroe, s->m0_ + k)[ix];
        vv = (k == 1) ? vk * vk : vv + vk * vk;
      }
      c[ix] = (gamma - 1) * (h[ix] - HALF * vv);
    }
    FORBOX(b, ix) c[ix] = fmax2(gamma * s->smallp / rr[ix], c[ix]);
    getpthermal(s, 1, wL, b, t);
    getpthermal(s, 1, wR, b, t2);
    FORBOX(b, ix) dpc[ix] = (t2[ix] - t[ix]) / c[ix];
    FORBOX(b, ix) c[ix] = sqrt(c[ix]);
    FORBOX(b, ix) dvc[ix] = (mRi[ix] / rR[ix] - mLi[ix] / rL[ix]) / c[ix];
  }
  double *a = R[ROE_A], *jump = R[ROE_JUMP];
  int idir = -1;
  switch (il) {
    case 0:
      FORBOX(b, ix) a[ix] = v[ix] + c[ix];
      FORBOX(b, ix) jump[ix] = HALF * (dpc[ix] + rr[ix] * dvc[ix]);
      break;
    case 1:
      FORBOX(b, ix) a[ix] = v[ix] - c[ix];
      FORBOX(b, ix) jump[ix] = HALF * (dpc[ix] - rr[ix] * dvc[ix]);
      break;
    case 2:
      FORBOX(b, ix) a[ix] = v[ix];
      FORBOX(b, ix) jump[ix] = -dpc[ix] + rR[ix] - rL[ix];
      break;
    default: {
      idir = il - 3;                /* 0-based il-shearW0_-1 */
      if (idir >= idim) idir++;
      const double *mLd = W(wL, s->m0_ + idir + 1), *mRd = W(wR, s->m0_ + idir + 1);
      FORBOX(b, ix) a[ix] = v[ix];
      FORBOX(b, ix) jump[ix] = rr[ix] * (mRd[ix] / rR[ix] - mLd[ix] / rL[ix]);
    }
  }
  const int te = s->p.typeentropy[il];
  double *aL = R[ROE_AL], *aR = R[ROE_AR], *smalla = R[ROE_SMALLA];
  if (te == VACGPU_ENTROPY_YEE) {
    const double cy = s->p.entropycoef[il];
    FORBOX(b, ix) smalla[ix] = cy;
  } else if (te == VACGPU_ENTROPY_HARTEN || te == VACGPU_ENTROPY_POWELL) {
    if (il == 0 || il == 1) {
      const double sg = il == 0 ? ONE : -ONE;
      getpthermal(s, 1, wL, b, aL);
      FORBOX(b, ix) aL[ix] = mLi[ix] / rL[ix] + sg * sqrt(gamma * aL[ix] / rL[ix]);
      getpthermal(s, 1, wR, b, aR);
      FORBOX(b, ix) aR[ix] = mRi[ix] / rR[ix] + sg * sqrt(gamma * aR[ix] / rR[ix]);
    } else {
      FORBOX(b, ix) aL[ix] = mLi[ix] / rL[ix];
      FORBOX(b, ix) aR[ix] = mRi[ix] / rR[ix];
    }
  }
  entropyfix(s, b, il, aL, aR, a, smalla);
}

/* rtimes, src/vacphys.mhdroe.t:284-449: rq = R(iw,il)*q at the Roe state */
static void rtimes_mhd(vo_state* s, const double* q, const double* wroe,
                       box b, int iw, int il, int idim, double* rq) {
  double** R = s->roe;
  const double gamma = s->p.eqpar[0];
  const int nd = s->ndir;
  int idir, jdir;
  roe_dirs(s, idim, &idir, &jdir);
  const double *cf = R[ROE_CF], *cs = R[ROE_CS], *af = R[ROE_AF],
               *as = R[ROE_AS], *cs2 = R[ROE_CS2];
  const double* sr = W(wroe, s->rho_);
  const double* bi = W(wroe, s->b0_ + idim + 1);
  const double* bI = W(wroe, s->b0_ + idir + 1);
  const double* bJ = W(wroe, s->b0_ + jdir + 1);
  const double* v = W(wroe, s->m0_ + idim + 1);
  const double* vI = W(wroe, s->m0_ + idir + 1);
  const double* vJ = W(wroe, s->m0_ + jdir + 1);
  if (iw == s->rho_) {
    switch (il) {
      case 0: case 1: FORBOX(b, ix) rq[ix] = q[ix] * af[ix]; break;
      case 2: case 3: FORBOX(b, ix) rq[ix] = q[ix] * as[ix]; break;
      case 4: FORBOX(b, ix) rq[ix] = q[ix]; break;
      default: FORBOX(b, ix) rq[ix] = ZERO; break;
    }
  } else if (iw == s->e_) {
    FORBOX(b, ix) {
      double vv = 0.0;
      for (int c = 1; c <= nd; c++) {
        const double vc = W(wroe, s->m0_ + c)[ix];
        vv = (c == 1) ? vc * vc : vv + vc * vc;
      }
      /* v2a2 and bv of the fast/slow waves (:310-327), bv of the Alfven
       * waves (:328-332) */
      const double v2a2 = HALF * vv + (2 - gamma) / (gamma - 1) * cs2[ix];
      double bv;
      if (il < 6) {
        bv = bI[ix] * vI[ix];
        if (nd == 3) bv = bv + bJ[ix] * vJ[ix];
        bv = bv * fsign(ONE, bi[ix]);
      } else {
        bv = bJ[ix] * vI[ix] - bI[ix] * vJ[ix];
      }
      switch (il) {
        case 0:
          rq[ix] = q[ix] * (-as[ix] * cs[ix] * bv +
                            af[ix] * (v2a2 + cf[ix] * (cf[ix] + v[ix])));
          break;
        case 1:
          rq[ix] = q[ix] * (+as[ix] * cs[ix] * bv +
                            af[ix] * (v2a2 + cf[ix] * (cf[ix] - v[ix])));
          break;
        case 2:
          rq[ix] = q[ix] * (+af[ix] * cf[ix] * bv +
                            as[ix] * (v2a2 + cs[ix] * (cs[ix] + v[ix])));
          break;
        case 3:
          rq[ix] = q[ix] * (-af[ix] * cf[ix] * bv +
                            as[ix] * (v2a2 + cs[ix] * (cs[ix] - v[ix])));
          break;
        case 4:
          rq[ix] = q[ix] * HALF * vv;
          break;
        case 5:
          rq[ix] = s->p.divbwave ? q[ix] * bi[ix] : ZERO;
          break;
        case 6:
          rq[ix] = +q[ix] * bv;
          break;
        default:
          rq[ix] = -q[ix] * bv;
          break;
      }
    }
  } else if (iw <= s->m0_ + nd) {
    const double* vw = W(wroe, iw);
    if (iw == s->m0_ + idim + 1) {
      switch (il) {
        case 0: FORBOX(b, ix) rq[ix] = q[ix] * af[ix] * (vw[ix] + cf[ix]); break;
        case 1: FORBOX(b, ix) rq[ix] = q[ix] * af[ix] * (vw[ix] - cf[ix]); break;
        case 2: FORBOX(b, ix) rq[ix] = q[ix] * as[ix] * (vw[ix] + cs[ix]); break;
        case 3: FORBOX(b, ix) rq[ix] = q[ix] * as[ix] * (vw[ix] - cs[ix]); break;
        case 4: FORBOX(b, ix) rq[ix] = q[ix] * vw[ix]; break;
        default: FORBOX(b, ix) rq[ix] = ZERO; break;
      }
    } else {
      const double* bw = W(wroe, s->b0_ - s->m0_ + iw);
      const int isI = iw == s->m0_ + idir + 1;
      switch (il) {
        case 0:
          FORBOX(b, ix) rq[ix] = q[ix] * (af[ix] * vw[ix] - as[ix] * cs[ix] * bw[ix] * fsign(ONE, bi[ix]));
          break;
        case 1:
          FORBOX(b, ix) rq[ix] = q[ix] * (af[ix] * vw[ix] + as[ix] * cs[ix] * bw[ix] * fsign(ONE, bi[ix]));
          break;
        case 2:
          FORBOX(b, ix) rq[ix] = q[ix] * (as[ix] * vw[ix] + af[ix] * cf[ix] * bw[ix] * fsign(ONE, bi[ix]));
          break;
        case 3:
          FORBOX(b, ix) rq[ix] = q[ix] * (as[ix] * vw[ix] - af[ix] * cf[ix] * bw[ix] * fsign(ONE, bi[ix]));
          break;
        case 4:
          FORBOX(b, ix) rq[ix] = q[ix] * vw[ix];
          break;
        case 5:
          FORBOX(b, ix) rq[ix] = ZERO;
          break;
        case 6:
          if (isI) FORBOX(b, ix) rq[ix] = +q[ix] * bJ[ix];
          else FORBOX(b, ix) rq[ix] = -q[ix] * bI[ix];
          break;
        default:
          if (isI) FORBOX(b, ix) rq[ix] = -q[ix] * bJ[ix];
          else FORBOX(b, ix) rq[ix] = +q[ix] * bI[ix];
          break;
      }
    }
  } else {
    if (iw == s->b0_ + idim + 1) {
      if (il == 5 && s->p.divbwave) FORBOX(b, ix) rq[ix] = q[ix];
      else FORBOX(b, ix) rq[ix] = ZERO;
    } else {
      const double* bw = W(wroe, iw);
      const int isI = iw == s->b0_ + idir + 1;
      switch (il) {
        case 0: case 1:
          FORBOX(b, ix) rq[ix] = +q[ix] * as[ix] * sqrt(cs2[ix]) * bw[ix] / sr[ix];
          break;
        case 2: case 3:
          FORBOX(b, ix) rq[ix] = -q[ix] * af[ix] * sqrt(cs2[ix]) * bw[ix] / sr[ix];
          break;
        case 4: case 5:
          FORBOX(b, ix) rq[ix] = ZERO;
          break;
        default:
          if (isI) FORBOX(b, ix) rq[ix] = -q[ix] * bJ[ix] / fsign(sr[ix], bi[ix]);
          else FORBOX(b, ix) rq[ix] = +q[ix] * bI[ix] / fsign(sr[ix], bi[ix]);
          break;
      }
    }
  }
}

/* rtimes, src/vacphys.hdroe.t:144-215 */
static void rtimes_hd(vo_state* s, const double* q, const double* wroe, box b,
                      int iw, int il, int idim, double* rq) {
  const double* c = s->roe[ROE_CS];
  const int shear = il >= 3;
  int idir = -1;
  if (shear) {
    idir = il - 3;
    if (idir >= idim) idir++;
  }
  const double* h = W(wroe, s->e_);
  const double* v = W(wroe, s->m0_ + idim + 1);
  if (iw == s->rho_) {
    if (shear) FORBOX(b, ix) rq[ix] = ZERO;
    else FORBOX(b, ix) rq[ix] = q[ix];
  } else if (iw == s->e_) {
    switch (il) {
      case 0: FORBOX(b, ix) rq[ix] = q[ix] * (h[ix] + v[ix] * c[ix]); break;
      case 1: FORBOX(b, ix) rq[ix] = q[ix] * (h[ix] - v[ix] * c[ix]); break;
      case 2:
        FORBOX(b, ix) {
          double vv = 0.0;
          for (int k = 1; k <= s->ndir; k++) {
            const double vk = W(wroe, s->m0_ + k)[ix];
            vv = (k == 1) ? vk * vk : vv + vk * vk;
          }
          rq[ix] = q[ix] * HALF * vv;
        }
        break;
      default: {
        const double* vd = W(wroe, s->m0_ + idir + 1);
        FORBOX(b, ix) rq[ix] = q[ix] * vd[ix];
      }
    }
  } else if (iw == s->m0_ + idim + 1) {
    switch (il) {
      case 0: FORBOX(b, ix) rq[ix] = q[ix] * (v[ix] + c[ix]); break;
      case 1: FORBOX(b, ix) rq[ix] = q[ix] * (v[ix] - c[ix]); break;
      case 2: FORBOX(b, ix) rq[ix] = q[ix] * v[ix]; break;
      default: FORBOX(b, ix) rq[ix] = ZERO; break;
    }
  } else {
    if (shear) {
      if (iw == s->m0_ + idir + 1) FORBOX(b, ix) rq[ix] = q[ix];
      else FORBOX(b, ix) rq[ix] = ZERO;
    } else {
      const double* vw = W(wroe, iw);
      FORBOX(b, ix) rq[ix] = q[ix] * vw[ix];
    }
  }
}

/* tvdlimit2, src/vactvd.t:86-206, with getphi's TVD-MUSCL branch
 * (src/vactvd.t:227-243): for each characteristic wave il, the dissipative
 * flux R(iw,il)*phi(il)*(dvolume(i)+dvolume(j))/4 enters wnew through
 * addflux(-1) (wnew += (F(ix)-F(ix-1))/dvolume). */
static void tvdlimit2(vo_state* s, double qdt, box ixC, box ixO, int idim,
                      const double* wL, const double* wR, double* wnew) {
  double** R = s->roe;
  box hxO = shift(ixO, idim, -1);
  const long sh = s->st[idim];
  if (s->mhd)
    average_mhd(s, wL, wR, ixC, idim, s->wroe);
  else
    average_hd(s, wL, wR, ixC, s->wroe);
  const double* dx = W(s->dx, idim);
  const double* dv = s->dvolume;
  for (int il = 0; il < s->nw; il++) {
    if (s->mhd)
      geteigenjump_mhd(s, wL, wR, s->wroe, ixC, il, idim);
    else
      geteigenjump_hd(s, wL, wR, s->wroe, ixC, il, idim);
    double *a = R[ROE_A], *smalla = R[ROE_SMALLA], *jump = R[ROE_JUMP];
    double *phi = R[ROE_PHI], *rphi = R[ROE_RPHI];
    const int te = s->p.typeentropy[il];
    FORBOX(ixC, ix) a[ix] = a[ix] * qdt * TWO / (dx[ix] + dx[ix + sh]);
    if (te == VACGPU_ENTROPY_HARTEN || te == VACGPU_ENTROPY_POWELL)
      FORBOX(ixC, ix) smalla[ix] = smalla[ix] * qdt * TWO / (dx[ix] + dx[ix + sh]);
    if ((il == 0 || il == 1) && s->courantpar > ZERO && s->istep == s->nstep) {
      double courantmax = 0.0;
      int first = 1;
      FORBOX_SEQ(ixC, ix) {
        const double q = fabs(a[ix]);
        if (first || q > courantmax) courantmax = q;
        first = 0;
      }
      if (courantmax > ONE) s->nerror[2]++;
      if (courantmax > SMALLDOUBLE) {
        const double c = qdt * s->courantpar / courantmax;
        if (c < s->dtcourant[idim]) s->dtcourant[idim] = c;
      }
    }
    if (te == VACGPU_ENTROPY_NUL || te == VACGPU_ENTROPY_RATIO) {
      FORBOX(ixC, ix) phi[ix] = fabs(a[ix]) * jump[ix];
    } else {
      FORBOX(ixC, ix) {
        if (fabs(a[ix]) >= smalla[ix])
          phi[ix] = fabs(a[ix]) * jump[ix];
        else
          phi[ix] = HALF * (smalla[ix] + a[ix] * a[ix] / smalla[ix]) * jump[ix];
      }
    }
    for (int iw = 0; iw < s->nw; iw++) {
      if (s->mhd)
        rtimes_mhd(s, phi, s->wroe, ixC, iw, il, idim, rphi);
      else
        rtimes_hd(s, phi, s->wroe, ixC, iw, il, idim, rphi);
      FORBOX(ixC, ix) rphi[ix] = rphi[ix] * QUARTER * (dv[ix + sh] + dv[ix]);
      addflux(s, -ONE, ixO, iw, idim, rphi, ixO, rphi, hxO, wnew);
    }
  }
}

/* ---------------------------------------------------------------- schemes */

/* hancock, src/vactvdlf.t:5-89 */
static void hancock(vo_state* s, double qdt, box ixO, int idimmin,
                    int idimmax, double* wCT, double* wnew) {
  for (int idim = idimmin; idim <= idimmax; idim++) {
    box hxO = shift(ixO, idim, -1);
    long sh = s->st[idim];
    for (int iw = 0; iw < s->nw; iw++) {
      double* r = W(s->wRC, iw);
      double* l = W(s->wLC, iw);
      const double* c = W(wCT, iw);
      FORBOX(hxO, ix) r[ix] = c[ix + sh];
      FORBOX(ixO, ix) l[ix] = c[ix];
    }
    upwindLR(s, ixO, hxO, idim, wCT, s->wLC, s->wRC);
    getv(s, s->wRC, hxO, idim, s->vRC);
    getv(s, s->wLC, ixO, idim, s->vLC);
    for (int iw = 0; iw < s->nw; iw++) {
      int tr = getflux(s, s->wRC, hxO, iw, idim, s->fRC);
      getflux(s, s->wLC, ixO, iw, idim, s->fLC);
      if (tr) {
        const double* r = W(s->wRC, iw);
        const double* l = W(s->wLC, iw);
        FORBOX(hxO, ix) s->fRC[ix] = s->fRC[ix] + s->vRC[ix] * r[ix];
        FORBOX(ixO, ix) s->fLC[ix] = s->fLC[ix] + s->vLC[ix] * l[ix];
      }
      addflux(s, qdt, ixO, iw, idim, s->fLC, ixO, s->fRC, hxO, wnew);
    }
  }
  if (s->p.sourceunsplit)
    addsource2(s, qdt * (idimmax - idimmin + ONE) / s->ndim, ixO, wCT, wnew);
}

/* tvdmusclf, addfluxok=.true., src/vactvdlf.t:92-299: method 'tvdlf' /
 * 'tvdlf1' (Lax-Friedrichs dissipation with the mean-state cmax) or 'tvdmu' /
 * 'tvdmu1' (central flux, then tvdlimit2's Roe dissipation) */
static void tvdmusclf(vo_state* s, double qdt, box ixO, int idimmin,
                      int idimmax, double* wCT, double* wnew) {
  const int tf = s->p.typefull;
  const int lf = tf == VACGPU_TVDLF || tf == VACGPU_TVDLF1;
  for (int idim = idimmin; idim <= idimmax; idim++) {
    box hxO = shift(ixO, idim, -1);
    box ixC = ixO;
    ixC.lo[idim] = hxO.lo[idim];
    long sh = s->st[idim];
    for (int iw = 0; iw < s->nw; iw++) {
      double* r = W(s->wRC, iw);
      double* l = W(s->wLC, iw);
      const double* c = W(wCT, iw);
      FORBOX(ixC, ix) r[ix] = c[ix + sh];
      FORBOX(ixC, ix) l[ix] = c[ix];
    }
    if (tf != VACGPU_TVDLF1 && tf != VACGPU_TVDMU1) {
      double* base;
      switch (s->p.typelimited) {
        case VACGPU_LIMITED_PREVIOUS: base = s->wold; break;
        case VACGPU_LIMITED_PREDICTOR: base = wCT; break;
        default: base = wnew; break;
      }
      upwindLR(s, ixC, ixC, idim, base, s->wLC, s->wRC);
    }
    if (lf) {
      /* mean state in wLC, cmax, CFL, wLC regained (src/vactvdlf.t:168-206) */
      for (int iw = 0; iw < s->nw; iw++) {
        double* l = W(s->wLC, iw);
        const double* r = W(s->wRC, iw);
        FORBOX(ixC, ix) l[ix] = HALF * (l[ix] + r[ix]);
      }
      int new_cmax = 1;
      getcmax(s, &new_cmax, s->wLC, ixC, idim, s->cmaxC);
      if (s->courantpar > ZERO && s->istep == s->nstep) {
        const double* dx = W(s->dx, idim);
        double courantmax = 0.0;
        int first = 1;
        FORBOX_SEQ(ixC, ix) {
          double q = s->cmaxC[ix] * TWO / (dx[ix] + dx[ix + sh]);
          if (first || q > courantmax) courantmax = q;
          first = 0;
        }
        if (qdt * courantmax > ONE) s->nerror[2]++;
        if (courantmax > SMALLDOUBLE) {
          double c = s->courantpar / courantmax;
          if (c < s->dtcourant[idim]) s->dtcourant[idim] = c;
        }
      }
      for (int iw = 0; iw < s->nw; iw++) {
        double* l = W(s->wLC, iw);
        const double* r = W(s->wRC, iw);
        FORBOX(ixC, ix) l[ix] = 2 * l[ix] - r[ix];
      }
    }
    getv(s, s->wLC, ixC, idim, s->vLC);
    getv(s, s->wRC, ixC, idim, s->vRC);
    for (int iw = 0; iw < s->nw; iw++) {
      const double* l = W(s->wLC, iw);
      const double* r = W(s->wRC, iw);
      int tr = getflux(s, s->wLC, ixC, iw, idim, s->fLC);
      getflux(s, s->wRC, ixC, iw, idim, s->fRC);
      if (tr) {
        FORBOX(ixC, ix) s->fLC[ix] = s->fLC[ix] + s->vLC[ix] * l[ix];
        FORBOX(ixC, ix) s->fRC[ix] = s->fRC[ix] + s->vRC[ix] * r[ix];
      }
      FORBOX(ixC, ix) s->fLC[ix] = HALF * (s->fLC[ix] + s->fRC[ix]);
      if (lf) {
        FORBOX(ixC, ix) s->fRC[ix] = -s->cmaxC[ix] * HALF * (r[ix] - l[ix]);
        FORBOX(ixC, ix) s->fLC[ix] = s->fLC[ix] + s->fRC[ix];
      }
      addflux(s, qdt, ixO, iw, idim, s->fLC, ixO, s->fLC, hxO, wnew);
    }
    if (!lf) tvdlimit2(s, qdt, ixC, ixO, idim, s->wLC, s->wRC, wnew);
  }
  if (s->p.sourceunsplit)
    addsource2(s, qdt * (idimmax - idimmin + ONE) / s->ndim, ixO, wCT, wnew);
}

/* advect1, src/vac.t:489-572 (method hancock/tvdlf; ixO = ixI shrunk by 2) */
static void advect1(vo_state* s, int pred, double qdt, int idimmin,
                    int idimmax, double* wCT, double* w) {
  s->istep++;
  if (pred)
    hancock(s, qdt, s->ixM, idimmin, idimmax, wCT, w);
  else
    tvdmusclf(s, qdt, s->ixM, idimmin, idimmax, wCT, w);
  getboundary(s, w, s->t + qdt);  /* qt+qdt, src/vac.t:567 */
}

/* advect, src/vac.t:363-486.  'tvdlf' and 'tvdmu' have the default
 * predictor 'hancock' (twostep); 'tvdlf1' and 'tvdmu1' have typepred1='nul',
 * which turns twostep into onestep (src/vacio.t:286-299,511): one substep
 * with wCT = a copy of w. */
static void advect(vo_state* s, int idimmin, int idimmax) {
  memcpy(s->w1, s->w, sizeof(double) * s->N * s->nw);
  s->istep = 0;
  /* qtC of each advect1 call (src/vac.t:407,426-427) */
  if (s->p.typefull == VACGPU_TVDLF1 || s->p.typefull == VACGPU_TVDMU1) {
    s->qtc = s->t;
    advect1(s, 0, s->dt, idimmin, idimmax, s->w1, s->w);
    return;
  }
  s->qtc = s->t;
  advect1(s, 1, s->dt / 2, idimmin, idimmax, s->w, s->w1);
  s->qtc = s->t + s->dt / 2;
  advect1(s, 0, s->dt, idimmin, idimmax, s->w1, s->w);
}

/* advance_expl, src/vac.t:283-360 */
static void advance_expl(vo_state* s) {
  if (s->p.dimsplit) {
    if ((s->it / 2) * 2 == s->it || s->p.typedimsplit == VACGPU_SPLIT_XY) {
      for (int d = 0; d < s->ndim; d++) advect(s, d, d);
    } else {
      for (int d = s->ndim - 1; d >= 0; d--) advect(s, d, d);
    }
  } else {
    advect(s, 0, s->ndim - 1);
  }
}

/* getdt_courant, src/vac.t:664-722 */
static void getdt_courant(vo_state* s) {
  s->dt = BIGDOUBLE;
  double courantmax = ZERO;
  int new_cmax = 1;
  for (int idim = 0; idim < s->ndim; idim++) {
    if (s->dtcourant[idim] < BIGDOUBLE) {
      if (s->dtcourant[idim] < s->dt) s->dt = s->dtcourant[idim];
    } else {
      getcmax(s, &new_cmax, s->w, s->ixM, idim, s->cmaxC);
      const double* dx = W(s->dx, idim);
      double m = 0.0;
      int first = 1;
      FORBOX_SEQ(s->ixM, ix) {
        double q = s->cmaxC[ix] / dx[ix];
        if (first || q > m) m = q;
        first = 0;
      }
      if (m > courantmax) courantmax = m;
    }
  }
  for (int idim = 0; idim < s->ndim; idim++) s->dtcourant[idim] = BIGDOUBLE;
  if (courantmax > SMALLDOUBLE) {
    double c = s->courantpar / courantmax;
    if (c < s->dt) s->dt = c;
  }
}

/* getdt_res, src/vacphys.mhdres.t:5-45: the diffusion limit, called from
 * getdt (src/vacphys.mhd0.t:83-103) on ixM: dtdiffpar*min(dx)^2/eta for
 * eqpar(eta_) > 0; for the specialeta field min over idim of
 * dtdiffpar/(smalldouble+max(eta/dx^2)), eta set from w at it==itmin and
 * otherwise the one of the last resistive source */
static void getdt_res(vo_state* s) {
  double dtdiff;
  if (s->p.eqpar[1] > ZERO) {
    double m = ZERO;
    int first = 1;
    for (int d = 0; d < s->ndim; d++) {
      const double* dx = W(s->dx, d);
      FORBOX_SEQ(s->ixM, i) {
        if (first || dx[i] < m) m = dx[i];
        first = 0;
      }
    }
    dtdiff = s->p.dtdiffpar * (m * m) / s->p.eqpar[1];
  } else {
    if (s->it == s->itmin) {
      const int idirmin = getcurrent(s, s->w, s->ixM);
      special_eta(s, s->w, s->ixM, idirmin);
    }
    dtdiff = BIGDOUBLE;
    for (int d = 0; d < s->ndim; d++) {
      const double* dx = W(s->dx, d);
      double m = ZERO;
      int first = 1;
      FORBOX_SEQ(s->ixM, i) {
        const double q = s->eta[i] / (dx[i] * dx[i]);
        if (first || q > m) m = q;
        first = 0;
      }
      const double c = s->p.dtdiffpar / (SMALLDOUBLE + m);
      if (c < dtdiff) dtdiff = c;
    }
  }
  if (dtdiff < s->dt) s->dt = dtdiff;
}

/* getdt_special: the user hook's dt=min(dt,dt_mine), or getdt_grav,
 * vacusr.gravity.t (dt limit of the gravity hook) */
static void getdt_special(vo_state* s) {
  if (s->dtsp_fn) {
    const double* x[3] = {W(s->x, 0), W(s->x, s->ndim > 1 ? 1 : 0),
                          W(s->x, s->ndim > 2 ? 2 : 0)};
    double d = s->dtsp_fn(s->src_user, s->w, s->ixM.lo, s->ixM.hi, s->st, s->N, x);
    if (d < s->dt) s->dt = d;
    return;
  }
  if (s->src_id != VACGPU_SRC_GRAVITY) return;
  if (s->it == s->itmin) {
    s->dtgrav = BIGDOUBLE;
    for (int idim = 0; idim < s->ndim; idim++) {
      double g = fabs(s->src_par[idim]);
      if (g > ZERO) {
        double m = 0.0;
        int first = 1;
        for (int jdim = 0; jdim < s->ndim; jdim++) {
          const double* dx = W(s->dx, jdim);
          FORBOX_SEQ(s->ixM, ix) {
            double q = g / dx[ix];
            if (first || q > m) m = q;
            first = 0;
          }
        }
        double c = ONE / sqrt(m);
        if (c < s->dtgrav) s->dtgrav = c;
      }
    }
  }
  if (s->dtgrav < s->dt) s->dt = s->dtgrav;
}

/* -------------------------------------------------------------- public API */

#define ERR(msg)                                   \
  do {                                             \
    snprintf(errbuf, sizeof(errbuf), "%s", msg);   \
    return NULL;                                   \
  } while (0)

static char errbuf[256];

/* Configurations the Roe solvers define: the MHD solver dies for ndir=1
 * (src/vacphys.mhdroe.t:25); the left/right speeds of the MHD entropy fixes
 * of the fastLW/slow waves and of alfvLW are saved by the fastRW and alfvRW
 * calls (src/vacphys.mhdroe.t:245-276), so those waves' fix needs the
 * fastRW's (alfvRW's); the HD 'ratio' fix reads speeds the HD solver never
 * sets (src/vacphys.hdroe.t:110-134). */
static const char* roe_check(const vacgpu_params* p, int nw) {
  const int mhd = p->physics == VACGPU_PHYS_MHD;
  if (mhd && p->ndir < 2) return "MHD Roe solver needs ndir>=2";
  for (int il = 0; il < nw; il++) {
    const int te = p->typeentropy[il];
    if (te < VACGPU_ENTROPY_NUL || te > VACGPU_ENTROPY_YEE)
      return "unknown typeentropy";
    if (!mhd && te == VACGPU_ENTROPY_RATIO)
      return "typeentropy='ratio' is undefined for the HD Roe solver";
  }
  if (mhd) {
#define USES_LR(il)                                      \
  (p->typeentropy[il] == VACGPU_ENTROPY_HARTEN ||        \
   p->typeentropy[il] == VACGPU_ENTROPY_POWELL ||        \
   p->typeentropy[il] == VACGPU_ENTROPY_RATIO)
    for (int il = 1; il < 4; il++)
      if (USES_LR(il) && !USES_LR(0))
        return "MHD entropy fix of a fast/slow wave needs the fastRW fix";
    if (nw == 8 && USES_LR(7) && !USES_LR(6))
      return "MHD entropy fix of alfvLW needs the alfvRW fix";
#undef USES_LR
  }
  return NULL;
}

const char* vo_last_error(void) { return errbuf; }

vo_state* vo_create(const vacgpu_params* p) {
  if (p->ndim < 1 || p->ndim > 3) ERR("ndim out of range");
  if (p->ndir < p->ndim || p->ndir > 3) ERR("ndir out of range");
  if (p->dixB != 2) ERR("dixB must be 2");
  int nw = p->physics == VACGPU_PHYS_MHD ? 2 + 2 * p->ndir : 2 + p->ndir;
  if (p->nw != nw) ERR("nw does not match physics and ndir");
  if (p->typefull == VACGPU_TVDMU || p->typefull == VACGPU_TVDMU1) {
    const char* why = roe_check(p, nw);
    if (why) ERR(why);
  }
  vo_state* s = (vo_state*)calloc(1, sizeof(vo_state));
  s->p = *p;
  s->ndim = p->ndim;
  s->ndir = p->ndir;
  s->nw = nw;
  s->mhd = p->physics == VACGPU_PHYS_MHD;
  s->rho_ = 0;
  s->m0_ = 0;
  s->e_ = 1 + p->ndir;
  s->b0_ = s->e_;
  for (int d = 0; d < 3; d++) {
    s->nG[d] = d < p->ndim ? p->nx[d] + 4 : 1;
    s->ixG.lo[d] = 0;
    s->ixG.hi[d] = s->nG[d] - 1;
    s->ixM.lo[d] = d < p->ndim ? 2 : 0;
    s->ixM.hi[d] = d < p->ndim ? s->nG[d] - 3 : 0;
  }
  s->st[0] = 1;
  s->st[1] = s->nG[0];
  s->st[2] = (long)s->nG[0] * s->nG[1];
  s->N = s->st[2] * s->nG[2];
  long N = s->N;
  s->x = calloc(N * 3, sizeof(double));
  s->dx = calloc(N * 3, sizeof(double));
  s->dvolume = calloc(N, sizeof(double));
  s->w = calloc(N * nw, sizeof(double));
  s->w1 = calloc(N * nw, sizeof(double));
  s->wold = calloc(N * nw, sizeof(double));
  s->wLC = calloc(N * nw, sizeof(double));
  s->wRC = calloc(N * nw, sizeof(double));
  double** t1[] = {&s->fLC, &s->fRC, &s->vLC, &s->vRC, &s->cmaxC,
                   &s->ldw, &s->dwC, &s->tmp, &s->tmp2, &s->divb,
                   &s->csound2, &s->cfast2, &s->pp};
  for (unsigned i = 0; i < sizeof(t1) / sizeof(t1[0]); i++)
    *t1[i] = calloc(N, sizeof(double));
  for (int c = 0; c < 3; c++) s->cur[c] = calloc(N, sizeof(double));
  if (s->mhd && p->eqpar[1] < ZERO) {
    s->eta = calloc(N, sizeof(double));
    for (int c = 0; c < 3; c++) s->gradeta[c] = calloc(N, sizeof(double));
  }
  s->smallp = p->smallp;
  s->smallrho = p->smallrho;
  s->courantpar = p->courantpar;
  s->dtpar = p->dtpar;
  /* onestep / twostep */
  s->nstep = (p->typefull == VACGPU_TVDLF1 || p->typefull == VACGPU_TVDMU1) ? 1 : 2;
  if (p->typefull == VACGPU_TVDMU || p->typefull == VACGPU_TVDMU1) {
    s->wroe = calloc(N * nw, sizeof(double));
    for (int i = 0; i < NROE; i++) s->roe[i] = calloc(N, sizeof(double));
  }
  /* startup, src/vac.t:160-220 */
  for (int d = 0; d < 3; d++) s->dtcourant[d] = BIGDOUBLE;
  if (s->dtpar > ZERO && p->slowsteps != 1) s->courantpar = -ONE;
  return s;
}

void vo_destroy(vo_state* s) {
  if (!s) return;
  double* a[] = {s->x, s->dx, s->dvolume, s->w, s->w1, s->wold, s->wLC,
                 s->wRC, s->fLC, s->fRC, s->vLC, s->vRC, s->cmaxC, s->ldw,
                 s->dwC, s->tmp, s->tmp2, s->divb, s->csound2, s->cfast2,
                 s->pp};
  for (unsigned i = 0; i < sizeof(a) / sizeof(a[0]); i++) free(a[i]);
  for (int iB = 0; iB < VACGPU_MAXB; iB++) free(s->fixB[iB]);
  for (int c = 0; c < 3; c++) free(s->cur[c]);
  free(s->wroe);
  free(s->eta);
  for (int c = 0; c < 3; c++) free(s->gradeta[c]);
  for (int i = 0; i < NROE; i++) free(s->roe[i]);
  free(s);
}

/* gridsetup1, src/vacgrid.t:457-593 (Cartesian slab, fullgridini=F).
 * xmesh: x(ixM^S,1:ndim) column-major. */
int vo_set_grid(vo_state* s, const double* xmesh) {
  int nd = s->ndim;
  int nQ[3], q0[3];
  for (int d = 0; d < 3; d++) {
    nQ[d] = d < nd ? s->nG[d] + 2 : 1;
    q0[d] = d < nd ? 1 : 0; /* qx index of G index 0 */
  }
  long qs1 = nQ[0], qs2 = (long)nQ[0] * nQ[1];
  long NQ = qs2 * nQ[2];
  double* qx = calloc(NQ * nd, sizeof(double));
#define QX(i1, i2, i3, jd) \
  qx[(long)(jd)*NQ + (i1) + qs1 * (i2) + qs2 * (i3)]
  /* qx(ixG)=x(ixG); x in the ghost cells is zero, as in VAC */
  long k = 0;
  for (int jd = 0; jd < nd; jd++)
    for (int i3 = s->ixM.lo[2]; i3 <= s->ixM.hi[2]; i3++)
      for (int i2 = s->ixM.lo[1]; i2 <= s->ixM.hi[1]; i2++)
        for (int i1 = s->ixM.lo[0]; i1 <= s->ixM.hi[0]; i1++)
          QX(i1 + q0[0], i2 + q0[1], i3 + q0[2], jd) = xmesh[k++];
  for (int idim = 0; idim < nd; idim++) {
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
      lo[d] = 0;
      hi[d] = nQ[d] - 1;
    }
    for (int pass = 0; pass < 2; pass++) {
      int ixe, ixf;
      if (pass == 0) { /* upper layers */
        lo[idim] = s->ixM.hi[idim] + 1 + q0[idim];
        hi[idim] = nQ[idim] - 1;
        ixe = lo[idim] - 1;
        ixf = ixe - 1;
      } else {
        lo[idim] = 0;
        hi[idim] = s->ixM.lo[idim] - 1 + q0[idim];
        ixe = hi[idim] + 1;
        ixf = ixe + 1;
      }
      for (int jd = 0; jd < nd; jd++)
        for (int ix = lo[idim]; ix <= hi[idim]; ix++) {
          int c = abs(ixe - ix);
          int a[3];
          for (a[2] = lo[2]; a[2] <= hi[2]; a[2]++)
            for (a[1] = lo[1]; a[1] <= hi[1]; a[1]++)
              for (a[0] = lo[0]; a[0] <= hi[0]; a[0]++) {
                if (a[idim] != lo[idim]) continue;
                int b[3] = {a[0], a[1], a[2]}, e[3] = {a[0], a[1], a[2]},
                    f[3] = {a[0], a[1], a[2]};
                b[idim] = ix;
                e[idim] = ixe;
                f[idim] = ixf;
                QX(b[0], b[1], b[2], jd) =
                    (1 + c) * QX(e[0], e[1], e[2], jd) -
                    c * QX(f[0], f[1], f[2], jd);
              }
        }
    }
  }
  for (int i3 = 0; i3 < s->nG[2]; i3++)
    for (int i2 = 0; i2 < s->nG[1]; i2++)
      for (int i1 = 0; i1 < s->nG[0]; i1++) {
        long ix = IDX(s, i1, i2, i3);
        int q[3] = {i1 + q0[0], i2 + q0[1], i3 + q0[2]};
        for (int jd = 0; jd < nd; jd++)
          W(s->x, jd)[ix] = QX(q[0], q[1], q[2], jd);
        for (int idim = 0; idim < nd; idim++) {
          int j[3] = {q[0], q[1], q[2]}, h[3] = {q[0], q[1], q[2]};
          j[idim]++;
          h[idim]--;
          W(s->dx, idim)[ix] = HALF * (QX(j[0], j[1], j[2], idim) -
                                       QX(h[0], h[1], h[2], idim));
        }
        double dv = W(s->dx, 0)[ix];
        for (int idim = 1; idim < nd; idim++) dv = dv * W(s->dx, idim)[ix];
        s->dvolume[ix] = dv;
      }
#undef QX
  free(qx);
  s->volume = 0.0;
  FORBOX_SEQ(s->ixM, ix) s->volume = s->volume + s->dvolume[ix];
  return 0;
}

/* w(ixM^S,1:nw) from the .ini; ghosts by getboundary (src/vac.t:54) */
void vo_set_state(vo_state* s, const double* wmesh, int it, double t) {
  long k = 0;
  for (int iw = 0; iw < s->nw; iw++) FORBOX_SEQ(s->ixM, ix) W(s->w, iw)[ix] = wmesh[k++];
  s->it = it;
  s->itmin = it;
  s->t = t;
  s->initialized = 0;  /* a new run: fixed boundaries store again */
  getboundary(s, s->w, s->t);
}

void vo_get_state(vo_state* s, double* wmesh) {
  long k = 0;
  for (int iw = 0; iw < s->nw; iw++) FORBOX_SEQ(s->ixM, ix) wmesh[k++] = W(s->w, iw)[ix];
}

/* full ixG state (test access to ghosts) */
void vo_get_state_full(vo_state* s, double* wfull) {
  memcpy(wfull, s->w, sizeof(double) * s->N * s->nw);
}

void vo_register_bound(vo_state* s,
                       void (*fn)(void*, double*, const int*, const int*,
                                  const long*, long, const double*, int, int,
                                  double),
                       void* user) {
  s->bound_fn = fn;
  s->bound_user = user;
}

void vo_register_eta(vo_state* s,
                     void (*fn)(void*, const double*, const double* const*,
                                double*, double* const*, const int*,
                                const int*, const long*, long,
                                const double* const*, int, double),
                     void* user) {
  s->eta_fn = fn;
  s->eta_user = user;
}

/* the user's specialsource and getdt_special (either may be NULL); they
 * replace a built-in source */
void vo_register_source_fn(
    vo_state* s,
    void (*src)(void*, double, double, const double*, double, double*, const int*,
                const int*, const long*, long, const double* const*),
    double (*dtsp)(void*, const double*, const int*, const int*, const long*, long,
                   const double* const*),
    void* user) {
  s->src_fn = src;
  s->dtsp_fn = dtsp;
  s->src_user = user;
  if (src || dtsp) s->src_id = VACGPU_SRC_NONE;
}

void vo_register_source(vo_state* s, int id, const double* par, int npar) {
  s->src_id = id;
  memset(s->src_par, 0, sizeof(s->src_par));
  for (int i = 0; i < npar && i < VACGPU_MAXSRCPAR; i++) s->src_par[i] = par[i];
}

/* The time loop body, src/vac.t:55-106.  Returns the number of steps done;
 * *finished=1 when timetofinish held. */
int vo_step(vo_state* s, int maxsteps, double tstop, int* finished) {
  int n = 0;
  *finished = 0;
  const vacgpu_params* p = &s->p;
  while (n < maxsteps) {
    double dtsave_dt = s->dt, dtold_save = s->dtold;
    double dtc[3] = {s->dtcourant[0], s->dtcourant[1], s->dtcourant[2]};
    if (s->dtpar > ZERO) {
      s->dt = s->dtpar;
    } else {
      if (s->courantpar > ZERO) getdt_courant(s);
      if (s->mhd && s->p.eqpar[1] != ZERO) getdt_res(s);
      getdt_special(s);
      if (p->dtcantgrow && s->it > s->itmin && s->dtold < s->dt) s->dt = s->dtold;
      s->dtold = s->dt;
    }
    /* timetofinish, src/vac.t:608-628 (residual checks off) */
    if (s->it >= p->itmax || s->t >= p->tmax || s->dt < p->dtmin) {
      *finished = 1;
      break;
    }
    if (s->t >= tstop) {
      /* caller saves before this step: the dt evaluation is repeated then */
      s->dt = dtsave_dt;
      s->dtold = dtold_save;
      for (int d = 0; d < 3; d++) s->dtcourant[d] = dtc[d];
      break;
    }
    if (p->slowsteps == 1 && s->it == s->itmin) s->dtpar = -ONE;
    if (p->slowsteps > s->it - s->itmin + 1) {
      double r = ONE - (s->it - s->itmin + ONE) / p->slowsteps;
      s->dt = s->dt * (ONE - r * r);
    }
    if (p->tmaxexact) {
      double c = p->tmax - s->t + SMALLDOUBLE;
      if (c < s->dt) s->dt = c;
    }
    memcpy(s->wold, s->w, sizeof(double) * s->N * s->nw);
    advance_expl(s);
    s->it = s->it + 1;
    s->t = s->t + s->dt;
    n++;
  }
  return n;
}

double vo_t(vo_state* s) { return s->t; }
int vo_it(vo_state* s) { return s->it; }
double vo_dt(vo_state* s) { return s->dt; }
double vo_smallp(vo_state* s) { return s->smallp; }
double vo_smallrho(vo_state* s) { return s->smallrho; }
double vo_volume(vo_state* s) { return s->volume; }
void vo_nerror(vo_state* s, int* n) { memcpy(n, s->nerror, sizeof(s->nerror)); }
long vo_ncells_full(vo_state* s) { return s->N; }

/* dx(ixG^S,idim) and x(ixG^S,idim), full grid */
void vo_get_dx(vo_state* s, int idim, double* out) {
  memcpy(out, W(s->dx, idim), sizeof(double) * s->N);
}
void vo_get_x(vo_state* s, int idim, double* out) {
  memcpy(out, W(s->x, idim), sizeof(double) * s->N);
}

/* savefilelog_default, src/vacio.t:1050-1105 */
void vo_sums(vo_state* s, double* wmean) {
  for (int iw = 0; iw < s->nw; iw++) {
    double acc = 0.0;
    FORBOX_SEQ(s->ixM, ix) acc = acc + s->dvolume[ix] * W(s->w, iw)[ix];
    wmean[iw] = acc / s->volume;
  }
}

// roe.cuh - the TVD-MUSCL corrector of methods 'tvdmu' and 'tvdmu1'
// (tvdmusclf, src/vactvdlf.t:92-299, with tvdlimit2 and getphi,
// src/vactvd.t:86-243): the central flux of the upwindLR face states plus
// Roe's characteristic dissipation, from the eight-wave MHD Roe solver
// (src/vacphys.mhdroe.t) or the gamma-law HD one (src/vacphys.hdroe.t).
//
// A face pass evaluates each face once (one thread per face): the face
// states, the central flux and the Roe decomposition, storing the central
// flux and the dissipative fluxes R(iw,il)*phi(il)*(dvolume(i)+dvolume(j))/4
// of every wave; a cell pass then applies them in the reference's order: the
// central fluxes of all variables (addflux with qdt), then wave by wave the
// dissipative ones (addflux with qdt=-1: += (F(i)-F(i-1))/dvolume).
// The FP64 instance (roe_fp64.cu, built without FMA contraction) keeps every
// array statement's operation order and is bit-identical to the CPU
// restatement.  The mixed instance (roe_mixed.cu, IEEE FP32 division and
// square root) runs the solver in FP32 with cancellation-free forms of the
// MHD average (average_mhd_f32), the thermal pressures from the
// double-float recovery of physics_mixed.cuh, and the HD average and the
// entropy-fix speeds in double.
#pragma once
#include "sweep.cuh"

namespace vacgpu {

template <class PH, int NDIM, int NDIR, bool MHD>
struct RoeSweep {
  typedef Sweep<PH, NDIM, NDIR, MHD> S;
  typedef typename PH::T T;
  typedef typename PH::R R;
  typedef Lay<NDIR, MHD> L;
  // R: the path's arithmetic (double on the FP64 path, float on the mixed
  // one); D: double, for the HD average and the entropy-fix speeds
  typedef double D;
  static constexpr int NW = L::NW;
  static constexpr int E = L::E;
  static constexpr int B0 = L::B0;

  // Roe state of one face after average and geteigenjump (the saved
  // quantities of src/vacphys.mhdroe.t:18-19,150-153 and
  // src/vacphys.hdroe.t:63-65) and the limiter function of every wave.
  struct Face {
    R v[NDIR];   // MHD: mean velocity; HD: Roe-averaged velocity
    R b[NDIR];   // MHD: B_idim (|B_idim| >= smalldouble), beta_idir, beta_jdir
    R sr;        // MHD: sqrt(mean rho); HD: sqrt(rhoL)*sqrt(rhoR)
    R cf, cs, af, as, cs2;  // MHD: fast/slow speeds, weights, sound^2
                            // HD: cs = sound speed c
    R h;         // HD: Roe-averaged enthalpy
    R dp, rhodv; // MHD: pR-pL (conservative form), rho*dv_idim
                 // HD: (pR-pL)/c^2, (vR-vL)_idim/c
    R phi[NW];   // getphi's TVD-MUSCL phi = |a*dt/dx|*jump (entropy fixed)
    // mixed cell pass only (prep_face): SIGN(1,B_idim), sqrt(cs2)/sr,
    // 1/SIGN(sr,B_idim), v^2 and v^2/2+(2-gamma)/(gamma-1)*cs2, formed once
    // per face instead of in each of rtimes' products
    R sgn, csr, isrs, vv, v2a2;
  };

  // Fortran SIGN(a,b), MAX and MIN as the oracle's selects
  static __device__ __forceinline__ D fsign(D a, D b) {
    return copysign(fabs(a), b);
  }
  static __device__ __forceinline__ D rmax(D a, D b) { return a > b ? a : b; }
  static __device__ __forceinline__ D rmin(D a, D b) { return a < b ? a : b; }
  // smalldouble of the reference
  static __device__ __forceinline__ D tiny() { return 1.0e-99; }

  // idir = idim+1-ndir*(idim/ndir) and jdir likewise, 1-based
  // (src/vacphys.mhdroe.t:97,145-146); 0-based here
  static __device__ __forceinline__ int dir_i(int d) {
    const int i1 = d + 1;
    return i1 + 1 - NDIR * (i1 / NDIR) - 1;
  }
  static __device__ __forceinline__ int dir_j(int d) {
    const int d1 = dir_i(d) + 1;
    return d1 + 1 - NDIR * (d1 / NDIR) - 1;
  }

  // getpthermal(.true.): p clipped at smallp, in double
  static __device__ __forceinline__ double pthd(const SweepArgs& a,
                                                const R* u, double smallp) {
    const double p = PH::template pthermal_raw<NDIR, MHD>(u, a.ph);
    return p >= smallp ? p : smallp;
  }
  // Eigenvalue a and jump L*dw of wave il with its entropy fix
  // (geteigenjump, src/vacphys.mhdroe.t:130-281 and
  // src/vacphys.hdroe.t:48-141; entropyfix, src/vactvd.t:422-451), then
  // phi of getphi's TVD-MUSCL branch (src/vactvd.t:227-243).  dxs =
  // dx(i)+dx(j); am receives |a*dt*2/dxs| of the two fast waves.
  template <int il>
  static __device__ __forceinline__ void wave(const SweepArgs& a, const R* wL,
                                              const R* wR, int d, double smallp,
                                              D qdt, R dxs, const R* bd,
                                              Face& f, D* am) {
    const R rL = wL[0], rR = wR[0];
    const R v = f.v[d];
    const R cf = f.cf, cs = f.cs, af = f.af, as = f.as;
    const R cs2 = f.cs2, rhodv = f.rhodv, dp = f.dp, sr = f.sr;
    R aa, jump;
    if (MHD) {
      // bd = {bdv, bdb} of the fast/slow waves, then of the Alfven waves
      const R bdv = il < 6 ? bd[0] : bd[2];
      const R bdb = il < 6 ? bd[1] : bd[3];
      switch (il) {
        case 0:
          aa = v + cf;
          jump = R(0.5) / cs2 *
                 (af * (+cf * rhodv + dp) + as * (-cs * bdv + bdb));
          break;
        case 1:
          aa = v - cf;
          jump = R(0.5) / cs2 *
                 (af * (-cf * rhodv + dp) + as * (+cs * bdv + bdb));
          break;
        case 2:
          aa = v + cs;
          jump = R(0.5) / cs2 *
                 (as * (+cs * rhodv + dp) + af * (+cf * bdv - bdb));
          break;
        case 3:
          aa = v - cs;
          jump = R(0.5) / cs2 *
                 (as * (-cs * rhodv + dp) + af * (-cf * bdv - bdb));
          break;
        case 4:
          aa = v;
          jump = rR - rL - dp / cs2;
          break;
        case 5:
          if (a.ph.divbwave) {
            aa = v;
            jump = R(wR[B0 + 1 + d]) - R(wL[B0 + 1 + d]);
          } else {
            aa = R(0);
            jump = R(0);
          }
          break;
        case 6:
          aa = v + R(fabs(f.b[d])) / sr;
          jump = +bdv - bdb;
          break;
        default:
          aa = v - R(fabs(f.b[d])) / sr;
          jump = -bdv - bdb;
          break;
      }
    } else {
      switch (il) {
        case 0:
          aa = v + cs;
          jump = R(0.5) * (dp + sr * rhodv);
          break;
        case 1:
          aa = v - cs;
          jump = R(0.5) * (dp - sr * rhodv);
          break;
        case 2:
          aa = v;
          jump = -dp + rR - rL;
          break;
        default: {
          int idir = il - 3;
          if (idir >= d) idir++;
          aa = v;
          jump = sr * (R(wR[1 + idir]) / rR - R(wL[1 + idir]) / rL);
        }
      }
    }
    // entropy fix: left and right eigenvalues, smalla or a modified a, in
    // double (the slow speeds of the left and right states cancel as the
    // averaged one does)
    const int te = a.ph.typeentropy[il];
    R smalla = R(0);
    if (te == VACGPU_ENTROPY_YEE) {
      smalla = R(a.ph.entropycoef[il]);
    } else if (te != VACGPU_ENTROPY_NUL) {
      const double g = a.ph.gamma;
      const double dL = wL[0], dR = wR[0];
      double aL = (double)wL[1 + d] / dL, aR = (double)wR[1 + d] / dR;
      if (MHD) {
        const double bLi = wL[B0 + 1 + d], bRi = wR[B0 + 1 + d];
        if (il < 4) {
          const double c2L = g * pthd(a, wL, smallp) / dL;
          const double c2R = g * pthd(a, wR, smallp) / dR;
          double bbL = (double)wL[B0 + 1] * (double)wL[B0 + 1];
          double bbR = (double)wR[B0 + 1] * (double)wR[B0 + 1];
#pragma unroll
          for (int c = 2; c <= NDIR; c++) {
            bbL = bbL + (double)wL[B0 + c] * (double)wL[B0 + c];
            bbR = bbR + (double)wR[B0 + c] * (double)wR[B0 + c];
          }
          const double ccL = c2L + bbL / dL, ccR = c2R + bbR / dR;
          const double qL = sqrt(ccL * ccL - 4.0 * c2L * (bLi * bLi) / dL);
          const double qR = sqrt(ccR * ccR - 4.0 * c2R * (bRi * bRi) / dR);
          if (il == 0) {
            aL = aL + sqrt(0.5 * (ccL + qL));
            aR = aR + sqrt(0.5 * (ccR + qR));
          } else if (il == 1) {
            aL = aL - sqrt(0.5 * (ccL + qL));
            aR = aR - sqrt(0.5 * (ccR + qR));
          } else if (il == 2) {
            aL = aL + sqrt(0.5 * (ccL - qL));
            aR = aR + sqrt(0.5 * (ccR - qR));
          } else {
            aL = aL - sqrt(0.5 * (ccL - qL));
            aR = aR - sqrt(0.5 * (ccR - qR));
          }
        } else if (il >= 6) {
          const double caL = fabs(bLi) / sqrt(dL), caR = fabs(bRi) / sqrt(dR);
          if (il == 6) {
            aL = aL + caL;
            aR = aR + caR;
          } else {
            aL = aL - caL;
            aR = aR - caR;
          }
        }
      } else if (il < 2) {
        const double sg = il == 0 ? 1.0 : -1.0;
        aL = (double)wL[1 + d] / dL + sg * sqrt(g * pthd(a, wL, smallp) / dL);
        aR = (double)wR[1 + d] / dR + sg * sqrt(g * pthd(a, wR, smallp) / dR);
      }
      const double ad = aa;
      if (te == VACGPU_ENTROPY_HARTEN) {
        const double m = 0.0 > ad - aL ? 0.0 : ad - aL;
        smalla = R(m > aR - ad ? m : aR - ad);
      } else if (te == VACGPU_ENTROPY_POWELL) {
        const double q = 2.0 * (aR - aL);
        smalla = R(0.0 > q ? 0.0 : q);
      } else if (aL < 0.0 && aR > 0.0) {  // 'ratio'
        aa = R(ad - 2.0 * aR * aL / (aR - aL));
      }
    }
    // normalisation by dt*2/(dx(i)+dx(j)) (src/vactvd.t:131-140); the
    // mixed path multiplies by the face's dt*2/(dx(i)+dx(j)) formed once
    R adt;
    if constexpr (sizeof(R) == 4)
      adt = aa * (R(qdt) * R(2) / dxs);
    else
      adt = aa * R(qdt) * R(2) / dxs;
    if (te == VACGPU_ENTROPY_HARTEN || te == VACGPU_ENTROPY_POWELL)
      smalla = smalla * R(qdt) * R(2) / dxs;
    if (il < 2) am[il] = fabs(adt);
    if (te == VACGPU_ENTROPY_NUL || te == VACGPU_ENTROPY_RATIO ||
        fabs(adt) >= smalla)
      f.phi[il] = fabs(adt) * jump;
    else
      f.phi[il] = R(0.5) * (smalla + adt * adt / smalla) * jump;
  }

  // The mixed instance's MHD average: FP32 with cancellation-free forms of
  // the reference's speeds and weights (its af^2=(cs2-cs^2)/(cf^2-cs^2)
  // and the slow speed cancel at low beta), the pressures from the
  // double-float recovery.
  // With a2=gamma p/rho, ca2=B_idim^2/rho, bt2=B_perp^2/rho, b2=ca2+bt2:
  // cf^2-cs^2 = sqrt((a2-b2)^2+4 a2 bt2), cs^2 = a2 ca2/cf^2, and
  // a2-cs^2, cf^2-a2 are formed as a sum of positive terms or from the
  // identity (x+y)(x-y) = 4 a2 bt2; af^2 = 0 where the speeds coincide,
  // as the reference's clipping of 0/0 gives.
  static __device__ __forceinline__ void average_mhd_f32(const SweepArgs& a,
                                                         const R* wL,
                                                         const R* wR, int d,
                                                         double smallp,
                                                         Face& f, R* bd) {
    const float rL = wL[0], rR = wR[0];
    const float irL = 1.0f / rL, irR = 1.0f / rR;
    const float rho = 0.5f * (rL + rR);
    float v[NDIR], B[NDIR];
#pragma unroll
    for (int c = 0; c < NDIR; c++) {
      v[c] = 0.5f * (wL[1 + c] * irL + wR[1 + c] * irR);
      B[c] = 0.5f * (wL[B0 + 1 + c] + wR[B0 + 1 + c]);
      f.v[c] = v[c];
    }
    const float sp = float(smallp);
    float pL = PH::template pthermal_f<NDIR, MHD>(wL, a.ph);
    float pR = PH::template pthermal_f<NDIR, MHD>(wR, a.ph);
    pL = pL >= sp ? pL : sp;
    pR = pR >= sp ? pR : sp;
    if (a.ph.roe_dpprim) {
      f.dp = pR - pL;
    } else {
      // (g-1)*(de - v.dm + v^2/2 drho - d(B^2)/2) with d(B^2) as a sum of
      // (bR-bL)(bR+bL): the differences of nearby FP32 values are exact
      float s1 = 0.0f, s2 = 0.0f, s3 = 0.0f;
#pragma unroll
      for (int c = 0; c < NDIR; c++) {
        s1 = fmaf(v[c], wR[1 + c] - wL[1 + c], s1);
        s2 = fmaf(v[c], v[c], s2);
        const float bR = wR[B0 + 1 + c], bL = wL[B0 + 1 + c];
        s3 = fmaf(bR - bL, bR + bL, s3);
      }
      f.dp = a.ph.gm1f * ((wR[E] - wL[E]) - s1 + 0.5f * s2 * (rR - rL) -
                          0.5f * s3);
    }
    f.rhodv = (wR[1 + d] - wL[1 + d]) - v[d] * (rR - rL);
    const float irho = 1.0f / rho;
    const float p = 0.5f * (pL + pR);
    const float a2 = a.ph.gammaf * p * irho;
    const float ca2 = B[d] * B[d] * irho;
    float bt2 = 0.0f;
#pragma unroll
    for (int c = 0; c < NDIR; c++)
      if (c != d) bt2 = fmaf(B[c], B[c], bt2);
    bt2 = bt2 * irho;
    const float b2 = ca2 + bt2;
    const float dd = a2 - b2;
    const float x4 = 4.0f * a2 * bt2;
    const float Dr = sqrtf(fmaf(dd, dd, x4));
    const float cf2 = 0.5f * (a2 + b2 + Dr);
    const float cs2s = cf2 > 0.0f ? a2 * ca2 / cf2 : 0.0f;
    const float na = dd >= 0.0f ? 0.5f * (dd + Dr) : x4 / (2.0f * (Dr - dd));
    const float ns = dd <= 0.0f ? 0.5f * (Dr - dd) : x4 / (2.0f * (Dr + dd));
    const float iDr = Dr > 0.0f ? 1.0f / Dr : 0.0f;
    float af2 = Dr > 0.0f ? na * iDr : 0.0f;
    float as2 = Dr > 0.0f ? ns * iDr : 1.0f;
    af2 = fminf(1.0f, fmaxf(af2, 0.0f));
    as2 = fminf(1.0f, fmaxf(as2, 0.0f));
    f.cs2 = a2;
    f.cf = sqrtf(cf2);
    f.cs = sqrtf(cs2s);
    f.af = sqrtf(af2);
    f.as = sqrtf(as2);
    const float sr = sqrtf(rho);
    f.sr = sr;
    const int I = dir_i(d), J = dir_j(d);
    float bI = B[I], bJ = NDIR == 3 ? B[J] : 0.0f;
    if (NDIR == 2) {
      bI = bI >= 0.0f ? 1.0f : -1.0f;
    } else {
      const float t = sqrtf(bI * bI + bJ * bJ);
      if (t > 1.0e-30f) {
        const float it = 1.0f / t;
        bI = bI * it;
        bJ = bJ * it;
      } else {
        bI = 0.70710678f;
        bJ = 0.70710678f;
      }
    }
    float bi = B[d];
    if (fabsf(bi) < 1.0e-30f) bi = 1.0e-30f;
#pragma unroll
    for (int c = 0; c < NDIR; c++) f.b[c] = B[c];
    f.b[d] = bi;
    f.b[I] = bI;
    if (NDIR == 3) f.b[J] = bJ;
    // bdv, bdb of the fast/slow and the Alfven waves
    const float dvI = wR[1 + I] * irR - wL[1 + I] * irL;
    const float dbI = wR[B0 + 1 + I] - wL[B0 + 1 + I];
    float bdv = bI * dvI, bdb = bI * dbI;
    if (NDIR == 3) {
      const float dvJ = wR[1 + J] * irR - wL[1 + J] * irL;
      const float dbJ = wR[B0 + 1 + J] - wL[B0 + 1 + J];
      bdv = fmaf(bJ, dvJ, bdv);
      bdb = fmaf(bJ, dbJ, bdb);
      bd[2] = (bJ * dvI - bI * dvJ) * 0.5f * rho;
      bd[3] = (bJ * dbI - bI * dbJ) * 0.5f * copysignf(sr, bi);
    }
    bd[0] = bdv * copysignf(rho, bi);
    bd[1] = bdb * sqrtf(a2) * sr;
  }

  // average (src/vacphys.mhdroe.t:4-127, src/vacphys.hdroe.t:4-45) and the
  // waves of tvdlimit2's il loop.
  static __device__ __forceinline__ void decompose(const SweepArgs& a,
                                                   const R* wL, const R* wR,
                                                   int d, double smallp, D qdt,
                                                   R dxs, Face& f, D* am) {
    // FP64 path: the reference's statements in double.  Mixed path: the
    // MHD average in FP32 with cancellation-free forms (average_mhd_f32),
    // the HD average in double.
    const D rL = wL[0], rR = wR[0];
    const double dL = rL, dR = rR;
    R bd[4] = {R(0), R(0), R(0), R(0)};
    if constexpr (MHD && sizeof(R) == 4) {
      average_mhd_f32(a, wL, wR, d, smallp, f, bd);
    } else if constexpr (MHD) {
      const double rho = 0.5 * (dL + dR);
      double B[NDIR];
#pragma unroll
      for (int c = 0; c < NDIR; c++) {
        f.v[c] = D(0.5) * (wL[1 + c] / rL + wR[1 + c] / rR);
        B[c] = 0.5 * ((double)wL[B0 + 1 + c] + (double)wR[B0 + 1 + c]);
      }
      const double pL = pthd(a, wL, smallp), pR = pthd(a, wR, smallp);
      const double p = 0.5 * (pL + pR);
      if (a.ph.roe_dpprim) {
        f.dp = D(pR - pL);
      } else {
        // (g-1)*(de - v.dm + v^2/2 drho - d(B^2)/2), conservative form
        double s1, s2, s3;
#pragma unroll
        for (int c = 0; c < NDIR; c++) {
          const double vc = f.v[c];
          const double t1 = vc * ((double)wR[1 + c] - (double)wL[1 + c]);
          const double bR = wR[B0 + 1 + c], bL = wL[B0 + 1 + c];
          if (c == 0) {
            s1 = t1;
            s2 = vc * vc;
            s3 = bR * bR - bL * bL;
          } else {
            s1 = s1 + t1;
            s2 = s2 + vc * vc;
            s3 = s3 + bR * bR - bL * bL;
          }
        }
        f.dp = D(a.ph.gm1 * ((double)wR[E] - (double)wL[E] - s1 +
                             0.5 * s2 * (dR - dL) - 0.5 * s3));
      }
      f.rhodv = D((double)wR[1 + d] - (double)wL[1 + d] -
                  (double)f.v[d] * (dR - dL));
      const double cs2 = a.ph.gamma * p / rho;
      double bb = B[0] * B[0];
#pragma unroll
      for (int c = 1; c < NDIR; c++) bb = bb + B[c] * B[c];
      double cf = bb / rho + cs2;
      const double bi = B[d];
      const double q = 0.5 * (cf - sqrt(cf * cf - 4.0 * cs2 * (bi * bi) / rho));
      double cs = 0.0 > q ? 0.0 : q;
      cf = cf - cs;
      double af = (cs2 - cs) / (cf - cs);
      af = af > 0.0 ? af : 0.0;
      af = 1.0 < af ? 1.0 : af;
      f.as = D(sqrt(1.0 - af));
      f.af = D(sqrt(af));
      f.cf = D(sqrt(cf));
      f.cs = D(sqrt(cs));
      f.cs2 = D(cs2);
      f.sr = D(sqrt(rho));
      const int I = dir_i(d), J = dir_j(d);
      if (NDIR == 2) {
        B[I] = B[I] >= 0.0 ? 1.0 : -1.0;
      } else {
        const double t = sqrt(B[I] * B[I] + B[J] * B[J]);
        if (t > 1.0e-99) {
          B[I] = B[I] / t;
          B[J] = B[J] / t;
        } else {
          B[I] = sqrt(0.5);
          B[J] = sqrt(0.5);
        }
      }
#pragma unroll
      for (int c = 0; c < NDIR; c++) f.b[c] = D(B[c]);
      // avoid sgn(b_idim)==0
      if (fabs(f.b[d]) < tiny()) f.b[d] = tiny();
      // bdv, bdb of the fast/slow waves (src/vacphys.mhdroe.t:155-170) and
      // of the Alfven waves (:172-184)
      const D dvI = wR[1 + I] / rR - wL[1 + I] / rL;
      const D dbI = wR[B0 + 1 + I] - wL[B0 + 1 + I];
      D bdv = f.b[I] * dvI;
      D bdb = f.b[I] * dbI;
      if (NDIR == 3) {
        const D dvJ = wR[1 + J] / rR - wL[1 + J] / rL;
        const D dbJ = wR[B0 + 1 + J] - wL[B0 + 1 + J];
        bdv = bdv + f.b[J] * dvJ;
        bdb = bdb + f.b[J] * dbJ;
        D av = f.b[J] * dvI - f.b[I] * dvJ;
        D ab = f.b[J] * dbI - f.b[I] * dbJ;
        bd[2] = av * D(0.5) * (f.sr * f.sr);
        bd[3] = ab * D(0.5) * fsign(f.sr, f.b[d]);
      }
      bd[0] = bdv * fsign(f.sr * f.sr, f.b[d]);
      bd[1] = bdb * sqrt(f.cs2) * f.sr;
    } else {
      const double t0 = sqrt(dL), t2 = sqrt(dR);
      const double sr = t0 * t2;
      f.sr = D(sr);
      const double t = t0 / t2;
      double v[NDIR];
#pragma unroll
      for (int c = 0; c < NDIR; c++) {
        v[c] = ((double)wL[1 + c] / dL * t + (double)wR[1 + c] / dR) / (1.0 + t);
        f.v[c] = D(v[c]);
      }
      const double pL = pthd(a, wL, smallp), pR = pthd(a, wR, smallp);
      const double hL = (pL + (double)wL[E]) / dL;
      const double hR = (pR + (double)wR[E]) / dR;
      const double h = (hL * t + hR) / (1.0 + t);
      f.h = D(h);
      double vv = v[0] * v[0];
#pragma unroll
      for (int c = 1; c < NDIR; c++) vv = vv + v[c] * v[c];
      double c2 = a.ph.gm1 * (h - 0.5 * vv);
      const double c2min = a.ph.gamma * smallp / sr;
      c2 = c2min > c2 ? c2min : c2;
      f.dp = D((pR - pL) / c2);
      const double c = sqrt(c2);
      f.cs = D(c);
      f.rhodv = D(((double)wR[1 + d] / dR - (double)wL[1 + d] / dL) / c);
    }
    wave<0>(a, wL, wR, d, smallp, qdt, dxs, bd, f, am);
    wave<1>(a, wL, wR, d, smallp, qdt, dxs, bd, f, am);
    wave<2>(a, wL, wR, d, smallp, qdt, dxs, bd, f, am);
    if (NW > 3) wave<(NW > 3 ? 3 : 0)>(a, wL, wR, d, smallp, qdt, dxs, bd, f, am);
    if (NW > 4) wave<(NW > 4 ? 4 : 0)>(a, wL, wR, d, smallp, qdt, dxs, bd, f, am);
    if (NW > 5) wave<(NW > 5 ? 5 : 0)>(a, wL, wR, d, smallp, qdt, dxs, bd, f, am);
    if (NW > 6) wave<(NW > 6 ? 6 : 0)>(a, wL, wR, d, smallp, qdt, dxs, bd, f, am);
    if (NW > 7) wave<(NW > 7 ? 7 : 0)>(a, wL, wR, d, smallp, qdt, dxs, bd, f, am);
  }

  // R(iw,il)*q at the Roe state (rtimes, src/vacphys.mhdroe.t:284-449 and
  // src/vacphys.hdroe.t:144-215)
  template <int iw, int il>
  static __device__ __forceinline__ R rtimes(const SweepArgs& a, const Face& f,
                                             R q, int d) {
    const R v = f.v[d];
    if (MHD) {
      const int I = dir_i(d), J = dir_j(d);
      if (iw == 0) {
        if (il <= 1) return q * f.af;
        if (il <= 3) return q * f.as;
        if (il == 4) return q;
        return R(0);
      }
      if (iw == E) {
        R vv, v2a2;
        if constexpr (sizeof(R) == 4) {
          vv = f.vv;
          v2a2 = f.v2a2;
        } else {
          vv = f.v[0] * f.v[0];
#pragma unroll
          for (int c = 1; c < NDIR; c++) vv = vv + f.v[c] * f.v[c];
          const R g = R(a.ph.gamma);
          v2a2 = R(0.5) * vv + (R(2) - g) / R(a.ph.gm1) * f.cs2;
        }
        R bv;
        if (il < 6) {
          bv = f.b[I] * f.v[I];
          if (NDIR == 3) bv = bv + f.b[J] * f.v[J];
          if constexpr (sizeof(R) == 4)
            bv = bv * f.sgn;
          else
            bv = bv * R(fsign(1.0, f.b[d]));
        } else {
          bv = f.b[J] * f.v[I] - f.b[I] * f.v[J];
        }
        switch (il) {
          case 0:
            return q * (-f.as * f.cs * bv + f.af * (v2a2 + f.cf * (f.cf + v)));
          case 1:
            return q * (+f.as * f.cs * bv + f.af * (v2a2 + f.cf * (f.cf - v)));
          case 2:
            return q * (+f.af * f.cf * bv + f.as * (v2a2 + f.cs * (f.cs + v)));
          case 3:
            return q * (-f.af * f.cf * bv + f.as * (v2a2 + f.cs * (f.cs - v)));
          case 4:
            return q * R(0.5) * vv;
          case 5:
            return a.ph.divbwave ? q * f.b[d] : R(0);
          case 6:
            return +q * bv;
          default:
            return -q * bv;
        }
      }
      if (iw <= NDIR) {
        const int c = iw - 1;
        const R vw = f.v[c];
        if (c == d) {
          switch (il) {
            case 0: return q * f.af * (vw + f.cf);
            case 1: return q * f.af * (vw - f.cf);
            case 2: return q * f.as * (vw + f.cs);
            case 3: return q * f.as * (vw - f.cs);
            case 4: return q * vw;
            default: return R(0);
          }
        }
        const R bw = f.b[c];
        R sg;
        if constexpr (sizeof(R) == 4)
          sg = f.sgn;
        else
          sg = R(fsign(1.0, f.b[d]));
        switch (il) {
          case 0: return q * (f.af * vw - f.as * f.cs * bw * sg);
          case 1: return q * (f.af * vw + f.as * f.cs * bw * sg);
          case 2: return q * (f.as * vw + f.af * f.cf * bw * sg);
          case 3: return q * (f.as * vw - f.af * f.cf * bw * sg);
          case 4: return q * vw;
          case 5: return R(0);
          case 6: return c == I ? +q * f.b[J] : -q * f.b[I];
          default: return c == I ? -q * f.b[J] : +q * f.b[I];
        }
      }
      const int c = iw - B0 - 1;
      if (c == d) return (il == 5 && a.ph.divbwave) ? q : R(0);
      const R bw = f.b[c];
      if constexpr (sizeof(R) == 4) {
        switch (il) {
          case 0:
          case 1:
            return +q * f.as * (f.csr * bw);
          case 2:
          case 3:
            return -q * f.af * (f.csr * bw);
          case 4:
          case 5:
            return R(0);
          default:
            if (c == I) return -q * f.b[J] * f.isrs;
            return +q * f.b[I] * f.isrs;
        }
      }
      switch (il) {
        case 0:
        case 1:
          return +q * f.as * sqrt(f.cs2) * bw / f.sr;
        case 2:
        case 3:
          return -q * f.af * sqrt(f.cs2) * bw / f.sr;
        case 4:
        case 5:
          return R(0);
        default:
          if (c == I) return -q * f.b[J] / R(fsign(f.sr, f.b[d]));
          return +q * f.b[I] / R(fsign(f.sr, f.b[d]));
      }
    } else {
      const bool shear = il >= 3;
      int idir = il - 3;
      if (idir >= d) idir++;
      if (iw == 0) return shear ? R(0) : q;
      if (iw == E) {
        switch (il) {
          case 0: return q * (f.h + v * f.cs);
          case 1: return q * (f.h - v * f.cs);
          case 2: {
            R vv = f.v[0] * f.v[0];
#pragma unroll
            for (int k = 1; k < NDIR; k++) vv = vv + f.v[k] * f.v[k];
            return q * R(0.5) * vv;
          }
          default: return q * f.v[idir];
        }
      }
      const int c = iw - 1;
      if (c == d) {
        if (il == 0) return q * (v + f.cs);
        if (il == 1) return q * (v - f.cs);
        if (il == 2) return q * v;
        return R(0);
      }
      if (shear) return c == idir ? q : R(0);
      return q * f.v[c];
    }
  }

  // One face in direction d between cell o (G index ci) and o+s: the
  // central flux of the face states and the Roe decomposition.
  static __device__ __forceinline__ void face(const SweepArgs& a,
                                              const T* __restrict__ w1,
                                              const T* __restrict__ base,
                                              long long o, long long s, int d,
                                              int ci, R smallp, double qsmallp,
                                              D qdt, bool limit, R* F, Face& f,
                                              D* am) {
    R wL[NW], wR[NW];
    S::face_states(a, w1, base, o, s, smallp, limit, wL, wR);
    R fL[NW], fR[NW];
    PH::template flux<NDIR, MHD>(wL, d, a.ph, smallp, fL);
    PH::template flux<NDIR, MHD>(wR, d, a.ph, smallp, fR);
#pragma unroll
    for (int iw = 0; iw < NW; iw++) F[iw] = R(0.5) * (fL[iw] + fR[iw]);
    const R dxs = PH::dx(a.a, d, ci) + PH::dx(a.a, d, ci + 1);
    decompose(a, wL, wR, d, qsmallp, qdt, dxs, f, am);
  }

  // dvolume(ix) = dx_1*dx_2*dx_3 (gridsetup1, src/vacgrid.t:573-576)
  static __device__ __forceinline__ R dvol(const SweepArgs& a, const int* c) {
    R v = PH::dx(a.a, 0, c[0]);
    if (NDIM > 1) v = v * PH::dx(a.a, 1, c[1]);
    if (NDIM > 2) v = v * PH::dx(a.a, 2, c[2]);
    return v;
  }

  // Face pass of direction d (a compile-time constant, so that the face
  // state and the Roe quantities stay in registers): once per face, the
  // central flux and, wave by wave, the dissipative fluxes
  // R(iw,il)*phi(il)*(dvolume(i)+dvolume(j))/4, with setnoflux applied to
  // both ('symm0' mesh faces), into buf[k*nf+f] (k = iw for the central
  // flux, NW+il*NW+iw for the dissipative ones); plus the CFL maxima of
  // the two fast waves.
  template <int NT, int d>
  static __device__ void face_pass(const SweepArgs& a, const T* __restrict__ w1,
                                   const T* __restrict__ base,
                                   R* __restrict__ buf) {
    __shared__ unsigned long long shk[NT / 32];
    Ctrl* ctrl = a.ctrl;
    if (ctrl->done) return;
    const DevGrid& g = a.g;
    const long long nf = face_count(g, d);
    const long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long key[2] = {0ULL, 0ULL};
    if (f < nf) {
      int cl[3];
      face_left_cell(g, d, f, cl);
      const long long st[3] = {1, g.P, g.plane};
      const long long o = gidx(g, cl[0], cl[1], cl[2]);
      const bool limit = a.ph.typefull != VACGPU_TVDMU1;
      Face fs;
      R F[NW];
      D am[2];
      face(a, w1, base, o, st[d], d, cl[d], R(ctrl->smallp), ctrl->smallp,
           ctrl->dt, limit, F, fs, am);
      if (a.ph.courantpar > 0.0) {
        key[0] = dkey((double)am[0]);
        key[1] = dkey((double)am[1]);
      }
      const int nof = cl[d] == 1 ? a.ph.noflux[d][0]
                      : cl[d] == g.nx[d] + 1 ? a.ph.noflux[d][1] : 0;
#pragma unroll
      for (int iw = 0; iw < NW; iw++)
        buf[iw * nf + f] = ((nof >> iw) & 1) ? R(0) : F[iw];
      if constexpr (sizeof(R) == 4) {
        // mixed path: the limiter functions and the Roe state the right
        // eigenvectors need; the cell pass forms R(iw,il)*phi(il)
        store_face(fs, nf, f, buf);
      } else {
        // FP64 path: the dissipative fluxes themselves (their right
        // eigenvectors take double divisions the cell pass need not repeat)
        int cr[3] = {cl[0], cl[1], cl[2]};
        cr[d] = cl[d] + 1;
        const R vf = dvol(a, cr) + dvol(a, cl);  // dvolume(j)+dvolume(i)
        store_waves<0>(a, fs, d, vf, nof, nf, f, buf);
        store_waves<1>(a, fs, d, vf, nof, nf, f, buf);
        store_waves<2>(a, fs, d, vf, nof, nf, f, buf);
        if (NW > 3) store_waves<(NW > 3 ? 3 : 0)>(a, fs, d, vf, nof, nf, f, buf);
        if (NW > 4) store_waves<(NW > 4 ? 4 : 0)>(a, fs, d, vf, nof, nf, f, buf);
        if (NW > 5) store_waves<(NW > 5 ? 5 : 0)>(a, fs, d, vf, nof, nf, f, buf);
        if (NW > 6) store_waves<(NW > 6 ? 6 : 0)>(a, fs, d, vf, nof, nf, f, buf);
        if (NW > 7) store_waves<(NW > 7 ? 7 : 0)>(a, fs, d, vf, nof, nf, f, buf);
      }
    }
    if (a.ph.courantpar > 0.0) {
#pragma unroll
      for (int k = 0; k < 2; k++) {
        const unsigned long long kk = block_max_key<NT>(key[k], shk);
        if (threadIdx.x == 0 && kk) {
          unsigned long long* slot = k == 0 ? &ctrl->face_cmax[d][blockIdx.x % NSLOT]
                                            : &ctrl->face_cmax2[d][blockIdx.x % NSLOT];
          atomic_max_key(slot, kk);
        }
      }
    }
  }
  // wave il's dissipative flux of variable iw at one face
  template <int il, int iw>
  static __device__ __forceinline__ void store_wave_var(const SweepArgs& a,
                                                        const Face& fs, int d,
                                                        R vf, int nof,
                                                        long long nf,
                                                        long long f, R* buf) {
    R r = rtimes<iw, il>(a, fs, fs.phi[il], d) * R(0.25) * vf;
    if ((nof >> iw) & 1) r = R(0);
    buf[(long long)(NW + il * NW + iw) * nf + f] = r;
  }
  template <int il>
  static __device__ __forceinline__ void store_waves(const SweepArgs& a,
                                                     const Face& fs, int d,
                                                     R vf, int nof, long long nf,
                                                     long long f, R* buf) {
    store_wave_var<il, 0>(a, fs, d, vf, nof, nf, f, buf);
    store_wave_var<il, 1>(a, fs, d, vf, nof, nf, f, buf);
    store_wave_var<il, 2>(a, fs, d, vf, nof, nf, f, buf);
    if (NW > 3) store_wave_var<il, (NW > 3 ? 3 : 0)>(a, fs, d, vf, nof, nf, f, buf);
    if (NW > 4) store_wave_var<il, (NW > 4 ? 4 : 0)>(a, fs, d, vf, nof, nf, f, buf);
    if (NW > 5) store_wave_var<il, (NW > 5 ? 5 : 0)>(a, fs, d, vf, nof, nf, f, buf);
    if (NW > 6) store_wave_var<il, (NW > 6 ? 6 : 0)>(a, fs, d, vf, nof, nf, f, buf);
    if (NW > 7) store_wave_var<il, (NW > 7 ? 7 : 0)>(a, fs, d, vf, nof, nf, f, buf);
  }

  // The mixed path's face record after the central flux: phi of every wave
  // and the Roe state of rtimes (MHD: v, b, sr, cf, cs, af, as, cs2; HD:
  // v, h, cs), at buf[(NW+k)*nf+f].
  static constexpr int NFF = MHD ? 2 * NDIR + 6 : NDIR + 2;
  static __device__ __forceinline__ void store_face(const Face& fs, long long nf,
                                                    long long f, R* buf) {
    R* b = buf + (long long)NW * nf + f;
    int k = 0;
#pragma unroll
    for (int il = 0; il < NW; il++) b[(k++) * nf] = fs.phi[il];
#pragma unroll
    for (int c = 0; c < NDIR; c++) b[(k++) * nf] = fs.v[c];
    if (MHD) {
#pragma unroll
      for (int c = 0; c < NDIR; c++) b[(k++) * nf] = fs.b[c];
      b[(k++) * nf] = fs.sr;
      b[(k++) * nf] = fs.cf;
      b[(k++) * nf] = fs.cs;
      b[(k++) * nf] = fs.af;
      b[(k++) * nf] = fs.as;
      b[(k++) * nf] = fs.cs2;
    } else {
      b[(k++) * nf] = fs.h;
      b[(k++) * nf] = fs.cs;
    }
  }
  static __device__ __forceinline__ void load_face(const R* buf, long long nf,
                                                   long long f, Face& fs) {
    const R* b = buf + (long long)NW * nf + f;
    int k = 0;
#pragma unroll
    for (int il = 0; il < NW; il++) fs.phi[il] = b[(k++) * nf];
#pragma unroll
    for (int c = 0; c < NDIR; c++) fs.v[c] = b[(k++) * nf];
    if (MHD) {
#pragma unroll
      for (int c = 0; c < NDIR; c++) fs.b[c] = b[(k++) * nf];
      fs.sr = b[(k++) * nf];
      fs.cf = b[(k++) * nf];
      fs.cs = b[(k++) * nf];
      fs.af = b[(k++) * nf];
      fs.as = b[(k++) * nf];
      fs.cs2 = b[(k++) * nf];
    } else {
      fs.h = b[(k++) * nf];
      fs.cs = b[(k++) * nf];
    }
  }
  // wave il's dissipative fluxes of every variable from the two faces' records
  // (the mixed path: the face's scale 0.25*(dvolume_i+dvolume_j)/dvolume
  // multiplies instead of one division per wave and variable)
  template <int il, int iw>
  static __device__ __forceinline__ void dissipate_var(
      const SweepArgs& a, const Face& fm, const Face& fp, int d, R sm, R sp,
      int nofm, int nofp, R* acc) {
    R rp = rtimes<iw, il>(a, fp, fp.phi[il], d) * sp;
    R rm = rtimes<iw, il>(a, fm, fm.phi[il], d) * sm;
    if ((nofp >> iw) & 1) rp = R(0);
    if ((nofm >> iw) & 1) rm = R(0);
    acc[iw] = acc[iw] + (rp - rm);
  }
  template <int il>
  static __device__ __forceinline__ void dissipate(const SweepArgs& a,
                                                   const Face& fm,
                                                   const Face& fp, int d,
                                                   R sm, R sp, int nofm,
                                                   int nofp, R* acc) {
    dissipate_var<il, 0>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    dissipate_var<il, 1>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    dissipate_var<il, 2>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    if (NW > 3) dissipate_var<il, (NW > 3 ? 3 : 0)>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    if (NW > 4) dissipate_var<il, (NW > 4 ? 4 : 0)>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    if (NW > 5) dissipate_var<il, (NW > 5 ? 5 : 0)>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    if (NW > 6) dissipate_var<il, (NW > 6 ? 6 : 0)>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    if (NW > 7) dissipate_var<il, (NW > 7 ? 7 : 0)>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
  }
  // the per-face constants of rtimes on the mixed path
  static __device__ __forceinline__ void prep_face(const SweepArgs& a, int d,
                                                   Face& f) {
    R vv = f.v[0] * f.v[0];
#pragma unroll
    for (int c = 1; c < NDIR; c++) vv = vv + f.v[c] * f.v[c];
    f.vv = vv;
    if (MHD) {
      f.sgn = copysignf(1.0f, f.b[d]);
      const R isr = R(1) / f.sr;
      f.isrs = f.sgn * isr;
      f.csr = sqrtf(f.cs2) * isr;
      f.v2a2 = R(0.5) * vv + a.ph.c2gf * f.cs2;
    }
  }
  // one direction of the mixed path's cell pass (compile-time d keeps the
  // two face records in registers)
  template <int d>
  static __device__ __forceinline__ void dissipate_dir(const SweepArgs& a,
                                                       const R* buf,
                                                       long long nf,
                                                       long long fm_i,
                                                       long long fp_i,
                                                       const int* c, R dv0,
                                                       R* acc) {
    Face fm, fp;
    load_face(buf, nf, fm_i, fm);
    load_face(buf, nf, fp_i, fp);
    prep_face(a, d, fm);
    prep_face(a, d, fp);
    int cn[3] = {c[0], c[1], c[2]};
    cn[d] = c[d] - 1;
    const R vm = dv0 + dvol(a, cn);  // dvolume(j)+dvolume(i), lower face
    cn[d] = c[d] + 1;
    const R vp = dvol(a, cn) + dv0;  // and upper face
    const R q = R(0.25) / dv0;
    const R sm = vm * q, sp = vp * q;
    const int nofp = c[d] == a.g.nx[d] + 1 ? a.ph.noflux[d][1] : 0;
    const int nofm = c[d] == 2 ? a.ph.noflux[d][0] : 0;
    dissipate<0>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    dissipate<1>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    dissipate<2>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    if (NW > 3) dissipate<(NW > 3 ? 3 : 0)>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    if (NW > 4) dissipate<(NW > 4 ? 4 : 0)>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    if (NW > 5) dissipate<(NW > 5 ? 5 : 0)>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    if (NW > 6) dissipate<(NW > 6 ? 6 : 0)>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
    if (NW > 7) dissipate<(NW > 7 ? 7 : 0)>(a, fm, fp, d, sm, sp, nofm, nofp, acc);
  }

  // Cell pass: per direction the central fluxes of all variables
  // (addflux with qdt), then wave by wave the dissipative fluxes (addflux
  // with qdt=-1: += (F(i+1/2)-F(i-1/2))/dvolume), then the sources.
  static __device__ void correct(const SweepArgs& a, const T* __restrict__ w,
                                 const T* __restrict__ w1,
                                 T* __restrict__ wout) {
    const Ctrl* ctrl = a.ctrl;
    if (ctrl->done) return;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.g.ncell) return;
    int c[3];
    cell_coords(a.g, n, c);
    const long long off = gidx(a.g, c[0], c[1], c[2]);
    const long long st[3] = {1, a.g.P, a.g.plane};
    const long long vs = a.g.vs;
    const double qdt = ctrl->dt;
    const R smallp = R(ctrl->smallp);
    R acc[NW];
#pragma unroll
    for (int iw = 0; iw < NW; iw++) acc[iw] = R(w[off + iw * vs]);
    if (a.ph.useprim && a.ph.typefull != VACGPU_TVDMU1) {
      // the limiter base (the state) leaves upwindLR round-tripped
      S::to_prim(a, smallp, acc);
      S::to_cons(a, acc);
    }
    const R dv0 = dvol(a, c);
    for (int d = a.d0; d <= a.d1; d++) {
      const R* buf = (const R*)a.faces + (long long)(d - a.d0) * a.face_stride;
      const long long nf = face_count(a.g, d);
      int cm[3] = {c[0], c[1], c[2]};
      cm[d] = c[d] - 1;
      const long long fm = face_index(a.g, d, cm), fp = face_index(a.g, d, c);
      const R cq = PH::qdx(qdt, a.a, d, c[d]);
#pragma unroll
      for (int iw = 0; iw < NW; iw++)
        acc[iw] = acc[iw] - cq * (buf[iw * nf + fp] - buf[iw * nf + fm]);
      if constexpr (sizeof(R) == 4) {
        if (d == 0)
          dissipate_dir<0>(a, buf, nf, fm, fp, c, dv0, acc);
        else if (NDIM > 1 && d == 1)
          dissipate_dir<(NDIM > 1 ? 1 : 0)>(a, buf, nf, fm, fp, c, dv0, acc);
        else if (NDIM > 2)
          dissipate_dir<(NDIM > 2 ? 2 : 0)>(a, buf, nf, fm, fp, c, dv0, acc);
      } else {
#pragma unroll
        for (int il = 0; il < NW; il++)
#pragma unroll
          for (int iw = 0; iw < NW; iw++) {
            const R* r = buf + (long long)(NW + il * NW + iw) * nf;
            acc[iw] = acc[iw] + (r[fp] - r[fm]) / dv0;
          }
      }
    }
    if (a.ph.sourceunsplit && !a.ph.src_hook) {
      R wc[NW];
#pragma unroll
      for (int iw = 0; iw < NW; iw++) wc[iw] = R(w1[off + iw * vs]);
      S::add_sources(a, S::src_qdt(a, qdt), wc, w1 + off, st,
                     c, acc);
    }
#pragma unroll
    for (int iw = 0; iw < NW; iw++) wout[off + iw * vs] = T(acc[iw]);
  }
};

template <class PH, int NDIM, int NDIR, bool MHD, int D>
__global__ void __launch_bounds__(128)
    k_roe_face(SweepArgs a, const typename PH::T* __restrict__ w1,
               const typename PH::T* __restrict__ base,
               typename PH::R* __restrict__ buf) {
  RoeSweep<PH, NDIM, NDIR, MHD>::template face_pass<128, D>(a, w1, base, buf);
}

// (the mixed cell pass is held to 128 registers: 4 CTAs per SM)
template <class PH, int NDIM, int NDIR, bool MHD>
__global__ void __launch_bounds__(128, sizeof(typename PH::R) == 4 ? 4 : 1)
    k_correct_roe(SweepArgs a, const typename PH::T* __restrict__ w,
                  const typename PH::T* __restrict__ w1,
                  typename PH::T* __restrict__ wout) {
  RoeSweep<PH, NDIM, NDIR, MHD>::correct(a, w, w1, wout);
}

template <class PH, int NDIM, int NDIR, bool MHD>
void launch_roe_instance(const SweepArgs& a, const typename PH::T* w,
                         const typename PH::T* w1, const typename PH::T* base,
                         typename PH::T* wout, cudaStream_t st) {
  for (int d = a.d0; d <= a.d1; d++) {
    typename PH::R* buf =
        (typename PH::R*)a.faces + (long long)(d - a.d0) * a.face_stride;
    const unsigned nbf = grid_for(face_count(a.g, d), 128);
    if (d == 0)
      k_roe_face<PH, NDIM, NDIR, MHD, 0><<<nbf, 128, 0, st>>>(a, w1, base, buf);
    else if (NDIM > 1 && d == 1)
      k_roe_face<PH, NDIM, NDIR, MHD, (NDIM > 1 ? 1 : 0)><<<nbf, 128, 0, st>>>(a, w1, base, buf);
    else if (NDIM > 2)
      k_roe_face<PH, NDIM, NDIR, MHD, (NDIM > 2 ? 2 : 0)><<<nbf, 128, 0, st>>>(a, w1, base, buf);
  }
  k_correct_roe<PH, NDIM, NDIR, MHD><<<grid_for(a.g.ncell, 128), 128, 0, st>>>(a, w, w1, wout);
}

// (ndim, ndir, physics) instances; the MHD Roe solver needs ndir >= 2
// (src/vacphys.mhdroe.t:25)
template <class PH>
void launch_correct_roe(const SweepArgs& a, const typename PH::T* w,
                        const typename PH::T* w1, const typename PH::T* base,
                        typename PH::T* wout, cudaStream_t st) {
#define KC(D, C, M) launch_roe_instance<PH, D, C, M>(a, w, w1, base, wout, st)
  if (a.mhd) {
    if (a.g.ndim == 2 && a.ndir == 2) KC(2, 2, true);
    else if (a.g.ndim == 2 && a.ndir == 3) KC(2, 3, true);
    else if (a.g.ndim == 3 && a.ndir == 3) KC(3, 3, true);
  } else {
    if (a.g.ndim == 1 && a.ndir == 1) KC(1, 1, false);
    else if (a.g.ndim == 2 && a.ndir == 2) KC(2, 2, false);
    else if (a.g.ndim == 2 && a.ndir == 3) KC(2, 3, false);
    else if (a.g.ndim == 3 && a.ndir == 3) KC(3, 3, false);
  }
#undef KC
}

}  // namespace vacgpu

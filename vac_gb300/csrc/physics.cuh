// physics.cuh - pointwise ideal-MHD / gamma-law HD physics of VAC 4.52 for
// the device, on one state vector u[NW] (conservative variables).
//
// The FP64 functions keep every Fortran array statement of the reference as
// the same sequence of IEEE operations (this header is compiled without FMA
// contraction for the FP64 path), so each value is bit-identical to the CPU
// restatement.  Variable layout (src/vacpar.t.mhd:9-26, src/vacpar.t.hd:9-26):
//   rho=0, m_c=c (c=1..NDIR), e=NDIR+1, b_c=NDIR+1+c.
#pragma once
#include <cuda_runtime.h>

#include "vacgpu_internal.h"

namespace vacgpu {

template <int NDIR, bool MHD>
struct Lay {
  static constexpr int NW = MHD ? 2 + 2 * NDIR : 2 + NDIR;
  static constexpr int RHO = 0;
  static constexpr int M0 = 0;
  static constexpr int E = NDIR + 1;
  static constexpr int B0 = NDIR + 1;
};

// Constant sub-expressions of gamma live in DevPhys, evaluated once on the
// host in FP64 with the same operations the reference applies (so they are
// the same bits): pt1 = one-half*gamma, gm1 = gamma-one,
// pt3 = half*(gamma-one).
typedef DevPhys PhysConst;

// ------------------------------------------------------------------ FP64

// getptotal, src/vacphys0.t.mhd:225-257 (unclipped total pressure)
template <int NDIR>
__device__ __forceinline__ double ptotal_mhd(const double* u,
                                             const PhysConst& k) {
  typedef Lay<NDIR, true> L;
  double bb = u[L::B0 + 1] * u[L::B0 + 1];
#pragma unroll
  for (int c = 2; c <= NDIR; c++) bb = bb + u[L::B0 + c] * u[L::B0 + c];
  double p = k.pt1 * bb;
  p = p + k.gm1 * u[L::E];
  double mm = u[1] * u[1];
#pragma unroll
  for (int c = 2; c <= NDIR; c++) mm = mm + u[c] * u[c];
  p = p - k.pt3 * mm / u[0];
  return p;
}

// getpthermal, src/vacphys0.t.mhd:165-222 (before clipping)
template <int NDIR>
__device__ __forceinline__ double pthermal_mhd_raw(const double* u,
                                                   const PhysConst& k) {
  typedef Lay<NDIR, true> L;
  double mm = u[1] * u[1];
#pragma unroll
  for (int c = 2; c <= NDIR; c++) mm = mm + u[c] * u[c];
  double p = mm / u[0];
#pragma unroll
  for (int c = 1; c <= NDIR; c++) p = p + u[L::B0 + c] * u[L::B0 + c];
  return k.gm1 * (u[L::E] - 0.5 * p);
}

// getpthermal, src/vacphys0.t.hd:103-134 (before clipping)
template <int NDIR>
__device__ __forceinline__ double pthermal_hd_raw(const double* u,
                                                  const PhysConst& k) {
  typedef Lay<NDIR, false> L;
  double mm = u[1] * u[1];
#pragma unroll
  for (int c = 2; c <= NDIR; c++) mm = mm + u[c] * u[c];
  return k.gm1 * (u[L::E] - 0.5 * mm / u[0]);
}

__device__ __forceinline__ double clip_p(double p, double smallp) {
  return (p >= smallp) ? p : smallp;
}

template <int NDIR, bool MHD>
__device__ __forceinline__ double pthermal_raw(const double* u,
                                               const PhysConst& k) {
  if (MHD) return pthermal_mhd_raw<NDIR>(u, k);
  return pthermal_hd_raw<NDIR>(u, k);
}

// getcmax, src/vacphys0.t.mhd:79-116 (fast speed) / src/vacphys0.t.hd:72-100
template <int NDIR, bool MHD>
__device__ __forceinline__ double cmax_fn(const double* u, int idim,
                                          const PhysConst& k, double smallp) {
  typedef Lay<NDIR, MHD> L;
  if (MHD) {
    double p = clip_p(pthermal_mhd_raw<NDIR>(u, k), smallp);
    double cs2 = k.gamma * p / u[0];
    double bb = u[L::B0 + 1] * u[L::B0 + 1];
#pragma unroll
    for (int c = 2; c <= NDIR; c++) bb = bb + u[L::B0 + c] * u[L::B0 + c];
    double cf2 = bb / u[0] + cs2;
    double bi = u[L::B0 + 1 + idim];
    return sqrt(0.5 * (cf2 + sqrt(cf2 * cf2 - 4.0 * cs2 * (bi * bi) / u[0]))) +
           fabs(u[1 + idim] / u[0]);
  } else {
    double p = clip_p(pthermal_hd_raw<NDIR>(u, k), smallp);
    double cs = sqrt(k.gamma * p / u[0]);
    return cs + fabs(u[1 + idim] / u[0]);
  }
}

// getflux + transport term, src/vacphys.mhd0.t:149-205 and
// src/vacphys.t.hd:49-75; the transport flux v*w is added after the
// non-transport part as in hancock/tvdmusclf (src/vactvdlf.t:67-70,220-223).
template <int NDIR, bool MHD>
__device__ __forceinline__ void flux_fn(const double* u, int idim,
                                        const PhysConst& k, double smallp,
                                        double* f) {
  typedef Lay<NDIR, MHD> L;
  const double rho = u[0];
  const double v = u[1 + idim] / rho;
  if (MHD) {
    const double pt = ptotal_mhd<NDIR>(u, k);
    const double bi = u[L::B0 + 1 + idim];
    f[0] = 0.0 + v * u[0];
#pragma unroll
    for (int c = 1; c <= NDIR; c++) {
      double bk = u[L::B0 + c];
      double fk = (c == idim + 1) ? pt - bk * bi : -bk * bi;
      f[c] = fk + v * u[c];
    }
    double bm = u[L::B0 + 1] * u[1];
#pragma unroll
    for (int c = 2; c <= NDIR; c++) bm = bm + u[L::B0 + c] * u[c];
    f[L::E] = (u[1 + idim] * pt - bi * bm) / rho + v * u[L::E];
#pragma unroll
    for (int c = 1; c <= NDIR; c++) {
      if (c == idim + 1)
        f[L::B0 + c] = 0.0;
      else
        f[L::B0 + c] = -u[c] / rho * bi + v * u[L::B0 + c];
    }
  } else {
    const double p = clip_p(pthermal_hd_raw<NDIR>(u, k), smallp);
    f[0] = 0.0 + v * u[0];
#pragma unroll
    for (int c = 1; c <= NDIR; c++) {
      double fk = (c == idim + 1) ? p : 0.0;
      f[c] = fk + v * u[c];
    }
    f[L::E] = u[1 + idim] / rho * p + v * u[L::E];
  }
}

// Fortran MAX/MIN of two values, written as the same selects the CPU oracle
// uses so that even the sign of a zero result agrees.
__device__ __forceinline__ double fmax2(double a, double b) {
  return a > b ? a : b;
}
__device__ __forceinline__ double fmin2(double a, double b) {
  return a < b ? a : b;
}

// dwlimiter2, src/vacgrid.t:938-996: a = dw(i+1/2), b = dw(i-1/2)
__device__ __forceinline__ double limiter_fn(int lim, double a, double b) {
  const double s = copysign(1.0, a);
  switch (lim) {
    case LIM_WOODWARD: {
      double m = fmin2(fmin2(fabs(a), s * b), s * 0.25 * (b + a));
      return 2.0 * s * fmax2(0.0, m);
    }
    case LIM_SUPERBEE: {
      double x = fmin2(2.0 * fabs(a), s * b);
      double y = fmin2(fabs(a), 2.0 * s * b);
      return s * fmax2(fmax2(0.0, x), y);
    }
    case LIM_VANLEER:
      return 2.0 * fmax2(b * a, 0.0) / (a + b + 1.0e-12);
    case LIM_ALBADA:
      return (b * (a * a + 1.0e-12) + a * (b * b + 1.0e-12)) /
             (a * a + b * b + 2.0e-12);
    default:
      return s * fmax2(0.0, fmin2(fabs(a), s * b));
  }
}

// The FP64 physics policy of the sweep templates (sweep_fp64.cu,
// roe_fp64.cu): storage and arithmetic in IEEE double.
struct PH64 {
  typedef double T;
  typedef double R;
  static __device__ __forceinline__ R limiter(int lim, R a, R b) {
    return limiter_fn(lim, a, b);
  }
  template <int NDIR, bool MHD>
  static __device__ __forceinline__ void flux(const R* u, int d,
                                              const DevPhys& k, R smallp,
                                              R* f) {
    flux_fn<NDIR, MHD>(u, d, k, smallp, f);
  }
  template <int NDIR, bool MHD>
  static __device__ __forceinline__ R cmax(const R* u, int d,
                                           const DevPhys& k, R smallp) {
    return cmax_fn<NDIR, MHD>(u, d, k, smallp);
  }
  template <int NDIR, bool MHD>
  static __device__ __forceinline__ double pthermal_raw(const R* u,
                                                        const DevPhys& k) {
    return vacgpu::pthermal_raw<NDIR, MHD>(u, k);
  }
  // dx(ix,idim) (gridsetup1, src/vacgrid.t:527-530)
  static __device__ __forceinline__ R dx(const DevArrays& a, int d, int i) {
    return a.dx[d][i];
  }
  // qdt/dx(ix,idim) of addflux (src/vacgrid.t:676-677)
  static __device__ __forceinline__ R qdx(double qdt, const DevArrays& a,
                                          int d, int i) {
    return qdt / a.dx[d][i];
  }
  // cmaxC*two/(dx(ixC)+dx(jxC)) (src/vactvdlf.t:188-190)
  static __device__ __forceinline__ double cfl(R cm, const DevArrays& a,
                                               int d, int i) {
    return cm * 2.0 / (a.dx[d][i] + a.dx[d][i + 1]);
  }
  // cmax/dx of getdt_courant (src/vac.t:701-702)
  static __device__ __forceinline__ double cell_ratio(R cm,
                                                      const DevArrays& a,
                                                      int d, int i) {
    return cm / a.dx[d][i];
  }
  static __device__ __forceinline__ R mul_qg(double qdt, double g) {
    return qdt * g;
  }
  static __device__ __forceinline__ R qdiv(double q) { return q; }
};

}  // namespace vacgpu

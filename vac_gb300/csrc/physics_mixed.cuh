// physics_mixed.cuh - pointwise MHD/HD physics of the mixed-precision path:
// FP32 state, fluxes and wave speeds; the thermal-pressure recovery
// p = (g-1)(e - m^2/(2 rho) - B^2/2) is evaluated at double precision.
//
// The recovery is where low-beta and high-Mach cells cancel
// catastrophically (e is dominated by the magnetic or kinetic energy), so
// its result must be accurate relative to p, not to e.  Three evaluations
// are provided:
//   PREC_FF   double-float arithmetic: each square is split exactly with the
//             FMA-based TwoProduct, the (non-negative) sums use Dekker's
//             Fast2Sum on the ordered pair, m^2/rho is a FP32 quotient plus
//             an FMA-computed remainder correction (Dekker 1971; Ogita, Rump
//             & Oishi 2005), and e - S/2 is one FMA, exact where it cancels.
//             Accurate to a few ulps of p itself; runs on the FP32 pipes.
//   PREC_F64  the same expression in native IEEE double on the FP64 pipe.
//   PREC_F32  plain FP32 (reference for the error study only).
// Total pressure uses ptot = p + B^2/2, which equals the reference's
// (1-g/2)B^2 + (g-1)e - (g-1)/2 m^2/rho (src/vacphys0.t.mhd:225-257).
#pragma once
#include <cuda_runtime.h>

#include "physics.cuh"

namespace vacgpu {

enum { PREC_F32 = 0, PREC_FF = 1, PREC_F64 = 2 };

__device__ __forceinline__ void two_prod(float a, float b, float& p,
                                         float& e) {
  p = a * b;
  e = fmaf(a, b, -p);
}
// s + e = a + b exactly for a, b >= 0 (Dekker's Fast2Sum on the ordered
// pair: the larger operand first).
__device__ __forceinline__ void two_sum_pos(float a, float b, float& s,
                                            float& e) {
  const float hi = fmaxf(a, b), lo = fminf(a, b);
  s = hi + lo;
  e = lo - (s - hi);
}

// Thermal pressure (unclipped) and the magnetic energy density B^2/2 of a
// FP32 state.  MHD when NB>0 (NB = number of field components).
template <int NDIR, int NB, int PM>
__device__ __forceinline__ float pressure_mixed(const float* u, float rinv,
                                                float gm1, float* half_bb) {
  const int E = NDIR + 1;
  if (PM == PREC_F64) {
    double rho = u[0];
    double mm = (double)u[1] * u[1], bb = 0.0;
#pragma unroll
    for (int c = 2; c <= NDIR; c++) mm = fma((double)u[c], (double)u[c], mm);
#pragma unroll
    for (int c = 1; c <= NB; c++)
      bb = fma((double)u[E + c], (double)u[E + c], bb);
    double r = (double)rinv;
    double q = mm * r;
    q = fma(fma(-q, rho, mm), r, q);  // one Newton step on mm/rho
    *half_bb = (float)(0.5 * bb);
    return (float)((double)gm1 * ((double)u[E] - 0.5 * (q + bb)));
  } else if (PM == PREC_FF) {
    // sums of squares as unevaluated pairs (hi + lo), all terms >= 0
    float mh, ml;
    two_prod(u[1], u[1], mh, ml);
#pragma unroll
    for (int c = 2; c <= NDIR; c++) {
      float ph, pl, t;
      two_prod(u[c], u[c], ph, pl);
      two_sum_pos(mh, ph, mh, t);
      ml = ml + (pl + t);
    }
    // q = mm/rho: FP32 quotient, exact FMA remainder, corrected low part
    float qh = mh * rinv;
    float rem = fmaf(-qh, u[0], mh);
    float ql = (rem + ml) * rinv;
    float sh = qh, sl = ql;
    if (NB > 0) {
      float bh, bl;
      two_prod(u[E + 1], u[E + 1], bh, bl);
#pragma unroll
      for (int c = 2; c <= NB; c++) {
        float ph, pl, t;
        two_prod(u[E + c], u[E + c], ph, pl);
        two_sum_pos(bh, ph, bh, t);
        bl = bl + (pl + t);
      }
      *half_bb = 0.5f * (bh + bl);
      float t;
      two_sum_pos(qh, bh, sh, t);
      sl = ql + bl + t;
    } else {
      *half_bb = 0.0f;
    }
    // e - (sh + sl)/2: the FMA is exact where the subtraction cancels
    // (e and sh/2 within a factor 2, Sterbenz) and rounds to the nearest
    // float of a result no smaller than sh/2 otherwise
    float d = fmaf(-0.5f, sh, u[E]);
    d = fmaf(-0.5f, sl, d);
    return gm1 * d;
  } else {
    float mm = u[1] * u[1], bb = 0.0f;
#pragma unroll
    for (int c = 2; c <= NDIR; c++) mm = fmaf(u[c], u[c], mm);
#pragma unroll
    for (int c = 1; c <= NB; c++) bb = fmaf(u[E + c], u[E + c], bb);
    *half_bb = 0.5f * bb;
    return gm1 * (u[E] - 0.5f * (mm * rinv + bb));
  }
}

template <int PM>
struct PHMixed {
  typedef float T;
  typedef float R;

  static __device__ __forceinline__ float limiter(int lim, float a, float b) {
    const float s = copysignf(1.0f, a);
    switch (lim) {
      case LIM_WOODWARD: {
        float m = fminf(fminf(fabsf(a), s * b), s * 0.25f * (b + a));
        return 2.0f * s * fmaxf(0.0f, m);
      }
      case LIM_SUPERBEE: {
        float x = fminf(2.0f * fabsf(a), s * b);
        float y = fminf(fabsf(a), 2.0f * s * b);
        return s * fmaxf(fmaxf(0.0f, x), y);
      }
      case LIM_VANLEER:
        return 2.0f * fmaxf(b * a, 0.0f) / (a + b + 1.0e-12f);
      case LIM_ALBADA:
        return fmaf(b, fmaf(a, a, 1.0e-12f), a * fmaf(b, b, 1.0e-12f)) /
               (fmaf(a, a, b * b) + 2.0e-12f);
      default:
        return s * fmaxf(0.0f, fminf(fabsf(a), s * b));
    }
  }

  // getflux + transport (src/vacphys.mhd0.t:149-205, src/vacphys.t.hd:49-75)
  template <int NDIR, bool MHD>
  static __device__ __forceinline__ void flux(const float* u, int d,
                                              const DevPhys& k, float smallp,
                                              float* f) {
    float p, rinv;
    flux_p<NDIR, MHD>(u, d, k, smallp, f, p, rinv);
  }
  // the same, also returning the unclipped thermal pressure and 1/rho
  template <int NDIR, bool MHD>
  static __device__ __forceinline__ void flux_p(const float* u, int d,
                                                const DevPhys& k, float smallp,
                                                float* f, float& p_raw,
                                                float& rinv_out) {
    const int E = NDIR + 1;
    const float rinv = 1.0f / u[0];
    const float v = u[1 + d] * rinv;
    float hbb;
    float p = pressure_mixed<NDIR, MHD ? NDIR : 0, PM>(u, rinv, k.gm1f,
                                                       &hbb);
    p_raw = p;
    rinv_out = rinv;
    if (MHD) {
      const float pt = p + hbb;
      const float bi = u[E + 1 + d];
      f[0] = v * u[0];
#pragma unroll
      for (int c = 1; c <= NDIR; c++) {
        float bk = u[E + c];
        float fk = (c == d + 1) ? pt - bk * bi : -bk * bi;
        f[c] = fmaf(v, u[c], fk);
      }
      float bm = u[E + 1] * u[1];
#pragma unroll
      for (int c = 2; c <= NDIR; c++) bm = fmaf(u[E + c], u[c], bm);
      f[E] = fmaf(fmaf(u[1 + d], pt, -(bi * bm)), rinv, v * u[E]);
#pragma unroll
      for (int c = 1; c <= NDIR; c++) {
        if (c == d + 1)
          f[E + c] = 0.0f;
        else
          f[E + c] = fmaf(v, u[E + c], -(u[c] * rinv * bi));
      }
    } else {
      p = p >= smallp ? p : smallp;
      f[0] = v * u[0];
#pragma unroll
      for (int c = 1; c <= NDIR; c++) {
        float fk = (c == d + 1) ? p : 0.0f;
        f[c] = fmaf(v, u[c], fk);
      }
      f[E] = v * (p + u[E]);
    }
  }

  // getcmax (src/vacphys0.t.mhd:79-116, src/vacphys0.t.hd:72-100).  The
  // discriminant cf2^2-4cs2 b_i^2/rho can round below zero in FP32; it is
  // clamped at zero here (the FP64 path keeps the reference's expression).
  // Sums of two products are written as explicit FMAs (here and in the
  // fluxes): left to the compiler, which product it fuses can differ from
  // one kernel to another, and the batched and single-grid kernels must
  // round alike.
  template <int NDIR, bool MHD>
  static __device__ __forceinline__ float cmax(const float* u, int d,
                                               const DevPhys& k,
                                               float smallp) {
    const int E = NDIR + 1;
    const float rinv = 1.0f / u[0];
    float hbb;
    float p = pressure_mixed<NDIR, MHD ? NDIR : 0, PM>(u, rinv, k.gm1f,
                                                       &hbb);
    p = p >= smallp ? p : smallp;
    const float cs2 = k.gammaf * p * rinv;
    if (MHD) {
      const float cf2 = fmaf(2.0f * hbb, rinv, cs2);
      const float bi = u[E + 1 + d];
      float disc = fmaf(cf2, cf2, -(4.0f * cs2 * (bi * bi) * rinv));
      disc = disc > 0.0f ? disc : 0.0f;
      return sqrtf(0.5f * (cf2 + sqrtf(disc))) + fabsf(u[1 + d] * rinv);
    }
    return sqrtf(cs2) + fabsf(u[1 + d] * rinv);
  }

  // getcmax at the mean M of two states L, R whose unclipped thermal
  // pressures pL, pR and inverse densities riL, riR are known.  With
  // K = m^2/(2 rho) and B^2/2 the mean's pressure is, exactly,
  //   p(M) = (pL+pR)/2 + (g-1) (rhoL rhoR |vL-vR|^2 / (4 (rhoL+rhoR))
  //                             + |BL-BR|^2 / 8),
  // where rhoL rhoR |vL-vR|^2 = |rhoR mL - rhoL mR|^2 / (rhoL rhoR).  Both
  // corrections are non-negative, so p(M) keeps the accuracy of pL and pR
  // without a recovery of its own.  M is (L+R)/2 up to rounding.
  template <int NDIR, bool MHD>
  static __device__ __forceinline__ float cmax_mean(
      const float* L, const float* R, const float* M, float pL, float pR,
      float riL, float riR, int d, const DevPhys& k, float smallp) {
    const int E = NDIR + 1;
    const float rinv = 1.0f / M[0];
    float kk = 0.0f;
#pragma unroll
    for (int c = 1; c <= NDIR; c++) {
      const float t = fmaf(R[0], L[c], -(L[0] * R[c]));
      kk = fmaf(t, t, kk);
    }
    // 1/(4 (rhoL+rhoR)) = rinv/8 with rhoL+rhoR = 2 rho_M
    float corr = kk * (riL * riR) * (0.125f * rinv);
    float bb = 0.0f;
    if (MHD) {
      float db = 0.0f;
#pragma unroll
      for (int c = 1; c <= NDIR; c++) {
        const float t = L[E + c] - R[E + c];
        db = fmaf(t, t, db);
        bb = fmaf(M[E + c], M[E + c], bb);
      }
      corr = fmaf(0.125f, db, corr);
    }
    float p = fmaf(k.gm1f, corr, 0.5f * (pL + pR));
    p = p >= smallp ? p : smallp;
    const float cs2 = k.gammaf * p * rinv;
    if (MHD) {
      const float cf2 = fmaf(bb, rinv, cs2);
      const float bi = M[E + 1 + d];
      float disc = fmaf(cf2, cf2, -(4.0f * cs2 * (bi * bi) * rinv));
      disc = disc > 0.0f ? disc : 0.0f;
      return sqrtf(0.5f * (cf2 + sqrtf(disc))) + fabsf(M[1 + d] * rinv);
    }
    return sqrtf(cs2) + fabsf(M[1 + d] * rinv);
  }

  // thermal pressure (unclipped) with the path's recovery, as FP32
  template <int NDIR, bool MHD>
  static __device__ __forceinline__ float pthermal_f(const float* u,
                                                     const DevPhys& k) {
    float hbb;
    return pressure_mixed<NDIR, MHD ? NDIR : 0, PM>(u, 1.0f / u[0], k.gm1f,
                                                    &hbb);
  }

  template <int NDIR, bool MHD>
  static __device__ __forceinline__ double pthermal_raw(const float* u,
                                                        const DevPhys& k) {
    double rho = u[0], mm = 0.0, bb = 0.0;
    for (int c = 1; c <= NDIR; c++) mm += (double)u[c] * u[c];
    if (MHD)
      for (int c = 1; c <= NDIR; c++) bb += (double)u[NDIR + 1 + c] * u[NDIR + 1 + c];
    return k.gm1 * ((double)u[NDIR + 1] - 0.5 * (mm / rho + bb));
  }

  static __device__ __forceinline__ float dx(const DevArrays& a, int d,
                                             int i) {
    return a.dxf[d][i];
  }
  static __device__ __forceinline__ float qdx(double qdt, const DevArrays& a,
                                              int d, int i) {
    return (float)qdt / a.dxf[d][i];
  }
  static __device__ __forceinline__ double cfl(float cm, const DevArrays& a,
                                               int d, int i) {
    return (double)(cm * 2.0f / (a.dxf[d][i] + a.dxf[d][i + 1]));
  }
  static __device__ __forceinline__ double cell_ratio(float cm,
                                                      const DevArrays& a,
                                                      int d, int i) {
    return (double)(cm / a.dxf[d][i]);
  }
  static __device__ __forceinline__ float mul_qg(double qdt, double g) {
    return (float)(qdt * g);
  }
  static __device__ __forceinline__ float qdiv(double q) { return (float)q; }
};

}  // namespace vacgpu

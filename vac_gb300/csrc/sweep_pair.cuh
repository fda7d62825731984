// sweep_pair.cuh - the fused sweep of the mixed-precision path for 3-D grids
// with two cells per thread in Blackwell's packed FP32 arithmetic.
//
// One split sweep of VAC's twostep Hancock/TVDLF scheme (src/vac.t:363-572,
// src/vactvdlf.t:5-299): Hancock predictor w1 (src/vactvdlf.t:5-89), TVDLF
// corrector with the limited slopes of the base state
// (src/vactvdlf.t:92-299), Powell and gravity sources, CFL maximum and the
// ghost cells of the new state, in one kernel.  A CTA of 128 threads owns a
// 32x8 (y and z sweeps) or 30x8 (x sweep) column tile and marches through a
// chunk of planes along the marching axis; each state plane of the tile and
// its 2-cell halo arrives in shared memory by one TMA tensor copy, two
// planes ahead of use.  Every thread owns two cells adjacent along x, whose
// arithmetic runs as one stream of .f32x2 instructions (pack2.cuh): the
// flux, pressure-recovery, limiter and update arithmetic of a pair costs the
// instruction slots of one cell.
//
// y and z sweeps (the sweep axis is the marching axis): a thread carries its
// column's state, predictor and face values from plane to plane in
// registers, so the face between planes j-1 and j needs no shared memory;
// only the transverse magnetic components of the predictor, which div B of
// the neighbours reads, go through shared memory.
//
// x sweep (in-plane): the face between the cells of a pair is the thread's
// own; the face to the right neighbour takes the neighbour's face state by a
// warp shuffle, and so does the left face flux of the update.
//
// Numerics: the mixed path's FP32 state and fluxes with the double-float
// thermal-pressure recovery of physics_mixed.cuh (exact FMA products,
// compensated sums) in all four flux evaluations of a cell; the face's fast
// speed takes the mean state's pressure from the two face pressures (an
// exact identity).  The mean-state restore wLC = 2 mean - wR of
// src/vactvdlf.t:205 is an FP64 bit-parity device that changes nothing but a
// rounding in FP32 and is left out here.
#pragma once
#include <cuda.h>

#include "pack2.cuh"
#include "sweep_fused.cuh"

namespace vacgpu {

constexpr int PT_NT = 128;  // threads per CTA

// per-CTA shared memory of the pair sweep (floats): state ring + two planes
// of the predictor's transverse B components over the 36x10 region
__host__ __device__ constexpr int pair_smem_floats(int nw) {
  return FWRING * fused_slot_floats(nw, 0) + 2 * 2 * 36 * 10;
}

// ------------------------------------------------------- packed physics

struct PairK {  // per-launch constants, splatted
  f2 gm1, gamma, half, mhalf, quarter, eighth;
  f2 mone;  // -1: x * mone negates x in one packed multiply (exact, -0 for +0)
  float smallp;
};

// Dekker's error-free sum of non-negative terms: Fast2Sum on the
// lane-wise ordered pair (two min/max, three FP32 operations; measured a
// little faster than Knuth's branch-free six-operation TwoSum here).
__device__ __forceinline__ void p_tsum(f2 a, f2 b, f2& s, f2& e) {
  const f2 hi = vmax(a, b), lo = vmin(a, b);
  s = hi + lo;
  e = lo - (s - hi);
}

// a*a = h + l exactly (FMA TwoProduct)
__device__ __forceinline__ void p_tsq(f2 a, f2& h, f2& l, const PairK& k) {
  h = a * a;
  l = ffma(a, a, h * k.mone);
}

// Variables of a state with ND vector components: rho, m_1..m_ND (u[1..ND]),
// e (u[ND+1]), B_1..B_ND (u[ND+2..2ND+1], MHD).

// Thermal pressure (unclipped) in double-float arithmetic; hbb receives
// B^2/2 (MHD).  The same steps as pressure_mixed<.., PREC_FF>.
template <bool MHD, int ND = 3>
__device__ __forceinline__ f2 p_pressure(const f2* u, f2 rinv, const PairK& k,
                                         f2& hbb) {
  f2 mh, ml;
  p_tsq(u[1], mh, ml, k);
#pragma unroll
  for (int c = 2; c <= ND; c++) {
    f2 ph, pl, t;
    p_tsq(u[c], ph, pl, k);
    p_tsum(mh, ph, mh, t);
    ml = ml + (pl + t);
  }
  // mm/rho: FP32 quotient, exact FMA remainder, corrected low part
  const f2 qh = mh * rinv;
  const f2 rem = ffma(qh, u[0] * k.mone, mh);
  const f2 ql = (rem + ml) * rinv;
  f2 sh = qh, sl = ql;
  if (MHD) {
    f2 bh, bl;
    p_tsq(u[ND + 2], bh, bl, k);
#pragma unroll
    for (int c = ND + 3; c <= 2 * ND + 1; c++) {
      f2 ph, pl, t;
      p_tsq(u[c], ph, pl, k);
      p_tsum(bh, ph, bh, t);
      bl = bl + (pl + t);
    }
    hbb = k.half * (bh + bl);
    f2 t;
    p_tsum(qh, bh, sh, t);
    sl = ql + bl + t;
  }
  f2 d = ffma(k.mhalf, sh, u[ND + 1]);
  d = ffma(k.mhalf, sl, d);
  return k.gm1 * d;
}

// getflux + transport along DD (src/vacphys.mhd0.t:149-205,
// src/vacphys.t.hd:49-75); p: unclipped thermal pressure, rinv: 1/rho.
// f[rho] is m_DD itself (v rho up to a rounding).
template <int DD, bool MHD, int ND = 3>
__device__ __forceinline__ void p_flux(const f2* u, const PairK& k, f2* f,
                                       f2& p, f2& rinv) {
  constexpr int E = ND + 1;  // e; B_c is u[E + c]
  rinv = vrcp(u[0]);
  const f2 v = u[1 + DD] * rinv;
  f2 hbb;
  p = p_pressure<MHD, ND>(u, rinv, k, hbb);
  f[0] = u[1 + DD];
  if (MHD) {
    const f2 pt = p + hbb;
    const f2 nbi = u[E + 1 + DD] * k.mone;
#pragma unroll
    for (int c = 1; c <= ND; c++) {
      const f2 fk = c == DD + 1 ? ffma(u[E + c], nbi, pt) : u[E + c] * nbi;
      f[c] = ffma(v, u[c], fk);
    }
    f2 bm = u[E + 1] * u[1];
#pragma unroll
    for (int c = 2; c <= ND; c++) bm = ffma(u[E + c], u[c], bm);
    const f2 t = ffma(nbi, bm, u[1 + DD] * pt);
    f[E] = ffma(t, rinv, v * u[E]);
#pragma unroll
    for (int c = 1; c <= ND; c++) {
      if (c == DD + 1)
        f[E + c] = f2s(0.0f);
      else
        f[E + c] = ffma(v, u[E + c], (u[c] * rinv) * nbi);
    }
  } else {
    const f2 pc = vclamp_lo(p, k.smallp);
#pragma unroll
    for (int c = 1; c <= ND; c++) f[c] = c == DD + 1 ? ffma(v, u[c], pc) : v * u[c];
    f[E] = v * (pc + u[E]);
  }
}

// getcmax at the mean M of the face states L, R (unclipped pressures pL, pR,
// inverse densities riL, riR), as PHMixed::cmax_mean: the mean's pressure
// (pL+pR)/2 + (g-1)(|rhoR mL - rhoL mR|^2/(4 rhoL rhoR (rhoL+rhoR))
// + |BL-BR|^2/8) has no cancellation.  Only M's rho, m_DD and B are read.
template <int DD, bool MHD, int ND = 3>
__device__ __forceinline__ f2 p_cmax_mean(const f2* L, const f2* R,
                                          const f2* M, f2 pL, f2 pR, f2 riL,
                                          f2 riR, const PairK& k) {
  constexpr int B1 = ND + 2;  // B_1
  const f2 rinv = vrcp(M[0]);
  f2 kk;
#pragma unroll
  for (int c = 1; c <= ND; c++) {
    const f2 t = ffma(R[0], L[c], (L[0] * R[c]) * k.mone);
    kk = c == 1 ? t * t : ffma(t, t, kk);
  }
  f2 corr = kk * (riL * riR) * (k.eighth * rinv);
  f2 bb;
  if (MHD) {
    f2 db;
#pragma unroll
    for (int c = B1; c < B1 + ND; c++) {
      const f2 t = L[c] - R[c];
      db = c == B1 ? t * t : ffma(t, t, db);
      bb = c == B1 ? M[c] * M[c] : ffma(M[c], M[c], bb);
    }
    corr = ffma(k.eighth, db, corr);
  }
  f2 p = ffma(k.gm1, corr, k.half * (pL + pR));
  p = vclamp_lo(p, k.smallp);
  const f2 cs2 = k.gamma * p * rinv;
  const f2 va = vabs(M[1 + DD] * rinv);
  if (MHD) {
    const f2 cf2 = ffma(bb, rinv, cs2);
    const f2 bi = M[B1 + DD];
    const f2 q = cs2 * (bi * bi) * rinv;
    f2 disc = ffma(cf2, cf2, f2s(-4.0f) * q);
    disc = vmax(disc, f2s(0.0f));
    return vsqrt(k.half * (cf2 + vsqrt(disc))) + va;
  }
  return vsqrt(cs2) + va;
}

// Half the limited slope, dwlimiter2 (src/vacgrid.t:938-996) of
// a = dw(i+1/2), b = dw(i-1/2) times 1/2: minmod s max(0, min(|a|, s b))/2;
// woodward s max(0, min(|a|, s b, s (a+b)/4)), s = sign(1, a).  s is
// formed by bit operations (+-1 or +-1/2 with a's sign) and applied by
// exact multiplications, so the result equals 0.5 * the limiter's value
// bit for bit (powers of two scale without rounding).
template <int LIMC>
__device__ __forceinline__ f2 p_hlim(f2 a, f2 b, const PairK& k) {
  float al, ah, bl, bh;
  if (LIMC == LIMC_WOODWARD) {
    f2 s;
    s.v = (a.v & 0x8000000080000000ull) | 0x3f8000003f800000ull;  // +-1
    const f2 sb = b * s, sc = (a + b) * (s * k.quarter);
    float sbl, sbh, scl, sch;
    f2u(a, al, ah);
    f2u(sb, sbl, sbh);
    f2u(sc, scl, sch);
    const f2 r = f2m(fmaxf(0.0f, fminf(fminf(fabsf(al), sbl), scl)),
                     fmaxf(0.0f, fminf(fminf(fabsf(ah), sbh), sch)));
    return r * s;
  }
  const f2 sb = vxorsign(b, a);
  f2 sh;
  sh.v = (a.v & 0x8000000080000000ull) | 0x3f0000003f000000ull;  // +-1/2
  float sbl, sbh;
  f2u(a, al, ah);
  f2u(sb, sbl, sbh);
  const f2 r = f2m(fmaxf(0.0f, fminf(fabsf(al), sbl)), fmaxf(0.0f, fminf(fabsf(ah), sbh)));
  return r * sh;
}

// ------------------------------------------------------------ the kernel

// getboundary's ghost images of one new cell value per variable (scalar,
// one lane): the composition of the region copies of src/vacgrid.t:195-413
// as in Fused::ghost_images (NDIM = 2: gc[2] = 0 and no z images).
template <int NW, int NDIM = 3>
__device__ __forceinline__ void pair_ghost_images(const FusedArgs& a,
                                                  const int* gc, long long off,
                                                  const float* acc) {
  const DevGrid& g = a.g;
  int x1, x2, fx, y1 = 0, y2 = 0, fy = 0, z1 = 0, z2 = 0, fz = 0;
  typedef Fused<3, 0, true, PREC_FF, LIMC_MINMOD> FX;
  const int nx_ = 1 + FX::preimages(a, 0, gc[0], x1, fx, x2);
  const int ny_ = 1 + FX::preimages(a, 1, gc[1], y1, fy, y2);
  const int nz_ = NDIM == 3 ? 1 + FX::preimages(a, 2, gc[2], z1, fz, z2) : 1;
#pragma unroll 1
  for (int k = 0; k < nz_; k++) {
    const int pz = k == 0 ? gc[2] : (k == 1 ? z1 : z2);
    const int sz = k == 1 ? fz : 0;
#pragma unroll 1
    for (int jj = 0; jj < ny_; jj++) {
      const int py = jj == 0 ? gc[1] : (jj == 1 ? y1 : y2);
      const int sy = jj == 1 ? fy : 0;
      const long long orow =
          off + (long long)(pz - gc[2]) * g.plane + (long long)(py - gc[1]) * g.P;
#pragma unroll 1
      for (int i = 0; i < nx_; i++) {
        if ((i | jj | k) == 0) continue;
        const int px = i == 0 ? gc[0] : (i == 1 ? x1 : x2);
        const int fl = (i == 1 ? fx : 0) ^ sy ^ sz;
        const long long o = orow + (px - gc[0]);
#pragma unroll
        for (int v = 0; v < NW; v++) a.wout[o + v * g.vs] = ((fl >> v) & 1) ? -acc[v] : acc[v];
      }
    }
  }
}

// One split sweep along D of a 3-D grid, two cells per thread.  GEN:
// the general form (gravity, non-periodic faces, sources or the CFL
// maximum switched off); false: the common case -- every face periodic,
// unsplit sources with Powell's terms for MHD, no gravity, CFL maximum --
// with those decisions fixed at compile time.
template <int D, bool MHD, int LIMC, bool GEN>
struct PairSweep {
  static constexpr int K = D == 0 ? 0 : 2;        // in-plane / marching
  static constexpr int AM = D == 0 ? 2 : D;        // marching axis
  static constexpr int AR = D == 2 ? 1 : (D == 1 ? 2 : 1);  // tile-row axis
  static constexpr int NW = MHD ? 8 : 5;
  static constexpr int TX = K == 0 ? 30 : 32;      // output columns
  static constexpr int TY = 8;                     // output rows
  static constexpr int BPL = FB_X * 12;            // floats per variable plane
  static constexpr int SLOT = fused_slot_floats(NW, 0);
  static constexpr int WBO = K == 0 ? 3 : 2;       // column offset in w1b
  static constexpr int WBP = 36;                   // w1b row pitch
  static constexpr int WBC = WBP * 10;             // w1b component plane

  // transverse B of the predictor: component c (0: B_x, 1: B_AR) of plane p
  static __device__ __forceinline__ float* wb(float* sm, int p, int c, int ly, int lx) {
    return sm + FWRING * SLOT + ((p & 1) * 2 + c) * WBC + (ly + 1) * WBP + lx + WBO;
  }

  // Hancock predictor of the magnetic component B_k alone at a pair of
  // cells: F_D[B_k] = v_D B_k - v_k B_D at the two face states and the
  // Powell term of B_k; c, pp, mm: the five variables rho, m_D, m_k, B_D,
  // B_k at the cells, their upper and lower neighbours along D.  Every
  // operation is the one the full predictor does for B_k (p_flux, sources),
  // so a cell's value is the same bits whichever of the two computes it.
  // nqdivb: -qs * div B.
  static __device__ __forceinline__ f2 bflux(const f2* x, const PairK& k) {
    const f2 ri = vrcp(x[0]);
    const f2 v = x[1] * ri;
    return ffma(v, x[4], (x[2] * ri) * (x[3] * k.mone));
  }
  static __device__ __forceinline__ f2 predict_b(const f2* c, const f2* pp,
                                                 const f2* mm, f2 cq, f2 nqdivb,
                                                 bool powell, const PairK& k) {
    f2 uL[5], uR[5];
#pragma unroll
    for (int i = 0; i < 5; i++) {
      const f2 hl = p_hlim<LIMC>(pp[i] - c[i], c[i] - mm[i], k);
      uR[i] = c[i] - hl;
      uL[i] = c[i] + hl;
    }
    const f2 fR = bflux(uR, k), fL = bflux(uL, k);
    f2 out = ffma(cq, fR - fL, c[4]);
    if (powell) out = ffma(c[2], vrcp(c[0]) * nqdivb, out);
    return out;
  }

  // addsource2 with wCT = wc: gravity (specialsource), then Powell's terms
  // (addsource) for nq = -qs * div B.
  static __device__ __forceinline__ void sources(const FusedArgs& a, f2 qs,
                                                 const f2* wc, f2 nq, bool powell,
                                                 f2* acc) {
    if (GEN && a.ph.src_id == VACGPU_SRC_GRAVITY) {
#pragma unroll
      for (int d = 1; d <= 3; d++)
        if (a.gravf[d - 1] != 0.0f) acc[d] = ffma(qs * f2s(a.gravf[d - 1]), wc[0], acc[d]);
#pragma unroll
      for (int d = 1; d <= 3; d++)
        if (a.gravf[d - 1] != 0.0f) acc[4] = ffma(qs * f2s(a.gravf[d - 1]), wc[d], acc[4]);
    }
    if (MHD && powell) {
      const f2 t = vrcp(wc[0]) * nq;
      f2 mb = wc[1] * wc[5];
      mb = ffma(wc[2], wc[6], mb);
      mb = ffma(wc[3], wc[7], mb);
#pragma unroll
      for (int c = 1; c <= 3; c++) {
        acc[c] = ffma(wc[4 + c], nq, acc[c]);
        acc[4 + c] = ffma(wc[c], t, acc[4 + c]);
      }
      acc[4] = ffma(mb, t, acc[4]);
    }
  }

  // TVDLF face flux 2F = F(L) + F(R) - cmax (R - L) and cmax of a pair of
  // faces with left states L and right states R.
  static __device__ __forceinline__ f2 face(const f2* L, const f2* R,
                                            const PairK& k, f2* G) {
    f2 fL[NW], fR[NW], pL, pR, riL, riR;
    p_flux<D, MHD>(L, k, fL, pL, riL);
    p_flux<D, MHD>(R, k, fR, pR, riR);
    f2 M[NW];
    M[0] = k.half * (L[0] + R[0]);
    M[1 + D] = k.half * (L[1 + D] + R[1 + D]);
    if (MHD)
#pragma unroll
      for (int c = 5; c <= 7; c++) M[c] = k.half * (L[c] + R[c]);
    const f2 cm = p_cmax_mean<D, MHD>(L, R, M, pL, pR, riL, riR, k);
#pragma unroll
    for (int v = 0; v < NW; v++) G[v] = ffma(cm, L[v] - R[v], fL[v] + fR[v]);
    return cm;
  }

  // the new state of a pair of cells to HBM (lane-masked), with the ghost
  // images of cells within two cells of a mesh face; off: element offset of
  // the first cell, ghost-range coordinates gx (x), gr (row axis), gm
  // (marching axis); nearxr: the pair is within two cells of an x or
  // row-axis face
  static __device__ __forceinline__ void store(const FusedArgs& a, const f2* acc,
                                               long long off, int gx, int gr, int gm,
                                               bool nearxr, bool ok0, bool ok1) {
    const DevGrid& g = a.g;
    if (ok0 && ok1) {
#pragma unroll
      for (int v = 0; v < NW; v++) st2(a.wout + off + v * g.vs, acc[v]);
    } else {
#pragma unroll
      for (int v = 0; v < NW; v++) {
        float lo, hi;
        f2u(acc[v], lo, hi);
        if (ok0) a.wout[off + v * g.vs] = lo;
        if (ok1) a.wout[off + 1 + v * g.vs] = hi;
      }
    }
    if (!(nearxr || gm < 4 || gm >= g.nx[AM])) return;
    int gc[3];
    gc[0] = gx;
    gc[AR] = gr;
    gc[AM] = gm;
#pragma unroll 1
    for (int h = 0; h < 2; h++) {
      if (!(h ? ok1 : ok0)) continue;
      int c2[3] = {gc[0] + h, gc[1], gc[2]};
      bool near = false;
#pragma unroll
      for (int d = 0; d < 3; d++) near = near || c2[d] < 4 || c2[d] >= g.nx[d];
      if (!near) continue;
      float s[NW];
#pragma unroll
      for (int v = 0; v < NW; v++) s[v] = h ? f2hi(acc[v]) : f2lo(acc[v]);
      pair_ghost_images<NW>(a, c2, off + h, s);
    }
  }

  // per-variable ghost fix of a predictor value (getboundary on w1 at a
  // non-periodic face): src for the variables not periodic in that
  // dimension, negated where 'asymm'
  static __device__ __forceinline__ float gfix(float own, float src, int v, int pmask,
                                               int amask) {
    if ((pmask >> v) & 1) return own;
    return ((amask >> v) & 1) ? -src : src;
  }

  static __device__ bool run(const CUtensorMap* map, const FusedArgs& a, float* sm,
                             int bx, int by, int bz, unsigned long long* bars,
                             int* uses, unsigned slotid) {
    Ctrl* ctrl = a.ctrl;
    if (ctrl->done) return true;
    __shared__ float shq[PT_NT / 32];
    const int tid = threadIdx.x;
    const DevGrid& g = a.g;
    const int nX = g.nx[0], nR = g.nx[AR], nM = g.nx[AM];
    const int x0 = K == 0 ? bx * TX - 1 : bx * TX, y0 = by * TY;
    const int z0 = bz * a.nzc;
    const int z1 = min(z0 + a.nzc, nM);
    const double dtd = ctrl->dt;
    const float qdt = (float)dtd;
    const f2 qdt2 = f2s((float)(dtd / 2));
    const f2 nqs1h = f2s(-((float)(dtd / 2 / 3) * 0.5f));  // -predictor source x 1/2
    const f2 qs2 = f2s((float)(dtd / 3));               // corrector source
    const f2 nqs2h = f2s(-((float)(dtd / 3) * 0.5f));
    const f2 qs1 = f2s((float)(dtd / 2 / 3));
    PairK k;
    k.gm1 = f2s(a.ph.gm1f);
    k.gamma = f2s(a.ph.gammaf);
    k.half = f2s(0.5f);
    k.mhalf = f2s(-0.5f);
    k.quarter = f2s(0.25f);
    k.eighth = f2s(0.125f);
    k.mone = f2s(-1.0f);
    k.smallp = (float)ctrl->smallp;
    const bool powell = MHD && (!GEN || (a.ph.divbfix && a.ph.sourceunsplit));
    const bool srcs = !GEN || a.ph.sourceunsplit;
    const bool cfl = !GEN || a.cfl;
    const int cstart = x0 + g.xpad - 2;
    const int sh = cstart & 3;
    const int colx = cstart - sh;
    const unsigned plane_bytes = NW * BPL * 4;
    const int all = (1 << NW) - 1;

    const int pbase = z0 - 2;
    auto slot = [&](int p) -> float* { return sm + ((p - pbase) % FWRING) * SLOT; };
    auto issue = [&](int p) {
      const int q = p - pbase;
      fence_proxy_async();
      mbar_expect_tx(&bars[q % FWRING], plane_bytes);
      tma_load_plane(map, slot(p), &bars[q % FWRING], colx, y0, p + 2);
    };
    auto wait_plane = [&](int p) -> bool {
      const int q = p - pbase;
      return mbar_wait(&bars[q % FWRING], (uses[q % FWRING] + q / FWRING) & 1);
    };

    // this thread's pair: row ly, columns lx0, lx0+1 (box column bc)
    const int lane = tid & 31, hl = lane & 15;
    const int ly = 2 * (tid >> 5) + (lane >> 4);
    const int lx0 = K == 0 ? 2 * hl - 1 : 2 * hl;
    const int bc = lx0 + 4 + sh;  // even
    const int br = ly + 2;
    const int ix0 = x0 + lx0, iy = y0 + ly;
    const bool rowok = iy < nR;
    const bool ok0 = rowok && ix0 >= 0 && ix0 < nX && (K != 0 || lx0 >= 0);
    const bool ok1 = rowok && ix0 + 1 >= 0 && ix0 + 1 < nX && (K != 0 || lx0 + 1 < TX);
    // 1/dx along x per lane and along the row axis (ghost-range indices)
    const int gx0 = min(max(ix0 + 2, 0), g.nG[0] - 1), gx1 = min(ix0 + 3, g.nG[0] - 1);
    const f2 idxx = f2m(a.idxf[0][gx0], a.idxf[0][gx1]);
    const f2 idxy = f2s(a.idxf[AR][min(iy + 2, g.nG[AR] - 1)]);
    // in-plane sweep: CFL factors 2/(dx_i+dx_i+1) of the pair's two faces
    f2 cflx = f2s(0.0f);
    if (K == 0)
      cflx = f2m(2.0f / (a.dxf[0][gx0] + a.dxf[0][gx1]),
                 2.0f / (a.dxf[0][gx1] + a.dxf[0][min(ix0 + 4, g.nG[0] - 1)]));
    // ghost fixes of the predictor at non-periodic faces
    const bool fix_x = GEN && a.periodic_mask[0] != all && (x0 <= 0 || x0 + TX + 1 >= nX);
    const bool fix_r = GEN && a.periodic_mask[AR] != all && (y0 == 0 || y0 + TY >= nR);
    const bool fix_m = GEN && a.periodic_mask[AM] != all;
    // the pair's output offset at marching-axis ghost index 0, the stride
    // along that axis, and whether it lies within two cells of an x or
    // row-axis face (ghost images)
    int gco[3];
    gco[0] = ix0 + 2;
    gco[AR] = iy + 2;
    gco[AM] = 0;
    const long long obase = gidx(g, gco[0], gco[1], gco[2]);
    const long long sam = AM == 2 ? g.plane : g.P;
    const bool nearxr = gco[AR] < 4 || gco[AR] >= g.nx[AR] || gco[0] < 4 || gco[0] + 1 >= g.nx[0];

    f2 qmax = f2s(0.0f);
    if (tid == 0) {
      issue(z0 - 2);
      issue(z0 - 1);
      issue(z0);
    }
    // carried along the march (planes j-1 / j)
    f2 u0[NW];        // state of plane j (marching sweeps)
    f2 dbxc = f2s(0.0f);          // in-plane: the same of w1(j)
    f2 w1p[NW];       // predictor of plane j-1
    f2 hlp[NW];       // half limited slope of plane j-1 (marching sweeps)
    f2 Gp[NW];        // 2 x face flux: marching (j-2|j-1); in-plane dG of j-1
    f2 dbxp = f2s(0.0f);          // in-plane: B_x(x+1)-B_x(x-1) of w1(j-1)
    f2 bzm2 = f2s(0.0f), bzm1 = f2s(0.0f);  // B_AM of w1(j-2), w1(j-1)
#pragma unroll
    for (int v = 0; v < NW; v++) u0[v] = w1p[v] = hlp[v] = Gp[v] = f2s(0.0f);

    const int pfirst = z0 - 1, plast = z1;
    // 1/dx and dx along the marching axis at planes j-1 and j, and the
    // next plane's, loaded one plane ahead of use (ghost-range indices
    // j+1 .. j+3 stay below nG = nM + 4)
    float idzp = a.idxf[AM][pfirst + 1], dxzp = a.dxf[AM][pfirst + 1];
    float idzc = a.idxf[AM][pfirst + 2], dxzc = a.dxf[AM][pfirst + 2];
    for (int j = pfirst; j <= plast; j++) {
      const float idzn = a.idxf[AM][j + 3], dxzn = a.dxf[AM][j + 3];
      bool ok = true;
      if (j == pfirst) ok = wait_plane(j - 1) && wait_plane(j);
      ok = ok && wait_plane(j + 1);
      if (__syncthreads_or(!ok)) {  // barrier A
        if (tid == 0) {
          atomicExch(&ctrl->fault, 1);
          // the copies of planes j-1 .. j+1 may still be in flight: wait for
          // them, again with a bound, so none lands after the CTA exits
          for (int p = max(j - 1, pbase); p <= j + 1; p++) {
            const int q = p - pbase;
            mbar_wait(&bars[q % FWRING], (uses[q % FWRING] + q / FWRING) & 1, 1LL << 28);
          }
        }
        return false;
      }
      if (tid == 0 && j + 2 <= z1 + 1) issue(j + 2);
      const float* pm = slot(j - 1);
      const float* p0 = slot(j);
      const float* pp = slot(j + 1);
      const f2 idxz = f2s(idzc);
      const bool edge = j == z0 - 1 || j == z1;
      const bool ring = powell && !edge;  // planes updated later need the ring

      f2 w1[NW], hl_[NW];
      f2 bz = f2s(0.0f);
      if (K == 2) {
        // ---------------- marching sweep: predictor of the column pair
        f2 um[NW], up[NW];
#pragma unroll
        for (int v = 0; v < NW; v++) {
          um[v] = ld2(pm + v * BPL + br * FB_X + bc);
          up[v] = ld2(pp + v * BPL + br * FB_X + bc);
          u0[v] = ld2(p0 + v * BPL + br * FB_X + bc);
        }
        f2 uL[NW], uR[NW];
#pragma unroll
        for (int v = 0; v < NW; v++) {
          hl_[v] = p_hlim<LIMC>(up[v] - u0[v], u0[v] - um[v], k);
          uR[v] = u0[v] - hl_[v];
          uL[v] = u0[v] + hl_[v];
        }
        f2 fL[NW], fR[NW], pt_, ri_;
        p_flux<D, MHD>(uR, k, fR, pt_, ri_);
        p_flux<D, MHD>(uL, k, fL, pt_, ri_);
        const f2 cq = qdt2 * idxz;
#pragma unroll
        for (int v = 0; v < NW; v++) w1[v] = ffma(cq, fR[v] - fL[v], u0[v]);
        if (srcs) {
          f2 nqdivb = f2s(0.0f);
          if (powell) {
            const float* bxr = p0 + 5 * BPL + br * FB_X + bc;
            const float* byr = p0 + (5 + AR) * BPL + br * FB_X + bc;
            float cl, ch;
            f2u(u0[5], cl, ch);
            const f2 dbx = f2m(ch - bxr[-1], bxr[2] - cl);
            const f2 dby = ld2(byr + FB_X) - ld2(byr - FB_X);
            const f2 dbz = up[5 + AM] - um[5 + AM];
            const f2 divb = ffma(dbz, idxz, ffma(dby, idxy, dbx * idxx));
            nqdivb = nqs1h * divb;
          }
          sources(a, qs1, u0, nqdivb, powell, w1);
        }
        // marching-axis ghost planes: w1(-1) from w1(0), w1(n) from w1(n-1)
        if (fix_m && j == 0) {
#pragma unroll
          for (int v = 0; v < NW; v++) {
            float ol, oh, sl, sh2;
            f2u(w1p[v], ol, oh);
            f2u(w1[v], sl, sh2);
            w1p[v] = f2m(gfix(ol, sl, v, a.periodic_mask[AM], a.asymm_lo[AM]),
                         gfix(oh, sh2, v, a.periodic_mask[AM], a.asymm_lo[AM]));
          }
          bzm1 = w1p[5 + AM];
        }
        if (fix_m && j == nM) {
#pragma unroll
          for (int v = 0; v < NW; v++) {
            float ol, oh, sl, sh2;
            f2u(w1[v], ol, oh);
            f2u(w1p[v], sl, sh2);
            w1[v] = f2m(gfix(ol, sl, v, a.periodic_mask[AM], a.asymm_hi[AM]),
                        gfix(oh, sh2, v, a.periodic_mask[AM], a.asymm_hi[AM]));
          }
        }
        bz = w1[5 + AM];
        if (ring) {
          st2(wb(sm, j, 0, ly, lx0), w1[5]);
          st2(wb(sm, j, 1, ly, lx0), w1[5 + AR]);
          // transverse B of the ring: rows -1 and TY (warp 0, B_AR), columns
          // -1 and TX (warp 1, lanes 0-7, B_x)
          const int wq = tid >> 5;
          if (wq == 0 || (wq == 1 && lane < 8)) {
            const int kk = wq == 0 ? AR : 0;
            const int iv[5] = {0, 1 + D, 1 + kk, 5 + D, 5 + kk};
            f2 c[5], cp[5], cm_[5];
            int rr, cL, cH;  // box row, box columns of the two cells
            if (wq == 0) {
              rr = lane < 16 ? 1 : TY + 2;
              cL = bc;
              cH = bc + 1;
            } else {
              rr = lane + 2;
              cL = 3 + sh;
              cH = TX + 4 + sh;
            }
#pragma unroll
            for (int i = 0; i < 5; i++) {
              const int o = iv[i] * BPL + rr * FB_X;
              c[i] = f2m(p0[o + cL], p0[o + cH]);
              cp[i] = f2m(pp[o + cL], pp[o + cH]);
              cm_[i] = f2m(pm[o + cL], pm[o + cH]);
            }
            // div B of w at the two ring cells
            const float* b0 = p0 + 5 * BPL + rr * FB_X;
            const float* b1 = p0 + (5 + AR) * BPL + rr * FB_X;
            const float* b2p = pp + (5 + AM) * BPL + rr * FB_X;
            const float* b2m = pm + (5 + AM) * BPL + rr * FB_X;
            const f2 dbx = f2m(b0[cL + 1] - b0[cL - 1], b0[cH + 1] - b0[cH - 1]);
            const f2 dby = f2m(b1[cL + FB_X] - b1[cL - FB_X], b1[cH + FB_X] - b1[cH - FB_X]);
            const f2 dbz = f2m(b2p[cL] - b2m[cL], b2p[cH] - b2m[cH]);
            const int rl = rr - 2;
            const int gxl = min(max(x0 + cL - 4 - sh + 2, 0), g.nG[0] - 1);
            const int gxh = min(max(x0 + cH - 4 - sh + 2, 0), g.nG[0] - 1);
            const f2 ix_ = f2m(a.idxf[0][gxl], a.idxf[0][gxh]);
            const f2 iy_ = f2s(a.idxf[AR][min(max(y0 + rl + 2, 0), g.nG[AR] - 1)]);
            const f2 divb = ffma(dbz, idxz, ffma(dby, iy_, dbx * ix_));
            const f2 o = predict_b(c, cp, cm_, qdt2 * idxz, nqs1h * divb, true, k);
            if (wq == 0) {
              st2(wb(sm, j, 1, rl, lx0), o);
            } else {
              *wb(sm, j, 0, rl, -1) = f2lo(o);
              *wb(sm, j, 0, rl, TX) = f2hi(o);
            }
          }
        }
      } else {
        // ---------------- in-plane x sweep
        const int o0 = br * FB_X + bc;
        if (edge) {
          // planes outside the chunk: only B_AM of the predictor
          if (powell) {
            const int iv[5] = {0, 1, 1 + AM, 5, 5 + AM};
            f2 c[5], cp[5], cm_[5];
#pragma unroll
            for (int i = 0; i < 5; i++) {
              const float* r = p0 + iv[i] * BPL + o0;
              c[i] = ld2(r);
              cp[i] = f2m(r[1], r[2]);
              cm_[i] = f2m(r[-1], r[0]);
            }
            const float* bxr = p0 + 5 * BPL + o0;
            const f2 dbx = f2m(bxr[1] - bxr[-1], bxr[2] - bxr[0]);
            const float* byr = p0 + (5 + AR) * BPL + o0;
            const f2 dby = ld2(byr + FB_X) - ld2(byr - FB_X);
            const f2 dbz = ld2(pp + (5 + AM) * BPL + o0) - ld2(pm + (5 + AM) * BPL + o0);
            const f2 divb = ffma(dbz, idxz, ffma(dby, idxy, dbx * idxx));
            bz = predict_b(c, cp, cm_, qdt2 * idxx, nqs1h * divb, true, k);
          }
        } else {
          f2 u[NW], hlv[NW], dbx = f2s(0.0f);
#pragma unroll
          for (int v = 0; v < NW; v++) {
            // the pair and its neighbours shifted by one cell each way, so
            // the slopes and B_x(x+1)-B_x(x-1) are packed differences
            const float* r = p0 + v * BPL + o0;
            const f2 c = ld2(r);
            const f2 cl = f2m(r[-1], r[0]), cr = f2m(r[1], r[2]);
            const f2 dp = cr - c, dm = c - cl;
            if (v == 5) dbx = cr - cl;
            u[v] = c;
            hlv[v] = p_hlim<LIMC>(dp, dm, k);
          }
          f2 uL[NW], uR[NW];
#pragma unroll
          for (int v = 0; v < NW; v++) {
            uR[v] = u[v] - hlv[v];
            uL[v] = u[v] + hlv[v];
          }
          f2 fL[NW], fR[NW], pt_, ri_;
          p_flux<D, MHD>(uR, k, fR, pt_, ri_);
          p_flux<D, MHD>(uL, k, fL, pt_, ri_);
          const f2 cq = qdt2 * idxx;
#pragma unroll
          for (int v = 0; v < NW; v++) w1[v] = ffma(cq, fR[v] - fL[v], u[v]);
          if (srcs) {
            f2 nqdivb = f2s(0.0f);
            if (powell) {
              const float* byr = p0 + (5 + AR) * BPL + o0;
              const f2 dby = ld2(byr + FB_X) - ld2(byr - FB_X);
              const f2 dbz = ld2(pp + (5 + AM) * BPL + o0) - ld2(pm + (5 + AM) * BPL + o0);
              const f2 divb = ffma(dbz, idxz, ffma(dby, idxy, dbx * idxx));
              nqdivb = nqs1h * divb;
            }
            sources(a, qs1, u, nqdivb, powell, w1);
          }
          // x-face ghost cells of the region: w1(-1) from w1(0), w1(n) from
          // w1(n-1) (the pair's first cell has an even index)
          if (fix_x) {
#pragma unroll
            for (int v = 0; v < NW; v++) {
              float lo, hi;
              f2u(w1[v], lo, hi);
              const float dn = __shfl_down_sync(0xffffffffu, lo, 1, 16);
              const float upv = __shfl_up_sync(0xffffffffu, hi, 1, 16);
              const int pmk = a.periodic_mask[0];
              if (ix0 + 1 == -1) hi = gfix(hi, dn, v, pmk, a.asymm_lo[0]);
              if (ix0 == nX) lo = gfix(lo, upv, v, pmk, a.asymm_hi[0]);
              if (ix0 + 1 == nX) hi = gfix(hi, lo, v, pmk, a.asymm_hi[0]);
              w1[v] = f2m(lo, hi);
            }
          }
          bz = w1[5 + AM];
#pragma unroll
          for (int v = 0; v < NW; v++) hl_[v] = hlv[v];
          if (ring) {
            st2(wb(sm, j, 1, ly, lx0), w1[5 + AR]);
            if ((tid >> 5) == 0) {
              // B_y of the ring rows -1 and TY
              const int rr = lane < 16 ? 1 : TY + 2;
              const int rl = rr - 2;
              const int ob = rr * FB_X + bc;
              const int iv[5] = {0, 1, 1 + AR, 5, 5 + AR};
              f2 c[5], cp[5], cm_[5];
#pragma unroll
              for (int i = 0; i < 5; i++) {
                const float* r = p0 + iv[i] * BPL + ob;
                c[i] = ld2(r);
                cp[i] = f2m(r[1], r[2]);
                cm_[i] = f2m(r[-1], r[0]);
              }
              const float* bxr = p0 + 5 * BPL + ob;
              const f2 dbx2 = f2m(bxr[1] - bxr[-1], bxr[2] - bxr[0]);
              const float* byr = p0 + (5 + AR) * BPL + ob;
              const f2 dby = ld2(byr + FB_X) - ld2(byr - FB_X);
              const f2 dbz = ld2(pp + (5 + AM) * BPL + ob) - ld2(pm + (5 + AM) * BPL + ob);
              const f2 iy_ = f2s(a.idxf[AR][min(max(y0 + rl + 2, 0), g.nG[AR] - 1)]);
              const f2 divb = ffma(dbz, idxz, ffma(dby, iy_, dbx2 * idxx));
              st2(wb(sm, j, 1, rl, lx0), predict_b(c, cp, cm_, qdt2 * idxx, nqs1h * divb, true, k));
            }
          }
        }
        // marching-axis ghost planes of B_AM
        if (fix_m && j == 0) {
          float ol, oh, sl, sh2;
          f2u(bzm1, ol, oh);
          f2u(bz, sl, sh2);
          bzm1 = f2m(gfix(ol, sl, 5 + AM, a.periodic_mask[AM], a.asymm_lo[AM]),
                     gfix(oh, sh2, 5 + AM, a.periodic_mask[AM], a.asymm_lo[AM]));
        }
        if (fix_m && j == nM) {
          float ol, oh, sl, sh2;
          f2u(bz, ol, oh);
          f2u(bzm1, sl, sh2);
          bz = f2m(gfix(ol, sl, 5 + AM, a.periodic_mask[AM], a.asymm_hi[AM]),
                   gfix(oh, sh2, 5 + AM, a.periodic_mask[AM], a.asymm_hi[AM]));
        }
      }
      // getboundary of the ring/tile predictor values at non-periodic x and
      // row faces (read at the next iteration's update).  The transverse B
      // of plane j in w1b is otherwise read only at the next iteration,
      // after its barrier A, so this barrier is needed only here.
      if (ring && (fix_r || (K == 2 && fix_x))) {
        __syncthreads();  // barrier B: w1b of plane j complete
        for (int c = tid; c < 36 * 10; c += PT_NT) {
          const int lx = c % 36 - WBO, lyy = c / 36 - 1;
          const int ixc = x0 + lx, iyc = y0 + lyy;
          int d = -1, slx = lx, sly = lyy, lo = 0;
          if (K == 2 && (ixc == -1 || ixc == nX) && iyc >= 0 && iyc < nR) {
            d = 0;
            lo = ixc == -1;
            slx = lx + (lo ? 1 : -1);
          } else if ((iyc == -1 || iyc == nR) && ixc >= 0 && ixc < nX) {
            d = AR;
            lo = iyc == -1;
            sly = lyy + (lo ? 1 : -1);
          }
          if (d < 0) continue;
          const int asy = lo ? a.asymm_lo[d] : a.asymm_hi[d];
#pragma unroll
          for (int cc = K == 2 ? 0 : 1; cc < 2; cc++) {
            const int v = cc == 0 ? 5 : 5 + AR;
            float* dst = wb(sm, j, cc, lyy, lx);
            *dst = gfix(*dst, *wb(sm, j, cc, sly, slx), v, a.periodic_mask[d], asy);
          }
        }
      }

      // ---------------- faces of plane j (in-plane) or between j-1 and j
      f2 G[NW];
#pragma unroll
      for (int v = 0; v < NW; v++) G[v] = f2s(0.0f);
      if (K == 2) {
        if (j >= z0) {
          f2 L[NW], R[NW];
#pragma unroll
          for (int v = 0; v < NW; v++) {
            L[v] = w1p[v] + hlp[v];
            R[v] = w1[v] - hl_[v];
          }
          const f2 cm = face(L, R, k, G);
          if (cfl) {
            const float cf = 2.0f / (dxzp + dxzc);
            float cl, ch, ql, qh;
            f2u(cm * f2s(cf), cl, ch);
            f2u(qmax, ql, qh);
            if (ok0) ql = (cl > ql || cl != cl) ? cl : ql;
            if (ok1) qh = (ch > qh || ch != ch) ? ch : qh;
            qmax = f2m(ql, qh);
          }
        }
      } else if (!edge) {
        f2 L[NW], R[NW];
#pragma unroll
        for (int v = 0; v < NW; v++) {
          float rl, rh;
          f2u(w1[v] - hl_[v], rl, rh);
          const float nb = __shfl_down_sync(0xffffffffu, rl, 1, 16);
          L[v] = w1[v] + hl_[v];
          R[v] = f2m(rh, nb);
        }
        const f2 cm = face(L, R, k, G);
        if (cfl) {
          // faces (-1|0) .. (n-1|n) of mesh rows inside the chunk
          float cl, ch, ql, qh;
          f2u(cm * cflx, cl, ch);
          f2u(qmax, ql, qh);
          const bool v0 = rowok && ix0 >= -1 && ix0 < nX;
          const bool v1 = rowok && ix0 + 1 >= -1 && ix0 + 1 < nX && hl < 15;
          if (v0) ql = (cl > ql || cl != cl) ? cl : ql;
          if (v1) qh = (ch > qh || ch != ch) ? ch : qh;
          qmax = f2m(ql, qh);
        }
        // flux differences of the pair's cells, and B_x(x+1)-B_x(x-1) of w1
#pragma unroll
        for (int v = 0; v < NW; v++) {
          float gl, gh;
          f2u(G[v], gl, gh);
          const float gm = __shfl_up_sync(0xffffffffu, gh, 1, 16);
          G[v] = f2m(gl - gm, gh - gl);
        }
        if (powell) {
          float bl, bh;
          f2u(w1[5], bl, bh);
          const float bm_ = __shfl_up_sync(0xffffffffu, bh, 1, 16);
          const float bp_ = __shfl_down_sync(0xffffffffu, bl, 1, 16);
          dbxc = f2m(bh - bm_, bp_ - bl);  // of plane j, used at j+1
        }
      }

      // ---------------- update of plane j-1
      const int jo = j - 1;
      if (jo >= z0 && jo < z1 && (ok0 || ok1)) {
        const float* pu = pm;  // state plane j-1
        f2 acc[NW];
        const f2 idxo = K == 2 ? f2s(idzp) : idxx;
        const f2 ncq = f2s(-0.5f * qdt) * idxo;
#pragma unroll
        for (int v = 0; v < NW; v++) {
          const f2 w = ld2(pu + v * BPL + br * FB_X + bc);
          acc[v] = K == 2 ? ffma(ncq, G[v] - Gp[v], w) : ffma(ncq, Gp[v], w);
        }
        if (srcs) {
          f2 nqdivb = f2s(0.0f);
          if (powell) {
            f2 dbx;
            if (K == 2) {
              float cl, ch;
              f2u(w1p[5], cl, ch);
              dbx = f2m(ch - *wb(sm, jo, 0, ly, lx0 - 1), *wb(sm, jo, 0, ly, lx0 + 2) - cl);
            } else {
              dbx = dbxp;
            }
            const f2 dby = ld2(wb(sm, jo, 1, ly + 1, lx0)) - ld2(wb(sm, jo, 1, ly - 1, lx0));
            const f2 dbz = bz - bzm2;
            const f2 divb = ffma(dbz, f2s(idzp), ffma(dby, idxy, dbx * idxx));
            nqdivb = nqs2h * divb;
          }
          sources(a, qs2, w1p, nqdivb, powell, acc);
        }
        store(a, acc, obase + (long long)(jo + 2) * sam, gco[0], gco[AR], jo + 2, nearxr, ok0,
              ok1);
      }
      // ---------------- carry to the next plane
      idzp = idzc;
      idzc = idzn;
      dxzp = dxzc;
      dxzc = dxzn;
      if (K == 0 && !edge) dbxp = dbxc;
      bzm2 = bzm1;
      bzm1 = bz;
      if (K == 2) {
#pragma unroll
        for (int v = 0; v < NW; v++) {
          w1p[v] = w1[v];
          hlp[v] = hl_[v];
          Gp[v] = G[v];
        }
      } else if (!edge) {
#pragma unroll
        for (int v = 0; v < NW; v++) {
          w1p[v] = w1[v];
          Gp[v] = G[v];
        }
      }
    }
    {  // phase bookkeeping: planes pbase .. z1+1 were loaded
      const int np = z1 + 2 - pbase;
#pragma unroll
      for (int s2 = 0; s2 < FWRING; s2++) uses[s2] += (np - s2 + FWRING - 1) / FWRING;
    }
    if (cfl) {
      float q = fmaxf(f2lo(qmax), f2hi(qmax));
      {
        const float l = f2lo(qmax), h = f2hi(qmax);
        q = (h > l || h != h) ? h : l;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float v = __shfl_xor_sync(0xffffffffu, q, o);
        q = (v > q || v != v) ? v : q;
      }
      if ((tid & 31) == 0) shq[tid >> 5] = q;
      __syncthreads();
      if (tid == 0) {
        for (int i = 1; i < PT_NT / 32; i++) q = (shq[i] > q || shq[i] != shq[i]) ? shq[i] : q;
        const unsigned long long key = dkey((double)q);
        if (q != 0.0f) atomicMax(&ctrl->face_cmax[D][slotid % NSLOT], key);
      }
    }
    return true;
  }
};

template <int D, bool MHD, int LIMC, bool GEN>
__global__ void __launch_bounds__(PT_NT, 3)
    k_sweep_pair(const __grid_constant__ CUtensorMap map, FusedArgs a) {
  extern __shared__ __align__(128) float dsm[];
  __shared__ __align__(8) unsigned long long bars[FWRING];
  init_bars(bars);
  int uses[FWRING] = {0, 0, 0, 0};
  const unsigned slotid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  PairSweep<D, MHD, LIMC, GEN>::run(&map, a, dsm, blockIdx.x, blockIdx.y, blockIdx.z, bars,
                                   uses, slotid);
}

}  // namespace vacgpu

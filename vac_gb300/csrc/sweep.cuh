// sweep.cuh - kernels of one dimensional sweep of VAC's twostep
// Hancock-predictor / TVDLF-corrector scheme (src/vac.t:363-572,
// src/vactvdlf.t:5-299), the ghost-cell fill (src/vacgrid.t:195-413) and the
// cell-centred CFL pass of getdt_courant (src/vac.t:664-722).
//
// Templated on a physics policy PH (storage type T, arithmetic type R and
// the pointwise physics), the dimensionality and the physics module.
#pragma once
#include "vacgpu_internal.h"

namespace vacgpu {

__device__ __forceinline__ void atomic_max_key(unsigned long long* a,
                                               unsigned long long k) {
  atomicMax(a, k);
}
__device__ __forceinline__ void atomic_min_key(unsigned long long* a,
                                               unsigned long long k) {
  atomicMin(a, k);
}

// Block-wide max of an ordered key; thread 0 returns the result.
template <int NT>
__device__ __forceinline__ unsigned long long block_max_key(
    unsigned long long k, unsigned long long* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long v = __shfl_xor_sync(0xffffffffu, k, o);
    k = v > k ? v : k;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = k;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < NT / 32; i++) k = sh[i] > k ? sh[i] : k;
  }
  __syncthreads();
  return k;
}

// Decompose a mesh-cell counter into ghost-box coordinates.
__device__ __forceinline__ void cell_coords(const DevGrid& g, long long n,
                                            int* c) {
  int ix = (int)(n % g.nx[0]);
  long long r = n / g.nx[0];
  int iy = (int)(r % g.nx[1]);
  int iz = (int)(r / g.nx[1]);
  c[0] = ix + g.gh[0];
  c[1] = iy + g.gh[1];
  c[2] = iz + g.gh[2];
}

template <class PH, int NDIM, int NDIR, bool MHD>
struct Sweep {
  typedef typename PH::T T;
  typedef typename PH::R R;
  typedef Lay<NDIR, MHD> L;
  static constexpr int NW = L::NW;

  // Levi-Civita symbol, 1-based indices
  static __host__ __device__ constexpr int lvc(int i, int j, int k) {
    return (i == j || j == k || i == k)
               ? 0
               : (((i == 1 && j == 2) || (i == 2 && j == 3) || (i == 3 && j == 1)) ? 1 : -1);
  }
  // first current component getcurrent fills (src/vacphys.mhdres.t:48-93)
  static constexpr int IDM0 = 7 - 2 * NDIR;

  // J_k = eps_kjl d_j B_l at the cell o (offset from the cell of wct) with
  // ghost-range coordinates cc, slab gradients (src/vacgrid.t:816-823)
  static __device__ __forceinline__ R current(const SweepArgs& a,
                                              const T* __restrict__ wct,
                                              long long o, const long long* st,
                                              const int* cc, int k) {
    R j = R(0);
#pragma unroll
    for (int jd = 1; jd <= NDIM; jd++)
#pragma unroll
      for (int kd = 1; kd <= NDIR; kd++) {
        const int l = lvc(k, jd, kd);
        if (!l) continue;
        const T* q = wct + o + (long long)(L::B0 + kd) * a.g.vs;
        const R g = R(0.5) * (R(q[st[jd - 1]]) - R(q[-st[jd - 1]])) /
                    PH::dx(a.a, jd - 1, cc[jd - 1]);
        j = l == 1 ? j + g : j - g;
      }
    return j;
  }

  // resistive terms of addsource: addsource_res2 (curl form,
  // src/vacphys.mhdres.t:236-315) or addsource_res1 (compactres, :96-233),
  // in the reference's term order; eta = eqpar(eta_) > 0 or, with a
  // specialeta field, eta (and gradeta) of the cell and its neighbours
  static __device__ __forceinline__ void add_resistive(
      const SweepArgs& a, double qdt, const R* wc, const T* __restrict__ wct,
      const long long* st, const int* c, R* acc) {
    const double* ef = a.etaf;
    const long long off = ef ? gidx(a.g, c[0], c[1], c[2]) : 0;
    const R eta = ef ? R(ef[off]) : R(a.ph.eta), q = PH::qdiv(qdt);
    const long long vs = a.g.vs;
    if (!a.ph.compactres) {
      // B_i -= eps_ijk d_j (eta J_k qdt)
#pragma unroll
      for (int idir = 1; idir <= NDIR; idir++)
#pragma unroll
        for (int jd = 1; jd <= NDIM; jd++)
#pragma unroll
          for (int kd = IDM0; kd <= 3; kd++) {
            const int l = lvc(idir, jd, kd);
            if (!l) continue;
            int cp[3] = {c[0], c[1], c[2]}, cm[3] = {c[0], c[1], c[2]};
            cp[jd - 1]++;
            cm[jd - 1]--;
            const long long s = st[jd - 1];
            const R ep = ef ? R(ef[off + s]) : eta, em = ef ? R(ef[off - s]) : eta;
            const R tp = current(a, wct, s, st, cp, kd) * ep * q;
            const R tm = current(a, wct, -s, st, cm, kd) * em * q;
            const R g = R(0.5) * (tp - tm) / PH::dx(a.a, jd - 1, c[jd - 1]);
            acc[L::B0 + idir] = l == 1 ? acc[L::B0 + idir] - g : acc[L::B0 + idir] + g;
          }
      // e += eps_ijk d_i (B_j eta J_k qdt)
#pragma unroll
      for (int idir = 1; idir <= NDIM; idir++)
#pragma unroll
        for (int jd = 1; jd <= NDIR; jd++)
#pragma unroll
          for (int kd = IDM0; kd <= 3; kd++) {
            const int l = lvc(idir, jd, kd);
            if (!l) continue;
            int cp[3] = {c[0], c[1], c[2]}, cm[3] = {c[0], c[1], c[2]};
            cp[idir - 1]++;
            cm[idir - 1]--;
            const long long s = st[idir - 1];
            const R ep = ef ? R(ef[off + s]) : eta, em = ef ? R(ef[off - s]) : eta;
            const T* bj = wct + (long long)(L::B0 + jd) * vs;
            const R tp = R(bj[s]) * current(a, wct, s, st, cp, kd) * ep * q;
            const R tm = R(bj[-s]) * current(a, wct, -s, st, cm, kd) * em * q;
            const R g = R(0.5) * (tp - tm) / PH::dx(a.a, idir - 1, c[idir - 1]);
            acc[L::E] = l == 1 ? acc[L::E] + g : acc[L::E] - g;
          }
    } else {
      // B_i += qdt (eta lap(B_i) - [grad(eta) x J]_i), e += the same B_i,
      // then e += qdt eta J^2
#pragma unroll
      for (int idir = 1; idir <= NDIR; idir++) {
        const T* qb = wct + (long long)(L::B0 + idir) * vs;
        R t = R(0);
#pragma unroll
        for (int d = 0; d < NDIM; d++) {
          const R dx = PH::dx(a.a, d, c[d]);
          t = t + (R(qb[st[d]]) - R(2) * R(qb[0]) + R(qb[-st[d]])) / (dx * dx);
        }
        t = t * eta;
        if (ef) {
#pragma unroll
          for (int jd = 1; jd <= NDIM; jd++)
#pragma unroll
            for (int kd = IDM0; kd <= 3; kd++) {
              const int l = lvc(idir, jd, kd);
              if (!l) continue;
              const R ge = R(a.gradetaf[jd - 1][off]);
              const R jk = current(a, wct, 0, st, c, kd);
              t = l == 1 ? t - ge * jk : t + ge * jk;
            }
        }
        acc[L::B0 + idir] = acc[L::B0 + idir] + q * t;
        acc[L::E] = acc[L::E] + q * t * wc[L::B0 + idir];
      }
      R jj = R(0);
#pragma unroll
      for (int k = IDM0; k <= 3; k++) {
        const R jk = current(a, wct, 0, st, c, k);
        jj = jj + jk * jk;
      }
      acc[L::E] = acc[L::E] + q * eta * jj;
    }
  }

  // getcurrent (src/vacphys.mhdres.t:48-93) into double fields over the
  // mesh and one layer around it, for the specialeta hook
  static __device__ void current_field(const SweepArgs& a, const T* __restrict__ w,
                                       double* const* cur) {
    const DevGrid& g = a.g;
    int ext[3], lo[3];
    for (int d = 0; d < 3; d++) {
      lo[d] = d < g.ndim ? 1 : 0;
      ext[d] = d < g.ndim ? g.nx[d] + 2 : 1;
    }
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= (long long)ext[0] * ext[1] * ext[2]) return;
    int c[3];
    c[0] = lo[0] + (int)(n % ext[0]);
    c[1] = lo[1] + (int)((n / ext[0]) % ext[1]);
    c[2] = lo[2] + (int)(n / ((long long)ext[0] * ext[1]));
    const long long off = gidx(g, c[0], c[1], c[2]);
    const long long st[3] = {1, g.P, g.plane};
#pragma unroll
    for (int k = IDM0; k <= 3; k++)
      cur[k - 1][off] = double(current(a, w + off, 0, st, c, k));
  }

  // qdt*(idimmax-idimmin+1)/ndim of the unsplit source call
  // (src/vactvdlf.t:85,292):
  // the reference's double expression on the FP64 path; formed in FP32 on
  // the mixed one, whose sources take it rounded to FP32 anyway (GB300's
  // FP64 pipe would spend a double division per cell on it)
  static __device__ __forceinline__ double src_qdt(const SweepArgs& a,
                                                   double qdt) {
    if constexpr (sizeof(R) == 4)
      return (double)((float)qdt * (float)((a.d1 - a.d0) + 1) / (float)NDIM);
    else
      return qdt * ((a.d1 - a.d0) + 1.0) / NDIM;
  }

  // addsource2 (src/vac.t:575-605): specialsource (uniform gravity,
  // vacusr.gravity.t:24-75) then addsource (resistive terms, then the
  // Powell divB source, src/vacphys.mhd0.t:208-280).  wc = wCT at the
  // cell, wct points at the cell in the wCT array (for the differences).
  static __device__ __forceinline__ void add_sources(
      const SweepArgs& a, double qdt, const R* wc, const T* __restrict__ wct,
      const long long* st, const int* c, R* acc) {
    if (a.ph.src_id == VACGPU_SRC_GRAVITY) {
#pragma unroll
      for (int d = 1; d <= NDIM; d++) {
        double gr = a.ph.src_par[d - 1];
        if (fabs(gr) > 1.0e-99) acc[d] = acc[d] + PH::mul_qg(qdt, gr) * wc[0];
      }
#pragma unroll
      for (int d = 1; d <= NDIM; d++) {
        double gr = a.ph.src_par[d - 1];
        if (fabs(gr) > 1.0e-99)
          acc[L::E] = acc[L::E] + PH::mul_qg(qdt, gr) * wc[d];
      }
    }
    if (MHD && fabs(a.ph.eta) > 1.0e-99) add_resistive(a, qdt, wc, wct, st, c, acc);
    if (MHD && a.ph.divbfix) {
      R divb = R(0);
#pragma unroll
      for (int d = 0; d < NDIM; d++) {
        const T* q = wct + (long long)(L::B0 + 1 + d) * a.g.vs;
        R gq = R(0.5) * (R(q[st[d]]) - R(q[-st[d]])) / PH::dx(a.a, d, c[d]);
        divb = divb + gq;
      }
      divb = PH::qdiv(qdt) * divb;
      R mb = wc[1] * wc[L::B0 + 1];
#pragma unroll
      for (int k = 2; k <= NDIR; k++) mb = mb + wc[k] * wc[L::B0 + k];
#pragma unroll
      for (int k = 1; k <= NDIR; k++) {
        acc[k] = acc[k] - wc[L::B0 + k] * divb;
        acc[L::B0 + k] = acc[L::B0 + k] - wc[k] / wc[0] * divb;
      }
      acc[L::E] = acc[L::E] - mb / wc[0] * divb;
    }
  }

  // primitive (src/vacphys0.t.mhd:31-52, src/vacphys0.t.hd:30-51): the
  // clipped thermal pressure into e, v = m/rho
  static __device__ __forceinline__ void to_prim(const SweepArgs& a, R smallp,
                                                 R* u) {
    R p = R(PH::template pthermal_raw<NDIR, MHD>(u, a.ph));
    p = (p >= smallp) ? p : smallp;
    u[L::E] = p;
#pragma unroll
    for (int k = 1; k <= NDIR; k++) u[k] = u[k] / u[0];
  }
  // conserve (src/vacphys0.t.mhd:5-27, src/vacphys0.t.hd:5-26)
  static __device__ __forceinline__ void to_cons(const SweepArgs& a, R* u) {
    R vv = u[1] * u[1];
#pragma unroll
    for (int k = 2; k <= NDIR; k++) vv = vv + u[k] * u[k];
    const R gm1 = R(a.ph.gm1);
    if (MHD) {
      R bb = u[L::B0 + 1] * u[L::B0 + 1];
#pragma unroll
      for (int k = 2; k <= NDIR; k++) bb = bb + u[L::B0 + k] * u[L::B0 + k];
      u[L::E] = u[L::E] / gm1 + R(0.5) * (u[0] * vv + bb);
    } else {
      u[L::E] = u[L::E] / gm1 + R(0.5) * u[0] * vv;
    }
#pragma unroll
    for (int k = 1; k <= NDIR; k++) u[k] = u[0] * u[k];
  }
  static __device__ __forceinline__ void load(const T* __restrict__ w,
                                              long long o, long long vs, R* u) {
#pragma unroll
    for (int iw = 0; iw < NW; iw++) u[iw] = R(w[o + iw * vs]);
  }

  // useprimitive's in-place round trip of the limiter base over the ghost
  // box: out = conserve(primitive(w)) (src/vactvdlf.t:325-330,357-362).
  static __device__ void roundtrip(const SweepArgs& a, const T* __restrict__ w,
                                   T* __restrict__ out) {
    const Ctrl* ctrl = a.ctrl;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nG = (long long)a.g.nG[0] * a.g.nG[1] * a.g.nG[2];
    if (ctrl->done || n >= nG) return;
    const int gx = (int)(n % a.g.nG[0]);
    const long long r = n / a.g.nG[0];
    const int gy = (int)(r % a.g.nG[1]), gz = (int)(r / a.g.nG[1]);
    const long long off = gidx(a.g, gx, gy, gz);
    R u[NW];
    load(w, off, a.g.vs, u);
    to_prim(a, R(ctrl->smallp), u);
    to_cons(a, u);
#pragma unroll
    for (int iw = 0; iw < NW; iw++) out[off + iw * a.g.vs] = T(u[iw]);
  }

  // One direction of the predictor, the direction a compile-time constant
  // (a runtime one puts the face states in a stack frame)
  template <int d>
  static __device__ __forceinline__ void predict_dir(
      const SweepArgs& a, const T* __restrict__ w, long long off,
      const long long* st, const int* c, double qdt, R smallp, const R* u,
      const R* pc, R* acc) {
    const long long vs = a.g.vs;
    R uL[NW], uR[NW];
    if (a.ph.useprim) {
      R pm[NW], pp[NW];
      load(w, off - st[d], vs, pm);
      load(w, off + st[d], vs, pp);
      to_prim(a, smallp, pm);
      to_prim(a, smallp, pp);
#pragma unroll
      for (int iw = 0; iw < NW; iw++) {
        R l = PH::limiter(a.ph.lim[iw], pp[iw] - pc[iw], pc[iw] - pm[iw]);
        uR[iw] = pc[iw] - R(0.5) * l;
        uL[iw] = pc[iw] + R(0.5) * l;
      }
      to_cons(a, uR);
      to_cons(a, uL);
    } else {
#pragma unroll
      for (int iw = 0; iw < NW; iw++) {
        R wm = R(w[off + iw * vs - st[d]]);
        R wp = R(w[off + iw * vs + st[d]]);
        R l = PH::limiter(a.ph.lim[iw], wp - u[iw], u[iw] - wm);
        uR[iw] = u[iw] - R(0.5) * l;
        uL[iw] = u[iw] + R(0.5) * l;
      }
    }
    R fL[NW], fR[NW];
    PH::template flux<NDIR, MHD>(uR, d, a.ph, smallp, fR);
    PH::template flux<NDIR, MHD>(uL, d, a.ph, smallp, fL);
    // 'symm0' faces (setnoflux, src/vacgrid.t:416-454): no flux through
    // the mesh edge
    if (c[d] == a.g.nx[d] + 1 && a.ph.noflux[d][1]) {
#pragma unroll
      for (int iw = 0; iw < NW; iw++)
        if ((a.ph.noflux[d][1] >> iw) & 1) fL[iw] = R(0);
    }
    if (c[d] == 2 && a.ph.noflux[d][0]) {
#pragma unroll
      for (int iw = 0; iw < NW; iw++)
        if ((a.ph.noflux[d][0] >> iw) & 1) fR[iw] = R(0);
    }
    const R cq = PH::qdx(qdt, a.a, d, c[d]);
#pragma unroll
    for (int iw = 0; iw < NW; iw++) acc[iw] = acc[iw] - cq * (fL[iw] - fR[iw]);
  }

  // Hancock predictor (src/vactvdlf.t:5-89): w1 = w - dt/2/dx*(F(w+ldw/2)
  // - F(w-ldw/2)) + dt/2*(nsweepdims/ndim)*S(w), on the mesh.  With
  // useprimitive the slopes and face states are formed in primitive
  // variables and the sources see the round-tripped state.
  static __device__ void predict(const SweepArgs& a, const T* __restrict__ w,
                                 T* __restrict__ w1) {
    const Ctrl* ctrl = a.ctrl;
    if (ctrl->done) return;
    long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.g.ncell) return;
    int c[3];
    cell_coords(a.g, n, c);
    const long long off = gidx(a.g, c[0], c[1], c[2]);
    const long long st[3] = {1, a.g.P, a.g.plane};
    const long long vs = a.g.vs;
    const double qdt = ctrl->dt / 2;
    const R smallp = R(ctrl->smallp);
    R u[NW], acc[NW];
#pragma unroll
    for (int iw = 0; iw < NW; iw++) {
      u[iw] = R(w[off + iw * vs]);
      acc[iw] = u[iw];
    }
    R pc[NW];  // useprimitive: primitive state of the cell
    if (a.ph.useprim) {
#pragma unroll
      for (int iw = 0; iw < NW; iw++) pc[iw] = u[iw];
      to_prim(a, smallp, pc);
    }
    for (int d = a.d0; d <= a.d1; d++) {
      if (d == 0)
        predict_dir<0>(a, w, off, st, c, qdt, smallp, u, pc, acc);
      else if (NDIM > 1 && d == 1)
        predict_dir<(NDIM > 1 ? 1 : 0)>(a, w, off, st, c, qdt, smallp, u, pc,
                                        acc);
      else if (NDIM > 2)
        predict_dir<(NDIM > 2 ? 2 : 0)>(a, w, off, st, c, qdt, smallp, u, pc,
                                        acc);
    }
    if (a.ph.sourceunsplit && !a.ph.src_hook) {
      // the round-tripped state (useprimitive) leaves rho and B unchanged
      if (a.ph.useprim) {
        to_cons(a, pc);
#pragma unroll
        for (int iw = 0; iw < NW; iw++) u[iw] = pc[iw];
      }
      add_sources(a, src_qdt(a, qdt), u, w + off, st, c,
                  acc);
    }
#pragma unroll
    for (int iw = 0; iw < NW; iw++) w1[off + iw * vs] = T(acc[iw]);
  }

  // Face states of upwindLR (src/vactvdlf.t:302-367) at the face between
  // cell `o` and `o+s`: wL = wCT(o)+ldw/2, wR = wCT(o+s)-ldw/2 with the
  // limited slopes of `base` (in primitive variables with useprimitive,
  // src/vactvdlf.t:325-362); the first order methods take wCT unlimited.
  static __device__ __forceinline__ void face_states(
      const SweepArgs& a, const T* __restrict__ w1, const T* __restrict__ base,
      long long o, long long s, R smallp, bool limit, R* wL, R* wR) {
    const long long vs = a.g.vs;
#pragma unroll
    for (int iw = 0; iw < NW; iw++) {
      wL[iw] = R(w1[o + iw * vs]);
      wR[iw] = R(w1[o + iw * vs + s]);
    }
    if (limit && a.ph.useprim) {
      R bm[NW], b0[NW], b1[NW], b2[NW];
      load(base, o - s, vs, bm);
      load(base, o, vs, b0);
      load(base, o + s, vs, b1);
      load(base, o + 2 * s, vs, b2);
      to_prim(a, smallp, bm);
      to_prim(a, smallp, b0);
      to_prim(a, smallp, b1);
      to_prim(a, smallp, b2);
      to_prim(a, smallp, wL);
      to_prim(a, smallp, wR);
#pragma unroll
      for (int iw = 0; iw < NW; iw++) {
        R ldL = PH::limiter(a.ph.lim[iw], b1[iw] - b0[iw], b0[iw] - bm[iw]);
        R ldR = PH::limiter(a.ph.lim[iw], b2[iw] - b1[iw], b1[iw] - b0[iw]);
        wR[iw] = wR[iw] - R(0.5) * ldR;
        wL[iw] = wL[iw] + R(0.5) * ldL;
      }
      to_cons(a, wL);
      to_cons(a, wR);
    } else if (limit) {
#pragma unroll
      for (int iw = 0; iw < NW; iw++) {
        const T* b = base + o + iw * vs;
        R bm = R(b[-s]), b0 = R(b[0]), b1 = R(b[s]), b2 = R(b[2 * s]);
        R ldL = PH::limiter(a.ph.lim[iw], b1 - b0, b0 - bm);
        R ldR = PH::limiter(a.ph.lim[iw], b2 - b1, b1 - b0);
        wR[iw] = wR[iw] - R(0.5) * ldR;
        wL[iw] = wL[iw] + R(0.5) * ldL;
      }
    }
  }

  // TVDLF numerical flux at the face between cell `o` and `o+st` in
  // direction d (src/vactvdlf.t:140-259); returns the face cmax.
  static __device__ __forceinline__ R face_flux(const SweepArgs& a,
                                                const T* __restrict__ w1,
                                                const T* __restrict__ base,
                                                long long o, long long s,
                                                int d, R smallp, R* F) {
    R wL[NW], wR[NW];
    face_states(a, w1, base, o, s, smallp, a.ph.typefull != VACGPU_TVDLF1, wL,
                wR);
    R mean[NW];
#pragma unroll
    for (int iw = 0; iw < NW; iw++) mean[iw] = R(0.5) * (wL[iw] + wR[iw]);
    const R cmax = PH::template cmax<NDIR, MHD>(mean, d, a.ph, smallp);
#pragma unroll
    for (int iw = 0; iw < NW; iw++) wL[iw] = R(2) * mean[iw] - wR[iw];
    R fL[NW], fR[NW];
    PH::template flux<NDIR, MHD>(wL, d, a.ph, smallp, fL);
    PH::template flux<NDIR, MHD>(wR, d, a.ph, smallp, fR);
#pragma unroll
    for (int iw = 0; iw < NW; iw++) {
      R f = R(0.5) * (fL[iw] + fR[iw]);
      R diss = -cmax * R(0.5) * (wR[iw] - wL[iw]);
      F[iw] = f + diss;
    }
    return cmax;
  }

  // TVDLF corrector (src/vactvdlf.t:92-299), face pass: the numerical flux
  // of every face of direction d, once per face, with setnoflux applied
  // ('symm0' mesh faces carry no flux of their variables), into
  // F[iw*nf+f]; plus the CFL maximum of the last substep
  // (src/vactvdlf.t:184-201).
  // (inlined into k_face, whose direction is a compile-time constant: a
  // runtime one puts the face states in a stack frame)
  template <int NT>
  static __device__ __forceinline__ void face_pass(const SweepArgs& a,
                                                   const T* __restrict__ w1,
                                                   const T* __restrict__ base,
                                                   int d, R* __restrict__ F) {
    __shared__ unsigned long long shk[NT / 32];
    Ctrl* ctrl = a.ctrl;
    if (ctrl->done) return;
    const DevGrid& g = a.g;
    const long long nf = face_count(g, d);
    const long long f = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long key = 0ULL;
    if (f < nf) {
      int cl[3];
      face_left_cell(g, d, f, cl);
      const long long st[3] = {1, g.P, g.plane};
      const long long o = gidx(g, cl[0], cl[1], cl[2]);
      R Ff[NW];
      const R cm = face_flux(a, w1, base, o, st[d], d, R(ctrl->smallp), Ff);
      if (a.ph.courantpar > 0.0) key = dkey(PH::cfl(cm, a.a, d, cl[d]));
      const int nof = cl[d] == 1 ? a.ph.noflux[d][0]
                      : cl[d] == g.nx[d] + 1 ? a.ph.noflux[d][1] : 0;
#pragma unroll
      for (int iw = 0; iw < NW; iw++)
        F[iw * nf + f] = ((nof >> iw) & 1) ? R(0) : Ff[iw];
    }
    if (a.ph.courantpar > 0.0) {
      const unsigned long long k = block_max_key<NT>(key, shk);
      if (threadIdx.x == 0 && k)
        atomic_max_key(&ctrl->face_cmax[d][blockIdx.x % NSLOT], k);
    }
  }

  // TVDLF corrector, cell pass: wnew = w - dt/dx (F(i+1/2) - F(i-1/2)) per
  // direction, then the unsplit sources (src/vactvdlf.t:250-296).
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
    if (a.ph.useprim && a.ph.typefull != VACGPU_TVDLF1) {
      // the limiter base (the state) leaves upwindLR round-tripped
      to_prim(a, smallp, acc);
      to_cons(a, acc);
    }
    for (int d = a.d0; d <= a.d1; d++) {
      const R* F = (const R*)a.faces + (long long)(d - a.d0) * a.face_stride;
      const long long nf = face_count(a.g, d);
      int cm[3] = {c[0], c[1], c[2]};
      cm[d] = c[d] - 1;
      const long long fm = face_index(a.g, d, cm), fp = face_index(a.g, d, c);
      const R cq = PH::qdx(qdt, a.a, d, c[d]);
#pragma unroll
      for (int iw = 0; iw < NW; iw++)
        acc[iw] = acc[iw] - cq * (F[iw * nf + fp] - F[iw * nf + fm]);
    }
    if (a.ph.sourceunsplit && !a.ph.src_hook) {
      R wc[NW];
#pragma unroll
      for (int iw = 0; iw < NW; iw++) wc[iw] = R(w1[off + iw * vs]);
      add_sources(a, src_qdt(a, qdt), wc, w1 + off, st, c,
                  acc);
    }
#pragma unroll
    for (int iw = 0; iw < NW; iw++) wout[off + iw * vs] = T(acc[iw]);
  }

  // addsource (src/vac.t:575-605 after specialsource) as a pass of its own
  // when the user's specialsource hook runs between the flux update and
  // it: w += addsource(wCT) on the mesh, with the operations the predictor
  // (pred) or corrector kernel performs in place otherwise.
  static __device__ void source_pass(const SweepArgs& a, const T* __restrict__ wct,
                                     T* __restrict__ w, int pred) {
    const Ctrl* ctrl = a.ctrl;
    if (ctrl->done) return;
    long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= a.g.ncell) return;
    int c[3];
    cell_coords(a.g, n, c);
    const long long off = gidx(a.g, c[0], c[1], c[2]);
    const long long st[3] = {1, a.g.P, a.g.plane};
    const long long vs = a.g.vs;
    const double qdt = pred ? ctrl->dt / 2 : ctrl->dt;
    R acc[NW], wc[NW];
#pragma unroll
    for (int iw = 0; iw < NW; iw++) {
      acc[iw] = R(w[off + iw * vs]);
      wc[iw] = R(wct[off + iw * vs]);
    }
    add_sources(a, src_qdt(a, qdt), wc, wct + off, st, c, acc);
#pragma unroll
    for (int iw = 0; iw < NW; iw++) w[off + iw * vs] = T(acc[iw]);
  }

  // getpthermal's one-time smallp: min/max of the unclipped pressure on the
  // mesh (src/vacphys0.t.mhd:202-217).
  template <int NT>
  // bid, nblk: this block's part of the grid's cells (default: the launch's
  // blocks); the control fields are read through L2, as a persistent
  // kernel needs when another SM set them earlier in the same launch
  static __device__ void pminmax(const SweepArgs& a, const T* __restrict__ w, int bid = -1,
                                 int nblk = 0) {
    __shared__ unsigned long long shk[NT / 32];
    Ctrl* ctrl = a.ctrl;
    if (__ldcg(&ctrl->done) || !__ldcg(&ctrl->need_smallp)) return;
    if (bid < 0) {
      bid = blockIdx.x;
      nblk = gridDim.x;
    }
    unsigned long long kmin = ~0ULL, kmax = 0ULL;
    for (long long n = (long long)bid * blockDim.x + threadIdx.x;
         n < a.g.ncell; n += (long long)nblk * blockDim.x) {
      int c[3];
      cell_coords(a.g, n, c);
      const long long off = gidx(a.g, c[0], c[1], c[2]);
      R u[NW];
#pragma unroll
      for (int iw = 0; iw < NW; iw++) u[iw] = R(__ldcg(w + off + iw * a.g.vs));
      const unsigned long long k = dkey(PH::template pthermal_raw<NDIR, MHD>(u, a.ph));
      kmin = k < kmin ? k : kmin;
      kmax = k > kmax ? k : kmax;
    }
    unsigned long long k = block_max_key<NT>(kmax, shk);
    if (threadIdx.x == 0) atomic_max_key(&ctrl->pmax[bid % NSLOT], k);
    k = ~block_max_key<NT>(~kmin, shk);
    if (threadIdx.x == 0) atomic_min_key(&ctrl->pmin[bid % NSLOT], k);
  }

  // keeppositive (smallfix), src/vacphys.t.mhd:9-53, src/vacphys.t.hd:
  // 176-219, src/vacproc.positive.t:2-34, in the reference's expression
  // order.  min(rho) for the one-time smallrho:
  template <int NT>
  static __device__ void kp_rhomin(const SweepArgs& a, const T* __restrict__ w) {
    __shared__ unsigned long long shk[NT / 32];
    Ctrl* ctrl = a.ctrl;
    if (ctrl->done || !ctrl->need_smallrho) return;
    unsigned long long kmin = ~0ULL;
    for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
         n < a.g.ncell; n += (long long)gridDim.x * blockDim.x) {
      int c[3];
      cell_coords(a.g, n, c);
      const unsigned long long k = dkey((double)w[gidx(a.g, c[0], c[1], c[2])]);
      kmin = k < kmin ? k : kmin;
    }
    const unsigned long long k = ~block_max_key<NT>(~kmin, shk);
    if (threadIdx.x == 0) atomic_min_key(&ctrl->rmin[blockIdx.x % NSLOT], k);
  }

  // density floor rho = max(rho, smallrho) (keeppositive_rho), or the
  // vacuum state where rho < smallrho (vacuumrho >= 0)
  static __device__ void kp_rho(const SweepArgs& a, T* __restrict__ w) {
    const Ctrl* ctrl = a.ctrl;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (ctrl->done || n >= a.g.ncell) return;
    int c[3];
    cell_coords(a.g, n, c);
    const long long off = gidx(a.g, c[0], c[1], c[2]);
    const double smallrho = ctrl->smallrho;
    const double rho = (double)w[off];
    if (a.ph.vacuumrho < 0.0) {
      if (rho < fmax2(0.0, smallrho)) atomicOr((int*)&a.ctrl->kp_r, 1);
      if (smallrho > 0.0) w[off] = T(fmax2(rho, smallrho));
    } else if (rho < smallrho) {
#pragma unroll
      for (int k = 1; k <= NDIR; k++) w[off + k * a.g.vs] = T(0.0);
      w[off] = T(a.ph.vacuumrho);
      double e = ctrl->smallp / a.ph.gm1;
      if (MHD) {
        double b1 = (double)w[off + (L::B0 + 1) * a.g.vs];
        double bb = b1 * b1;
#pragma unroll
        for (int k = 2; k <= NDIR; k++) {
          const double bk = (double)w[off + (L::B0 + k) * a.g.vs];
          bb = bb + bk * bk;
        }
        e = e + 0.5 * bb;
      }
      w[off + L::E * a.g.vs] = T(e);
    }
  }

  // any unclipped pressure below max(0, smallp)?
  static __device__ void kp_pcheck(const SweepArgs& a, const T* __restrict__ w) {
    const Ctrl* ctrl = a.ctrl;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (ctrl->done || n >= a.g.ncell) return;
    int c[3];
    cell_coords(a.g, n, c);
    const long long off = gidx(a.g, c[0], c[1], c[2]);
    R u[NW];
#pragma unroll
    for (int iw = 0; iw < NW; iw++) u[iw] = R(w[off + iw * a.g.vs]);
    const double p = PH::template pthermal_raw<NDIR, MHD>(u, a.ph);
    if (p < fmax2(0.0, ctrl->smallp)) atomicOr((int*)&a.ctrl->kp_p, 1);
  }

  // if so (and smallp > 0): e from max(p, smallp) in every mesh cell
  static __device__ void kp_pfix(const SweepArgs& a, T* __restrict__ w) {
    const Ctrl* ctrl = a.ctrl;
    const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (ctrl->done || !ctrl->kp_p || !(ctrl->smallp > 0.0) || n >= a.g.ncell) return;
    int c[3];
    cell_coords(a.g, n, c);
    const long long off = gidx(a.g, c[0], c[1], c[2]);
    R u[NW];
#pragma unroll
    for (int iw = 0; iw < NW; iw++) u[iw] = R(w[off + iw * a.g.vs]);
    const double smallp = ctrl->smallp;
    const double p = PH::template pthermal_raw<NDIR, MHD>(u, a.ph);
    double mm = (double)u[1] * (double)u[1];
#pragma unroll
    for (int k = 2; k <= NDIR; k++) mm = mm + (double)u[k] * (double)u[k];
    const double x = fmax2(p, smallp) / a.ph.gm1;
    double e;
    if (MHD) {
      double bb = (double)u[L::B0 + 1] * (double)u[L::B0 + 1];
#pragma unroll
      for (int k = 2; k <= NDIR; k++)
        bb = bb + (double)u[L::B0 + k] * (double)u[L::B0 + k];
      e = x + 0.5 * (mm / (double)u[0] + bb);
    } else {
      e = x + 0.5 / (double)u[0] * mm;
    }
    w[off + L::E * a.g.vs] = T(e);
  }

  // Cell-centred max(cmax/dx) of getdt_courant for the dimensions whose
  // dtcourant is unset (src/vac.t:690-711).
  template <int NT>
  static __device__ void cell_cmax(const SweepArgs& a, const T* __restrict__ w, int bid = -1,
                                   int nblk = 0) {
    __shared__ unsigned long long shk[NT / 32];
    Ctrl* ctrl = a.ctrl;
    if (__ldcg(&ctrl->done)) return;
    int need[3];
    for (int d = 0; d < 3; d++) need[d] = __ldcg(&ctrl->need_cell[d]);
    if (!(need[0] | need[1] | need[2])) return;
    if (bid < 0) {
      bid = blockIdx.x;
      nblk = gridDim.x;
    }
    const R smallp = R(__ldcg(&ctrl->smallp));
    unsigned long long key[3] = {0ULL, 0ULL, 0ULL};
    for (long long n = (long long)bid * blockDim.x + threadIdx.x;
         n < a.g.ncell; n += (long long)nblk * blockDim.x) {
      int c[3];
      cell_coords(a.g, n, c);
      const long long off = gidx(a.g, c[0], c[1], c[2]);
      R u[NW];
#pragma unroll
      for (int iw = 0; iw < NW; iw++) u[iw] = R(__ldcg(w + off + iw * a.g.vs));
      for (int d = 0; d < NDIM; d++) {
        if (!need[d]) continue;
        R cm = PH::template cmax<NDIR, MHD>(u, d, a.ph, smallp);
        unsigned long long k = dkey(PH::cell_ratio(cm, a.a, d, c[d]));
        key[d] = k > key[d] ? k : key[d];
      }
    }
    for (int d = 0; d < NDIM; d++) {
      if (!need[d]) continue;
      unsigned long long k = block_max_key<NT>(key[d], shk);
      if (threadIdx.x == 0)
        atomic_max_key(&ctrl->cell_cmax[d][bid % NSLOT], k);
    }
  }
};

// Ghost-cell fill: ghost(i,j,k) = sign * w(map_x(i), map_y(j), map_z(k)),
// the composition of getboundary's per-region copies (src/vacgrid.t:195-413:
// regions are filled x first, then y, then z, each over the full extent of
// the other dimensions, from mesh cells), for 'periodic', 'cont', 'symm' and
// 'asymm'.
__device__ __forceinline__ int bc_map(int gi, int n, int tlo, int thi,
                                      int* sgn) {
  if (gi < 2) {
    switch (tlo) {
      case VACGPU_BC_PERIODIC: return gi + n;
      case VACGPU_BC_CONT: return 2;
      case VACGPU_BC_ASYMM: *sgn = -*sgn; return 3 - gi;
      default: return 3 - gi;
    }
  }
  if (gi >= n + 2) {
    switch (thi) {
      case VACGPU_BC_PERIODIC: return gi - n;
      case VACGPU_BC_CONT: return n + 1;
      case VACGPU_BC_ASYMM: *sgn = -*sgn; return 2 * n + 3 - gi;
      default: return 2 * n + 3 - gi;
    }
  }
  return gi;
}

template <typename T, int NW>
__device__ __forceinline__ void ghost_cell(T* __restrict__ w, const DevGrid& g,
                                           const DevPhys& ph, long long t) {
  const int ndim = g.ndim;
  const long long nzs = ndim == 3 ? 4LL * g.nG[1] * g.nG[0] : 0;
  const long long nys = ndim >= 2 ? 4LL * g.nx[2] * g.nG[0] : 0;
  const long long nxs = 4LL * g.nx[1] * g.nx[2];
  int c[3];
  if (t < nzs) {
    int l = (int)(t / ((long long)g.nG[1] * g.nG[0]));
    long long r = t % ((long long)g.nG[1] * g.nG[0]);
    c[2] = l < 2 ? l : g.nG[2] - 4 + l;
    c[1] = (int)(r / g.nG[0]);
    c[0] = (int)(r % g.nG[0]);
  } else if (t < nzs + nys) {
    long long u = t - nzs;
    int l = (int)(u / ((long long)g.nx[2] * g.nG[0]));
    long long r = u % ((long long)g.nx[2] * g.nG[0]);
    c[1] = l < 2 ? l : g.nG[1] - 4 + l;
    c[2] = (int)(r / g.nG[0]) + g.gh[2];
    c[0] = (int)(r % g.nG[0]);
  } else if (t < nzs + nys + nxs) {
    long long u = t - nzs - nys;
    int l = (int)(u % 4);
    long long r = u / 4;
    c[0] = l < 2 ? l : g.nG[0] - 4 + l;
    c[1] = (int)(r % g.nx[1]) + g.gh[1];
    c[2] = (int)(r / g.nx[1]) + g.gh[2];
  } else {
    return;
  }
  const long long dst = gidx(g, c[0], c[1], c[2]);
  bool uni = true;
  for (int d = 0; d < ndim; d++)
    uni = uni && ph.gmap[d][0] != GMAP_MIXED && ph.gmap[d][1] != GMAP_MIXED;
  if (uni) {
    // one source cell for every variable; asymm flips per variable
    int s[3] = {c[0], c[1], c[2]};
    int flip = 0;
    for (int d = 0; d < ndim; d++) {
      const int side = c[d] < 2 ? 0 : (c[d] >= g.nx[d] + 2 ? 1 : -1);
      if (side < 0) continue;
      s[d] = gmap_src(c[d], g.nx[d], ph.gmap[d][side]);
      flip ^= ph.asym[d][side];
    }
    const long long src = gidx(g, s[0], s[1], s[2]);
#pragma unroll
    for (int iw = 0; iw < NW; iw++) {
      T v = w[src + iw * g.vs];
      w[dst + iw * g.vs] = ((flip >> iw) & 1) ? -v : v;
    }
    return;
  }
#pragma unroll
  for (int iw = 0; iw < NW; iw++) {
    int sgn = 1, s[3] = {c[0], c[1], c[2]};
    for (int d = 0; d < ndim; d++)
      s[d] = bc_map(c[d], g.nx[d], ph.typeB[2 * d][iw], ph.typeB[2 * d + 1][iw],
                    &sgn);
    T v = w[gidx(g, s[0], s[1], s[2]) + iw * g.vs];
    w[dst + iw * g.vs] = sgn < 0 ? -v : v;
  }
}

template <typename T, int NW>
__global__ void k_ghost(T* __restrict__ w, DevGrid g, DevPhys ph,
                        const Ctrl* ctrl) {
  if (ctrl && ctrl->done) return;
  ghost_cell<T, NW>(w, g, ph, (long long)blockIdx.x * blockDim.x + threadIdx.x);
}

// Ordered ghost fill for grids with 'fixed', 'fixed1', 'cont1' or 'grad1'
// faces: the body of getboundary's region loop (src/vacgrid.t:230-366) for
// region iB -- the two ghost layers of dimension iB/2 over the full ghost
// box of the other dimensions -- launched in iB order so corners see the
// earlier regions' values as in the reference.  restore: the stored values
// of the fixed types (src/vacgrid.t:253-305) are used; otherwise they are
// computed ('fixed' as 'cont', 'fixed1'/'grad1' as 'cont1').
__device__ __forceinline__ long long face_cells(const DevGrid& g, int iB,
                                                int* lo, int* ext) {
  const int idim = iB / 2, upper = iB % 2;
  for (int d = 0; d < 3; d++) {
    lo[d] = 0;
    ext[d] = g.nG[d];
  }
  ext[idim] = 2;
  lo[idim] = upper ? g.nx[idim] + 2 : 0;
  return (long long)ext[0] * ext[1] * ext[2];
}

template <typename T, int NW>
__global__ void k_ghost_face(T* __restrict__ w, DevGrid g, DevPhys ph,
                             const Ctrl* ctrl, int iB,
                             const T* __restrict__ fixb, int restore) {
  if (ctrl && ctrl->done) return;
  int lo[3], ext[3];
  const long long tot = face_cells(g, iB, lo, ext);
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= tot) return;
  const int idim = iB / 2, upper = iB % 2;
  int c[3];
  c[0] = lo[0] + (int)(n % ext[0]);
  const long long r = n / ext[0];
  c[1] = lo[1] + (int)(r % ext[1]);
  c[2] = lo[2] + (int)(r / ext[1]);
  const int k = c[idim], nx = g.nx[idim];
  const int ixe = upper ? nx + 1 : 2;  // edge mesh layer
  const int ixf = upper ? ixe - 1 : ixe + 1;
  auto at = [&](int kk) {
    int cc[3] = {c[0], c[1], c[2]};
    cc[idim] = kk;
    return gidx(g, cc[0], cc[1], cc[2]);
  };
  const long long dst = gidx(g, c[0], c[1], c[2]);
  const long long oe = at(ixe), of = at(ixf);
  const int dk = k > ixe ? k - ixe : ixe - k;
#pragma unroll
  for (int iw = 0; iw < NW; iw++) {
    const int t = ph.typeB[iB][iw];
    if (t == VACGPU_BC_SPECIAL) continue;  // the specialbound hook's
    const long long vo = (long long)iw * g.vs;
    const bool fixedtype = t == VACGPU_BC_FIXED || t == VACGPU_BC_FIXED1 ||
                           t == VACGPU_BC_GRAD1;
    T v;
    if (fixedtype && restore) {
      v = fixb[iw * tot + n];
      if (t == VACGPU_BC_GRAD1) v = v + w[oe + vo];
    } else if (t == VACGPU_BC_CONT || t == VACGPU_BC_FIXED) {
      v = w[oe + vo];
    } else if (fixedtype || t == VACGPU_BC_CONT1) {
      v = T(dk + 1) * w[oe + vo] - T(dk) * w[of + vo];
    } else if (t == VACGPU_BC_PERIODIC) {
      v = w[at(upper ? k - nx : k + nx) + vo];
    } else {  // symm, symm0, asymm
      const int ixm = upper ? 2 * nx + 3 : 3;
      v = w[at(ixm - k) + vo];
      if (t == VACGPU_BC_ASYMM) v = -v;
    }
    w[dst + vo] = v;
  }
}

// The first fill's values of the fixed types (grad1: minus the edge),
// src/vacgrid.t:373-409.
template <typename T, int NW>
__global__ void k_fix_store(const T* __restrict__ w, DevGrid g, DevPhys ph,
                            int iB, T* __restrict__ fixb) {
  int lo[3], ext[3];
  const long long tot = face_cells(g, iB, lo, ext);
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= tot) return;
  const int idim = iB / 2, upper = iB % 2;
  int c[3];
  c[0] = lo[0] + (int)(n % ext[0]);
  const long long r = n / ext[0];
  c[1] = lo[1] + (int)(r % ext[1]);
  c[2] = lo[2] + (int)(r / ext[1]);
  int ce[3] = {c[0], c[1], c[2]};
  ce[idim] = upper ? g.nx[idim] + 1 : 2;
  const long long dst = gidx(g, c[0], c[1], c[2]);
  const long long oe = gidx(g, ce[0], ce[1], ce[2]);
#pragma unroll
  for (int iw = 0; iw < NW; iw++) {
    const int t = ph.typeB[iB][iw];
    const long long vo = (long long)iw * g.vs;
    if (t == VACGPU_BC_GRAD1)
      fixb[iw * tot + n] = w[dst + vo] - w[oe + vo];
    else if (t == VACGPU_BC_FIXED || t == VACGPU_BC_FIXED1)
      fixb[iw * tot + n] = w[dst + vo];
  }
}

// Elements of the fixed-boundary store of face iB (offset of face iB: the
// sum over the earlier faces).
inline long long fix_face_elems(const DevGrid& g, int iB, int nw) {
  const int idim = iB / 2;
  long long n = 2;
  for (int d = 0; d < 3; d++)
    if (d != idim) n *= g.nG[d];
  return n * nw;
}

inline long long ghost_count(const DevGrid& g) {
  long long nzs = g.ndim == 3 ? 4LL * g.nG[1] * g.nG[0] : 0;
  long long nys = g.ndim >= 2 ? 4LL * g.nx[2] * g.nG[0] : 0;
  return nzs + nys + 4LL * g.nx[1] * g.nx[2];
}

// ---------------------------------------------------------------- wrappers

template <class PH, int NDIM, int NDIR, bool MHD>
__global__ void __launch_bounds__(128)
    k_current_field(SweepArgs a, const typename PH::T* __restrict__ w,
                    double* c0, double* c1, double* c2) {
  double* cur[3] = {c0, c1, c2};
  if (MHD) Sweep<PH, NDIM, NDIR, MHD>::current_field(a, w, cur);
}

// (register bounds: 96 for the FP32 state, 128 for FP64 -- the
// predictor waits on its stencil loads and wants the resident warps)
template <class PH, int NDIM, int NDIR, bool MHD>
__global__ void __launch_bounds__(128, sizeof(typename PH::R) == 4 ? 5 : 4)
    k_predict(SweepArgs a, const typename PH::T* __restrict__ w,
              typename PH::T* __restrict__ w1) {
  Sweep<PH, NDIM, NDIR, MHD>::predict(a, w, w1);
}

template <class PH, int NDIM, int NDIR, bool MHD, int D>
__global__ void __launch_bounds__(128)
    k_face(SweepArgs a, const typename PH::T* __restrict__ w1,
           const typename PH::T* __restrict__ base,
           typename PH::R* __restrict__ F) {
  Sweep<PH, NDIM, NDIR, MHD>::template face_pass<128>(a, w1, base, D, F);
}

// the face pass of direction d
template <class PH, int NDIM, int NDIR, bool MHD>
void launch_face_dir(const SweepArgs& a, const typename PH::T* w1,
                     const typename PH::T* base, int d, typename PH::R* F,
                     unsigned nb, cudaStream_t st) {
  if (d == 0)
    k_face<PH, NDIM, NDIR, MHD, 0><<<nb, 128, 0, st>>>(a, w1, base, F);
  else if (NDIM > 1 && d == 1)
    k_face<PH, NDIM, NDIR, MHD, (NDIM > 1 ? 1 : 0)><<<nb, 128, 0, st>>>(a, w1, base, F);
  else if (NDIM > 2)
    k_face<PH, NDIM, NDIR, MHD, (NDIM > 2 ? 2 : 0)><<<nb, 128, 0, st>>>(a, w1, base, F);
}

template <class PH, int NDIM, int NDIR, bool MHD>
__global__ void __launch_bounds__(128)
    k_source_pass(SweepArgs a, const typename PH::T* __restrict__ wct,
                  typename PH::T* __restrict__ w, int pred) {
  Sweep<PH, NDIM, NDIR, MHD>::source_pass(a, wct, w, pred);
}

template <class PH, int NDIM, int NDIR, bool MHD>
__global__ void __launch_bounds__(128)
    k_correct(SweepArgs a, const typename PH::T* __restrict__ w,
              const typename PH::T* __restrict__ w1,
              typename PH::T* __restrict__ wout) {
  Sweep<PH, NDIM, NDIR, MHD>::correct(a, w, w1, wout);
}

template <class PH, int NDIM, int NDIR, bool MHD>
__global__ void __launch_bounds__(128)
    k_pminmax(SweepArgs a, const typename PH::T* __restrict__ w) {
  Sweep<PH, NDIM, NDIR, MHD>::template pminmax<128>(a, w);
}

template <class PH, int NDIM, int NDIR, bool MHD>
__global__ void __launch_bounds__(128)
    k_cell_cmax(SweepArgs a, const typename PH::T* __restrict__ w) {
  Sweep<PH, NDIM, NDIR, MHD>::template cell_cmax<128>(a, w);
}

template <class PH, int NDIM, int NDIR, bool MHD>
__global__ void __launch_bounds__(128)
    k_roundtrip(SweepArgs a, const typename PH::T* __restrict__ w,
                typename PH::T* __restrict__ out) {
  Sweep<PH, NDIM, NDIR, MHD>::roundtrip(a, w, out);
}

template <class PH, int NDIM, int NDIR, bool MHD>
__global__ void __launch_bounds__(128)
    k_kp_rhomin(SweepArgs a, const typename PH::T* __restrict__ w) {
  Sweep<PH, NDIM, NDIR, MHD>::template kp_rhomin<128>(a, w);
}
template <class PH, int NDIM, int NDIR, bool MHD>
__global__ void __launch_bounds__(128)
    k_kp_rho(SweepArgs a, typename PH::T* __restrict__ w) {
  Sweep<PH, NDIM, NDIR, MHD>::kp_rho(a, w);
}
template <class PH, int NDIM, int NDIR, bool MHD>
__global__ void __launch_bounds__(128)
    k_kp_pcheck(SweepArgs a, const typename PH::T* __restrict__ w) {
  Sweep<PH, NDIM, NDIR, MHD>::kp_pcheck(a, w);
}
template <class PH, int NDIM, int NDIR, bool MHD>
__global__ void __launch_bounds__(128)
    k_kp_pfix(SweepArgs a, typename PH::T* __restrict__ w) {
  Sweep<PH, NDIM, NDIR, MHD>::kp_pfix(a, w);
}

// Dispatch on (ndim, ndir, physics) to a template instance.
#define VACGPU_DISPATCH(a, KCALL)                                        \
  do {                                                                   \
    if ((a).mhd) {                                                       \
      if ((a).g.ndim == 1 && (a).ndir == 1) { KCALL(1, 1, true); }       \
      else if ((a).g.ndim == 2 && (a).ndir == 2) { KCALL(2, 2, true); }  \
      else if ((a).g.ndim == 2 && (a).ndir == 3) { KCALL(2, 3, true); }  \
      else if ((a).g.ndim == 3 && (a).ndir == 3) { KCALL(3, 3, true); }  \
    } else {                                                             \
      if ((a).g.ndim == 1 && (a).ndir == 1) { KCALL(1, 1, false); }      \
      else if ((a).g.ndim == 2 && (a).ndir == 2) { KCALL(2, 2, false); } \
      else if ((a).g.ndim == 2 && (a).ndir == 3) { KCALL(2, 3, false); } \
      else if ((a).g.ndim == 3 && (a).ndir == 3) { KCALL(3, 3, false); } \
    }                                                                    \
  } while (0)

inline unsigned grid_for(long long n, int nt) {
  return (unsigned)((n + nt - 1) / nt);
}

template <class PH>
struct Launch {
  typedef typename PH::T T;
  static void predict(const SweepArgs& a, const T* w, T* w1, cudaStream_t st) {
    unsigned nb = grid_for(a.g.ncell, 128);
#define KC(D, C, M) k_predict<PH, D, C, M><<<nb, 128, 0, st>>>(a, w, w1)
    VACGPU_DISPATCH(a, KC);
#undef KC
  }
  // face pass per direction into the face buffer, then the cell pass
  static void correct(const SweepArgs& a, const T* w, const T* w1,
                      const T* base, T* wout, cudaStream_t st) {
    for (int d = a.d0; d <= a.d1; d++) {
      typename PH::R* F = (typename PH::R*)a.faces + (long long)(d - a.d0) * a.face_stride;
      const unsigned nbf = grid_for(face_count(a.g, d), 128);
#define KC(D, C, M) launch_face_dir<PH, D, C, M>(a, w1, base, d, F, nbf, st)
      VACGPU_DISPATCH(a, KC);
#undef KC
    }
    const unsigned nb = grid_for(a.g.ncell, 128);
#define KC(D, C, M) k_correct<PH, D, C, M><<<nb, 128, 0, st>>>(a, w, w1, wout)
    VACGPU_DISPATCH(a, KC);
#undef KC
  }
  static void source_pass(const SweepArgs& a, const T* wct, T* w, int pred,
                          cudaStream_t st) {
    const unsigned nb = grid_for(a.g.ncell, 128);
#define KC(D, C, M) k_source_pass<PH, D, C, M><<<nb, 128, 0, st>>>(a, wct, w, pred)
    VACGPU_DISPATCH(a, KC);
#undef KC
  }
  static void ghost(const SweepArgs& a, T* w, cudaStream_t st) {
    long long n = ghost_count(a.g);
    unsigned nb = grid_for(n, 128);
    int nw = a.mhd ? 2 + 2 * a.ndir : 2 + a.ndir;
    switch (nw) {
      case 3: k_ghost<T, 3><<<nb, 128, 0, st>>>(w, a.g, a.ph, a.ctrl); break;
      case 4: k_ghost<T, 4><<<nb, 128, 0, st>>>(w, a.g, a.ph, a.ctrl); break;
      case 5: k_ghost<T, 5><<<nb, 128, 0, st>>>(w, a.g, a.ph, a.ctrl); break;
      case 6: k_ghost<T, 6><<<nb, 128, 0, st>>>(w, a.g, a.ph, a.ctrl); break;
      case 8: k_ghost<T, 8><<<nb, 128, 0, st>>>(w, a.g, a.ph, a.ctrl); break;
    }
  }
  static void pminmax(const SweepArgs& a, const T* w, cudaStream_t st) {
    unsigned nb = grid_for(a.g.ncell, 128);
    if (nb > 1216) nb = 1216;  // grid-stride: a no-op step costs one wave
#define KC(D, C, M) k_pminmax<PH, D, C, M><<<nb, 128, 0, st>>>(a, w)
    VACGPU_DISPATCH(a, KC);
#undef KC
  }
  static void cell_cmax(const SweepArgs& a, const T* w, cudaStream_t st) {
    unsigned nb = grid_for(a.g.ncell, 128);
    if (nb > 1216) nb = 1216;
#define KC(D, C, M) k_cell_cmax<PH, D, C, M><<<nb, 128, 0, st>>>(a, w)
    VACGPU_DISPATCH(a, KC);
#undef KC
  }
  // getboundary face by face (grids with fixed/extrapolating faces)
  static void ghost_faces(const SweepArgs& a, T* w, T* fixb, int restore,
                          cudaStream_t st) {
    for (int iB = 0; iB < 2 * a.g.ndim; iB++) ghost_face(a, w, fixb, restore, iB, st);
  }
  // region iB alone (its stored values follow those of the regions before)
  static void ghost_face(const SweepArgs& a, T* w, T* fixb, int restore, int iB,
                         cudaStream_t st) {
    const int nw = a.mhd ? 2 + 2 * a.ndir : 2 + a.ndir;
    long long off = 0;
    for (int j = 0; j < iB; j++) off += fix_face_elems(a.g, j, nw);
    const long long tot = fix_face_elems(a.g, iB, 1);
    const unsigned nb = grid_for(tot, 128);
    T* fb = fixb + off;
    switch (nw) {
      case 3: k_ghost_face<T, 3><<<nb, 128, 0, st>>>(w, a.g, a.ph, a.ctrl, iB, fb, restore); break;
      case 4: k_ghost_face<T, 4><<<nb, 128, 0, st>>>(w, a.g, a.ph, a.ctrl, iB, fb, restore); break;
      case 5: k_ghost_face<T, 5><<<nb, 128, 0, st>>>(w, a.g, a.ph, a.ctrl, iB, fb, restore); break;
      case 6: k_ghost_face<T, 6><<<nb, 128, 0, st>>>(w, a.g, a.ph, a.ctrl, iB, fb, restore); break;
      case 8: k_ghost_face<T, 8><<<nb, 128, 0, st>>>(w, a.g, a.ph, a.ctrl, iB, fb, restore); break;
    }
  }
  static void current_field(const SweepArgs& a, const T* w, double* const* cur,
                            cudaStream_t st) {
    long long n = 1;
    for (int d = 0; d < 3; d++) n *= d < a.g.ndim ? a.g.nx[d] + 2 : 1;
    const unsigned nb = grid_for(n, 128);
#define KC(D, C, M) \
  k_current_field<PH, D, C, M><<<nb, 128, 0, st>>>(a, w, cur[0], cur[1], cur[2])
    VACGPU_DISPATCH(a, KC);
#undef KC
  }
  static void fix_store(const SweepArgs& a, const T* w, T* fixb, cudaStream_t st) {
    const int nw = a.mhd ? 2 + 2 * a.ndir : 2 + a.ndir;
    long long off = 0;
    for (int iB = 0; iB < 2 * a.g.ndim; iB++) {
      const unsigned nb = grid_for(fix_face_elems(a.g, iB, 1), 128);
      T* fb = fixb + off;
      switch (nw) {
        case 3: k_fix_store<T, 3><<<nb, 128, 0, st>>>(w, a.g, a.ph, iB, fb); break;
        case 4: k_fix_store<T, 4><<<nb, 128, 0, st>>>(w, a.g, a.ph, iB, fb); break;
        case 5: k_fix_store<T, 5><<<nb, 128, 0, st>>>(w, a.g, a.ph, iB, fb); break;
        case 6: k_fix_store<T, 6><<<nb, 128, 0, st>>>(w, a.g, a.ph, iB, fb); break;
        case 8: k_fix_store<T, 8><<<nb, 128, 0, st>>>(w, a.g, a.ph, iB, fb); break;
      }
      off += fix_face_elems(a.g, iB, nw);
    }
  }
  static void roundtrip(const SweepArgs& a, const T* w, T* out, cudaStream_t st) {
    const long long n = (long long)a.g.nG[0] * a.g.nG[1] * a.g.nG[2];
#define KC(D, C, M) k_roundtrip<PH, D, C, M><<<grid_for(n, 128), 128, 0, st>>>(a, w, out)
    VACGPU_DISPATCH(a, KC);
#undef KC
  }
  // keeppositive on the mesh of w (getboundary with smallfix=T,
  // src/vacgrid.t:213); decisions stay on the device.
  static void keeppositive(const SweepArgs& a, T* w, cudaStream_t st) {
    const unsigned nb = grid_for(a.g.ncell, 128);
    const unsigned nr = nb > 1216 ? 1216 : nb;
    const bool floor = a.ph.vacuumrho < 0.0;
    launch_kp_begin(a.ctrl, floor, st);
    if (floor) {
#define KC(D, C, M) k_kp_rhomin<PH, D, C, M><<<nr, 128, 0, st>>>(a, w)
      VACGPU_DISPATCH(a, KC);
#undef KC
      launch_kp_smallrho(a.ctrl, a.ph.smallrhocoeff, st);
    }
#define KC(D, C, M) k_kp_rho<PH, D, C, M><<<nb, 128, 0, st>>>(a, w)
    VACGPU_DISPATCH(a, KC);
#undef KC
    pminmax(a, w, st);  // getpthermal's one-time smallp, if still unset
    launch_smallp(a.ctrl, a.mhd, a.ph.smallpcoeff, st);
#define KC(D, C, M) k_kp_pcheck<PH, D, C, M><<<nb, 128, 0, st>>>(a, w)
    VACGPU_DISPATCH(a, KC);
#undef KC
#define KC(D, C, M) k_kp_pfix<PH, D, C, M><<<nb, 128, 0, st>>>(a, w)
    VACGPU_DISPATCH(a, KC);
#undef KC
    launch_kp_end(a.ctrl, st);
  }
};

#define VACGPU_DEFINE_LAUNCHERS(SUF, PH)                                      \
  void launch_predict_##SUF(const SweepArgs& s, const PH::T* w, PH::T* w1,   \
                            cudaStream_t st) {                               \
    Launch<PH>::predict(s, w, w1, st);                                       \
  }                                                                          \
  void launch_correct_##SUF(const SweepArgs& s, const PH::T* w,              \
                            const PH::T* w1, const PH::T* base, PH::T* wout, \
                            cudaStream_t st) {                               \
    Launch<PH>::correct(s, w, w1, base, wout, st);                           \
  }                                                                          \
  void launch_ghost_##SUF(const SweepArgs& s, PH::T* w, cudaStream_t st) {   \
    Launch<PH>::ghost(s, w, st);                                             \
  }                                                                          \
  void launch_source_pass_##SUF(const SweepArgs& s, const PH::T* wct,        \
                                PH::T* w, int pred, cudaStream_t st) {       \
    Launch<PH>::source_pass(s, wct, w, pred, st);                            \
  }                                                                          \
  void launch_pminmax_##SUF(const SweepArgs& s, const PH::T* w,              \
                            cudaStream_t st) {                               \
    Launch<PH>::pminmax(s, w, st);                                           \
  }                                                                          \
  void launch_cell_cmax_##SUF(const SweepArgs& s, const PH::T* w,            \
                              cudaStream_t st) {                             \
    Launch<PH>::cell_cmax(s, w, st);                                         \
  }                                                                          \
  void launch_keeppositive_##SUF(const SweepArgs& s, PH::T* w,               \
                                 cudaStream_t st) {                          \
    Launch<PH>::keeppositive(s, w, st);                                      \
  }                                                                          \
  void launch_roundtrip_##SUF(const SweepArgs& s, const PH::T* w,            \
                              PH::T* out, cudaStream_t st) {                 \
    Launch<PH>::roundtrip(s, w, out, st);                                    \
  }                                                                          \
  void launch_ghost_faces_##SUF(const SweepArgs& s, PH::T* w, PH::T* fixb,    \
                                int restore, cudaStream_t st) {              \
    Launch<PH>::ghost_faces(s, w, fixb, restore, st);                        \
  }                                                                          \
  void launch_ghost_face_##SUF(const SweepArgs& s, PH::T* w, PH::T* fixb,     \
                               int restore, int iB, cudaStream_t st) {       \
    Launch<PH>::ghost_face(s, w, fixb, restore, iB, st);                     \
  }                                                                          \
  void launch_fix_store_##SUF(const SweepArgs& s, const PH::T* w,            \
                              PH::T* fixb, cudaStream_t st) {                \
    Launch<PH>::fix_store(s, w, fixb, st);                                   \
  }                                                                          \
  void launch_current_field_##SUF(const SweepArgs& s, const PH::T* w,        \
                                  double* const* cur, cudaStream_t st) {     \
    Launch<PH>::current_field(s, w, cur, st);                                \
  }

}  // namespace vacgpu

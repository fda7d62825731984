// control.cuh - device functions of VAC's time-loop control
// (src/vac.t:59-106): the dt choice of getdt_courant (src/vac.t:664-722),
// getdt_special, dtcantgrow, slowsteps and tmaxexact, the timetofinish
// test (src/vac.t:608-628), and the step epilogue (CFL bookkeeping of
// src/vactvdlf.t:184-201, it+1, t+dt).  Each runs on one 128-thread block
// for one grid's control block; the control kernels (control.cu) and the
// persistent batched step (sweep_line2.cu) call them.  The reduction slots
// (face_cmax, cell_cmax, pmin, pmax) are filled by atomics from every SM,
// so they are read through L2 (ld.global.cg): a kernel that runs several
// steps must not see a line its SM cached from an earlier step.
#pragma once
#include "vacgpu_internal.h"

namespace vacgpu {

static constexpr double BIG = 1.0e99;
static constexpr double SMALL = 1.0e-99;

// max/min of NSLOT ordered keys with one 128-thread block (thread 0 result)
__device__ __forceinline__ unsigned long long fold_max(const unsigned long long* s) {
  __shared__ unsigned long long sh[NSLOT];
  unsigned long long k = __ldcg(s + threadIdx.x);
  sh[threadIdx.x] = k;
  __syncthreads();
  for (int o = NSLOT / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      unsigned long long v = sh[threadIdx.x + o];
      if (v > sh[threadIdx.x]) sh[threadIdx.x] = v;
    }
    __syncthreads();
  }
  unsigned long long r = sh[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ void dt_begin_dev(Ctrl* c, int ndim) {
  __shared__ int stop;
  if (threadIdx.x == 0) {
    stop = c->done;
    if (!stop && c->steps >= c->maxsteps) {
      c->done = 3;
      stop = 1;
    }
    if (!stop) {
      const bool courant = !(c->dtpar > 0.0) && c->courantpar > 0.0;
      int any = 0;
      for (int d = 0; d < 3; d++) {
        c->need_cell[d] = (d < ndim && courant && !(c->dtcourant[d] < BIG));
        any |= c->need_cell[d];
      }
      c->need_smallp = any && c->smallp < 0.0;
    }
  }
  __syncthreads();
  if (stop) return;
  const int i = threadIdx.x;
  for (int d = 0; d < 3; d++) {
    c->face_cmax[d][i] = 0ULL;
    c->face_cmax2[d][i] = 0ULL;
    c->cell_cmax[d][i] = 0ULL;
  }
  c->pmin[i] = ~0ULL;
  c->pmax[i] = 0ULL;
}

// smallp = minval(p)*smallpcoeff at the first getpthermal call; MHD falls
// back to maxval(p)*smallpcoeff for a negative minimum
// (src/vacphys0.t.mhd:202-217, src/vacphys0.t.hd:123-126).
__device__ __forceinline__ void smallp_dev(Ctrl* c, int mhd, double coeff) {
  if (c->done || !c->need_smallp) return;
  unsigned long long kmax = fold_max(c->pmax);
  __shared__ unsigned long long sh[NSLOT];
  sh[threadIdx.x] = ~__ldcg(c->pmin + threadIdx.x);
  __syncthreads();
  for (int o = NSLOT / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o && sh[threadIdx.x + o] > sh[threadIdx.x])
      sh[threadIdx.x] = sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double pmin = dkey_inv(~sh[0]);
    double pmax = dkey_inv(kmax);
    double sp = pmin * coeff;
    if (mhd && sp < 0.0) sp = pmax * coeff;
    c->smallp = sp;
    c->need_smallp = 0;
  }
}

struct DtEndArgs {
  int ndim, itmax, slowsteps, dtcantgrow, tmaxexact;
  double tmax, dtmin;
  int etafield;       // specialeta: dtdiff from the field's max eta/dx^2
  double dtdiffpar;
};
DtEndArgs dt_end_args(const vacgpu_params& p);  // control.cu

__device__ __forceinline__ void dt_end_dev(Ctrl* c, const DtEndArgs& p) {
  if (c->done) return;
  unsigned long long km[3] = {0, 0, 0};
  for (int d = 0; d < p.ndim; d++)
    if (c->need_cell[d]) km[d] = fold_max(c->cell_cmax[d]);
  if (threadIdx.x != 0) return;
  double dt;
  double dtc_save[3] = {c->dtcourant[0], c->dtcourant[1], c->dtcourant[2]};
  const double dtold_save = c->dtold;
  const bool courant = c->courantpar > 0.0;
  if (c->dtpar > 0.0) {
    dt = c->dtpar;
  } else {
    dt = c->dt;
    if (courant) {
      // getdt_courant
      dt = BIG;
      double courantmax = 0.0;
      for (int d = 0; d < p.ndim; d++) {
        if (c->dtcourant[d] < BIG) {
          if (c->dtcourant[d] < dt) dt = c->dtcourant[d];
        } else {
          double m = dkey_inv(km[d]);
          if (m > courantmax) courantmax = m;
        }
      }
      for (int d = 0; d < 3; d++) c->dtcourant[d] = BIG;
      if (courantmax > SMALL) {
        double q = c->courantpar / courantmax;
        if (q < dt) dt = q;
      }
    }
    // getdt: the resistive diffusion limit (getdt_res,
    // src/vacphys.mhdres.t:5-45), fixed by the grid
    if (p.etafield) {
      // min over idim of dtdiffpar/(smalldouble+max(eta/dx^2))
      double dtdiff = BIG;
      for (int d = 0; d < p.ndim; d++) {
        const double q = p.dtdiffpar / (SMALL + dkey_inv(c->etak[d]));
        if (q < dtdiff) dtdiff = q;
      }
      if (dtdiff < dt) dt = dtdiff;
    } else if (c->dtdiff < dt) {
      dt = c->dtdiff;
    }
    // getdt_special (uniform gravity: dtgrav fixed at the first step; the
    // user's hook: its limit of this step)
    if (c->dtgrav < dt) dt = c->dtgrav;
    if (c->dtspecial < dt) dt = c->dtspecial;
    if (p.dtcantgrow && c->it > c->itmin && c->dtold < dt) dt = c->dtold;
    c->dtold = dt;
  }
  // timetofinish (residual tests off)
  if (c->it >= p.itmax || c->t >= p.tmax || dt < p.dtmin) {
    c->dt = dt;
    c->done = 1;
    return;
  }
  if (c->t >= c->tstop) {
    // the caller saves before this step; the dt choice is made again then
    for (int d = 0; d < 3; d++) c->dtcourant[d] = dtc_save[d];
    c->dtold = dtold_save;
    c->done = 2;
    return;
  }
  if (p.slowsteps == 1 && c->it == c->itmin) c->dtpar = -1.0;
  if (p.slowsteps > c->it - c->itmin + 1) {
    double r = 1.0 - (c->it - c->itmin + 1.0) / p.slowsteps;
    // explicit roundings: the same bits whatever the unit's contraction flags
    dt = __dmul_rn(dt, __dsub_rn(1.0, __dmul_rn(r, r)));
  }
  if (p.tmaxexact) {
    double q = p.tmax - c->t + SMALL;
    if (q < dt) dt = q;
  }
  c->dt = dt;
}

// After the last sweep: fold the correctors' CFL maxima into dtcourant
// (src/vactvdlf.t:184-201; 'tvdmu': the fast waves' normalised
// eigenvalues, src/vactvd.t:144-160), count Courant violations, it+1, t+dt.
// toggle: the number of buffer swaps of one step (batched grids).
__device__ __forceinline__ void step_end_dev(Ctrl* c, int ndim, int toggle) {
  if (c->done) return;
  unsigned long long km[3] = {0, 0, 0}, km2[3] = {0, 0, 0};
  if (c->courantpar > 0.0)
    for (int d = 0; d < ndim; d++) {
      km[d] = fold_max(c->face_cmax[d]);
      if (c->roe) km2[d] = fold_max(c->face_cmax2[d]);
    }
  if (threadIdx.x != 0) return;
  for (int d = 0; d < ndim; d++) {
    if (c->roe) {
      // courantmax = max|a*dt*2/(dx+dx)| per wave; dtcourant =
      // min(dtcourant, dt*courantpar/courantmax)
      const unsigned long long ks[2] = {km[d], km2[d]};
      for (int k = 0; k < 2; k++) {
        if (!ks[k]) continue;
        double cm = dkey_inv(ks[k]);
        if (cm > 1.0) c->nerror[2]++;
        if (cm > SMALL) {
          double q = c->dt * c->courantpar / cm;
          if (q < c->dtcourant[d]) c->dtcourant[d] = q;
        }
      }
      continue;
    }
    if (!km[d]) continue;
    double cm = dkey_inv(km[d]);
    if (c->dt * cm > 1.0) c->nerror[2]++;
    if (cm > SMALL) {
      double q = c->courantpar / cm;
      if (q < c->dtcourant[d]) c->dtcourant[d] = q;
    }
  }
  c->it = c->it + 1;
  c->t = c->t + c->dt;
  c->steps = c->steps + 1;
  c->cur ^= toggle;
}

}  // namespace vacgpu

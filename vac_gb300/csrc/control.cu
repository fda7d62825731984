// control.cu - device side of VAC's time loop (src/vac.t:59-106): the dt
// choice of getdt_courant (src/vac.t:664-722), getdt_special, dtcantgrow,
// slowsteps and tmaxexact, the timetofinish test (src/vac.t:608-628), and the
// step epilogue (CFL bookkeeping of src/vactvdlf.t:184-201, it+1, t+dt).
// Single-block kernels: a few hundred words of control state.
#include "vacgpu_internal.h"

namespace vacgpu {

static constexpr double BIG = 1.0e99;
static constexpr double SMALL = 1.0e-99;

// max/min of NSLOT ordered keys with one 128-thread block (thread 0 result)
__device__ unsigned long long fold_max(const unsigned long long* s) {
  __shared__ unsigned long long sh[NSLOT];
  unsigned long long k = s[threadIdx.x];
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

__device__ void dt_begin_dev(Ctrl* c, int ndim) {
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
__device__ void smallp_dev(Ctrl* c, int mhd, double coeff) {
  if (c->done || !c->need_smallp) return;
  unsigned long long kmax = fold_max(c->pmax);
  __shared__ unsigned long long sh[NSLOT];
  sh[threadIdx.x] = ~c->pmin[threadIdx.x];
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

__device__ void dt_end_dev(Ctrl* c, const DtEndArgs& p) {
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
    dt = dt * (1.0 - r * r);
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
__device__ void step_end_dev(Ctrl* c, int ndim, int toggle) {
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

__global__ void k_dt_begin(Ctrl* c, int ndim) { dt_begin_dev(c, ndim); }
// getboundary's qt: t (before the loop), qt+qdt = t+dt/2 after the
// predictor and t+dt after the corrector (src/vac.t:54,567)
__global__ void k_set_qt(Ctrl* c, int mode) {
  c->qt = mode == 0 ? c->t : mode == 1 ? c->t + c->dt / 2 : c->t + c->dt;
}
__global__ void k_smallp(Ctrl* c, int mhd, double coeff) {
  smallp_dev(c, mhd, coeff);
}
__global__ void k_dt_end(Ctrl* c, DtEndArgs p) { dt_end_dev(c, p); }
__global__ void k_step_end(Ctrl* c, int ndim) { step_end_dev(c, ndim, 0); }

// batched: block b serves grid b
__global__ void kb_dt_begin(Ctrl* const* cs, int ndim) {
  dt_begin_dev(cs[blockIdx.x], ndim);
}
__global__ void kb_smallp(Ctrl* const* cs, int mhd, double coeff) {
  smallp_dev(cs[blockIdx.x], mhd, coeff);
}
__global__ void kb_dt_end(Ctrl* const* cs, DtEndArgs p) {
  dt_end_dev(cs[blockIdx.x], p);
}
__global__ void kb_step_end(Ctrl* const* cs, int ndim, int toggle) {
  step_end_dev(cs[blockIdx.x], ndim, toggle);
}
__global__ void kb_call_begin(Ctrl* const* cs, int maxsteps, double tstop) {
  Ctrl* c = cs[blockIdx.x];
  if (threadIdx.x == 0) {
    c->done = 0;
    c->steps = 0;
    c->maxsteps = maxsteps;
    c->tstop = tstop;
  }
}

// the arguments of a specialsource hook call, in the reference's double
// arithmetic: qdt*(idimmax-idimmin+1)/ndim with qdt = dt/2 (predictor) or
// dt, and qtC = t or t+dt/2 (src/vac.t:407,426-427, src/vactvdlf.t:85,292)
__global__ void k_src_args(Ctrl* c, int pred, int half, int nsweep, int ndim) {
  if (c->done) return;
  const double qdt = pred ? c->dt / 2 : c->dt;
  c->src_qdt = qdt * (double)nsweep / ndim;
  c->src_qtc = half ? c->t + c->dt / 2 : c->t;
}
__global__ void k_dtspecial_begin(Ctrl* c) { c->dtspecial = BIG; }

void launch_src_args(Ctrl* c, int pred, int half, int nsweep, int ndim, cudaStream_t st) {
  k_src_args<<<1, 1, 0, st>>>(c, pred, half, nsweep, ndim);
}
void launch_dtspecial_begin(Ctrl* c, cudaStream_t st) { k_dtspecial_begin<<<1, 1, 0, st>>>(c); }

void launch_dt_begin(Ctrl* c, int ndim, cudaStream_t st) {
  k_dt_begin<<<1, NSLOT, 0, st>>>(c, ndim);
}
void launch_smallp(Ctrl* c, int mhd, double coeff, cudaStream_t st) {
  k_smallp<<<1, NSLOT, 0, st>>>(c, mhd, coeff);
}

// keeppositive (src/vacphys.t.mhd:9-53, src/vacproc.positive.t:2-34):
// the one-time smallrho (min(rho)*smallrhocoeff, when the density floor is
// in use and smallrho is still -1) and smallp (getpthermal's first call)
// minima are due when their value is unset.
__global__ void k_kp_begin(Ctrl* c, int rho_floor) {
  __shared__ int need_r, need_p;
  if (threadIdx.x == 0) {
    need_r = need_p = 0;
    if (!c->done) {
      need_r = rho_floor && c->smallrho == -1.0;
      need_p = c->smallp < 0.0;
      c->need_smallrho = need_r;
      c->need_smallp = need_p;
    }
  }
  __syncthreads();
  const int i = threadIdx.x;
  if (need_r) c->rmin[i] = ~0ULL;
  if (need_p) {
    c->pmin[i] = ~0ULL;
    c->pmax[i] = 0ULL;
  }
}
__global__ void k_kp_smallrho(Ctrl* c, double coeff) {
  if (c->done || !c->need_smallrho) return;
  __shared__ unsigned long long sh[NSLOT];
  sh[threadIdx.x] = ~c->rmin[threadIdx.x];
  __syncthreads();
  for (int o = NSLOT / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o && sh[threadIdx.x + o] > sh[threadIdx.x])
      sh[threadIdx.x] = sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    c->smallrho = dkey_inv(~sh[0]) * coeff;
    c->need_smallrho = 0;
  }
}
__global__ void k_kp_end(Ctrl* c) {
  if (c->done) return;
  c->nerror[0] += c->kp_p;  // toosmallp_
  c->nerror[1] += c->kp_r;  // toosmallr_
  c->kp_p = 0;
  c->kp_r = 0;
}
void launch_kp_begin(Ctrl* c, int rho_floor, cudaStream_t st) {
  k_kp_begin<<<1, NSLOT, 0, st>>>(c, rho_floor);
}
void launch_kp_smallrho(Ctrl* c, double coeff, cudaStream_t st) {
  k_kp_smallrho<<<1, NSLOT, 0, st>>>(c, coeff);
}
void launch_kp_end(Ctrl* c, cudaStream_t st) { k_kp_end<<<1, 1, 0, st>>>(c); }
// Ctrl::etak = max over the mesh of eta/dx_d^2 (getdt_res,
// src/vacphys.mhdres.t:31-35); first_only: only at it==itmin
__global__ void k_eta_reset(Ctrl* c, int first_only) {
  if (c->done || (first_only && c->it != c->itmin)) return;
  for (int d = 0; d < 3; d++) c->etak[d] = 0ULL;
}
__global__ void k_eta_max(SweepArgs a, int first_only) {
  Ctrl* c = a.ctrl;
  if (c->done || (first_only && c->it != c->itmin)) return;
  const DevGrid& g = a.g;
  unsigned long long key[3] = {0ULL, 0ULL, 0ULL};
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
       n < g.ncell; n += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(n % g.nx[0]);
    const long long r = n / g.nx[0];
    const int iy = (int)(r % g.nx[1]), iz = (int)(r / g.nx[1]);
    const int cc[3] = {ix + g.gh[0], iy + g.gh[1], iz + g.gh[2]};
    const double e = a.etaf[gidx(g, cc[0], cc[1], cc[2])];
    for (int d = 0; d < g.ndim; d++) {
      const double dx = a.a.dx[d][cc[d]];
      const unsigned long long k = dkey(e / (dx * dx));
      if (k > key[d]) key[d] = k;
    }
  }
  for (int d = 0; d < g.ndim; d++) {
    unsigned long long k = key[d];
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long v = __shfl_xor_sync(0xffffffffu, k, o);
      k = v > k ? v : k;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(&c->etak[d], k);
  }
}

void launch_eta_max(const SweepArgs& a, int first_only, cudaStream_t st) {
  k_eta_reset<<<1, 1, 0, st>>>(a.ctrl, first_only);
  k_eta_max<<<2 * 152, 256, 0, st>>>(a, first_only);
}

void launch_set_qt(Ctrl* c, int mode, cudaStream_t st) {
  k_set_qt<<<1, 1, 0, st>>>(c, mode);
}

void launch_dt_end(Ctrl* c, const vacgpu_params& p, cudaStream_t st) {
  DtEndArgs a;
  a.etafield = p.physics == VACGPU_PHYS_MHD && p.eqpar[1] < 0.0;
  a.dtdiffpar = p.dtdiffpar;
  a.ndim = p.ndim;
  a.itmax = p.itmax;
  a.slowsteps = p.slowsteps;
  a.dtcantgrow = p.dtcantgrow;
  a.tmaxexact = p.tmaxexact;
  a.tmax = p.tmax;
  a.dtmin = p.dtmin;
  k_dt_end<<<1, NSLOT, 0, st>>>(c, a);
}
void launch_step_end(Ctrl* c, int ndim, cudaStream_t st) {
  k_step_end<<<1, NSLOT, 0, st>>>(c, ndim);
}

static DtEndArgs dt_end_args(const vacgpu_params& p) {
  DtEndArgs a;
  a.etafield = p.physics == VACGPU_PHYS_MHD && p.eqpar[1] < 0.0;
  a.dtdiffpar = p.dtdiffpar;
  a.ndim = p.ndim;
  a.itmax = p.itmax;
  a.slowsteps = p.slowsteps;
  a.dtcantgrow = p.dtcantgrow;
  a.tmaxexact = p.tmaxexact;
  a.tmax = p.tmax;
  a.dtmin = p.dtmin;
  return a;
}

void launchb_control(int which, Ctrl* const* cs, int n, const vacgpu_params& p,
                     int toggle, int maxsteps, double tstop, cudaStream_t st) {
  switch (which) {
    case 0: kb_dt_begin<<<n, NSLOT, 0, st>>>(cs, p.ndim); break;
    case 1:
      kb_smallp<<<n, NSLOT, 0, st>>>(cs, p.physics == VACGPU_PHYS_MHD,
                                     p.smallpcoeff);
      break;
    case 2: kb_dt_end<<<n, NSLOT, 0, st>>>(cs, dt_end_args(p)); break;
    case 3: kb_step_end<<<n, NSLOT, 0, st>>>(cs, p.ndim, toggle); break;
    case 4: kb_call_begin<<<n, 32, 0, st>>>(cs, maxsteps, tstop); break;
  }
}

}  // namespace vacgpu

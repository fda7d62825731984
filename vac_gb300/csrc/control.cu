// control.cu - device side of VAC's time loop (src/vac.t:59-106): the dt
// choice of getdt_courant (src/vac.t:664-722), getdt_special, dtcantgrow,
// slowsteps and tmaxexact, the timetofinish test (src/vac.t:608-628), and the
// step epilogue (CFL bookkeeping of src/vactvdlf.t:184-201, it+1, t+dt).
// Single-block kernels: a few hundred words of control state.
#include "control.cuh"

namespace vacgpu {

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

DtEndArgs dt_end_args(const vacgpu_params& p) {
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

void launch_dt_end(Ctrl* c, const vacgpu_params& p, cudaStream_t st) {
  k_dt_end<<<1, NSLOT, 0, st>>>(c, dt_end_args(p));
}
void launch_step_end(Ctrl* c, int ndim, cudaStream_t st) {
  k_step_end<<<1, NSLOT, 0, st>>>(c, ndim);
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

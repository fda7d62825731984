// vacgpu.cu - the C ABI of include/vacgpu.h: handle life cycle, grid set-up
// (gridsetup1), state transfer, the device-resident time loop and the
// conservation sums.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "vacgpu_internal.h"

using namespace vacgpu;

namespace {

thread_local std::string g_err;

int fail(const std::string& m) {
  g_err = m;
  return 1;
}

#define CK(call)                                                        \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess)                                              \
      return fail(std::string("CUDA error: ") + cudaGetErrorString(e_) + \
                  " at " #call);                                        \
  } while (0)

const double BIGD = 1.0e99;

// mesh <-> padded state transfer (VAC column-major mesh blocks per variable)
template <typename T>
__global__ void k_scatter(const double* __restrict__ src, T* __restrict__ w,
                          DevGrid g, int nw) {
  long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.ncell * nw) return;
  int iw = (int)(n / g.ncell);
  long long m = n % g.ncell;
  int ix = (int)(m % g.nx[0]);
  long long r = m / g.nx[0];
  int iy = (int)(r % g.nx[1]);
  int iz = (int)(r / g.nx[1]);
  w[gidx(g, ix + g.gh[0], iy + g.gh[1], iz + g.gh[2]) + iw * g.vs] = (T)src[n];
}

template <typename T>
__global__ void k_gather(const T* __restrict__ w, double* __restrict__ dst,
                         DevGrid g, int nw) {
  long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.ncell * nw) return;
  int iw = (int)(n / g.ncell);
  long long m = n % g.ncell;
  int ix = (int)(m % g.nx[0]);
  long long r = m / g.nx[0];
  int iy = (int)(r % g.nx[1]);
  int iz = (int)(r / g.nx[1]);
  dst[n] = (double)w[gidx(g, ix + g.gh[0], iy + g.gh[1], iz + g.gh[2]) +
                     iw * g.vs];
}

// Volume sums: per block partial sums of dvolume*w in FP64, folded in a
// fixed order by a second kernel (deterministic).
template <typename T>
__global__ void k_sums_partial(const T* __restrict__ w, DevGrid g, int nw,
                               const double* dx0, const double* dx1,
                               const double* dx2, double* part) {
  __shared__ double sh[8][256 / 32];
  long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double acc[8];
  for (int iw = 0; iw < 8; iw++) acc[iw] = 0.0;
  if (n < g.ncell) {
    int ix = (int)(n % g.nx[0]);
    long long r = n / g.nx[0];
    int iy = (int)(r % g.nx[1]);
    int iz = (int)(r / g.nx[1]);
    int gx = ix + g.gh[0], gy = iy + g.gh[1], gz = iz + g.gh[2];
    double dv = dx0[gx];
    if (g.ndim > 1) dv = dv * dx1[gy];
    if (g.ndim > 2) dv = dv * dx2[gz];
    long long off = gidx(g, gx, gy, gz);
    for (int iw = 0; iw < nw; iw++) acc[iw] = dv * (double)w[off + iw * g.vs];
  }
  for (int iw = 0; iw < nw; iw++) {
    double v = acc[iw];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[iw][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < nw) {
    double s = 0.0;
    for (int i = 0; i < 256 / 32; i++) s += sh[threadIdx.x][i];
    part[(long long)blockIdx.x * nw + threadIdx.x] = s;
  }
}

__global__ void k_sums_final(const double* part, long long nblk, int nw,
                             double* out) {
  int iw = threadIdx.x;
  if (iw >= nw) return;
  double s = 0.0;
  for (long long b = 0; b < nblk; b++) s += part[b * nw + iw];
  out[iw] = s;
}

__global__ void k_call_begin(Ctrl* c, int maxsteps, double tstop) {
  c->done = 0;
  c->steps = 0;
  c->maxsteps = maxsteps;
  c->tstop = tstop;
}

}  // namespace

int vacgpu_internal_fail(const char* msg) { return fail(msg); }

struct HandleView {
  DevGrid g;
  DevPhys ph;
  SweepArgs sa;
  float* buf[2];
  const float* dxf[3];
  const float* idxf[3];
  Ctrl* ctrl;
  const void* tmap[2][2];  // [state buffer][box: x/z sweeps, y sweep]
  int nzc;
  bool fused;
};

struct vacgpu_handle {
  vacgpu_params p;
  DevGrid g;
  DevPhys ph;
  int nw;
  size_t elem;
  void* buf[3];      // two state buffers (ping-pong) + predictor output
  void* wold;        // step-start copy for typelimited='previous' when split
  void* fixb;        // stored ghost values of fixed/fixed1/grad1 faces
  vacgpu_bound_fn bound_fn;  // specialbound hook
  void* bound_user;
  bool hook_failed;  // a hook returned non-zero while a step was issued
  // A bounded device wait of the fused sweep gave up (Ctrl::fault): some
  // tiles of that sweep were not written, so the state is invalid.  Steps
  // are refused until vacgpu_upload gives the handle a new state.
  bool faulted;
  vacgpu_eta_fn eta_fn;  // specialeta hook (eqpar(eta_) < 0)
  void* eta_user;
  vacgpu_source_fn src_fn;       // the user's specialsource
  vacgpu_dtspecial_fn dtsp_fn;   // the user's getdt_special
  void* src_user;
  double* etaf;      // its eta field, gradeta (compactres) and the current
  double* gradetaf[3];
  double* curf[3];
  void* faces;       // the split correctors' face buffer
  long long face_stride;
  bool any_special;
  unsigned special[VACGPU_MAXB];  // per region: bit iw 'special'
  double* xg[3];     // cell centres over the ghost box (specialbound hooks)
  int cur;           // which of buf[0], buf[1] holds the state
  double* dx[3];
  float* dxf[3];
  std::vector<double> hdx[3];
  double volume;
  double* stage;     // mesh-ordered FP64 transfer buffer
  double* part;      // sums partials
  double* sums;
  Ctrl* ctrl;
  cudaStream_t st;
  int it_host;
  double dtgrav;
  double dtdiff;     // resistive diffusion dt limit (getdt_res), BIG if ideal
  bool have_grid, have_state;
  int pmode;         // mixed pressure variant (0 ff, 1 native f64, 2 f32)
  cudaStream_t own_st;
  // kernel statistics
  long long nlaunch[VACGPU_K_NCLASS];
  double kms[VACGPU_K_NCLASS];
  bool timing;
  struct Ev {
    int k;
    cudaEvent_t a, b;
  };
  std::vector<Ev> pending;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t open_ev;
  int open_k;
  // fused mixed sweep: TMA descriptors of the two state buffers, 1/dx
  // CUDA graphs of two consecutive steps, keyed by (state buffer, parity
  // of it): replayed instead of re-issuing ~20 launches per step.
  cudaGraphExec_t gexec[2][2];
  long long glaunch[2][2][VACGPU_K_NCLASS];  // kernels per replay, by class
  bool warmed;
  bool fused;
  CUtensorMap tmap[2][2];  // [state buffer][x/z sweeps, y sweep]
  float* idxf[3];
  int nzc;
  // z-chunk tuning of the fused 3-D sweep (results do not depend on the
  // chunk): pending until the first vacgpu_step call, which times one step
  // per candidate from a snapshot of the state and keeps the fastest
  bool tuning;
  int tncand;
  int tcand[6];
  // asynchronous snapshots (vacgpu_snapshot_begin/wait): per slot the
  // mesh-ordered FP64 copy on the device, its page-locked host copy, and
  // the events that order the gather (on st) and the download (on cst)
  struct Snap {
    double* dev;
    double* host;
    cudaEvent_t gathered, copied;
    bool pending;
    bool ready;  // host holds a completed snapshot (until the next begin)
  };
  Snap snap[2];
  cudaStream_t cst;  // copy stream of the snapshot downloads
};

namespace {

cudaEvent_t get_event(vacgpu_handle* h) {
  if (!h->pool.empty()) {
    cudaEvent_t e = h->pool.back();
    h->pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

// Bracket the next launch of class k (events only while timing is on).
void kbegin(vacgpu_handle* h, int k) {
  h->nlaunch[k]++;
  if (!h->timing) return;
  h->open_ev = get_event(h);
  h->open_k = k;
  cudaEventRecord(h->open_ev, h->st);
}
void kend(vacgpu_handle* h) {
  if (!h->timing) return;
  cudaEvent_t b = get_event(h);
  cudaEventRecord(b, h->st);
  h->pending.push_back({h->open_k, h->open_ev, b});
}

void drain_events(vacgpu_handle* h) {
  for (auto& e : h->pending) {
    cudaEventSynchronize(e.b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e.a, e.b);
    h->kms[e.k] += ms;
    h->pool.push_back(e.a);
    h->pool.push_back(e.b);
  }
  h->pending.clear();
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library links the CUDA runtime statically and not libcuda).
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                         cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

// 4-D map over one FP32 state buffer: (column, gy, gz, variable), box
// {40, rows, 1, nw} = one plane of a tile with its 2-cell halo.  With yz
// the two middle axes swap, (column, gz, gy, variable): the 3-D y sweep's
// planes are x-z slabs at fixed gy.
bool make_tmap(vacgpu_handle* h, void* base, int rows, bool yz, CUtensorMap* m) {
  auto fn = encode_fn();
  if (!fn) return false;
  const DevGrid& g = h->g;
  cuuint64_t dims[4] = {(cuuint64_t)g.P, (cuuint64_t)g.nG[1],
                        (cuuint64_t)g.nG[2], (cuuint64_t)h->nw};
  cuuint64_t strides[3] = {(cuuint64_t)g.P * 4, (cuuint64_t)g.plane * 4,
                           (cuuint64_t)g.vs * 4};
  if (yz) {
    dims[1] = (cuuint64_t)g.nG[2];
    dims[2] = (cuuint64_t)g.nG[1];
    strides[0] = (cuuint64_t)g.plane * 4;
    strides[1] = (cuuint64_t)g.P * 4;
  }
  cuuint32_t box[4] = {40, (cuuint32_t)rows, 1, (cuuint32_t)h->nw};
  cuuint32_t es[4] = {1, 1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dims, strides,
                  box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

// getboundary's ghost fill of w: composed index maps, or face by face
// (restore: reuse the stored values of fixed/fixed1/grad1 faces) when the
// grid has fixed or extrapolating faces.
// getboundary's region loop with the specialbound hook: each region's
// standard types, then the hook for its 'special' variables, region by
// region (src/vacgrid.t:228-372).  qtmode: the fill's qt (launch_set_qt).
int special_fill(vacgpu_handle* h, const SweepArgs& a, void* w, int restore,
                 int qtmode) {
  const DevGrid& g = h->g;
  launch_set_qt(h->ctrl, qtmode, h->st);
  for (int iB = 0; iB < 2 * g.ndim; iB++) {
    if (h->elem == 8)
      launch_ghost_face_fp64(a, (double*)w, (double*)h->fixb, restore, iB, h->st);
    else
      launch_ghost_face_mixed(a, (float*)w, (float*)h->fixb, restore, iB, h->st);
    if (!h->special[iB]) continue;
    vacgpu_region r;
    memset(&r, 0, sizeof(r));
    r.iB = iB;
    r.iw_mask = h->special[iB];
    const int idim = iB / 2, upper = iB % 2;
    for (int d = 0; d < 3; d++) {
      r.lo[d] = 0;
      r.hi[d] = g.nG[d] - 1;
      r.nx[d] = g.nx[d];
      r.nG[d] = g.nG[d];
      r.x[d] = h->xg[d];
    }
    r.lo[idim] = upper ? g.nx[idim] + 2 : 0;
    r.hi[idim] = upper ? g.nx[idim] + 3 : 1;
    r.offset0 = g.xpad;
    r.stride[0] = 1;
    r.stride[1] = g.P;
    r.stride[2] = g.plane;
    r.var_stride = g.vs;
    r.elem = (int)h->elem;
    r.qt = &h->ctrl->qt;
    if (h->bound_fn(h->bound_user, w, &r, (void*)h->st)) {
      h->hook_failed = true;
      return fail("the specialbound hook failed for region " + std::to_string(iB + 1));
    }
  }
  return 0;
}

void fill_ghosts(vacgpu_handle* h, const SweepArgs& a, void* w, int restore,
                 int qtmode) {
  if (h->bound_fn && h->ph.genbc) {
    special_fill(h, a, w, restore, qtmode);
    return;
  }
  if (h->ph.genbc) {
    if (h->elem == 8)
      launch_ghost_faces_fp64(a, (double*)w, (double*)h->fixb, restore, h->st);
    else
      launch_ghost_faces_mixed(a, (float*)w, (float*)h->fixb, restore, h->st);
  } else if (h->elem == 8) {
    launch_ghost_fp64(a, (double*)w, h->st);
  } else {
    launch_ghost_mixed(a, (float*)w, h->st);
  }
}

SweepArgs make_args(vacgpu_handle* h, int d0, int d1) {
  SweepArgs a;
  a.g = h->g;
  a.ph = h->ph;
  for (int d = 0; d < 3; d++) {
    a.a.dx[d] = h->dx[d];
    a.a.dxf[d] = h->dxf[d];
  }
  a.ctrl = h->ctrl;
  a.etaf = h->etaf;
  for (int d = 0; d < 3; d++) a.gradetaf[d] = h->gradetaf[d];
  a.faces = h->faces;
  a.face_stride = h->face_stride;
  a.ndir = h->p.ndir;
  a.mhd = h->p.physics == VACGPU_PHYS_MHD;
  a.d0 = d0;
  a.d1 = d1;
  a.typelimited = h->p.typelimited;
  return a;
}

// specialeta before a resistive source evaluation on w (the source's wCT):
// the current field, the hook, and the eta/dx^2 maxima of getdt_res
// (first_only: the step-start call, which counts at it==itmin only).
void eta_hook(vacgpu_handle* h, const SweepArgs& a, const void* w, int first_only) {
  if (!h->etaf || !h->eta_fn) return;
  const DevGrid& g = h->g;
  kbegin(h, VACGPU_K_DT);
  if (h->elem == 8)
    launch_current_field_fp64(a, (const double*)w, h->curf, h->st);
  else
    launch_current_field_mixed(a, (const float*)w, h->curf, h->st);
  vacgpu_eta_args e;
  memset(&e, 0, sizeof(e));
  vacgpu_region& r = e.box;
  r.iB = -1;
  for (int d = 0; d < 3; d++) {
    r.lo[d] = d < g.ndim ? 1 : 0;
    r.hi[d] = d < g.ndim ? g.nx[d] + 2 : 0;
    r.nx[d] = g.nx[d];
    r.nG[d] = g.nG[d];
    r.x[d] = h->xg[d];
  }
  r.offset0 = g.xpad;
  r.stride[0] = 1;
  r.stride[1] = g.P;
  r.stride[2] = g.plane;
  r.var_stride = g.vs;
  r.elem = (int)h->elem;
  r.qt = &h->ctrl->t;
  e.w = w;
  for (int k = 0; k < 3; k++) e.current[k] = h->curf[k];
  e.idirmin = 7 - 2 * h->p.ndir;
  e.eta = h->etaf;
  for (int k = 0; k < 3; k++) e.gradeta[k] = h->gradetaf[k];
  if (h->eta_fn(h->eta_user, &e, (void*)h->st)) h->hook_failed = true;
  launch_eta_max(a, first_only, h->st);
  kend(h);
}

// the mesh of the state as a hook region
static void mesh_region(const vacgpu_handle* h, vacgpu_region& r) {
  const DevGrid& g = h->g;
  memset(&r, 0, sizeof(r));
  r.iB = -1;
  for (int d = 0; d < 3; d++) {
    r.lo[d] = d < g.ndim ? 2 : 0;
    r.hi[d] = d < g.ndim ? g.nx[d] + 1 : 0;
    r.nx[d] = g.nx[d];
    r.nG[d] = g.nG[d];
    r.x[d] = h->xg[d];
  }
  r.offset0 = g.xpad;
  r.stride[0] = 1;
  r.stride[1] = g.P;
  r.stride[2] = g.plane;
  r.var_stride = g.vs;
  r.elem = (int)h->elem;
  r.qt = &h->ctrl->t;
}

// addsource2 with the user's specialsource (src/vac.t:575-605): the hook,
// then addsource as a pass of its own (the predictor and corrector kernels
// leave it out while a hook is installed).  pred: after the Hancock
// predictor (qdt = dt/2); half: qtC = t+dt/2 (the corrector of twostep).
template <typename T>
void source_hook(vacgpu_handle* h, const SweepArgs& a, int pred, int half, const T* wct,
                 T* w) {
  if (!h->src_fn || !h->p.sourceunsplit) return;
  kbegin(h, VACGPU_K_CONTROL);
  launch_src_args(h->ctrl, pred, half, a.d1 - a.d0 + 1, h->p.ndim, h->st);
  kend(h);
  vacgpu_source_args s;
  memset(&s, 0, sizeof(s));
  mesh_region(h, s.box);
  s.qdt = &h->ctrl->src_qdt;
  s.qtC = &h->ctrl->src_qtc;
  s.wCT = wct;
  s.w = w;
  s.nw = h->nw;
  s.ndir = h->p.ndir;
  if (h->src_fn(h->src_user, &s, (void*)h->st)) h->hook_failed = true;
  kbegin(h, pred ? VACGPU_K_PREDICT : VACGPU_K_CORRECT);
  if (sizeof(T) == 8)
    launch_source_pass_fp64(a, (const double*)wct, (double*)w, pred, h->st);
  else if (h->pmode == 1)
    launch_source_pass_mixedf64(a, (const float*)wct, (float*)w, pred, h->st);
  else if (h->pmode == 2)
    launch_source_pass_mixedf32(a, (const float*)wct, (float*)w, pred, h->st);
  else
    launch_source_pass_mixed(a, (const float*)wct, (float*)w, pred, h->st);
  kend(h);
}

template <typename T>
void run_sweep(vacgpu_handle* h, int d0, int d1) {
  SweepArgs a = make_args(h, d0, d1);
  T* w = (T*)h->buf[h->cur];
  T* wout = (T*)h->buf[h->cur ^ 1];
  T* w1 = (T*)h->buf[2];
  const T* base = w;
  if (h->p.typelimited == VACGPU_LIMITED_PREDICTOR) base = w1;
  if (h->p.typelimited == VACGPU_LIMITED_PREVIOUS && h->p.dimsplit)
    base = (const T*)h->wold;
  // useprimitive: the predictor's upwindLR leaves the state round-tripped
  // through primitive variables (src/vactvdlf.t:325-362); the corrector
  // limits and updates that copy
  const T* wc = w;
  if (h->ph.useprim) {
    kbegin(h, VACGPU_K_PREDICT);
    if (sizeof(T) == 8)
      launch_roundtrip_fp64(a, (const double*)w, (double*)h->wold, h->st);
    else if (h->pmode == 1)
      launch_roundtrip_mixedf64(a, (const float*)w, (float*)h->wold, h->st);
    else if (h->pmode == 2)
      launch_roundtrip_mixedf32(a, (const float*)w, (float*)h->wold, h->st);
    else
      launch_roundtrip_mixed(a, (const float*)w, (float*)h->wold, h->st);
    kend(h);
    wc = base = (const T*)h->wold;
  }
  const bool roe = h->p.typefull == VACGPU_TVDMU || h->p.typefull == VACGPU_TVDMU1;
  if (h->p.typefull == VACGPU_TVDLF1 || h->p.typefull == VACGPU_TVDMU1) {
    // typepred1='nul': onestep, the corrector alone with wCT = w
    // (src/vacio.t:286-299,511); no limiter, so the base is unused
    if (h->p.sourceunsplit) eta_hook(h, a, w, 0);
    kbegin(h, VACGPU_K_CORRECT);
    if (sizeof(T) == 8 && roe)
      launch_correct_roe_fp64(a, (const double*)w, (const double*)w,
                              (const double*)w, (double*)wout, h->st);
    else if (sizeof(T) == 8)
      launch_correct_fp64(a, (const double*)w, (const double*)w,
                          (const double*)w, (double*)wout, h->st);
    else if (roe)
      launch_correct_roe_mixed(a, (const float*)w, (const float*)w,
                               (const float*)w, (float*)wout, h->st);
    else
      launch_correct_mixed(a, (const float*)w, (const float*)w,
                           (const float*)w, (float*)wout, h->st);
    kend(h);
    source_hook<T>(h, a, 0, 0, w, wout);
    if (h->p.smallfix) {
      kbegin(h, VACGPU_K_GHOST);
      if (sizeof(T) == 8)
        launch_keeppositive_fp64(a, (double*)wout, h->st);
      else
        launch_keeppositive_mixed(a, (float*)wout, h->st);
      kend(h);
    }
    kbegin(h, VACGPU_K_GHOST);
    fill_ghosts(h, a, wout, 1, 2);
    kend(h);
  } else if (sizeof(T) == 8) {
    if (h->p.sourceunsplit) eta_hook(h, a, w, 0);
    kbegin(h, VACGPU_K_PREDICT);
    launch_predict_fp64(a, (const double*)w, (double*)w1, h->st);
    kend(h);
    source_hook<T>(h, a, 1, 0, w, w1);
    kbegin(h, VACGPU_K_GHOST);
    if (h->p.smallfix) launch_keeppositive_fp64(a, (double*)w1, h->st);
    fill_ghosts(h, a, w1, 1, 1);
    kend(h);
    if (h->p.sourceunsplit) eta_hook(h, a, w1, 0);
    kbegin(h, VACGPU_K_CORRECT);
    if (roe)
      launch_correct_roe_fp64(a, (const double*)wc, (const double*)w1,
                              (const double*)base, (double*)wout, h->st);
    else
      launch_correct_fp64(a, (const double*)wc, (const double*)w1,
                          (const double*)base, (double*)wout, h->st);
    kend(h);
    source_hook<T>(h, a, 0, 1, (const T*)w1, wout);
    kbegin(h, VACGPU_K_GHOST);
    if (h->p.smallfix) launch_keeppositive_fp64(a, (double*)wout, h->st);
    fill_ghosts(h, a, wout, 1, 2);
    kend(h);
  } else if (h->fused && h->pmode == 0 && d0 == d1 && !h->src_fn) {
    kbegin(h, VACGPU_K_SWEEP);
    // the fused sweep also writes the ghost cells of its output
    launch_sweep_fused(a, &h->tmap[h->cur][d0 == 1], (const float*)w, (float*)wout, h->idxf,
                       h->nzc, h->st);
    kend(h);
  } else {
    const float* fw = (const float*)w;
    const float* fwc = (const float*)wc;
    float* fw1 = (float*)w1;
    float* fo = (float*)wout;
    const float* fb = (const float*)base;
#define MIXED_SWEEP(SUF)                                \
  if (h->p.sourceunsplit) eta_hook(h, a, fw, 0);        \
  kbegin(h, VACGPU_K_PREDICT);                          \
  launch_predict_##SUF(a, fw, fw1, h->st);              \
  kend(h);                                              \
  source_hook<T>(h, a, 1, 0, w, w1);                    \
  kbegin(h, VACGPU_K_GHOST);                            \
  if (h->p.smallfix) launch_keeppositive_##SUF(a, fw1, h->st); \
  fill_ghosts(h, a, fw1, 1, 1);                         \
  kend(h);                                              \
  if (h->p.sourceunsplit) eta_hook(h, a, fw1, 0);       \
  kbegin(h, VACGPU_K_CORRECT);                          \
  if (roe)                                              \
    launch_correct_roe_mixed(a, fwc, fw1, fb, fo, h->st); \
  else                                                  \
    launch_correct_##SUF(a, fwc, fw1, fb, fo, h->st);   \
  kend(h);                                              \
  source_hook<T>(h, a, 0, 1, (const T*)w1, wout);       \
  kbegin(h, VACGPU_K_GHOST);                            \
  if (h->p.smallfix) launch_keeppositive_##SUF(a, fo, h->st); \
  fill_ghosts(h, a, fo, 1, 2);                          \
  kend(h);
    switch (h->pmode) {
      case 1: MIXED_SWEEP(mixedf64) break;
      case 2: MIXED_SWEEP(mixedf32) break;
      default: MIXED_SWEEP(mixed)
    }
#undef MIXED_SWEEP
  }
  h->cur ^= 1;
}

template <typename T>
void run_step(vacgpu_handle* h, int parity_odd) {
  const vacgpu_params& p = h->p;
  SweepArgs a = make_args(h, 0, p.ndim - 1);
  kbegin(h, VACGPU_K_CONTROL);
  launch_dt_begin(h->ctrl, p.ndim, h->st);
  kend(h);
  const T* w = (const T*)h->buf[h->cur];
  if (sizeof(T) == 8) {
    kbegin(h, VACGPU_K_DT);
    launch_pminmax_fp64(a, (const double*)w, h->st);
    kend(h);
    kbegin(h, VACGPU_K_CONTROL);
    launch_smallp(h->ctrl, a.mhd, p.smallpcoeff, h->st);
    kend(h);
    kbegin(h, VACGPU_K_DT);
    launch_cell_cmax_fp64(a, (const double*)w, h->st);
    kend(h);
  } else {
    kbegin(h, VACGPU_K_DT);
    launch_pminmax_mixed(a, (const float*)w, h->st);
    kend(h);
    kbegin(h, VACGPU_K_CONTROL);
    launch_smallp(h->ctrl, a.mhd, p.smallpcoeff, h->st);
    kend(h);
    kbegin(h, VACGPU_K_DT);
    launch_cell_cmax_mixed(a, (const float*)w, h->st);
    kend(h);
  }
  // getdt_res with the specialeta field: eta from the state at it==itmin
  eta_hook(h, a, w, 1);
  // getdt_special: the user's limit of this step from the state
  if (h->dtsp_fn) {
    kbegin(h, VACGPU_K_CONTROL);
    launch_dtspecial_begin(h->ctrl, h->st);
    kend(h);
    vacgpu_dtspecial_args d;
    memset(&d, 0, sizeof(d));
    mesh_region(h, d.box);
    d.w = w;
    d.dt = &h->ctrl->dtspecial;
    if (h->dtsp_fn(h->src_user, &d, (void*)h->st)) h->hook_failed = true;
  }
  kbegin(h, VACGPU_K_CONTROL);
  launch_dt_end(h->ctrl, p, h->st);
  kend(h);
  if (p.typelimited == VACGPU_LIMITED_PREVIOUS && p.dimsplit)
    cudaMemcpyAsync(h->wold, h->buf[h->cur], h->elem * h->g.vs * h->nw,
                    cudaMemcpyDeviceToDevice, h->st);
  if (p.dimsplit) {
    if (!parity_odd || p.typedimsplit == VACGPU_SPLIT_XY) {
      for (int d = 0; d < p.ndim; d++) run_sweep<T>(h, d, d);
    } else {
      for (int d = p.ndim - 1; d >= 0; d--) run_sweep<T>(h, d, d);
    }
  } else {
    run_sweep<T>(h, 0, p.ndim - 1);
  }
  kbegin(h, VACGPU_K_CONTROL);
  launch_step_end(h->ctrl, p.ndim, h->st);
  kend(h);
}

// Issue k steps on the handle's stream without waiting: two-step units
// are replayed from captured CUDA graphs keyed by (state buffer, parity of
// it); h->cur follows the swaps of steps that execute.
// z-chunk tuning of the fused 3-D sweep: one step per candidate from a
// snapshot of the state (kept in the predictor buffer, which the fused
// sweep does not use) and of the control block, restored after each trial,
// so the run itself is untouched; the fastest candidate is kept.
int tune_nzc(vacgpu_handle* h) {
  h->tuning = false;
  const size_t bytes = (size_t)h->g.vs * h->nw * h->elem;
  const int cur0 = h->cur;
  long long nl[VACGPU_K_NCLASS];
  memcpy(nl, h->nlaunch, sizeof(nl));
  Ctrl saved;
  CK(cudaMemcpyAsync(&saved, h->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(h->buf[2], h->buf[cur0], bytes, cudaMemcpyDeviceToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  float best = 1e30f;
  int nbest = h->nzc;
  for (int i = 0; i < h->tncand; i++) {
    h->nzc = h->tcand[i];
    k_call_begin<<<1, 1, 0, h->st>>>(h->ctrl, 1, 1e300);
    cudaEventRecord(e0, h->st);
    run_step<float>(h, h->it_host & 1);
    cudaEventRecord(e1, h->st);
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      nbest = h->tcand[i];
    }
    CK(cudaMemcpyAsync(h->buf[cur0], h->buf[2], bytes, cudaMemcpyDeviceToDevice, h->st));
    CK(cudaMemcpyAsync(h->ctrl, &saved, sizeof(Ctrl), cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    h->cur = cur0;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  memcpy(h->nlaunch, nl, sizeof(nl));
  h->nzc = nbest;
  CK(cudaGetLastError());
  return 0;
}

// Captured graphs hold the launch arguments and hooks of their capture.
void drop_graphs(vacgpu_handle* h) {
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      if (h->gexec[i][j]) {
        cudaGraphExecDestroy(h->gexec[i][j]);
        h->gexec[i][j] = nullptr;
      }
}

int issue_steps(vacgpu_handle* h, int k, int it_base) {
  const int nsw = h->p.dimsplit ? h->p.ndim : 1;
  const bool graphs = !h->timing && h->st != nullptr &&
                      !(getenv("VACGPU_GRAPH") && atoi(getenv("VACGPU_GRAPH")) == 0);
  for (int s = 0; s < k;) {
    const int par = (it_base + s) & 1;
    if (graphs && h->warmed && k - s >= 2) {
      cudaGraphExec_t& ex = h->gexec[h->cur][par];
      const int cur0 = h->cur;
      if (!ex) {
        cudaGraph_t gr;
        long long before[VACGPU_K_NCLASS];
        memcpy(before, h->nlaunch, sizeof(before));
        CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
        for (int q = 0; q < 2; q++) {
          if (h->elem == 8)
            run_step<double>(h, (par + q) & 1);
          else
            run_step<float>(h, (par + q) & 1);
        }
        CK(cudaStreamEndCapture(h->st, &gr));
        CK(cudaGraphInstantiate(&ex, gr, 0));
        cudaGraphDestroy(gr);
        for (int k = 0; k < VACGPU_K_NCLASS; k++) {
          h->glaunch[cur0][par][k] = h->nlaunch[k] - before[k];
          h->nlaunch[k] = before[k];  // counted when the graph runs
        }
        h->cur = cur0;
      }
      CK(cudaGraphLaunch(ex, h->st));
      for (int k = 0; k < VACGPU_K_NCLASS; k++) h->nlaunch[k] += h->glaunch[cur0][par][k];
      h->cur = cur0 ^ ((2 * nsw) & 1);
      s += 2;
    } else {
      if (h->elem == 8)
        run_step<double>(h, par);
      else
        run_step<float>(h, par);
      h->warmed = true;
      s += 1;
    }
  }
  return 0;
}

int check_params(const vacgpu_params* p) {
  if (p->ndim < 1 || p->ndim > 3) return fail("ndim must be 1..3");
  if (p->ndir < p->ndim || p->ndir > 3) return fail("ndir must be ndim..3");
  bool ok = (p->ndim == p->ndir) || (p->ndim == 2 && p->ndir == 3);
  if (!ok) return fail("supported (ndim,ndir): (1,1) (2,2) (2,3) (3,3)");
  if (p->physics != VACGPU_PHYS_HD && p->physics != VACGPU_PHYS_MHD)
    return fail("physics must be VACGPU_PHYS_HD or VACGPU_PHYS_MHD");
  int nw = p->physics == VACGPU_PHYS_MHD ? 2 + 2 * p->ndir : 2 + p->ndir;
  if (p->nw != nw) return fail("nw does not match physics and ndir");
  if (p->dixB != 2) return fail("dixB must be 2 (VAC's dixBlo=dixBhi=2)");
  for (int d = 0; d < p->ndim; d++)
    if (p->nx[d] < 2) return fail("nx must be >= 2 in every dimension");
  if (!(p->eqpar[0] > 0.0)) return fail("eqpar(gamma_) must be positive");
  if (p->physics == VACGPU_PHYS_MHD && p->eqpar[1] < 0.0 && p->useprimitive)
    return fail("eqpar(eta_)<0 (specialeta) with useprimitive=T is not supported");
  if (p->typefull < VACGPU_TVDLF || p->typefull > VACGPU_TVDMU1)
    return fail("typefull must be tvdlf, tvdlf1, tvdmu or tvdmu1");
  const bool roe = p->typefull == VACGPU_TVDMU || p->typefull == VACGPU_TVDMU1;
  if (roe) {
    // the configurations the Roe solvers define (src/vacphys.mhdroe.t:25,
    // :245-276; src/vacphys.hdroe.t:110-134)
    const bool mhd = p->physics == VACGPU_PHYS_MHD;
    if (mhd && p->ndir < 2) return fail("MHD Roe solver needs ndir>=2");
    for (int il = 0; il < nw; il++) {
      const int te = p->typeentropy[il];
      if (te < VACGPU_ENTROPY_NUL || te > VACGPU_ENTROPY_YEE)
        return fail("unknown typeentropy");
      if (!mhd && te == VACGPU_ENTROPY_RATIO)
        return fail("typeentropy='ratio' is undefined for the HD Roe solver");
    }
    if (mhd) {
      auto lr = [&](int il) {
        const int te = p->typeentropy[il];
        return te == VACGPU_ENTROPY_HARTEN || te == VACGPU_ENTROPY_POWELL ||
               te == VACGPU_ENTROPY_RATIO;
      };
      for (int il = 1; il < 4; il++)
        if (lr(il) && !lr(0))
          return fail("MHD entropy fix of a fast/slow wave needs the fastRW fix");
      if (nw == 8 && lr(7) && !lr(6))
        return fail("MHD entropy fix of alfvLW needs the alfvRW fix");
    }
  }
  const bool first_order =
      p->typefull == VACGPU_TVDLF1 || p->typefull == VACGPU_TVDMU1;
  for (int iw = 0; iw < nw; iw++)
    if (p->typelimiter[iw] < 0 || p->typelimiter[iw] > VACGPU_LIM_ALBADA)
      return fail("unknown typelimiter");
  if (p->typelimited < 0 || p->typelimited > VACGPU_LIMITED_PREDICTOR)
    return fail("unknown typelimited");
  if (!p->dimsplit && p->typelimited == VACGPU_LIMITED_ORIGINAL && !first_order)
    return fail("Error in TVDMUSCLF: Unsplit dim. and original is limited");
  if (p->useprimitive && !first_order) {
    if (!p->dimsplit || p->typelimited != VACGPU_LIMITED_ORIGINAL)
      return fail("useprimitive=T is supported with dimsplit and typelimited='original'");
    if (p->smallp < 0.0 && !(p->dtpar <= 0.0 && p->courantpar > 0.0))
      return fail("useprimitive=T with a fixed dt needs smallp given (its first "
                  "getpthermal call would set smallp over the ghost box)");
  }
  if (p->physics == VACGPU_PHYS_MHD && p->divbfix && !p->sourceunsplit)
    return fail("divbfix=T requires unsplitsource=T or splitsource=T !");
  for (int d = 0; d < p->ndim; d++)
    for (int iw = 0; iw < nw; iw++) {
      int lo = p->typeB[2 * d][iw], hi = p->typeB[2 * d + 1][iw];
      if (lo < 0 || lo > VACGPU_BC_SPECIAL || hi < 0 || hi > VACGPU_BC_SPECIAL)
        return fail("unsupported boundary type");
      if ((lo == VACGPU_BC_PERIODIC) != (hi == VACGPU_BC_PERIODIC))
        return fail("Error in BoundSetup: No periodic pair");
    }
  if (p->smallp < 0.0 && (p->dtpar > 0.0 || !(p->courantpar > 0.0)))
    return fail("smallp<0 with a fixed dt: give smallp explicitly");
  if (p->precision != VACGPU_PREC_FP64 && p->precision != VACGPU_PREC_MIXED)
    return fail("precision must be VACGPU_PREC_FP64 or VACGPU_PREC_MIXED");
  return 0;
}

}  // namespace

// Internal views used by batch.cu.
int vacgpu_internal_view(vacgpu_handle* h, HandleView* v) {
  v->g = h->g;
  v->ph = h->ph;
  v->sa = make_args(h, 0, h->p.ndim - 1);
  v->buf[0] = (float*)h->buf[0];
  v->buf[1] = (float*)h->buf[1];
  for (int d = 0; d < 3; d++) {
    v->dxf[d] = h->dxf[d];
    v->idxf[d] = h->idxf[d];
  }
  v->ctrl = h->ctrl;
  for (int i = 0; i < 2; i++)
    for (int k = 0; k < 2; k++) v->tmap[i][k] = &h->tmap[i][k];
  v->nzc = h->nzc;
  v->fused = h->fused;
  return 0;
}
int vacgpu_internal_set_cur(vacgpu_handle* h, int cur) {
  h->cur = cur;
  return 0;
}

// Server support: issue k steps that all execute (no stop condition in
// between) without any host synchronisation.
int vacgpu_internal_step_async(vacgpu_handle* h, int k) {
  h->tuning = false;  // served solves keep the default z chunk
  k_call_begin<<<1, 1, 0, h->st>>>(h->ctrl, k, 1e300);
  if (issue_steps(h, k, h->it_host)) return 1;
  h->it_host += k;
  CK(cudaGetLastError());
  return 0;
}
void* vacgpu_internal_stream(vacgpu_handle* h) { return (void*)h->st; }

// Device bytes vacgpu_create allocates for p (admission control).
size_t vacgpu_internal_device_bytes(const vacgpu_params* p) {
  size_t elem = p->precision == VACGPU_PREC_FP64 ? 8 : 4;
  long long nG[3], ncell = 1;
  for (int d = 0; d < 3; d++) {
    nG[d] = d < p->ndim ? p->nx[d] + 4 : 1;
    ncell *= d < p->ndim ? p->nx[d] : 1;
  }
  const long long align = 128 / elem;
  const long long P = ((align - 2 + nG[0] + align - 1) / align) * align;
  const size_t vs = (size_t)P * nG[1] * nG[2];
  size_t b = 3 * elem * vs * p->nw + 8 * (size_t)ncell * p->nw;
  {
    // the split correctors' face buffer (the fused mixed sweep needs none;
    // counted regardless)
    const bool roe = p->typefull == VACGPU_TVDMU || p->typefull == VACGPU_TVDMU1;
    long long mf = 0;
    for (int d = 0; d < p->ndim; d++) {
      long long f = 1;
      for (int k = 0; k < 3; k++) f *= (k < p->ndim ? p->nx[k] : 1) + (k == d ? 1 : 0);
      if (f > mf) mf = f;
    }
    b += elem * (size_t)mf * (roe ? p->nw * (p->nw + 1) : p->nw) *
         (p->dimsplit ? 1 : p->ndim);
  }
  b += 8 * ((ncell + 255) / 256) * p->nw + sizeof(Ctrl) + 64 * 1024;
  return b;
}

extern "C" {

// split corrector: per sweep direction the faces' fluxes (and, for the Roe
// dissipation, R(iw,il)*phi(il) of every wave)
static int alloc_faces(vacgpu_handle* h) {
  const vacgpu_params* p = &h->p;
  const DevGrid& g = h->g;
  const bool roe = p->typefull == VACGPU_TVDMU || p->typefull == VACGPU_TVDMU1;
  const long long K = roe ? (long long)h->nw * (h->nw + 1) : h->nw;
  long long mf = 0;
  for (int d = 0; d < p->ndim; d++)
    if (face_count(g, d) > mf) mf = face_count(g, d);
  h->face_stride = K * mf;
  const int nsw = p->dimsplit ? 1 : p->ndim;
  if (cudaMalloc(&h->faces, h->elem * (size_t)h->face_stride * nsw) != cudaSuccess)
    return fail("device allocation of the corrector's face buffer failed");
  return 0;
}

void vacgpu_default_params(vacgpu_params* p, int ndim, int ndir, int physics,
                           const int* nx) {
  memset(p, 0, sizeof(*p));
  p->ndim = ndim;
  p->ndir = ndir;
  p->physics = physics;
  p->nw = physics == VACGPU_PHYS_MHD ? 2 + 2 * ndir : 2 + ndir;
  for (int d = 0; d < 3; d++) p->nx[d] = d < ndim ? nx[d] : 1;
  p->dixB = 2;
  p->eqpar[0] = 5.0 / 3.0;
  p->typefull = VACGPU_TVDLF;
  for (int iw = 0; iw < VACGPU_MAXNW; iw++) p->typelimiter[iw] = VACGPU_LIM_MINMOD;
  p->typelimited = VACGPU_LIMITED_ORIGINAL;
  p->dimsplit = 1;
  p->typedimsplit = VACGPU_SPLIT_XYYX;
  p->divbfix = 1;
  p->sourceunsplit = 1;
  p->courantpar = 0.8;
  p->dtpar = -1.0;
  p->smallpcoeff = 1.0e-6;
  p->smallp = -1.0;
  p->itmax = 1000000;
  p->tmax = 1.0e99;
  p->dtmin = 1.0e-99;
  for (int b = 0; b < VACGPU_MAXB; b++)
    for (int iw = 0; iw < VACGPU_MAXNW; iw++) p->typeB[b][iw] = VACGPU_BC_CONT;
  p->precision = VACGPU_PREC_FP64;
  p->smallfix = 0;
  p->smallrho = -1.0;
  p->smallrhocoeff = 1.0e-6;
  p->vacuumrho = -1.0;
  p->compactres = 0;
  p->dtdiffpar = 0.5;
  // physini's entropycoef: the default-real literals 0.2 and 0.4
  // (src/vacphys.mhd0.t:18-28, src/vacphys.t.hd:21-29), widened to double
  for (int il = 0; il < VACGPU_MAXNW; il++) {
    p->typeentropy[il] = VACGPU_ENTROPY_NUL;
    double c = -1.0;
    if (physics == VACGPU_PHYS_MHD) {
      if (il < 4) c = (double)0.2f;
      if (il == 6 || il == 7) c = (double)0.4f;
    } else if (il < 2) {
      c = (double)0.2f;
    }
    p->entropycoef[il] = c;
  }
  p->divbwave = 1;
}

int vacgpu_create(const vacgpu_params* p, vacgpu_handle** out) {
  *out = nullptr;
  if (check_params(p)) return 1;
  vacgpu_handle* h = new vacgpu_handle();  // value-initialised: zeroed
  h->p = *p;
  h->nw = p->nw;
  h->elem = p->precision == VACGPU_PREC_FP64 ? 8 : 4;
  const char* pm = getenv("VACGPU_MIXED_PRESSURE");
  h->pmode = 0;
  if (pm && !strcmp(pm, "f64")) h->pmode = 1;
  if (pm && !strcmp(pm, "f32")) h->pmode = 2;
  if (h->pmode && p->precision == VACGPU_PREC_MIXED &&
      (p->typefull == VACGPU_TVDMU || p->typefull == VACGPU_TVDMU1)) {
    delete h;
    return fail("the Roe corrector's mixed path has the double-float "
                "pressure recovery only (VACGPU_MIXED_PRESSURE unset)");
  }
  DevGrid& g = h->g;
  g.ndim = p->ndim;
  g.ncell = 1;
  for (int d = 0; d < 3; d++) {
    g.nx[d] = d < p->ndim ? p->nx[d] : 1;
    g.gh[d] = d < p->ndim ? 2 : 0;
    g.nG[d] = g.nx[d] + 2 * g.gh[d];
    g.ncell *= g.nx[d];
  }
  const int align = (int)(128 / h->elem);
  g.xpad = align - 2;
  g.P = ((g.xpad + g.nG[0] + align - 1) / align) * align;
  g.plane = g.P * g.nG[1];
  g.vs = g.plane * g.nG[2];
  DevPhys& ph = h->ph;
  ph.gamma = p->eqpar[0];
  ph.pt1 = 1.0 - 0.5 * p->eqpar[0];
  ph.gm1 = p->eqpar[0] - 1.0;
  ph.gammaf = (float)ph.gamma;
  ph.gm1f = (float)ph.gm1;
  ph.c2gf = (2.0f - ph.gammaf) / ph.gm1f;
  ph.pt3 = 0.5 * (p->eqpar[0] - 1.0);
  ph.smallpcoeff = p->smallpcoeff;
  double courantpar = p->courantpar;
  if (p->dtpar > 0.0 && p->slowsteps != 1) courantpar = -1.0;  // startup
  ph.courantpar = courantpar;
  for (int iw = 0; iw < VACGPU_MAXNW; iw++) ph.lim[iw] = p->typelimiter[iw];
  memcpy(ph.typeB, p->typeB, sizeof(ph.typeB));
  ph.typefull = p->typefull;
  ph.divbfix = p->divbfix;
  ph.sourceunsplit = p->sourceunsplit;
  ph.smallfix = p->smallfix;
  ph.vacuumrho = p->vacuumrho;
  ph.smallrhocoeff = p->smallrhocoeff;
  const bool first_order =
      p->typefull == VACGPU_TVDLF1 || p->typefull == VACGPU_TVDMU1;
  ph.useprim = p->useprimitive && !first_order;
  for (int il = 0; il < VACGPU_MAXNW; il++) {
    ph.typeentropy[il] = p->typeentropy[il];
    ph.entropycoef[il] = p->entropycoef[il];
  }
  ph.divbwave = p->divbwave;
  ph.roe_dpprim = p->useprimitive;
  ph.eta = p->physics == VACGPU_PHYS_MHD ? p->eqpar[1] : 0.0;
  ph.compactres = p->compactres;
  ph.src_id = VACGPU_SRC_NONE;
  set_gmaps(ph, p->ndim, p->nw);
  for (int iB = 0; iB < 2 * p->ndim; iB++)
    for (int iw = 0; iw < p->nw; iw++)
      if (p->typeB[iB][iw] == VACGPU_BC_SPECIAL) h->special[iB] |= 1u << iw;
  for (int iB = 0; iB < VACGPU_MAXB; iB++) h->any_special |= h->special[iB] != 0;
  size_t bytes = h->elem * (size_t)g.vs * h->nw;
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 3 && e == cudaSuccess; i++) {
    e = cudaMalloc(&h->buf[i], bytes);
    if (e == cudaSuccess) e = cudaMemset(h->buf[i], 0, bytes);
  }
  // wold: the step-start copy ('previous') or useprimitive's round-tripped
  // limiter base
  if (e == cudaSuccess && ((p->typelimited == VACGPU_LIMITED_PREVIOUS && p->dimsplit) ||
                           ph.useprim))
    e = cudaMalloc(&h->wold, bytes);
  for (int d = 0; d < 3 && e == cudaSuccess; d++) {
    e = cudaMalloc(&h->xg[d], sizeof(double) * g.nG[d]);
    if (e == cudaSuccess) e = cudaMemset(h->xg[d], 0, sizeof(double) * g.nG[d]);
    if (e == cudaSuccess) e = cudaMalloc(&h->dx[d], sizeof(double) * g.nG[d]);
    if (e == cudaSuccess) e = cudaMalloc(&h->dxf[d], sizeof(float) * g.nG[d]);
  }
  if (e == cudaSuccess && p->physics == VACGPU_PHYS_MHD && p->eqpar[1] < 0.0) {
    // specialeta: the field, gradeta for the compact form, the current
    const size_t fb = sizeof(double) * g.vs;
    e = cudaMalloc(&h->etaf, fb);
    if (e == cudaSuccess) e = cudaMemset(h->etaf, 0, fb);
    for (int k = 0; k < 3 && e == cudaSuccess; k++) {
      e = cudaMalloc(&h->curf[k], fb);
      if (e == cudaSuccess) e = cudaMemset(h->curf[k], 0, fb);
      if (e == cudaSuccess && p->compactres) {
        e = cudaMalloc(&h->gradetaf[k], fb);
        if (e == cudaSuccess) e = cudaMemset(h->gradetaf[k], 0, fb);
      }
    }
  }
  if (e == cudaSuccess)
    e = cudaMalloc(&h->stage, sizeof(double) * g.ncell * h->nw);
  if (e == cudaSuccess && ph.genbc) {
    // stored ghost values: per face its two layers over the other
    // dimensions' ghost box, all variables
    size_t n = 0;
    for (int iB = 0; iB < 2 * g.ndim; iB++) {
      size_t f = 2;
      for (int d = 0; d < 3; d++)
        if (d != iB / 2) f *= g.nG[d];
      n += f * h->nw;
    }
    e = cudaMalloc(&h->fixb, n * h->elem);
  }
  long long nblk = (g.ncell + 255) / 256;
  if (e == cudaSuccess)
    e = cudaMalloc(&h->part, sizeof(double) * nblk * h->nw);
  if (e == cudaSuccess) e = cudaMalloc(&h->sums, sizeof(double) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&h->ctrl, sizeof(Ctrl));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
  h->own_st = h->st;
  if (e != cudaSuccess) {
    vacgpu_destroy(h);
    return fail(std::string("device allocation failed: ") + cudaGetErrorString(e));
  }
  h->nzc = 32;
  if (const char* nz = getenv("VACGPU_NZC")) h->nzc = atoi(nz) > 0 ? atoi(nz) : 32;
  h->fused = p->precision == VACGPU_PREC_MIXED && p->dimsplit &&
             (p->ndim == 2 || p->ndim == 3) && p->ndir == p->ndim &&
             p->typelimited == VACGPU_LIMITED_ORIGINAL &&
             p->typefull == VACGPU_TVDLF && !p->smallfix && !p->useprimitive &&
             !(p->physics == VACGPU_PHYS_MHD && p->eqpar[1] != 0.0);
  if (const char* fz = getenv("VACGPU_FUSED")) h->fused = h->fused && atoi(fz) != 0;
  // its ghost writes need uniform copy maps, periodic faces in pairs and
  // n >= 4; 'symm0' needs the split kernels' zero face fluxes
  for (int d = 0; d < p->ndim; d++)
    if (ph.gmap[d][0] == GMAP_MIXED || ph.gmap[d][1] == GMAP_MIXED || g.nx[d] < 4 ||
        (ph.gmap[d][0] == GMAP_PERIODIC) != (ph.gmap[d][1] == GMAP_PERIODIC) ||
        ph.noflux[d][0] || ph.noflux[d][1])
      h->fused = false;
  if (h->fused && p->ndim == 3 && !getenv("VACGPU_NZC") && g.ncell >= (1LL << 21)) {
    static const int cands[5] = {16, 24, 32, 48, 64};
    for (int i = 0; i < 5; i++)
      if (cands[i] < g.nx[2]) h->tcand[h->tncand++] = cands[i];
    h->tuning = h->tncand > 1;
  }
  if (h->fused) {
    bool ok = true;
    for (int i = 0; i < 2 && ok; i++)
      for (int k = 0; k < 2 && ok; k++)
        ok = make_tmap(h, h->buf[i], FUSED_BOX_ROWS[p->ndim == 3 ? 0 : k],
                       p->ndim == 3 && k == 1, &h->tmap[i][k]);
    for (int d = 0; d < 3 && ok; d++)
      ok = cudaMalloc(&h->idxf[d], sizeof(float) * g.nG[d]) == cudaSuccess;
    if (!ok) {
      vacgpu_destroy(h);
      return fail("TMA descriptor set-up failed");
    }
  }
  if ((h->elem == 8 || !h->fused || h->pmode != 0) && alloc_faces(h)) {
    vacgpu_destroy(h);
    return 1;
  }
  Ctrl c;
  memset(&c, 0, sizeof(c));
  c.roe = p->typefull == VACGPU_TVDMU || p->typefull == VACGPU_TVDMU1;
  c.dtpar = p->dtpar;
  c.courantpar = courantpar;
  c.smallp = p->smallp;
  c.dtgrav = BIGD;
  c.dtspecial = BIGD;
  c.dtdiff = BIGD;
  for (int d = 0; d < 3; d++) c.dtcourant[d] = BIGD;
  c.tstop = 1e300;
  e = cudaMemcpy(h->ctrl, &c, sizeof(c), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    vacgpu_destroy(h);
    return fail(std::string("cudaMemcpy: ") + cudaGetErrorString(e));
  }
  *out = h;
  return 0;
}

// gridsetup1 (src/vacgrid.t:457-593) for a Cartesian product grid: the
// ghost coordinates of each line are extrapolated linearly from the two
// edge cells, dx = (x(i+1)-x(i-1))/2, dvolume = dx1*dx2*dx3 and volume is
// summed in column-major order.
int vacgpu_set_grid(vacgpu_handle* h, const double* x) {
  if (!h) return fail("null handle");
  const DevGrid& g = h->g;
  const int nd = h->p.ndim;
  const long long n = g.ncell;
  const long long st[3] = {1, g.nx[0], (long long)g.nx[0] * g.nx[1]};
  for (int d = 0; d < nd; d++) {
    // product-grid check: x_d must depend on ix_d only
    const double* xd = x + d * n;
    for (long long m = 0; m < n; m++) {
      long long i = (m / st[d]) % g.nx[d];
      if (xd[m] != xd[i * st[d]])
        return fail("x is not a Cartesian product grid");
    }
    int N = g.nx[d];
    std::vector<double> q(N + 6);  // qx over [ixGmin-1, ixGmax+1]
    for (int i = 0; i < N; i++) q[i + 3] = xd[(long long)i * st[d]];
    int ixe = N + 2, ixf = ixe - 1;  // upper layers
    for (int ix = N + 3; ix <= N + 5; ix++) {
      int c = std::abs(ixe - ix);
      q[ix] = (1 + c) * q[ixe] - c * q[ixf];
    }
    ixe = 3;
    ixf = 4;  // lower layers
    for (int ix = 0; ix <= 2; ix++) {
      int c = std::abs(ixe - ix);
      q[ix] = (1 + c) * q[ixe] - c * q[ixf];
    }
    // cell centres over the ghost box (q covers one more cell each side)
    CK(cudaMemcpy(h->xg[d], q.data() + 1, sizeof(double) * (N + 4),
                  cudaMemcpyHostToDevice));
    h->hdx[d].assign(N + 4, 0.0);
    std::vector<float> f(N + 4);
    for (int i = 0; i < N + 4; i++) {
      h->hdx[d][i] = 0.5 * (q[i + 2] - q[i]);
      f[i] = (float)h->hdx[d][i];
      if (!(h->hdx[d][i] > 0.0)) return fail("grid spacing must be positive");
    }
    CK(cudaMemcpy(h->dx[d], h->hdx[d].data(), sizeof(double) * (N + 4),
                  cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->dxf[d], f.data(), sizeof(float) * (N + 4),
                  cudaMemcpyHostToDevice));
    if (h->idxf[d]) {
      std::vector<float> fi(N + 4);
      for (int i = 0; i < N + 4; i++) fi[i] = (float)(1.0 / h->hdx[d][i]);
      CK(cudaMemcpy(h->idxf[d], fi.data(), sizeof(float) * (N + 4),
                    cudaMemcpyHostToDevice));
    }
  }
  for (int d = nd; d < 3; d++) {
    double one = 1.0;
    float onef = 1.0f;
    CK(cudaMemcpy(h->dx[d], &one, sizeof(double), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->dxf[d], &onef, sizeof(float), cudaMemcpyHostToDevice));
    if (h->idxf[d])
      CK(cudaMemcpy(h->idxf[d], &onef, sizeof(float), cudaMemcpyHostToDevice));
  }
  double vol = 0.0;
  for (int iz = 0; iz < g.nx[2]; iz++)
    for (int iy = 0; iy < g.nx[1]; iy++)
      for (int ix = 0; ix < g.nx[0]; ix++) {
        double dv = h->hdx[0][ix + 2];
        if (nd > 1) dv = dv * h->hdx[1][iy + 2];
        if (nd > 2) dv = dv * h->hdx[2][iz + 2];
        vol = vol + dv;
      }
  h->volume = vol;
  // getdt_res (src/vacphys.mhdres.t:5-45): dtdiffpar*min(dx)^2/eta, a
  // constant of the grid for a constant eta (the specialeta field's limit
  // is formed on the device)
  h->dtdiff = BIGD;
  if (h->ph.eta > 0.0) {
    double m = h->hdx[0][2];
    for (int d = 0; d < nd; d++)
      for (int i = 0; i < g.nx[d]; i++)
        if (h->hdx[d][i + 2] < m) m = h->hdx[d][i + 2];
    h->dtdiff = h->p.dtdiffpar * (m * m) / h->ph.eta;
  }
  CK(cudaMemcpy(&h->ctrl->dtdiff, &h->dtdiff, sizeof(double), cudaMemcpyHostToDevice));
  h->have_grid = true;
  return 0;
}

static const char* NO_ETA =
    "eqpar(eta_)<0 needs the user's specialeta (vacgpu_register_eta)";
static const char* NO_SPECIAL =
    "Special boundary is not defined (typeB 'special' needs a hook: "
    "vacgpu_register_bound)";

int vacgpu_upload(vacgpu_handle* h, const double* w, int it, double t) {
  if (!h) return fail("null handle");
  if (h->any_special && !h->bound_fn) return fail(NO_SPECIAL);
  if (h->etaf && !h->eta_fn) return fail(NO_ETA);
  h->hook_failed = false;
  h->faulted = false;
  const DevGrid& g = h->g;
  long long n = g.ncell * h->nw;
  // it, t, itmin (startup, src/vac.t:176) and the dt state of a fresh run
  Ctrl c;
  CK(cudaMemcpyAsync(&c, h->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  c.it = it;
  c.itmin = it;
  c.t = t;
  c.dt = 0.0;
  c.dtold = 0.0;
  c.done = 0;
  c.dtpar = h->p.dtpar;
  c.courantpar = h->ph.courantpar;
  c.smallp = h->p.smallp;
  c.smallrho = h->p.smallrho;
  c.kp_r = c.kp_p = 0;
  for (int d = 0; d < 3; d++) c.dtcourant[d] = BIGD;
  for (int i = 0; i < 4; i++) c.nerror[i] = 0;
  c.dtgrav = h->dtgrav > 0 ? h->dtgrav : BIGD;
  c.dtspecial = BIGD;
  c.dtdiff = h->have_grid ? h->dtdiff : BIGD;
  c.cur = 0;
  c.fault = 0;
  CK(cudaMemcpyAsync(h->ctrl, &c, sizeof(Ctrl), cudaMemcpyHostToDevice, h->st));
  CK(cudaMemcpyAsync(h->stage, w, sizeof(double) * n, cudaMemcpyHostToDevice,
                     h->st));
  unsigned nb = (unsigned)((n + 255) / 256);
  // the getboundary before the time loop (src/vac.t:54), keeppositive first
  // when smallfix
  SweepArgs a = make_args(h, 0, 0);
  if (h->elem == 8) {
    k_scatter<double><<<nb, 256, 0, h->st>>>(h->stage, (double*)h->buf[0], g, h->nw);
    if (h->p.smallfix) launch_keeppositive_fp64(a, (double*)h->buf[0], h->st);
    fill_ghosts(h, a, h->buf[0], 0, 0);
    if (h->ph.genbc)
      launch_fix_store_fp64(a, (const double*)h->buf[0], (double*)h->fixb, h->st);
  } else {
    k_scatter<float><<<nb, 256, 0, h->st>>>(h->stage, (float*)h->buf[0], g, h->nw);
    if (h->p.smallfix) launch_keeppositive_mixed(a, (float*)h->buf[0], h->st);
    fill_ghosts(h, a, h->buf[0], 0, 0);
    if (h->ph.genbc)
      launch_fix_store_mixed(a, (const float*)h->buf[0], (float*)h->fixb, h->st);
  }
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->st));
  if (h->hook_failed) return fail("the specialbound hook failed");
  h->cur = 0;
  h->it_host = it;
  h->have_state = true;
  return 0;
}

int vacgpu_download(vacgpu_handle* h, double* w) {
  if (!h) return fail("null handle");
  const DevGrid& g = h->g;
  long long n = g.ncell * h->nw;
  unsigned nb = (unsigned)((n + 255) / 256);
  if (h->elem == 8)
    k_gather<double><<<nb, 256, 0, h->st>>>((const double*)h->buf[h->cur], h->stage, g, h->nw);
  else
    k_gather<float><<<nb, 256, 0, h->st>>>((const float*)h->buf[h->cur], h->stage, g, h->nw);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(w, h->stage, sizeof(double) * n, cudaMemcpyDeviceToHost,
                     h->st));
  CK(cudaStreamSynchronize(h->st));
  return 0;
}

int vacgpu_snapshot_begin(vacgpu_handle* h, int slot) {
  if (!h) return fail("null handle");
  if (slot < 0 || slot > 1) return fail("snapshot slot must be 0 or 1");
  if (!h->have_state) return fail("vacgpu_snapshot_begin before vacgpu_upload");
  vacgpu_handle::Snap& sn = h->snap[slot];
  if (sn.pending)
    return fail("snapshot slot " + std::to_string(slot) +
                " is still in flight (call vacgpu_snapshot_wait first)");
  const DevGrid& g = h->g;
  const long long n = g.ncell * h->nw;
  if (!h->cst) CK(cudaStreamCreateWithFlags(&h->cst, cudaStreamNonBlocking));
  if (!sn.dev) {
    CK(cudaMalloc(&sn.dev, sizeof(double) * n));
    CK(cudaMallocHost(&sn.host, sizeof(double) * n));
    CK(cudaEventCreateWithFlags(&sn.gathered, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&sn.copied, cudaEventDisableTiming));
  }
  sn.ready = false;
  // the gather follows the steps issued so far on the handle's stream; the
  // download waits for it on the copy stream, so later steps overlap it
  const unsigned nb = (unsigned)((n + 255) / 256);
  if (h->elem == 8)
    k_gather<double><<<nb, 256, 0, h->st>>>((const double*)h->buf[h->cur], sn.dev, g, h->nw);
  else
    k_gather<float><<<nb, 256, 0, h->st>>>((const float*)h->buf[h->cur], sn.dev, g, h->nw);
  CK(cudaGetLastError());
  CK(cudaEventRecord(sn.gathered, h->st));
  CK(cudaStreamWaitEvent(h->cst, sn.gathered, 0));
  CK(cudaMemcpyAsync(sn.host, sn.dev, sizeof(double) * n, cudaMemcpyDeviceToHost, h->cst));
  CK(cudaEventRecord(sn.copied, h->cst));
  sn.pending = true;
  return 0;
}

int vacgpu_snapshot_wait(vacgpu_handle* h, int slot, double* w) {
  if (!h) return fail("null handle");
  if (slot < 0 || slot > 1) return fail("snapshot slot must be 0 or 1");
  vacgpu_handle::Snap& sn = h->snap[slot];
  if (!sn.pending) return fail("no snapshot in flight in slot " + std::to_string(slot));
  CK(cudaEventSynchronize(sn.copied));
  if (w) memcpy(w, sn.host, sizeof(double) * h->g.ncell * h->nw);
  sn.pending = false;
  sn.ready = true;
  return 0;
}

const double* vacgpu_snapshot_data(vacgpu_handle* h, int slot) {
  if (!h || slot < 0 || slot > 1) {
    fail("bad handle or snapshot slot");
    return nullptr;
  }
  const vacgpu_handle::Snap& sn = h->snap[slot];
  if (!sn.ready) {
    fail("no completed snapshot in slot " + std::to_string(slot));
    return nullptr;
  }
  return sn.host;
}

int vacgpu_step(vacgpu_handle* h, int maxsteps, double tstop, double* t,
                int* it, double* dt, int* finished) {
  if (!h) return fail("null handle");
  if (!h->have_grid || !h->have_state)
    return fail("vacgpu_step before vacgpu_set_grid/vacgpu_upload");
  if (maxsteps < 0) return fail("maxsteps must be >= 0");
  if (h->faulted)
    return fail("the state is invalid after a timed-out device wait; upload a state first");
  if (h->any_special && !h->bound_fn) return fail(NO_SPECIAL);
  if (h->etaf && !h->eta_fn) return fail(NO_ETA);
  if (h->tuning && maxsteps > 0 && !h->timing && tune_nzc(h)) return 1;
  const int nsw = h->p.dimsplit ? h->p.ndim : 1;
  const int start_cur = h->cur;
  kbegin(h, VACGPU_K_CONTROL);
  k_call_begin<<<1, 1, 0, h->st>>>(h->ctrl, maxsteps, tstop);
  kend(h);
  CK(cudaGetLastError());
  int issued = 0, chunk = 4;
  Ctrl c;
  while (issued < maxsteps) {
    int k = maxsteps - issued < chunk ? maxsteps - issued : chunk;
    if (issue_steps(h, k, h->it_host + issued)) return 1;
    issued += k;
    CK(cudaGetLastError());
    if (h->hook_failed) {
      h->hook_failed = false;
      drop_graphs(h);
      CK(cudaStreamSynchronize(h->st));
      return fail("a user hook (specialbound, specialeta, specialsource or getdt_special) failed");
    }
    int done = 0;
    CK(cudaMemcpyAsync(&done, &h->ctrl->done, sizeof(int),
                       cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (done) break;
    if (chunk < 64) chunk *= 2;
  }
  CK(cudaMemcpyAsync(&c, h->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  // every executed step swapped the buffers nsw times; skipped ones none
  h->cur = start_cur ^ ((c.steps * nsw) & 1);
  if (c.fault) {
    h->faulted = true;
    return fail("a device wait timed out (TMA copy never completed); the state is invalid");
  }
  h->it_host = c.it;
  if (t) *t = c.t;
  if (it) *it = c.it;
  if (dt) *dt = c.dt;
  if (finished) *finished = c.done == 1;
  return 0;
}

int vacgpu_sums(vacgpu_handle* h, double* wmean) {
  if (!h) return fail("null handle");
  const DevGrid& g = h->g;
  long long nblk = (g.ncell + 255) / 256;
  if (h->elem == 8)
    k_sums_partial<double><<<(unsigned)nblk, 256, 0, h->st>>>(
        (const double*)h->buf[h->cur], g, h->nw, h->dx[0], h->dx[1], h->dx[2], h->part);
  else
    k_sums_partial<float><<<(unsigned)nblk, 256, 0, h->st>>>(
        (const float*)h->buf[h->cur], g, h->nw, h->dx[0], h->dx[1], h->dx[2], h->part);
  k_sums_final<<<1, 32, 0, h->st>>>(h->part, nblk, h->nw, h->sums);
  CK(cudaGetLastError());
  double s[8];
  CK(cudaMemcpyAsync(s, h->sums, sizeof(double) * h->nw, cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (int iw = 0; iw < h->nw; iw++) wmean[iw] = s[iw] / h->volume;
  return 0;
}

int vacgpu_error_counts(vacgpu_handle* h, int* nerror) {
  if (!h) return fail("null handle");
  Ctrl c;
  CK(cudaMemcpyAsync(&c, h->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  for (int i = 0; i < 4; i++) nerror[i] = c.nerror[i];
  return 0;
}

int vacgpu_register_eta(vacgpu_handle* h, vacgpu_eta_fn fn, void* user) {
  if (!h) return fail("null handle");
  if (h->st) CK(cudaStreamSynchronize(h->st));
  drop_graphs(h);
  h->eta_fn = fn;
  h->eta_user = user;
  return 0;
}

int vacgpu_register_bound(vacgpu_handle* h, vacgpu_bound_fn fn, void* user) {
  if (!h) return fail("null handle");
  if (h->st) CK(cudaStreamSynchronize(h->st));
  drop_graphs(h);
  h->bound_fn = fn;
  h->bound_user = user;
  return 0;
}

int vacgpu_register_source(vacgpu_handle* h, int source_id,
                           const double* params, int nparams) {
  if (!h) return fail("null handle");
  if (h->st) CK(cudaStreamSynchronize(h->st));
  drop_graphs(h);
  if (source_id != VACGPU_SRC_NONE && source_id != VACGPU_SRC_GRAVITY)
    return fail("unknown source id");
  if (nparams < 0 || nparams > VACGPU_MAXSRCPAR) return fail("bad nparams");
  if (!h->have_grid) return fail("register the source after vacgpu_set_grid");
  h->ph.src_id = source_id;
  for (int i = 0; i < VACGPU_MAXSRCPAR; i++)
    h->ph.src_par[i] = i < nparams ? params[i] : 0.0;
  // getdt_grav (vacusr.gravity.t): dtgrav = min_idim 1/sqrt(max(|g|/dx))
  h->dtgrav = BIGD;
  if (source_id == VACGPU_SRC_GRAVITY) {
    for (int d = 0; d < h->p.ndim; d++) {
      double gg = std::fabs(h->ph.src_par[d]);
      if (gg > 0.0) {
        double m = 0.0;
        bool first = true;
        for (int j = 0; j < h->p.ndim; j++)
          for (int i = 2; i < h->g.nx[j] + 2; i++) {
            double q = gg / h->hdx[j][i];
            if (first || q > m) m = q;
            first = false;
          }
        double c = 1.0 / std::sqrt(m);
        if (c < h->dtgrav) h->dtgrav = c;
      }
    }
  }
  double v = h->dtgrav;
  CK(cudaMemcpy(&h->ctrl->dtgrav, &v, sizeof(double), cudaMemcpyHostToDevice));
  return 0;
}

int vacgpu_register_source_fn(vacgpu_handle* h, vacgpu_source_fn src,
                              vacgpu_dtspecial_fn dt, void* user) {
  if (!h) return fail("null handle");
  if (src && h->ph.useprim)
    return fail("a specialsource hook with useprimitive is not supported");
  if (h->st) CK(cudaStreamSynchronize(h->st));
  drop_graphs(h);
  if (src && !h->faces && alloc_faces(h)) return 1;
  h->src_fn = src;
  h->dtsp_fn = dt;
  h->src_user = user;
  h->ph.src_hook = src != nullptr;
  if (src) h->tuning = false;  // the split kernels run; no z chunk to tune
  if (src || dt) {
    // the hooks replace a built-in source
    h->ph.src_id = VACGPU_SRC_NONE;
    h->dtgrav = BIGD;
    double v = BIGD;
    CK(cudaMemcpy(&h->ctrl->dtgrav, &v, sizeof(double), cudaMemcpyHostToDevice));
  }
  return 0;
}

void vacgpu_destroy(vacgpu_handle* h) {
  if (!h) return;
  if (h->st) cudaStreamSynchronize(h->st);
  if (h->own_st) cudaStreamSynchronize(h->own_st);
  if (h->cst) {
    cudaStreamSynchronize(h->cst);
    cudaStreamDestroy(h->cst);
  }
  for (auto& sn : h->snap) {
    cudaFree(sn.dev);
    cudaFreeHost(sn.host);
    if (sn.gathered) cudaEventDestroy(sn.gathered);
    if (sn.copied) cudaEventDestroy(sn.copied);
  }
  for (int i = 0; i < 3; i++) cudaFree(h->buf[i]);
  cudaFree(h->wold);
  cudaFree(h->fixb);
  cudaFree(h->faces);
  cudaFree(h->etaf);
  for (int k = 0; k < 3; k++) {
    cudaFree(h->curf[k]);
    cudaFree(h->gradetaf[k]);
  }
  for (int d = 0; d < 3; d++) {
    cudaFree(h->xg[d]);
    cudaFree(h->dx[d]);
    cudaFree(h->dxf[d]);
    cudaFree(h->idxf[d]);
  }
  cudaFree(h->stage);
  cudaFree(h->part);
  cudaFree(h->sums);
  cudaFree(h->ctrl);
  drain_events(h);
  for (auto e : h->pool) cudaEventDestroy(e);
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 2; j++)
      if (h->gexec[i][j]) cudaGraphExecDestroy(h->gexec[i][j]);
  if (h->own_st) cudaStreamDestroy(h->own_st);
  delete h;
}

int vacgpu_set_stream(vacgpu_handle* h, void* stream) {
  if (!h) return fail("null handle");
  CK(cudaStreamSynchronize(h->st));
  h->st = stream ? (cudaStream_t)stream : h->own_st;
  return 0;  // graphs launch on whichever stream is current
}

int vacgpu_timing(vacgpu_handle* h, int enable) {
  if (!h) return fail("null handle");
  CK(cudaStreamSynchronize(h->st));
  drain_events(h);
  if (enable) {
    for (int k = 0; k < VACGPU_K_NCLASS; k++) {
      h->nlaunch[k] = 0;
      h->kms[k] = 0.0;
    }
  }
  h->timing = enable != 0;
  return 0;
}

int vacgpu_kernel_stats(vacgpu_handle* h, int kclass, long long* launches,
                        double* ms) {
  if (!h) return fail("null handle");
  if (kclass < 0 || kclass >= VACGPU_K_NCLASS) return fail("bad kernel class");
  CK(cudaStreamSynchronize(h->st));
  drain_events(h);
  if (launches) *launches = h->nlaunch[kclass];
  if (ms) *ms = h->kms[kclass];
  return 0;
}

int vacgpu_last_error(char* buf, int len) {
  int n = (int)g_err.size();
  if (buf && len > 0) {
    int m = n < len - 1 ? n : len - 1;
    memcpy(buf, g_err.data(), m);
    buf[m] = 0;
  }
  return n;
}

const char* vacgpu_version(void) { return "vacgpu 0.1 (sm_103a)"; }

}  // extern "C"

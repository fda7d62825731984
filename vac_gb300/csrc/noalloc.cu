// noalloc.cu - vacgpu_sweep_noalloc: one FP64 split sweep on caller-owned
// device arrays with no device allocation.  The predictor output w1 and the
// control block (dt, smallp, CFL reduction slots) live in file-scope static
// device arrays; host code reaches them only through the device address
// cudaGetSymbolAddress returns (the symbol itself is a host-side stand-in).
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "vacgpu_internal.h"

using namespace vacgpu;

// Scratch shared by every call on a device: the predictor state (8 FP64
// variables x VACGPU_NOALLOC_MAX_GCELLS cells = 16 MiB) and one Ctrl block.
static __device__ __align__(256) double g_na_w1[VACGPU_NOALLOC_MAX_GCELLS * VACGPU_MAXNW];
// the corrector's face fluxes: at most (nx_d+1)*prod(nx_other) <= the
// ghost-box cells per variable
static __device__ __align__(256) double g_na_faces[VACGPU_NOALLOC_MAX_GCELLS * VACGPU_MAXNW];
static __device__ __align__(256) Ctrl g_na_ctrl;

namespace {

constexpr int MAXDEV = 64;
struct NaAddr {
  double* w1;
  double* faces;
  Ctrl* ctrl;
};
NaAddr g_addr[MAXDEV];
bool g_ready[MAXDEV];
std::mutex g_mu;

// Every call starts from a clean control block: the scratch keeps the last
// call's contents, so the CFL slots must be zeroed and done cleared.
__global__ void k_na_begin(Ctrl* c, double dt, double smallp) {
  if (threadIdx.x == 0) {
    c->done = 0;
    c->dt = dt;
    c->smallp = smallp;
  }
  for (int d = 0; d < 3; d++) c->face_cmax[d][threadIdx.x] = 0ULL;
}

__global__ void k_na_end(const Ctrl* c, int idim, double* out) {
  __shared__ unsigned long long sh[NSLOT];
  sh[threadIdx.x] = c->face_cmax[idim][threadIdx.x];
  __syncthreads();
  for (int o = NSLOT / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o && sh[threadIdx.x + o] > sh[threadIdx.x])
      sh[threadIdx.x] = sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0] ? dkey_inv(sh[0]) : 0.0;
}

}  // namespace

// Error reporting lives in vacgpu.cu.
int vacgpu_internal_fail(const char* msg);

extern "C" int vacgpu_sweep_noalloc(const vacgpu_params* p, const double* w,
                                    double* wout, const double* dx0,
                                    const double* dx1, const double* dx2,
                                    double dt, int idim, double* courantmax,
                                    void* stream) {
  if (!p || !w || !wout) return vacgpu_internal_fail("null argument");
  if (p->precision != VACGPU_PREC_FP64)
    return vacgpu_internal_fail("vacgpu_sweep_noalloc is FP64 only");
  if (p->ndim < 1 || p->ndim > 3 || idim < 0 || idim >= p->ndim)
    return vacgpu_internal_fail("idim out of range");
  bool combo = (p->ndim == p->ndir) || (p->ndim == 2 && p->ndir == 3);
  int nw = p->physics == VACGPU_PHYS_MHD ? 2 + 2 * p->ndir : 2 + p->ndir;
  if (!combo || p->nw != nw || p->dixB != 2)
    return vacgpu_internal_fail("unsupported ndim/ndir/nw/dixB");
  if (!p->dimsplit || p->typelimited == VACGPU_LIMITED_PREVIOUS)
    return vacgpu_internal_fail(
        "vacgpu_sweep_noalloc needs dimsplit and typelimited original or "
        "predictor");
  if (!(p->smallp >= 0.0))
    return vacgpu_internal_fail("vacgpu_sweep_noalloc needs smallp >= 0");
  if (p->typefull != VACGPU_TVDLF && p->typefull != VACGPU_TVDLF1)
    return vacgpu_internal_fail(
        "vacgpu_sweep_noalloc runs the tvdlf and tvdlf1 correctors");
  if (p->smallfix || p->useprimitive ||
      (p->physics == VACGPU_PHYS_MHD && p->eqpar[1] != 0.0))
    return vacgpu_internal_fail(
        "vacgpu_sweep_noalloc supports neither smallfix, useprimitive nor "
        "resistivity");
  const double* dxs[3] = {dx0, dx1, dx2};
  // cells with ghosts, checked against the limit after every factor so that
  // no product can wrap (each factor is at most the limit + 4)
  long long gcells = 1;
  for (int d = 0; d < p->ndim && gcells <= VACGPU_NOALLOC_MAX_GCELLS; d++) {
    if (p->nx[d] < 2) return vacgpu_internal_fail("nx must be >= 2");
    if (!dxs[d]) return vacgpu_internal_fail("dx of a used dimension is NULL");
    const long long f = p->nx[d] > VACGPU_NOALLOC_MAX_GCELLS
                            ? (long long)VACGPU_NOALLOC_MAX_GCELLS + 1
                            : (long long)p->nx[d] + 4;
    gcells *= f;
  }
  if (gcells > VACGPU_NOALLOC_MAX_GCELLS)
    return vacgpu_internal_fail(
        ("grid of " + std::to_string(gcells) +
         " cells (with ghosts) exceeds VACGPU_NOALLOC_MAX_GCELLS=" +
         std::to_string(VACGPU_NOALLOC_MAX_GCELLS))
            .c_str());

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAXDEV)
    return vacgpu_internal_fail("cudaGetDevice failed");
  NaAddr a;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ready[dev]) {
      // set-up once per device, with that device current
      void* pw = nullptr;
      void* pc = nullptr;
      void* pf = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&pw, g_na_w1);
      if (e == cudaSuccess) e = cudaGetSymbolAddress(&pc, g_na_ctrl);
      if (e == cudaSuccess) e = cudaGetSymbolAddress(&pf, g_na_faces);
      if (e != cudaSuccess)
        return vacgpu_internal_fail(
            (std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e))
                .c_str());
      g_addr[dev].w1 = (double*)pw;
      g_addr[dev].faces = (double*)pf;
      g_addr[dev].ctrl = (Ctrl*)pc;
      g_ready[dev] = true;
    }
    a = g_addr[dev];
  }

  SweepArgs s;
  memset(&s, 0, sizeof(s));
  DevGrid& g = s.g;
  g.ndim = p->ndim;
  g.ncell = 1;
  for (int d = 0; d < 3; d++) {
    g.nx[d] = d < p->ndim ? p->nx[d] : 1;
    g.gh[d] = d < p->ndim ? 2 : 0;
    g.nG[d] = g.nx[d] + 2 * g.gh[d];
    g.ncell *= g.nx[d];
  }
  g.xpad = 0;  // VAC's unpadded ixG layout
  g.P = g.nG[0];
  g.plane = g.P * g.nG[1];
  g.vs = g.plane * g.nG[2];
  DevPhys& ph = s.ph;
  ph.gamma = p->eqpar[0];
  ph.pt1 = 1.0 - 0.5 * p->eqpar[0];
  ph.gm1 = p->eqpar[0] - 1.0;
  ph.gammaf = (float)ph.gamma;
  ph.gm1f = (float)ph.gm1;
  ph.c2gf = (2.0f - ph.gammaf) / ph.gm1f;
  ph.pt3 = 0.5 * (p->eqpar[0] - 1.0);
  ph.smallpcoeff = p->smallpcoeff;
  ph.courantpar = courantmax ? 1.0 : -1.0;
  for (int iw = 0; iw < VACGPU_MAXNW; iw++) ph.lim[iw] = p->typelimiter[iw];
  memcpy(ph.typeB, p->typeB, sizeof(ph.typeB));
  ph.typefull = p->typefull;
  ph.divbfix = p->divbfix;
  ph.sourceunsplit = p->sourceunsplit;
  ph.src_id = VACGPU_SRC_NONE;
  set_gmaps(ph, p->ndim, p->nw);
  for (int d = 0; d < p->ndim; d++)
    if (ph.genbc || ph.noflux[d][0] || ph.noflux[d][1])
      return vacgpu_internal_fail(
          "vacgpu_sweep_noalloc supports cont, periodic, symm and asymm faces");
  for (int d = 0; d < 3; d++) s.a.dx[d] = dxs[d];
  s.ctrl = a.ctrl;
  s.ndir = p->ndir;
  s.mhd = p->physics == VACGPU_PHYS_MHD;
  s.d0 = s.d1 = idim;
  s.typelimited = p->typelimited;
  s.faces = a.faces;
  s.face_stride = (long long)p->nw * face_count(g, idim);

  cudaStream_t st = (cudaStream_t)stream;
  k_na_begin<<<1, NSLOT, 0, st>>>(a.ctrl, dt, p->smallp);
  if (p->typefull == VACGPU_TVDLF1) {
    // onestep (typepred1='nul'): the corrector alone with wCT = w and no
    // limiter (src/vacio.t:286-299,511)
    launch_correct_fp64(s, w, w, w, wout, st);
  } else {
    launch_predict_fp64(s, w, a.w1, st);
    launch_ghost_fp64(s, a.w1, st);
    const double* base = p->typelimited == VACGPU_LIMITED_PREDICTOR ? a.w1 : w;
    launch_correct_fp64(s, w, a.w1, base, wout, st);
  }
  launch_ghost_fp64(s, wout, st);
  if (courantmax) k_na_end<<<1, NSLOT, 0, st>>>(a.ctrl, idim, courantmax);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return vacgpu_internal_fail(
        (std::string("launch failed: ") + cudaGetErrorString(e)).c_str());
  return 0;
}

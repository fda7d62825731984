// vacgpu_internal.h - device data layout, the device-resident control block
// and the kernel launchers shared by the FP64 and mixed translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "../../include/vacgpu.h"

namespace vacgpu {

enum {
  LIM_MINMOD = VACGPU_LIM_MINMOD,
  LIM_WOODWARD = VACGPU_LIM_WOODWARD,
  LIM_SUPERBEE = VACGPU_LIM_SUPERBEE,
  LIM_VANLEER = VACGPU_LIM_VANLEER,
  LIM_ALBADA = VACGPU_LIM_ALBADA
};

// Number of slots the grid-level max/min reductions spread their atomics
// over (a block writes slot blockIdx % NSLOT); the step kernel folds them.
constexpr int NSLOT = 128;

// State layout in HBM: one padded box per variable (structure of arrays,
// like VAC's w(ixG^T,nw)), x fastest.  A row holds the nG[0] cells of
// ghost+mesh+ghost starting at column xpad, chosen so the first mesh cell
// (gx=2) sits on a 128-byte boundary; rows have pitch P elements.
struct DevGrid {
  int ndim;
  int nx[3];         // mesh cells (1 in unused dimensions)
  int nG[3];         // with ghost layers (nx+4, or 1)
  int gh[3];         // ghost width: 2 in used dimensions, 0 otherwise
  int xpad;          // column of gx=0
  long long P;       // row pitch (elements)
  long long plane;   // P*nG[1]
  long long vs;      // variable stride (elements)
  long long ncell;   // mesh cells
};

__host__ __device__ inline long long gidx(const DevGrid& g, int gx, int gy,
                                          int gz) {
  return ((long long)gz * g.nG[1] + gy) * g.P + gx + g.xpad;
}

struct DevPhys {
  double gamma, pt1, gm1, pt3;
  float gammaf, gm1f;  // the same, rounded once for the FP32 physics
  float c2gf;           // (2-gammaf)/gm1f, the FP32 Roe eigenvectors' constant
  double smallpcoeff;
  double courantpar;  // <=0: no CFL evaluation (dtpar set)
  int lim[VACGPU_MAXNW];
  int typeB[VACGPU_MAXB][VACGPU_MAXNW];
  int typefull;       // VACGPU_TVDLF / _TVDLF1 / _TVDMU / _TVDMU1
  int divbfix;
  int sourceunsplit;
  int smallfix;          // keeppositive before each ghost fill
  double vacuumrho, smallrhocoeff;
  int useprim;           // limit primitive variables (useprimitive)
  double eta;            // resistivity eqpar(eta_) (0: ideal MHD)
  int compactres;        // resistive source in the Laplacian form
  int src_id;
  // a user specialsource hook runs between the flux update and addsource:
  // the predictor/corrector kernels leave the sources to k_add_sources
  int src_hook;
  double src_par[VACGPU_MAXSRCPAR];
  // Boundary index map per face [dim][lo/hi] when every variable shares it:
  // GMAP_PERIODIC, GMAP_CONT or GMAP_MIRROR ('symm' and 'asymm'); GMAP_MIXED
  // when variables differ.  asym: bit iw set where variable iw is 'asymm'.
  int gmap[3][2];
  int asym[3][2];
  // bit iw set: 'symm0' face, zero flux of iw through it (setnoflux)
  int noflux[3][2];
  // some face is 'fixed', 'fixed1', 'cont1', 'grad1' or 'special': ghost
  // cells are filled face by face in getboundary's order (k_ghost_face)
  int genbc;
  // Roe dissipation of 'tvdmu'/'tvdmu1' (src/vactvd.t:86-243)
  int typeentropy[VACGPU_MAXNW];
  double entropycoef[VACGPU_MAXNW];
  int divbwave;
  int roe_dpprim;     // useprimitive: the MHD average takes dp = pR - pL
};

enum { GMAP_MIXED = -1, GMAP_PERIODIC = 0, GMAP_CONT = 1, GMAP_MIRROR = 2 };

// Fill gmap/asym/noflux/genbc of ph from its typeB table.
inline void set_gmaps(DevPhys& ph, int ndim, int nw) {
  ph.genbc = 0;
  for (int d = 0; d < 3; d++)
    for (int s = 0; s < 2; s++) {
      int m = GMAP_PERIODIC;
      int asy = 0, nof = 0;
      for (int v = 0; v < nw && d < ndim; v++) {
        int t = ph.typeB[2 * d + s][v];
        const bool gen = t == VACGPU_BC_FIXED || t == VACGPU_BC_FIXED1 ||
                         t == VACGPU_BC_CONT1 || t == VACGPU_BC_GRAD1 ||
                         t == VACGPU_BC_SPECIAL;
        int mv = gen ? GMAP_MIXED
                 : t == VACGPU_BC_PERIODIC ? GMAP_PERIODIC
                 : t == VACGPU_BC_CONT     ? GMAP_CONT
                                           : GMAP_MIRROR;
        if (gen) ph.genbc = 1;
        if (t == VACGPU_BC_ASYMM) asy |= 1 << v;
        if (t == VACGPU_BC_SYMM0) nof |= 1 << v;
        if (v == 0)
          m = mv;
        else if (mv != m)
          m = GMAP_MIXED;
      }
      ph.gmap[d][s] = m;
      ph.asym[d][s] = asy;
      ph.noflux[d][s] = nof;
    }
}

// Ghost position gi (G coordinate, n mesh cells) -> source mesh position
// under index map m of its face.
__host__ __device__ inline int gmap_src(int gi, int n, int m) {
  if (gi < 2)
    return m == GMAP_PERIODIC ? gi + n : m == GMAP_CONT ? 2 : 3 - gi;
  return m == GMAP_PERIODIC ? gi - n : m == GMAP_CONT ? n + 1 : 2 * n + 3 - gi;
}

// Device-resident time-loop state: dt, it and t never leave the device
// between steps, so a sequence of steps runs without host round trips (and
// can be captured as one CUDA graph).
struct Ctrl {
  double t, dt, dtold, dtpar, courantpar;
  double smallp;
  double dtgrav;
  double dtspecial;   // the user's getdt_special limit of this step (BIG: none)
  double src_qdt, src_qtc;  // qdt and qtC of the source call being issued
  double dtdiff;      // resistive diffusion dt limit (BIG without resistivity)
  double qt;          // time of the current ghost fill (specialbound hooks)
  // specialeta: max over the mesh of eta/dx_d^2 (ordered keys), of the
  // last field the hook produced (the first step's: from the state)
  unsigned long long etak[3];
  double tstop;
  double dtcourant[3];
  int it, itmin;
  int done;           // 0 running, 1 timetofinish, 2 tstop, 3 maxsteps
  int steps;          // steps done in the current vacgpu_step call
  int maxsteps;
  int need_cell[3];   // this step's dt needs the cell-centred cmax pass
  int need_smallp;    // smallp<0 at this step's first pressure evaluation
  int nerror[4];
  int fault;          // a bounded device wait gave up (TMA never completed)
  int cur;            // batched grids: which state buffer holds the state
  double smallrho;    // keeppositive_rho: -1 until set from min(rho)
  int need_smallrho;  // this keeppositive call sets smallrho
  int kp_r, kp_p;     // this keeppositive call found small rho / p
  // grid-level reductions (ordered-integer keys, atomicMax/atomicMin)
  unsigned long long face_cmax[3][NSLOT];  // corrector max cmax*2/(dx+dx)
  // 'tvdmu': max |a|*dt*2/(dx+dx) of the fastRW (face_cmax) and fastLW
  // (face_cmax2) waves of tvdlimit2 (src/vactvd.t:144-160)
  unsigned long long face_cmax2[3][NSLOT];
  int roe;
  unsigned long long cell_cmax[3][NSLOT];  // getdt_courant max cmax/dx
  unsigned long long pmin[NSLOT], pmax[NSLOT];
  unsigned long long rmin[NSLOT];          // keeppositive_rho min(rho)
};

// Faces of direction d: the nx_d+1 faces of each mesh line; the face with
// left cell (ghost-box coordinates) cl has index ((i2*e1)+i1)*e0+i0 with
// i_d = cl_d-1, i_k = cl_k-gh_k otherwise, e_d = nx_d+1, e_k = nx_k.
__host__ __device__ inline long long face_count(const DevGrid& g, int d) {
  long long n = 1;
  for (int k = 0; k < 3; k++) n *= g.nx[k] + (k == d ? 1 : 0);
  return n;
}
__host__ __device__ inline long long face_index(const DevGrid& g, int d,
                                                const int* cl) {
  long long idx = 0;
  for (int k = 2; k >= 0; k--) {
    const int e = g.nx[k] + (k == d ? 1 : 0);
    const int i = k == d ? cl[k] - 1 : cl[k] - g.gh[k];
    idx = idx * e + i;
  }
  return idx;
}
// Left cell of face f of direction d.
__host__ __device__ inline void face_left_cell(const DevGrid& g, int d,
                                               long long f, int* cl) {
  for (int k = 0; k < 3; k++) {
    const int e = g.nx[k] + (k == d ? 1 : 0);
    const int i = (int)(f % e);
    f /= e;
    cl[k] = k == d ? i + 1 : i + g.gh[k];
  }
}

// Order-preserving map of a double onto unsigned 64-bit integers.
__host__ __device__ inline unsigned long long dkey(double v) {
  long long b;
#ifdef __CUDA_ARCH__
  b = __double_as_longlong(v);
#else
  memcpy(&b, &v, 8);
#endif
  return b < 0 ? ~(unsigned long long)b
               : ((unsigned long long)b | 0x8000000000000000ULL);
}
__host__ __device__ inline double dkey_inv(unsigned long long k) {
  long long b = (k & 0x8000000000000000ULL)
                    ? (long long)(k & 0x7fffffffffffffffULL)
                    : (long long)~k;
  double v;
#ifdef __CUDA_ARCH__
  v = __longlong_as_double(b);
#else
  memcpy(&v, &b, 8);
#endif
  return v;
}

// Pointers of one grid's device arrays.
struct DevArrays {
  const double* dx[3];  // dx over the ghost-extended range, per dimension
  const float* dxf[3];  // FP32 copies for the mixed path
};

// Launchers (sweep_fp64.cu, sweep_mixed.cu).  `w` is the state at the start
// of the sweep, `w1` the predictor output, `wout` the corrected state.
struct SweepArgs {
  DevGrid g;
  DevPhys ph;
  DevArrays a;
  Ctrl* ctrl;
  // specialeta field (eqpar(eta_) < 0): eta and, for the compact form,
  // gradeta in the state's cell indexing; nullptr for a constant eta
  const double* etaf;
  const double* gradetaf[3];
  // corrector face buffer (the path's arithmetic type): per sweep
  // direction d0..d1 a block of face_stride elements holding, for every
  // face of the direction, its numerical flux (and the Roe dissipative
  // fluxes) variable-major
  void* faces;
  long long face_stride;
  int ndir, mhd;
  int d0, d1;           // sweep dimensions (d0==d1 when split)
  int typelimited;
};

// Precision-specific launchers (sweep_fp64.cu, sweep_mixed.cu).
#define VACGPU_DECLARE_LAUNCHERS(SUF, T)                                      \
  void launch_predict_##SUF(const SweepArgs& s, const T* w, T* w1,           \
                            cudaStream_t st);                                \
  void launch_correct_##SUF(const SweepArgs& s, const T* w, const T* w1,     \
                            const T* base, T* wout, cudaStream_t st);        \
  void launch_ghost_##SUF(const SweepArgs& s, T* w, cudaStream_t st);        \
  void launch_source_pass_##SUF(const SweepArgs& s, const T* wct, T* w,     \
                                int pred, cudaStream_t st);                  \
  void launch_pminmax_##SUF(const SweepArgs& s, const T* w, cudaStream_t st); \
  void launch_cell_cmax_##SUF(const SweepArgs& s, const T* w,                \
                              cudaStream_t st);                              \
  void launch_keeppositive_##SUF(const SweepArgs& s, T* w, cudaStream_t st); \
  void launch_roundtrip_##SUF(const SweepArgs& s, const T* w, T* out,       \
                              cudaStream_t st);                              \
  void launch_ghost_faces_##SUF(const SweepArgs& s, T* w, T* fixb,            \
                                int restore, cudaStream_t st);               \
  void launch_ghost_face_##SUF(const SweepArgs& s, T* w, T* fixb,             \
                               int restore, int iB, cudaStream_t st);        \
  void launch_fix_store_##SUF(const SweepArgs& s, const T* w, T* fixb,        \
                              cudaStream_t st);                              \
  void launch_current_field_##SUF(const SweepArgs& s, const T* w,            \
                                  double* const* cur, cudaStream_t st);
VACGPU_DECLARE_LAUNCHERS(fp64, double)
VACGPU_DECLARE_LAUNCHERS(mixed, float)
VACGPU_DECLARE_LAUNCHERS(mixedf64, float)
VACGPU_DECLARE_LAUNCHERS(mixedf32, float)

// TVD-MUSCL corrector ('tvdmu'/'tvdmu1') with the Roe dissipation
// (roe_fp64.cu, roe_mixed.cu); same arguments as launch_correct_*.
void launch_correct_roe_fp64(const SweepArgs& s, const double* w,
                             const double* w1, const double* base,
                             double* wout, cudaStream_t st);
void launch_correct_roe_mixed(const SweepArgs& s, const float* w,
                              const float* w1, const float* base, float* wout,
                              cudaStream_t st);

// Fused single-kernel sweep of the mixed path (sweep_fused.cu): returns
// false when no fused instance exists for the configuration.  `tmap` is the
// CUtensorMap (as bytes) of the input state buffer with the box of the sweep
// direction (fused_box_rows).
bool launch_sweep_fused(const SweepArgs& s, const void* tmap, const float* win,
                        float* wout,
                        const float* const* idxf, int nzc, cudaStream_t st);
// rows of the fused sweep's TMA box: x and z sweeps and the 3-D y sweep
// (k=0), the 2-D y sweep (k=1)
constexpr int FUSED_BOX_ROWS[2] = {12, 10};
int fused_smem_bytes(int nw, int kind);

// Precision-independent time-loop kernels (control.cu).
void launch_dt_begin(Ctrl* c, int ndim, cudaStream_t st);
void launch_smallp(Ctrl* c, int mhd, double smallpcoeff, cudaStream_t st);
// keeppositive bookkeeping: start (which one-time minima are due), the
// smallrho fold, and the end (nerror counts of the call).
void launch_kp_begin(Ctrl* c, int rho_floor, cudaStream_t st);
void launch_kp_smallrho(Ctrl* c, double coeff, cudaStream_t st);
void launch_kp_end(Ctrl* c, cudaStream_t st);
void launch_dt_end(Ctrl* c, const vacgpu_params& p, cudaStream_t st);
// the user source hook's call arguments: qdt = (pred ? dt/2 : dt) *
// (d1-d0+1)/ndim, qtC = t (+dt/2 for the corrector, pred = 0, half = 1)
void launch_src_args(Ctrl* c, int pred, int half, int nsweep, int ndim, cudaStream_t st);
// getdt_special: Ctrl::dtspecial = BIG before the user's dt hook
void launch_dtspecial_begin(Ctrl* c, cudaStream_t st);
// qt of a ghost fill: mode 0 t, 1 t+dt/2, 2 t+dt (src/vac.t:54,567)
void launch_set_qt(Ctrl* c, int mode, cudaStream_t st);
// specialeta: Ctrl::etak from the field (first_only: at it==itmin only)
void launch_eta_max(const SweepArgs& a, int first_only, cudaStream_t st);
void launch_step_end(Ctrl* c, int ndim, cudaStream_t st);
// Batched control: which = 0 dt_begin, 1 smallp, 2 dt_end, 3 step_end
// (toggle = buffer swaps per step), 4 call_begin; one block per grid.
void launchb_control(int which, Ctrl* const* cs, int n, const vacgpu_params& p,
                     int toggle, int maxsteps, double tstop, cudaStream_t st);

}  // namespace vacgpu

// batch.cu - many independent grids of uneven sizes advanced together.
//
// Every grid keeps its own state, dt, it and t (its own CFL condition, as
// separate VAC runs would).  One step of the whole batch is a fixed sequence
// of batched launches -- dt choice for all grids, one persistent sweep
// kernel per direction over the (grid, tile) work list of all grids (it also
// fills the ghost cells), the step epilogue for all grids -- and a call
// of vacgpu_batch_step captures its steps into one CUDA graph that is
// launched once.  The state buffer parity of each grid lives on the device
// (Ctrl::cur), so a grid that finishes early simply stops swapping.
//
// The persistent-kernel shape (CTAs and work-list order) is chosen by a
// small autotuner that times the candidates on the batch itself.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "batch_items.cuh"
#include "physics_mixed.cuh"
#include "sweep.cuh"
#include "sweep_fused.cuh"
#include "vacgpu_internal.h"

using namespace vacgpu;

int vacgpu_internal_fail(const char* msg);

// internal accessors of vacgpu.cu
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
int vacgpu_internal_view(vacgpu_handle* h, HandleView* v);
int vacgpu_internal_set_cur(vacgpu_handle* h, int cur);

namespace {

// rows per work item of the 2-D line sweep (the autotuner's item shapes)
// (negative: a guided list of base -r: items of -r rows, then toward the
// end of the list items of -r/2, -r/4 and -r/8 rows, two of each per grid
// and strip, so the sweep ends on short items)
constexpr int LINE2_SHAPES[3] = {16, -32, -16};

typedef PHMixed<PREC_FF> PHB;

template <int NDIM, int D, bool MHD, int LIMC>
__global__ void __launch_bounds__(FT_NT, 2)
    kb_sweep(const BItem* __restrict__ items, int nitems,
             const BInst* __restrict__ insts, const CUtensorMap* maps,
             int sweep) {
  extern __shared__ __align__(128) float dsm[];
  __shared__ __align__(8) unsigned long long bars[FWRING];
  __shared__ __align__(16) FusedArgs fa;
  __shared__ int mapidx;
  init_bars(bars);
  int uses[FWRING] = {0, 0, 0, 0};
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const BItem item = items[it];
    const BInst* in = insts + item.inst;
    {  // the grid's arguments into shared memory (word copy)
      const int* src = (const int*)&in->fa;
      int* dst = (int*)&fa;
      for (int k = threadIdx.x; k < (int)(sizeof(FusedArgs) / 4); k += blockDim.x)
        dst[k] = src[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int src = in->fa.ctrl->cur ^ (sweep & 1);
      fa.wout = in->buf[src ^ 1];
      mapidx = item.inst * 4 + src * 2 + (D == 1);
    }
    __syncthreads();
    bool ok = Fused<NDIM, D, MHD, PREC_FF, LIMC, PREC_FF>::run(
        &maps[mapidx], fa, dsm, item.bx, item.by, item.bz, bars, uses,
        (unsigned)it);
    __syncthreads();
    if (!ok) return;
  }
}

template <int NDIM, bool MHD>
__global__ void __launch_bounds__(128) kb_pminmax(const BInst* insts) {
  const BInst* in = insts + blockIdx.y;
  Sweep<PHB, NDIM, NDIM, MHD>::template pminmax<128>(in->sa, in->buf[in->sa.ctrl->cur]);
}

template <int NDIM, bool MHD>
__global__ void __launch_bounds__(128) kb_cell_cmax(const BInst* insts) {
  const BInst* in = insts + blockIdx.y;
  Sweep<PHB, NDIM, NDIM, MHD>::template cell_cmax<128>(in->sa, in->buf[in->sa.ctrl->cur]);
}

}  // namespace

struct vacgpu_batch {
  int n;
  vacgpu_params p0;
  std::vector<vacgpu_handle*> h;
  BInst* d_insts;
  CUtensorMap* d_maps;  // per grid: [state buffer][box: x/z, y]
  Ctrl** d_ctrls;
  // work lists per sweep direction (tile shapes differ), work-list order
  // (0 interleaved over grids, 1 grid-major) and item shape (2-D line
  // sweeps: rows per item, LINE2_SHAPES; one shape otherwise)
  BItem* d_items[3][2][3];
  int nitems[3][3];
  int nshape, shape;
  cudaStream_t st;
  int nw;
  bool ready;
  // launch shape (autotuned): persistent CTAs (0: one per work item) and
  // work-list order
  int ctas, order;
  bool pair;     // 3-D grids on the two-cells-per-thread sweep
  bool line2;    // 2-D grids on the warp-marching sweep
  bool pairgen;  // ... either in its general form
  bool tuned;
  // 2-D line sweeps: all steps of a call in one cooperative launch
  // (kb_steps_line2) instead of the graph of launches; chosen by the tuner
  bool onelaunch;
  int steps_ctas;
  int nparts;  // blocks per grid of the first-step passes (largest grid / 8192 cells)
  GridSync* d_gs;
  double tune_ms[24];
  int it0;
  struct G {
    int nsteps, par;
    double tstop;
    bool onelaunch;
    cudaGraphExec_t ex;
  };
  bool nograph_one;  // the cooperative launch could not be captured: launch it directly
  // 2-D line sweeps: host copies of the work lists (the phase lists of a
  // call on grids at different parities of it are built from them) and
  // the device buffers of those phase lists
  std::vector<BItem> h_items[2][2][3];
  BItem* d_plist[2];
  int nplist[2];
  std::vector<int> its;  // it of every grid after the last call
  std::vector<G> graphs;
};

namespace {

int bfail(const std::string& m) { return vacgpu_internal_fail(m.c_str()); }

#define BCK(call)                                                         \
  do {                                                                    \
    cudaError_t e_ = (call);                                              \
    if (e_ != cudaSuccess)                                                \
      return bfail(std::string("CUDA error: ") + cudaGetErrorString(e_) + \
                   " at " #call);                                         \
  } while (0)

template <int NDIM, bool MHD>
void launch_sweep_b(vacgpu_batch* b, int D, int LIMC, int sweep, int ctas,
                    int order) {
  constexpr int NW = MHD ? 2 + 2 * NDIM : 2 + NDIM;
  const int smem = fused_smem_floats(NW, fused_kind(NDIM, D)) * 4;
  const int n = b->nitems[D][0];
  const BItem* items = b->d_items[D][order][0];
  if (ctas <= 0 || ctas > n) ctas = n;
#define KB(DD, LL)                                                          \
  {                                                                         \
    auto k = kb_sweep<NDIM, DD, MHD, LL>;                                   \
    static bool attr = false;                                               \
    if (!attr) {                                                            \
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                           smem);                                           \
      attr = true;                                                          \
    }                                                                       \
    k<<<ctas, FT_NT, smem, b->st>>>(items, n, b->d_insts, b->d_maps, sweep); \
  }
#define KBL(DD)                                 \
  if (LIMC == LIMC_WOODWARD) KB(DD, LIMC_WOODWARD) \
  else if (LIMC == LIMC_MINMOD) KB(DD, LIMC_MINMOD) \
  else KB(DD, LIMC_RUNTIME)
  if (D == 0) { KBL(0) }
  else if (D == 1) { KBL(1) }
  else if (NDIM == 3) { KBL(2 % NDIM) }
#undef KBL
#undef KB
}

void launch_sweep_any(vacgpu_batch* b, int D, int sweep, int ctas, int order, int shape) {
  const vacgpu_params& p = b->p0;
  if (b->line2) {
    launch_batch_line2(b->d_items[D][order][shape], b->nitems[D][shape], b->d_insts, sweep, D,
                       p.physics == VACGPU_PHYS_MHD, p.typelimiter[0], b->pairgen, ctas,
                       b->st);
    return;
  }
  if (b->pair) {
    launch_batch_pair(b->d_items[D][order][0], b->nitems[D][0], b->d_insts, b->d_maps, sweep, D,
                      p.physics == VACGPU_PHYS_MHD, p.typelimiter[0], b->pairgen, ctas,
                      b->st);
    return;
  }
  int l0 = p.typelimiter[0];
  bool uni = p.typefull != VACGPU_TVDLF1;
  for (int v = 1; v < b->nw; v++) uni = uni && p.typelimiter[v] == l0;
  const int LIMC = !uni ? LIMC_RUNTIME
                   : l0 == VACGPU_LIM_WOODWARD ? LIMC_WOODWARD
                   : l0 == VACGPU_LIM_MINMOD ? LIMC_MINMOD
                                             : LIMC_RUNTIME;
  const bool mhd = p.physics == VACGPU_PHYS_MHD;
  if (p.ndim == 2) {
    if (mhd) launch_sweep_b<2, true>(b, D, LIMC, sweep, ctas, order);
    else launch_sweep_b<2, false>(b, D, LIMC, sweep, ctas, order);
  } else {
    if (mhd) launch_sweep_b<3, true>(b, D, LIMC, sweep, ctas, order);
    else launch_sweep_b<3, false>(b, D, LIMC, sweep, ctas, order);
  }
}

// One step of every grid (the body of VAC's time loop, batched).
void issue_step(vacgpu_batch* b, int parity, int ctas, int order, int shape) {
  const vacgpu_params& p = b->p0;
  const int n = b->n;
  const bool mhd = p.physics == VACGPU_PHYS_MHD;
  launchb_control(0, b->d_ctrls, n, p, 0, 0, 0.0, b->st);
  dim3 pg(b->nparts, n);
#define PASS(K)                                                             \
  if (p.ndim == 2) {                                                        \
    if (mhd) K<2, true><<<pg, 128, 0, b->st>>>(b->d_insts);                 \
    else K<2, false><<<pg, 128, 0, b->st>>>(b->d_insts);                    \
  } else {                                                                  \
    if (mhd) K<3, true><<<pg, 128, 0, b->st>>>(b->d_insts);                 \
    else K<3, false><<<pg, 128, 0, b->st>>>(b->d_insts);                    \
  }
  PASS(kb_pminmax)
  launchb_control(1, b->d_ctrls, n, p, 0, 0, 0.0, b->st);
  PASS(kb_cell_cmax)
#undef PASS
  launchb_control(2, b->d_ctrls, n, p, 0, 0, 0.0, b->st);
  const int nsw = p.ndim;
  for (int s = 0; s < nsw; s++) {
    const int D = (!parity || p.typedimsplit == VACGPU_SPLIT_XY) ? s : nsw - 1 - s;
    launch_sweep_any(b, D, s, ctas, order, shape);  // also fills the ghost cells
  }
  launchb_control(3, b->d_ctrls, n, p, nsw & 1, 0, 0.0, b->st);
}

// nsteps steps of every grid of a 2-D line-sweep batch in one cooperative
// launch (kb_steps_line2): the call's begin, then per step the dt choice,
// the first-step passes where a grid needs them, the two sweeps and the
// step's end, separated by grid-wide barriers.  The barrier's counters are
// cleared before every launch, so a launch after a timed-out barrier starts
// clean.
int issue_steps_lists(vacgpu_batch* b, int nsteps, double tstop, int par, int xy,
                      const BItem* l0, int n0, const BItem* l1, int n1) {
  const vacgpu_params& p = b->p0;
  Line2Steps ls;
  ls.items[0] = l0;
  ls.nitems[0] = n0;
  ls.items[1] = l1;
  ls.nitems[1] = n1;
  ls.insts = b->d_insts;
  ls.ctrls = b->d_ctrls;
  ls.n = b->n;
  ls.nsteps = nsteps;
  ls.tstop = tstop;
  ls.par0 = par;
  ls.xy = xy;
  ls.dte = dt_end_args(p);
  ls.smallpcoeff = p.smallpcoeff;
  ls.nparts = b->nparts;
  ls.gs = b->d_gs;
  BCK(cudaMemsetAsync(b->d_gs, 0, sizeof(GridSync), b->st));
  if (!launch_line2_steps(ls, p.physics == VACGPU_PHYS_MHD, p.typelimiter[0], b->pairgen,
                          b->steps_ctas, b->st))
    return bfail(std::string("cooperative launch of the batched steps failed: ") +
                 cudaGetErrorString(cudaGetLastError()));
  return 0;
}

int issue_steps_one(vacgpu_batch* b, int nsteps, double tstop, int par, int order, int shape) {
  return issue_steps_lists(b, nsteps, tstop, par, b->p0.typedimsplit == VACGPU_SPLIT_XY,
                           b->d_items[0][order][shape], b->nitems[0][shape],
                           b->d_items[1][order][shape], b->nitems[1][shape]);
}

// A call on 2-D grids whose it differ in parity ('xyyx' splitting: each
// grid starts its step with the sweep its own it selects).  Phase list q
// serves the first sweep of the launch's steps s with s%2 == q and the
// second sweep of the others: grid g's x items where (it_g + q) is even,
// its y items otherwise, the two lists merged by position so that the
// short items of a guided list stay at the end.
int issue_steps_mixed(vacgpu_batch* b, int nsteps, double tstop) {
  const std::vector<BItem>& X = b->h_items[0][b->order][b->shape];
  const std::vector<BItem>& Y = b->h_items[1][b->order][b->shape];
  for (int q = 0; q < 2; q++) {
    std::vector<BItem> P;
    P.reserve(X.size() + Y.size());
    size_t ix = 0, iy = 0;
    auto takex = [&](const BItem& it) { return ((b->its[it.inst] + q) & 1) == 0; };
    while (ix < X.size() || iy < Y.size()) {
      const bool fromx = iy >= Y.size() ||
                         (ix < X.size() && (double)ix * Y.size() <= (double)iy * X.size());
      if (fromx) {
        if (takex(X[ix])) P.push_back(X[ix]);
        ix++;
      } else {
        if (!takex(Y[iy])) P.push_back(Y[iy]);
        iy++;
      }
    }
    if (!b->d_plist[q]) BCK(cudaMalloc(&b->d_plist[q], sizeof(BItem) * (X.size() + Y.size())));
    BCK(cudaMemcpyAsync(b->d_plist[q], P.data(), sizeof(BItem) * P.size(),
                        cudaMemcpyHostToDevice, b->st));
    BCK(cudaStreamSynchronize(b->st));  // P leaves scope
    b->nplist[q] = (int)P.size();
  }
  return issue_steps_lists(b, nsteps, tstop, 0, 0, b->d_plist[0], b->nplist[0], b->d_plist[1],
                           b->nplist[1]);
}

int prepare(vacgpu_batch* b) {
  if (b->ready) return 0;
  const int n = b->n;
  std::vector<BInst> ins(n);
  std::vector<CUtensorMap> maps(4 * n);
  std::vector<Ctrl*> ctrls(n);
  for (int i = 0; i < n; i++) {
    HandleView v;
    if (vacgpu_internal_view(b->h[i], &v)) return 1;
    if (!v.fused)
      return bfail("batched grids need the fused mixed-precision sweep "
                   "(dimsplit, ndir=ndim, uniform boundary maps)");
    BInst& bi = ins[i];
    memset(&bi, 0, sizeof(bi));
    FusedArgs& a = bi.fa;
    a.g = v.g;
    a.ph = v.ph;
    for (int d = 0; d < 3; d++) {
      a.dxf[d] = v.dxf[d];
      a.idxf[d] = v.idxf[d];
    }
    a.ctrl = v.ctrl;
    a.nzc = v.nzc;
    for (int d = 0; d < 3; d++) a.gravf[d] = (float)v.ph.src_par[d];
    a.cfl = v.ph.courantpar > 0.0;
    for (int d = 0; d < 3; d++)
      for (int w = 0; w < b->nw; w++) {
        if (v.ph.typeB[2 * d][w] == VACGPU_BC_PERIODIC) a.periodic_mask[d] |= 1 << w;
        if (v.ph.typeB[2 * d][w] == VACGPU_BC_ASYMM) a.asymm_lo[d] |= 1 << w;
        if (v.ph.typeB[2 * d + 1][w] == VACGPU_BC_ASYMM) a.asymm_hi[d] |= 1 << w;
      }
    bi.sa = v.sa;
    bi.buf[0] = v.buf[0];
    bi.buf[1] = v.buf[1];
    for (int k = 0; k < 4; k++)
      memcpy(&maps[4 * i + k], v.tmap[k / 2][k % 2], sizeof(CUtensorMap));
    ctrls[i] = v.ctrl;
  }
  // the pair sweep when it applies to every grid: the single-grid path
  // runs it on each of them, so the batch gives the same bits
  const bool mhd = b->p0.physics == VACGPU_PHYS_MHD;
  b->pair = b->p0.ndim == 3;
  b->line2 = b->p0.ndim == 2;
  b->pairgen = false;
  for (int i = 0; i < n; i++) {
    b->pair = b->pair && pair_applies(ins[i].fa, mhd);
    b->line2 = b->line2 && line2_applies(ins[i].fa, mhd);
    b->pairgen = b->pairgen || pair_general(ins[i].fa, mhd);
  }
  b->nshape = b->line2 ? 3 : 1;
  b->shape = 0;
  long long maxcell = 0;
  for (int i = 0; i < n; i++) maxcell = std::max(maxcell, (long long)ins[i].sa.g.ncell);
  b->nparts = (int)std::min(256LL, std::max(8LL, (maxcell + 8191) / 8192));
  BCK(cudaMalloc(&b->d_insts, sizeof(BInst) * n));
  BCK(cudaMalloc(&b->d_maps, sizeof(CUtensorMap) * 4 * n));
  BCK(cudaMalloc(&b->d_ctrls, sizeof(Ctrl*) * n));
  if (b->line2) {
    BCK(cudaMalloc(&b->d_gs, sizeof(GridSync)));
    BCK(cudaMemset(b->d_gs, 0, sizeof(GridSync)));
    b->steps_ctas = line2_steps_ctas(mhd, b->p0.typelimiter[0], b->pairgen);
  }
  BCK(cudaMemcpy(b->d_insts, ins.data(), sizeof(BInst) * n, cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(b->d_maps, maps.data(), sizeof(CUtensorMap) * 4 * n, cudaMemcpyHostToDevice));
  BCK(cudaMemcpy(b->d_ctrls, ctrls.data(), sizeof(Ctrl*) * n, cudaMemcpyHostToDevice));
  // work lists: every (grid, tile, z chunk) of the tile shape of each sweep
  // direction; order 0 round-robin over grids (neighbouring CTAs work on
  // different grids), order 1 grid-major, largest grid first
  for (int D = 0; D < b->p0.ndim; D++) {
    // tiles over x and the row axis, z chunks along the marching axis
    const int kind = fused_kind(b->p0.ndim, D);
    const int tx = kind == 0 ? TileCfg<0>::TX : TileCfg<1>::TX;
    const int ty = kind == 1 ? TileCfg<1>::TY : TileCfg<0>::TY;
    const int ar = kind == 2 && D == 1 ? 2 : 1, am = kind == 2 ? D : 2;
    // the pair sweep's x tiles start one column left of the mesh: nx + 1
    // columns of faces
    const int xext = b->pair && D == 0 ? 1 : 0;
    for (int sh = 0; sh < b->nshape; sh++) {
    // per grid, per level (guided lists: item size B, B/2, B/4, B/8)
    std::vector<std::vector<BItem>> per[4];
    for (auto& l : per) l.resize(n);
    for (int i = 0; i < n; i++) {
      const DevGrid& g = ins[i].fa.g;
      if (b->line2) {  // (strip, first and end row), strips fastest
        const int ns = line2_strips(D, mhd, g.nx[0]), r = LINE2_SHAPES[sh];
        const int ny = g.nx[1], B = r > 0 ? r : -r;
        // row chunks (first row, rows, level): the last rows in short chunks
        std::vector<int> tail;  // sizes from the top row down
        int rem = ny;
        if (r < 0)
          for (int lv = 3; lv >= 1; lv--)
            for (int k = 0; k < 2 && rem > 0; k++) {
              const int c = std::min(std::max(B >> lv, 1), rem);
              tail.push_back(c | lv << 16);
              rem -= c;
            }
        // (the item's sweep direction in bit 30 of bx, the strip below it)
        auto add = [&](int y0, int rows, int lv) {
          for (int x = 0; x < ns; x++)
            per[lv][i].push_back({i, x | D << 30, 2 + y0, 2 + y0 + rows});
        };
        for (int y = 0; y < rem; y += B) add(y, std::min(B, rem - y), 0);
        int y = rem;
        for (int k = (int)tail.size() - 1; k >= 0; k--) {
          add(y, tail[k] & 0xffff, tail[k] >> 16);
          y += tail[k] & 0xffff;
        }
        continue;
      }
      const int nbx = (g.nx[0] + xext + tx - 1) / tx, nby = (g.nx[ar] + ty - 1) / ty;
      const int nbz = g.ndim == 3 ? (g.nx[am] + ins[i].fa.nzc - 1) / ins[i].fa.nzc : 1;
      for (int z = 0; z < nbz; z++)
        for (int y = 0; y < nby; y++)
          for (int x = 0; x < nbx; x++) per[0][i].push_back({i, x, y, z});
    }
    std::vector<BItem> rr, gm;
    for (int lv = 0; lv < 4; lv++) {
      size_t maxk = 0;
      for (auto& v : per[lv]) maxk = std::max(maxk, v.size());
      for (size_t k = 0; k < maxk; k++)
        for (int i = 0; i < n; i++)
          if (k < per[lv][i].size()) rr.push_back(per[lv][i][k]);
      std::vector<int> idx(n);
      for (int i = 0; i < n; i++) idx[i] = i;
      std::stable_sort(idx.begin(), idx.end(), [&](int a, int c) {
        return ins[a].fa.g.ncell > ins[c].fa.g.ncell;
      });
      for (int i : idx) gm.insert(gm.end(), per[lv][i].begin(), per[lv][i].end());
    }
    b->nitems[D][sh] = (int)rr.size();
    for (int o = 0; o < 2; o++) {
      const std::vector<BItem>& l = o ? gm : rr;
      if (b->line2) b->h_items[D][o][sh] = l;
      BCK(cudaMalloc(&b->d_items[D][o][sh], sizeof(BItem) * l.size()));
      BCK(cudaMemcpy(b->d_items[D][o][sh], l.data(), sizeof(BItem) * l.size(),
                     cudaMemcpyHostToDevice));
    }
    }
  }
  b->ready = true;
  return 0;
}

// Autotuner: time two steps of every candidate launch shape on the batch
// itself, after one untimed step (state and control blocks restored after
// each trial), and keep the fastest.  Candidates: persistent CTAs (per SM:
// 1 and 2 for the one-cell sweep, whose 103 KB CTAs fit twice; 2 and 3 for
// the pair sweep; 4 and 8 CTAs of four warps for the 2-D line sweep) or one
// CTA (line sweep: one warp) per work item, times two work-list orders,
// times the item shapes (2-D line sweep: LINE2_SHAPES, 16 rows per item or
// a guided list); for 2-D line-sweep batches also the one-launch form of
// every item shape and order (VACGPU_ONELAUNCH=0 leaves it out, =1 takes
// it).
int autotune(vacgpu_batch* b) {
  if (b->tuned) return 0;
  const int n = b->n;
  std::vector<HandleView> v(n);
  size_t tot = 0;
  for (int i = 0; i < n; i++) {
    vacgpu_internal_view(b->h[i], &v[i]);
    tot += 2 * (size_t)v[i].g.vs * b->nw * sizeof(float) + sizeof(Ctrl);
  }
  char* snap = nullptr;
  BCK(cudaMalloc(&snap, tot));
  auto copy = [&](bool save) -> int {
    size_t off = 0;
    for (int i = 0; i < n; i++) {
      size_t bytes = (size_t)v[i].g.vs * b->nw * sizeof(float);
      for (int k = 0; k < 2; k++) {
        void* a = snap + off;
        if (save)
          BCK(cudaMemcpyAsync(a, v[i].buf[k], bytes, cudaMemcpyDeviceToDevice, b->st));
        else
          BCK(cudaMemcpyAsync(v[i].buf[k], a, bytes, cudaMemcpyDeviceToDevice, b->st));
        off += bytes;
      }
      if (save)
        BCK(cudaMemcpyAsync(snap + off, v[i].ctrl, sizeof(Ctrl), cudaMemcpyDeviceToDevice, b->st));
      else
        BCK(cudaMemcpyAsync(v[i].ctrl, snap + off, sizeof(Ctrl), cudaMemcpyDeviceToDevice, b->st));
      off += sizeof(Ctrl);
    }
    return 0;
  };
  if (copy(true)) return 1;
  int sms = 152;
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  const int per_sm[2] = {b->line2 ? 4 : b->pair ? 2 : 1, b->line2 ? 8 : b->pair ? 3 : 2};
  const int cand_ctas[3] = {per_sm[0] * sms, per_sm[1] * sms, 0};  // 0: one per item
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // one trial: from the saved state, one untimed step (it runs the
  // first-step passes where a grid needs them, as only a run's first step
  // does), then two timed steps; then the state and control blocks restored
  const int par = b->it0 & 1;
  auto trial = [&](int mode, int ctas, int o, int sh, float* ms) -> int {
    if (mode == 0) {
      launchb_control(4, b->d_ctrls, n, b->p0, 0, 1 << 30, 1e300, b->st);
      issue_step(b, par, ctas, o, sh);
      cudaEventRecord(e0, b->st);
      issue_step(b, par ^ 1, ctas, o, sh);
      issue_step(b, par, ctas, o, sh);
      cudaEventRecord(e1, b->st);
    } else {
      if (issue_steps_one(b, 1, 1e300, par, o, sh)) return 1;
      cudaEventRecord(e0, b->st);
      if (issue_steps_one(b, 2, 1e300, par ^ 1, o, sh)) return 1;
      cudaEventRecord(e1, b->st);
    }
    if (copy(false)) return 1;
    BCK(cudaEventSynchronize(e1));
    BCK(cudaEventElapsedTime(ms, e0, e1));
    return 0;
  };
  float best = 1e30f;
  int bc = cand_ctas[1], bo = 0, bs = 0, bm = 0, k = 0;
  for (int k = 0; k < 24; k++) b->tune_ms[k] = 0.0;
  for (int sh = 0; sh < b->nshape; sh++)
    for (int c = 0; c < 3; c++)
      for (int o = 0; o < 2; o++, k++) {
        float ms = 0.f;
        if (trial(0, cand_ctas[c], o, sh, &ms)) return 1;
        b->tune_ms[k] = ms;
        if (ms < best) {
          best = ms;
          bc = cand_ctas[c];
          bo = o;
          bs = sh;
        }
      }
  const char* ol = getenv("VACGPU_ONELAUNCH");
  if (b->line2 && !(ol && atoi(ol) == 0))
    for (int sh = 0; sh < b->nshape; sh++)
      for (int o = 0; o < 2; o++) {
        float ms = 0.f;
        if (trial(1, 0, o, sh, &ms)) return 1;
        b->tune_ms[18 + 2 * sh + o] = ms;
        if (ms < best || (ol && atoi(ol) == 1 && !bm)) {
          best = ms;
          bo = o;
          bs = sh;
          bm = 1;
        }
      }
  BCK(cudaStreamSynchronize(b->st));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(snap);
  BCK(cudaGetLastError());
  b->ctas = bm ? b->steps_ctas : bc;
  b->order = bo;
  b->shape = bs;
  b->onelaunch = bm;
  b->tuned = true;
  return 0;
}

}  // namespace

extern "C" {

int vacgpu_batch_create(const vacgpu_params* params, int n,
                        vacgpu_batch** out) {
  *out = nullptr;
  if (n < 1) return bfail("a batch needs at least one grid");
  for (int i = 0; i < n; i++) {
    const vacgpu_params& p = params[i];
    const vacgpu_params& q = params[0];
    if (p.precision != VACGPU_PREC_MIXED)
      return bfail("batched grids run the mixed-precision path");
    if (p.ndim != q.ndim || p.ndir != q.ndir || p.physics != q.physics ||
        p.typedimsplit != q.typedimsplit || p.itmax != q.itmax ||
        p.typefull != q.typefull ||
        memcmp(p.typelimiter, q.typelimiter, sizeof(p.typelimiter)) != 0)
      return bfail("grids of a batch share physics, dimensionality, method, "
                   "limiters and itmax");
  }
  vacgpu_batch* b = new vacgpu_batch();
  b->n = n;
  b->p0 = params[0];
  b->nw = params[0].nw;
  b->ctas = 304;
  for (int i = 0; i < n; i++) {
    vacgpu_handle* h = nullptr;
    if (vacgpu_create(&params[i], &h)) {
      vacgpu_batch_destroy(b);
      return 1;
    }
    b->h.push_back(h);
  }
  if (cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess) {
    vacgpu_batch_destroy(b);
    return bfail("stream creation failed");
  }
  *out = b;
  return 0;
}

int vacgpu_batch_set_grid(vacgpu_batch* b, int i, const double* x) {
  if (!b || i < 0 || i >= b->n) return bfail("bad batch index");
  return vacgpu_set_grid(b->h[i], x);
}

int vacgpu_batch_upload(vacgpu_batch* b, int i, const double* w, int it,
                        double t) {
  if (!b || i < 0 || i >= b->n) return bfail("bad batch index");
  if (vacgpu_upload(b->h[i], w, it, t)) return 1;
  if (i == 0) b->it0 = it;
  if (it != b->it0) return bfail("grids of a batch start at the same it");
  if (b->its.size() != (size_t)b->n) b->its.assign(b->n, it);
  b->its[i] = it;
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.ex);
  b->graphs.clear();
  return 0;
}

int vacgpu_batch_download(vacgpu_batch* b, int i, double* w) {
  if (!b || i < 0 || i >= b->n) return bfail("bad batch index");
  BCK(cudaStreamSynchronize(b->st));
  HandleView v;
  vacgpu_internal_view(b->h[i], &v);
  int cur = 0;
  BCK(cudaMemcpy(&cur, &v.ctrl->cur, sizeof(int), cudaMemcpyDeviceToHost));
  vacgpu_internal_set_cur(b->h[i], cur);
  return vacgpu_download(b->h[i], w);
}

int vacgpu_batch_step(vacgpu_batch* b, int nsteps, double tstop) {
  if (!b) return bfail("null batch");
  if (prepare(b)) return 1;
  const char* tz = getenv("VACGPU_TUNE");
  if (!b->tuned && !(tz && atoi(tz) == 0))
    if (autotune(b)) return 1;
  if (b->its.size() != (size_t)b->n) b->its.assign(b->n, b->it0);
  // 'xyyx' grids that a stop time left at different parities of it
  bool mixed = false;
  if (b->p0.typedimsplit != VACGPU_SPLIT_XY)
    for (int i = 1; i < b->n; i++) mixed = mixed || ((b->its[i] ^ b->its[0]) & 1);
  if (mixed && !b->line2)
    return bfail("grids of a 3-D batch are at different parities of it (a stop time ended "
                 "them at different steps); upload them again to continue");
  const int par = b->its[0] & 1;
  cudaGraphExec_t ex = nullptr;
  for (auto& g : b->graphs)
    if (g.nsteps == nsteps && g.par == par && g.tstop == tstop && g.onelaunch == b->onelaunch)
      ex = g.ex;
  if (mixed) {
    if (issue_steps_mixed(b, nsteps, tstop)) return 1;
  } else if (!ex && !(b->onelaunch && b->nograph_one)) {
    // the call's launches captured once and replayed (the one-launch form:
    // the clears of its counters and the cooperative launch)
    cudaGraph_t gr = nullptr;
    BCK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    if (b->onelaunch) {
      rc = issue_steps_one(b, nsteps, tstop, par, b->order, b->shape);
    } else {
      launchb_control(4, b->d_ctrls, b->n, b->p0, 0, nsteps, tstop, b->st);
      for (int s = 0; s < nsteps; s++)
        issue_step(b, (par + s) & 1, b->ctas, b->order, b->shape);
    }
    const cudaError_t e = cudaStreamEndCapture(b->st, &gr);
    cudaGraphExec_t gx = nullptr;
    if (!rc && e == cudaSuccess && cudaGraphInstantiate(&gx, gr, 0) == cudaSuccess) {
      ex = gx;
      b->graphs.push_back({nsteps, par, tstop, b->onelaunch, ex});
    } else if (b->onelaunch) {
      b->nograph_one = true;  // launched directly below
    } else {
      if (gr) cudaGraphDestroy(gr);
      (void)cudaGetLastError();
      return rc ? 1 : bfail("capture of the batched steps failed");
    }
    if (gr) cudaGraphDestroy(gr);
    (void)cudaGetLastError();
  }
  if (mixed) {
  } else if (ex) {
    BCK(cudaGraphLaunch(ex, b->st));
  } else if (issue_steps_one(b, nsteps, tstop, par, b->order, b->shape)) {
    return 1;
  }
  BCK(cudaStreamSynchronize(b->st));
  if (b->onelaunch || mixed) {
    GridSync gs;
    BCK(cudaMemcpy(&gs, b->d_gs, sizeof(gs), cudaMemcpyDeviceToHost));
    if (gs.fault) return bfail("a grid-wide barrier of the batched steps timed out");
  }
  // every grid advanced the same number of steps unless it finished early
  for (int i = 0; i < b->n; i++) {
    HandleView v;
    vacgpu_internal_view(b->h[i], &v);
    Ctrl c;
    BCK(cudaMemcpy(&c, v.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost));
    if (c.fault) return bfail("a device wait timed out (TMA copy never completed)");
    b->its[i] = c.it;
  }
  b->it0 = b->its[0];
  return 0;
}

int vacgpu_batch_status(vacgpu_batch* b, int i, double* t, int* it,
                        double* dt, int* finished) {
  if (!b || i < 0 || i >= b->n) return bfail("bad batch index");
  HandleView v;
  vacgpu_internal_view(b->h[i], &v);
  Ctrl c;
  BCK(cudaStreamSynchronize(b->st));
  BCK(cudaMemcpy(&c, v.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost));
  if (t) *t = c.t;
  if (it) *it = c.it;
  if (dt) *dt = c.dt;
  if (finished) *finished = c.done == 1;
  return 0;
}

int vacgpu_batch_tune(vacgpu_batch* b, int* ctas, int* order, int* rows, int* onelaunch,
                      double* ms) {
  if (!b) return bfail("null batch");
  if (prepare(b) || autotune(b)) return 1;
  const int ni = b->nitems[0][b->shape];
  if (ctas) *ctas = b->ctas > 0 ? b->ctas : (b->line2 ? (ni + 3) / 4 : ni);
  if (order) *order = b->order;
  if (rows) *rows = b->line2 ? LINE2_SHAPES[b->shape] : 0;
  if (onelaunch) {
    bool graphed = false;
    for (auto& g : b->graphs) graphed = graphed || g.onelaunch;
    *onelaunch = !b->onelaunch ? 0 : graphed ? 2 : 1;
  }
  if (ms)
    for (int k = 0; k < 24; k++) ms[k] = b->tune_ms[k];
  return 0;
}

void vacgpu_batch_destroy(vacgpu_batch* b) {
  if (!b) return;
  if (b->st) cudaStreamSynchronize(b->st);
  for (auto& g : b->graphs) cudaGraphExecDestroy(g.ex);
  for (auto* h : b->h) vacgpu_destroy(h);
  cudaFree(b->d_insts);
  cudaFree(b->d_maps);
  cudaFree(b->d_ctrls);
  cudaFree(b->d_gs);
  cudaFree(b->d_plist[0]);
  cudaFree(b->d_plist[1]);
  for (int D = 0; D < 3; D++)
    for (int o = 0; o < 2; o++)
      for (int sh = 0; sh < 3; sh++) cudaFree(b->d_items[D][o][sh]);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

}  // extern "C"

// sweep_line2.cu - instances and launchers of the warp-marching fused sweep
// of 2-D grids (mixed precision), single grids and batches.
#include <cstdlib>
#include <string>

#include "batch_items.cuh"
#include "physics_mixed.cuh"
#include "sweep.cuh"
#include "sweep_line2.cuh"

namespace vacgpu {

bool pair_enabled();
bool pair_general(const FusedArgs& a, bool mhd);

// One work item per warp: item = strip + nstrips * chunk.
// register bound: four CTAs per SM for HD (128 registers), two for MHD
template <int D, bool MHD, int LIMC, bool GEN>
__global__ void __launch_bounds__(L2_NT, MHD ? 2 : 4)
    k_sweep_line2(const FusedArgs a, const float* __restrict__ win, int nstrips, int nitems) {
  const int item = blockIdx.x * (L2_NT / 32) + (threadIdx.x >> 5);
  if (item >= nitems) return;
  constexpr int RF = line2_ring_floats(MHD ? 6 : 4);
  __shared__ __align__(16) float ring[L2_NT / 32][RF];
  const int sx = item % nstrips, ch = item / nstrips;
  const int gya = 2 + ch * L2_ROWS, gyb = min(gya + L2_ROWS, a.g.nx[1] + 2);
  Line2<D, MHD, LIMC, GEN>::run(a, win, a.wout, ring[threadIdx.x >> 5], sx, gya, gyb,
                                (unsigned)item);
}

// Batched grids: each warp takes items gw, gw + W, ... of the work list
// (W warps in the launch); an item is (grid, strip bx, output rows by ..
// bz-1 in ghost-range indices).
// (register bound: the work-list loop of the general y sweep needs more than
// 128 registers, so it runs three CTAs per SM rather than spill)
template <int D, bool MHD, int LIMC, bool GEN>
__global__ void __launch_bounds__(L2_NT, MHD ? 2 : (D == 1 && GEN ? 3 : 4))
    kb_sweep_line2(const BItem* __restrict__ items, int nitems, const BInst* __restrict__ insts,
                   int sweep) {
  constexpr int RF = line2_ring_floats(MHD ? 6 : 4);
  __shared__ __align__(16) float ring[L2_NT / 32][RF];
  const int nwarps = gridDim.x * (L2_NT / 32);
  for (int it = blockIdx.x * (L2_NT / 32) + (threadIdx.x >> 5); it < nitems; it += nwarps) {
    const BItem item = items[it];
    const BInst* in = insts + item.inst;
    const int src = in->fa.ctrl->cur ^ (sweep & 1);
    Line2<D, MHD, LIMC, GEN>::run(in->fa, in->buf[src], in->buf[src ^ 1],
                                  ring[threadIdx.x >> 5], item.bx & L2_STRIP, item.by,
                                  item.bz, (unsigned)it);
  }
}

// The warp-marching sweep applies to a 2-D grid with one limiter for every
// variable (minmod or woodward), rows that start 2 elements before a
// 16-byte boundary and fewer than 2^31 elements in the state; also false
// when
// VACGPU_PAIR=0 (the one-cell kernels for every grid).
bool line2_applies(const FusedArgs& a, bool mhd) {
  if (!pair_enabled()) return false;
  const int nw = mhd ? 6 : 4;
  const int l0 = a.ph.lim[0];
  bool uniform = a.ph.typefull != VACGPU_TVDLF1;
  for (int v = 1; v < nw; v++) uniform = uniform && a.ph.lim[v] == l0;
  if (!uniform || (l0 != VACGPU_LIM_WOODWARD && l0 != VACGPU_LIM_MINMOD)) return false;
  // the kernel indexes variables with 32-bit element offsets and stages
  // rows in 16-byte chunks from 4-column boundaries (mesh column 0 on one)
  return a.g.ndim == 2 && (a.g.xpad + 2) % 4 == 0 && a.g.P % 4 == 0 &&
         a.g.vs * nw < (1LL << 31);
}

// single-grid work items: strips x chunks of L2_ROWS rows
static int line2_items(int D, bool mhd, const DevGrid& g, int* nstrips) {
  *nstrips = line2_strips(D, mhd, g.nx[0]);
  return *nstrips * ((g.nx[1] + L2_ROWS - 1) / L2_ROWS);
}

template <int D, bool MHD, int LIMC, bool GEN>
static void launch_l2(const FusedArgs& a, const float* win, cudaStream_t st) {
  int ns;
  const int n = line2_items(D, MHD, a.g, &ns);
  const int per = L2_NT / 32;
  k_sweep_line2<D, MHD, LIMC, GEN><<<(n + per - 1) / per, L2_NT, 0, st>>>(a, win, ns, n);
}

bool launch_sweep_line2(const FusedArgs& a, const float* win, int D, bool mhd,
                        cudaStream_t st) {
  if (!line2_applies(a, mhd)) return false;
  const bool gen = pair_general(a, mhd);
  const int l0 = a.ph.lim[0];
#define L2G(DD, M, L)                                                        \
  {                                                                          \
    if (gen)                                                                 \
      launch_l2<DD, M, L, true>(a, win, st);                                 \
    else                                                                     \
      launch_l2<DD, M, L, false>(a, win, st);                                \
    return true;                                                             \
  }
#define L2D(DD)                                                              \
  if (D == DD) {                                                             \
    if (mhd) {                                                               \
      if (l0 == VACGPU_LIM_WOODWARD) L2G(DD, true, LIMC_WOODWARD)            \
      else L2G(DD, true, LIMC_MINMOD)                                        \
    } else {                                                                 \
      if (l0 == VACGPU_LIM_WOODWARD) L2G(DD, false, LIMC_WOODWARD)           \
      else L2G(DD, false, LIMC_MINMOD)                                       \
    }                                                                        \
  }
  L2D(0) L2D(1)
#undef L2D
#undef L2G
  return false;
}

template <int D, bool MHD, int LIMC, bool GEN>
static void launch_kb_l2(const BItem* items, int nitems, const BInst* insts, int sweep,
                         int ctas, cudaStream_t st) {
  kb_sweep_line2<D, MHD, LIMC, GEN><<<ctas, L2_NT, 0, st>>>(items, nitems, insts, sweep);
}

bool launch_batch_line2(const BItem* items, int nitems, const BInst* insts, int sweep, int D,
                        bool mhd, int lim, bool gen, int ctas, cudaStream_t st) {
  const int per = L2_NT / 32;
  if (ctas <= 0 || ctas * per > nitems) ctas = (nitems + per - 1) / per;
#define KL(DD, M, L)                                                         \
  {                                                                          \
    if (gen)                                                                 \
      launch_kb_l2<DD, M, L, true>(items, nitems, insts, sweep, ctas, st);   \
    else                                                                     \
      launch_kb_l2<DD, M, L, false>(items, nitems, insts, sweep, ctas, st);  \
    return true;                                                             \
  }
#define KLD(DD)                                                              \
  if (D == DD) {                                                             \
    if (mhd) {                                                               \
      if (lim == VACGPU_LIM_WOODWARD) KL(DD, true, LIMC_WOODWARD)            \
      else KL(DD, true, LIMC_MINMOD)                                         \
    } else {                                                                 \
      if (lim == VACGPU_LIM_WOODWARD) KL(DD, false, LIMC_WOODWARD)           \
      else KL(DD, false, LIMC_MINMOD)                                        \
    }                                                                        \
  }
  KLD(0) KLD(1)
#undef KLD
#undef KL
  return false;
}

}  // namespace vacgpu

// ------------------------------------------------- one launch, many steps

namespace vacgpu {

// Grid-wide barrier of a cooperative launch (every CTA resident): the last
// CTA to arrive resets the count and advances the generation; the others
// wait for the generation to move, at most `limit` cycles (about a second
// by default), after which the barrier reports failure and sets the fault
// flag.  Writes before the barrier are visible after it (CTA barrier, then
// a device-scope fence by the arriving thread, and a fence after the wait).
__device__ __forceinline__ bool grid_sync(GridSync* gs, unsigned nb,
                                          long long limit = 1LL << 31) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    volatile unsigned* vgen = &gs->gen;
    const unsigned g = *vgen;
    __threadfence();
    if (atomicAdd(&gs->count, 1u) == nb - 1) {
      atomicExch(&gs->count, 0u);
      __threadfence();
      atomicAdd(&gs->gen, 1u);
    } else {
      const long long t0 = clock64();
      while (*vgen == g) {
        if (clock64() - t0 > limit) {
          atomicExch(&gs->fault, 1);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    if (*(volatile int*)&gs->fault) ok = 0;
  }
  __syncthreads();
  return ok != 0;
}

// Every step of a batch of 2-D grids (the body of VAC's time loop for each
// grid, as issue_step issues it with separate launches): CTA b runs the
// control of grids b, b + gridDim.x, ...; the sweeps' warps take the work
// items in turn.  A step takes three grid-wide barriers: the owner of a
// grid chooses its dt right after the previous step's end (dt_begin, and
// dt_end unless the grid needs the first-step passes, which then run
// between barriers of their own), then the two sweeps.  Control fields
// written on one SM are read on others through L2 (the control functions,
// Line2::run and the first-step passes use ld.global.cg), and the rows of
// the state arrive by cp.async.cg, so no stale L1 line from an earlier step
// is read.  (HD: four CTAs per SM at 128 registers; on 64 uneven HD grids
// that ran about 3 % faster than three CTAs per SM.)
template <bool MHD, int LIMC, bool GEN>
__global__ void __launch_bounds__(L2_NT, MHD ? 2 : 4) kb_steps_line2(const Line2Steps ls) {
  constexpr int RF = line2_ring_floats(MHD ? 6 : 4);
  __shared__ __align__(16) float ring[L2_NT / 32][RF];
  __shared__ int defer;
  typedef Sweep<PHMixed<PREC_FF>, 2, 2, MHD> SW;
  const unsigned nb = gridDim.x;
  const int tid = threadIdx.x, warp = tid >> 5;
  GridSync* gs = ls.gs;
  // the next work item of a sweep, for the whole warp
  auto claim = [&](int* ctr) {
    int t = 0;
    if ((tid & 31) == 0) t = atomicAdd(ctr, 1);
    return __shfl_sync(0xffffffffu, t, 0);
  };
  // the dt choice of step s for grid g: dt_begin, then dt_end unless the
  // grid needs the first-step passes (flagged for the whole launch)
  auto choose_dt = [&](Ctrl* c, int s) {
    dt_begin_dev(c, 2);
    if (tid == 0) {
      defer = !c->done && (c->need_smallp | c->need_cell[0] | c->need_cell[1]);
      if (defer) atomicOr(&gs->need[s & 1], 1);
    }
    __syncthreads();
    if (!defer) dt_end_dev(c, ls.dte);
    __syncthreads();
  };
  // (the host clears *gs, need flags included, before the launch)
  for (int g = blockIdx.x; g < ls.n; g += nb) {  // call_begin, then step 0's dt
    Ctrl* c = ls.ctrls[g];
    if (tid == 0) {
      c->done = 0;
      c->steps = 0;
      c->maxsteps = ls.nsteps;
      c->tstop = ls.tstop;
    }
    __syncthreads();
    if (ls.nsteps > 0) choose_dt(c, 0);
  }
  for (int s = 0; s < ls.nsteps; s++) {
    const int par = (ls.par0 + s) & 1;
    if (!grid_sync(gs, nb)) return;
    // every CTA read need[(s+1)&1] in step s-1, before this barrier
    if (blockIdx.x == 0 && tid == 0) gs->need[(s + 1) & 1] = 0;
    if (__ldcg(&gs->need[s & 1])) {
      // the first-step passes: nparts parts of each grid's cells
      const int np = ls.nparts;
      for (int u = blockIdx.x; u < np * ls.n; u += nb) {
        const BInst* in = ls.insts + u / np;
        SW::template pminmax<L2_NT>(in->sa, in->buf[__ldcg(&in->sa.ctrl->cur)], u % np, np);
      }
      if (!grid_sync(gs, nb)) return;
      for (int g = blockIdx.x; g < ls.n; g += nb) smallp_dev(ls.ctrls[g], MHD, ls.smallpcoeff);
      if (!grid_sync(gs, nb)) return;
      for (int u = blockIdx.x; u < np * ls.n; u += nb) {
        const BInst* in = ls.insts + u / np;
        SW::template cell_cmax<L2_NT>(in->sa, in->buf[__ldcg(&in->sa.ctrl->cur)], u % np, np);
      }
      if (!grid_sync(gs, nb)) return;
      for (int g = blockIdx.x; g < ls.n; g += nb) {
        Ctrl* c = ls.ctrls[g];
        if (!c->done && (c->need_cell[0] | c->need_cell[1])) dt_end_dev(c, ls.dte);
      }
      if (!grid_sync(gs, nb)) return;
    }
    for (int sw = 0; sw < 2; sw++) {
      // the list of this sweep (each item carries its own direction: the
      // lists of a call on grids at different parities of it mix both)
      const BItem* items = ls.items[(!par || ls.xy) ? sw : 1 - sw];
      const int nit = ls.nitems[(!par || ls.xy) ? sw : 1 - sw];
      // items claimed one at a time (the next claim in flight while an item
      // runs); next[sw] is cleared for the following step once every warp
      // is past this sweep's barrier
      int it = claim(&gs->next[sw]);
      while (it < nit) {
        const int nx = claim(&gs->next[sw]);
        const BItem item = items[it];
        const BInst* in = ls.insts + item.inst;
        const int src = __ldcg(&in->fa.ctrl->cur) ^ (sw & 1);
        if (!(item.bx >> 30))
          Line2<0, MHD, LIMC, GEN>::run(in->fa, in->buf[src], in->buf[src ^ 1], ring[warp],
                                        item.bx & L2_STRIP, item.by, item.bz, (unsigned)it);
        else
          Line2<1, MHD, LIMC, GEN>::run(in->fa, in->buf[src], in->buf[src ^ 1], ring[warp],
                                        item.bx & L2_STRIP, item.by, item.bz, (unsigned)it);
        it = nx;
      }
      if (!grid_sync(gs, nb)) return;
      if (blockIdx.x == 0 && tid == 0) gs->next[sw] = 0;
    }
    for (int g = blockIdx.x; g < ls.n; g += nb) {
      Ctrl* c = ls.ctrls[g];
      step_end_dev(c, 2, 0);
      __syncthreads();
      if (s + 1 < ls.nsteps) choose_dt(c, s + 1);
    }
  }
}

template <bool MHD, int LIMC, bool GEN>
static int steps_ctas() {
  static int ctas = 0;
  if (!ctas) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kb_steps_line2<MHD, LIMC, GEN>, L2_NT,
                                                  0);
    ctas = sms * per;
  }
  return ctas;
}

template <bool MHD, int LIMC, bool GEN>
static bool launch_steps(const Line2Steps& ls, int ctas, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(L2_NT);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kb_steps_line2<MHD, LIMC, GEN>, ls) == cudaSuccess;
}

#define L2S_DISPATCH(F, ...)                                                  \
  if (mhd) {                                                                  \
    if (lim == VACGPU_LIM_WOODWARD)                                           \
      return gen ? F<true, LIMC_WOODWARD, true>(__VA_ARGS__)                  \
                 : F<true, LIMC_WOODWARD, false>(__VA_ARGS__);                \
    return gen ? F<true, LIMC_MINMOD, true>(__VA_ARGS__)                      \
               : F<true, LIMC_MINMOD, false>(__VA_ARGS__);                    \
  }                                                                           \
  if (lim == VACGPU_LIM_WOODWARD)                                             \
    return gen ? F<false, LIMC_WOODWARD, true>(__VA_ARGS__)                   \
               : F<false, LIMC_WOODWARD, false>(__VA_ARGS__);                 \
  return gen ? F<false, LIMC_MINMOD, true>(__VA_ARGS__)                       \
             : F<false, LIMC_MINMOD, false>(__VA_ARGS__);

int line2_steps_ctas(bool mhd, int lim, bool gen) { L2S_DISPATCH(steps_ctas) }

bool launch_line2_steps(const Line2Steps& ls, bool mhd, int lim, bool gen, int ctas,
                        cudaStream_t st) {
  L2S_DISPATCH(launch_steps, ls, ctas, st)
}
#undef L2S_DISPATCH

// ------------------------------------------ bounded waits, run out on purpose

// An mbarrier phase that nothing completes (no arrival, no copy): the
// bounded wait of the TMA-fed sweeps gives up after `limit` cycles.
__global__ void k_wait_mbar_out(int* out, long long limit) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    out[0] = mbar_wait(&bar, 0, limit) ? 0 : 1;
  }
}

// A grid-wide barrier that CTA 1 never reaches: CTA 0's wait gives up after
// `limit` cycles and sets the fault flag.
__global__ void k_wait_grid_out(GridSync* gs, int* out, long long limit) {
  if (blockIdx.x != 0) return;
  const bool ok = grid_sync(gs, gridDim.x, limit);
  if (threadIdx.x == 0) out[1] = (!ok && gs->fault) ? 1 : 0;
}

}  // namespace vacgpu

int vacgpu_internal_fail(const char* msg);

extern "C" int vacgpu_test_bounded_waits(int* mbar_timed_out, int* grid_timed_out) {
  using namespace vacgpu;
  int* d = nullptr;
  GridSync* gs = nullptr;
  int h[2] = {0, 0};
  cudaError_t e = cudaMalloc(&d, 2 * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&gs, sizeof(GridSync));
  if (e == cudaSuccess) e = cudaMemset(d, 0, 2 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(gs, 0, sizeof(GridSync));
  const long long limit = 1LL << 22;  // about 2 ms
  if (e == cudaSuccess) {
    k_wait_mbar_out<<<1, 32>>>(d, limit);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.gridDim = dim3(2);
    cfg.blockDim = dim3(32);
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, k_wait_grid_out, gs, d, limit);
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  cudaFree(gs);
  if (e != cudaSuccess) {
    std::string m = std::string("bounded-wait test: ") + cudaGetErrorString(e);
    return vacgpu_internal_fail(m.c_str());
  }
  if (mbar_timed_out) *mbar_timed_out = h[0];
  if (grid_timed_out) *grid_timed_out = h[1];
  return 0;
}

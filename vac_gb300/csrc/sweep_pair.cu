// sweep_pair.cu - instances and launcher of the two-cells-per-thread fused
// sweep of 3-D grids (mixed precision).
#include <cstdlib>
#include <cstring>

#include "batch_items.cuh"
#include "sweep_pair.cuh"

namespace vacgpu {

template <int D, bool MHD, int LIMC, bool GEN>
static void launch_pair_one(const CUtensorMap* map, const FusedArgs& a, dim3 grid,
                            cudaStream_t st) {
  constexpr int NW = MHD ? 8 : 5;
  const int smem = pair_smem_floats(NW) * 4;
  auto k = k_sweep_pair<D, MHD, LIMC, GEN>;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr = true;
  }
  k<<<grid, PT_NT, smem, st>>>(*map, a);
}

// The grid needs the general form of the pair sweep (PairSweep's GEN):
// gravity, a non-periodic face, split sources, no Powell terms for MHD, or
// no CFL maximum.
bool pair_general(const FusedArgs& a, bool mhd) {
  const int all = (1 << (mhd ? 8 : 5)) - 1;
  bool gen = a.ph.src_id != VACGPU_SRC_NONE || !a.ph.sourceunsplit || !a.cfl ||
             (mhd && !a.ph.divbfix);
  for (int d = 0; d < 3; d++) gen = gen || a.periodic_mask[d] != all;
  return gen;
}

template <int D, bool MHD, int LIMC>
static void launch_pair_gen(const CUtensorMap* map, const FusedArgs& a, dim3 grid,
                           cudaStream_t st) {
  if (pair_general(a, MHD))
    launch_pair_one<D, MHD, LIMC, true>(map, a, grid, st);
  else
    launch_pair_one<D, MHD, LIMC, false>(map, a, grid, st);
}

// VACGPU_PAIR=0 keeps the one-cell kernel for every grid (read once)
bool pair_enabled() {
  static const bool on = [] {
    const char* e = getenv("VACGPU_PAIR");
    return !(e && atoi(e) == 0);
  }();
  return on;
}

// The pair sweep runs 3-D sweeps with one limiter for every variable
// (minmod or woodward).
bool pair_applies(const FusedArgs& a, bool mhd) {
  if (!pair_enabled()) return false;
  const int nw = mhd ? 8 : 5;
  const int l0 = a.ph.lim[0];
  bool uniform = a.ph.typefull != VACGPU_TVDLF1;
  for (int v = 1; v < nw; v++) uniform = uniform && a.ph.lim[v] == l0;
  if (!uniform || (l0 != VACGPU_LIM_WOODWARD && l0 != VACGPU_LIM_MINMOD)) return false;
  // the pairs' 8-byte shared and global accesses need an even first column
  // (state rows start at xpad, a multiple of 32 minus 2 for FP32 states)
  return a.g.ndim == 3 && !(a.g.xpad & 1) && !(a.g.P & 1);
}

// False: not applicable, use the one-cell kernel.
bool launch_sweep_pair(const FusedArgs& a, int D, bool mhd, const void* tmap, int nzc,
                       cudaStream_t st) {
  if (!pair_applies(a, mhd)) return false;
  const int l0 = a.ph.lim[0];
  const int tx = D == 0 ? 30 : 32;
  const int ar = D == 1 ? 2 : 1, am = D == 0 ? 2 : D;
  const int nxt = D == 0 ? (a.g.nx[0] + 1 + tx - 1) / tx : (a.g.nx[0] + tx - 1) / tx;
  dim3 grid(nxt, (a.g.nx[ar] + 7) / 8, (a.g.nx[am] + nzc - 1) / nzc);
  const CUtensorMap* map = (const CUtensorMap*)tmap;
#define LP(DD, M, L) launch_pair_gen<DD, M, L>(map, a, grid, st)
#define LPD(DD)                                                              \
  if (D == DD) {                                                             \
    if (mhd) {                                                               \
      if (l0 == VACGPU_LIM_WOODWARD) LP(DD, true, LIMC_WOODWARD);            \
      else LP(DD, true, LIMC_MINMOD);                                        \
    } else {                                                                 \
      if (l0 == VACGPU_LIM_WOODWARD) LP(DD, false, LIMC_WOODWARD);           \
      else LP(DD, false, LIMC_MINMOD);                                       \
    }                                                                        \
    return true;                                                             \
  }
  LPD(0) LPD(1) LPD(2)
#undef LPD
#undef LP
  return false;
}

// ------------------------------------------------------- batched grids

// The pair sweep over a batch work list: each CTA takes items
// blockIdx.x, blockIdx.x + gridDim.x, ... in turn, with the item's grid
// arguments copied to shared memory; the TMA barriers' phases carry over
// from item to item.
template <int D, bool MHD, int LIMC, bool GEN>
__global__ void __launch_bounds__(PT_NT, 3)
    kb_sweep_pair(const BItem* __restrict__ items, int nitems,
                  const BInst* __restrict__ insts, const CUtensorMap* maps, int sweep) {
  extern __shared__ __align__(128) float dsm[];
  __shared__ __align__(8) unsigned long long bars[FWRING];
  __shared__ __align__(16) FusedArgs fa;
  __shared__ int mapidx;
  init_bars(bars);
  int uses[FWRING] = {0, 0, 0, 0};
  for (int it = blockIdx.x; it < nitems; it += gridDim.x) {
    const BItem item = items[it];
    const BInst* in = insts + item.inst;
    {
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
    const bool ok = PairSweep<D, MHD, LIMC, GEN>::run(&maps[mapidx], fa, dsm, item.bx, item.by,
                                                     item.bz, bars, uses, (unsigned)it);
    __syncthreads();
    if (!ok) return;
  }
}

template <int D, bool MHD, int LIMC, bool GEN>
static void launch_kb_pair(const BItem* items, int nitems, const BInst* insts,
                           const CUtensorMap* maps, int sweep, int ctas, cudaStream_t st) {
  constexpr int NW = MHD ? 8 : 5;
  const int smem = pair_smem_floats(NW) * 4;
  auto k = kb_sweep_pair<D, MHD, LIMC, GEN>;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr = true;
  }
  k<<<ctas, PT_NT, smem, st>>>(items, nitems, insts, maps, sweep);
}

bool launch_batch_pair(const BItem* items, int nitems, const BInst* insts,
                       const CUtensorMap* maps, int sweep, int D, bool mhd, int lim,
                       bool gen, int ctas, cudaStream_t st) {
  if (ctas <= 0 || ctas > nitems) ctas = nitems;
#define KP(DD, M, L)                                                          \
  {                                                                           \
    if (gen)                                                                  \
      launch_kb_pair<DD, M, L, true>(items, nitems, insts, maps, sweep, ctas, st); \
    else                                                                      \
      launch_kb_pair<DD, M, L, false>(items, nitems, insts, maps, sweep, ctas, st); \
    return true;                                                              \
  }
#define KPD(DD)                                                               \
  if (D == DD) {                                                              \
    if (mhd) {                                                                \
      if (lim == VACGPU_LIM_WOODWARD) KP(DD, true, LIMC_WOODWARD)             \
      else KP(DD, true, LIMC_MINMOD)                                          \
    } else {                                                                  \
      if (lim == VACGPU_LIM_WOODWARD) KP(DD, false, LIMC_WOODWARD)            \
      else KP(DD, false, LIMC_MINMOD)                                         \
    }                                                                         \
  }
  KPD(0) KPD(1) KPD(2)
#undef KPD
#undef KP
  return false;
}

}  // namespace vacgpu

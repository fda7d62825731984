// sweep_line2.cu - instances and launchers of the warp-marching fused sweep
// of 2-D grids (mixed precision), single grids and batches.
#include <cstdlib>

#include "batch_items.cuh"
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
                                  ring[threadIdx.x >> 5], item.bx, item.by, item.bz,
                                  (unsigned)it);
  }
}

// The warp-marching sweep applies to a 2-D grid with one limiter for every
// variable (minmod or woodward), even row offsets and fewer than 2^31
// elements in the state; also false when
// VACGPU_PAIR=0 (the one-cell kernels for every grid).
bool line2_applies(const FusedArgs& a, bool mhd) {
  if (!pair_enabled()) return false;
  const int nw = mhd ? 6 : 4;
  const int l0 = a.ph.lim[0];
  bool uniform = a.ph.typefull != VACGPU_TVDLF1;
  for (int v = 1; v < nw; v++) uniform = uniform && a.ph.lim[v] == l0;
  if (!uniform || (l0 != VACGPU_LIM_WOODWARD && l0 != VACGPU_LIM_MINMOD)) return false;
  // the kernel indexes variables with 32-bit element offsets
  return a.g.ndim == 2 && !(a.g.xpad & 1) && !(a.g.P & 1) &&
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

// sweep_pair.cu - instances and launcher of the two-cells-per-thread fused
// sweep of 3-D grids (mixed precision).
#include <cstdlib>
#include <cstring>

#include "sweep_pair.cuh"

namespace vacgpu {

template <int D, bool MHD, int LIMC, int TS>
static void launch_pair_one(const CUtensorMap* map, const FusedArgs& a, dim3 grid,
                            cudaStream_t st) {
  constexpr int NW = MHD ? 8 : 5;
  const int smem = pair_smem_floats(NW) * 4;
  auto k = k_sweep_pair<D, MHD, LIMC, TS>;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr = true;
  }
  k<<<grid, PT_NT, smem, st>>>(*map, a);
}

// Error-free sum of the pressure recovery: VACGPU_PAIR_TWOSUM=knuth selects
// Knuth's branch-free TwoSum instead of Fast2Sum on the ordered pair.
static int pair_twosum() {
  static const int t = [] {
    const char* e = getenv("VACGPU_PAIR_TWOSUM");
    return e && !strcmp(e, "knuth") ? 1 : 0;
  }();
  return t;
}

template <int D, bool MHD, int LIMC>
static void launch_pair_ts(const CUtensorMap* map, const FusedArgs& a, dim3 grid,
                           cudaStream_t st) {
  if (pair_twosum())
    launch_pair_one<D, MHD, LIMC, 1>(map, a, grid, st);
  else
    launch_pair_one<D, MHD, LIMC, 0>(map, a, grid, st);
}

// The pair sweep runs 3-D sweeps with one limiter for every variable
// (minmod or woodward); false: not applicable, use the one-cell kernel.
bool launch_sweep_pair(const FusedArgs& a, int D, bool mhd, const void* tmap, int nzc,
                       cudaStream_t st) {
  const int nw = mhd ? 8 : 5;
  const int l0 = a.ph.lim[0];
  bool uniform = a.ph.typefull != VACGPU_TVDLF1;
  for (int v = 1; v < nw; v++) uniform = uniform && a.ph.lim[v] == l0;
  if (!uniform || (l0 != VACGPU_LIM_WOODWARD && l0 != VACGPU_LIM_MINMOD)) return false;
  // the pairs' 8-byte shared and global accesses need an even first column
  // (state rows start at xpad, a multiple of 32 minus 2 for FP32 states)
  if (a.g.ndim != 3 || (a.g.xpad & 1) || (a.g.P & 1)) return false;
  const int tx = D == 0 ? 30 : 32;
  const int ar = D == 1 ? 2 : 1, am = D == 0 ? 2 : D;
  const int nxt = D == 0 ? (a.g.nx[0] + 1 + tx - 1) / tx : (a.g.nx[0] + tx - 1) / tx;
  dim3 grid(nxt, (a.g.nx[ar] + 7) / 8, (a.g.nx[am] + nzc - 1) / nzc);
  const CUtensorMap* map = (const CUtensorMap*)tmap;
#define LP(DD, M, L) launch_pair_ts<DD, M, L>(map, a, grid, st)
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

}  // namespace vacgpu

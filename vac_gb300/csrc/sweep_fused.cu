// sweep_fused.cu - instances and launcher of the fused mixed-precision sweep.
#include <cstdlib>
#include <cstring>

#include "sweep_fused.cuh"

namespace vacgpu {

int fused_smem_bytes(int nw, int k) { return fused_smem_floats(nw, k) * 4; }

bool launch_sweep_pair(const FusedArgs& a, int D, bool mhd, const void* tmap, int nzc,
                       cudaStream_t st);
bool launch_sweep_line2(const FusedArgs& a, const float* win, int D, bool mhd,
                        cudaStream_t st);

template <int NDIM, int D, bool MHD, int LIMC, int PMF>
static void launch_pmf(const CUtensorMap* map, const FusedArgs& a, dim3 grid,
                       cudaStream_t st) {
  constexpr int NW = MHD ? 2 + 2 * NDIM : 2 + NDIM;
  const int smem = fused_smem_floats(NW, fused_kind(NDIM, D)) * 4;
  auto k = k_sweep_fused<NDIM, D, MHD, PREC_FF, LIMC, PMF>;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    attr = true;
  }
  k<<<grid, FT_NT, smem, st>>>(*map, a);
}

// VACGPU_FLUX_PRESSURE=f32: FP32 pressure recovery in the fluxes (the wave
// speeds keep the double-float recovery).  Read once per process.
static bool flux_pressure_f32() {
  static const bool f = [] {
    const char* e = getenv("VACGPU_FLUX_PRESSURE");
    return e && !strcmp(e, "f32");
  }();
  return f;
}

template <int NDIM, int D, bool MHD, int LIMC>
static void launch_lim(const CUtensorMap* map, const FusedArgs& a, dim3 grid,
                       cudaStream_t st) {
  if (flux_pressure_f32())
    launch_pmf<NDIM, D, MHD, LIMC, PREC_F32>(map, a, grid, st);
  else
    launch_pmf<NDIM, D, MHD, LIMC, PREC_FF>(map, a, grid, st);
}

template <int NDIM, int D, bool MHD>
static void launch_one(const CUtensorMap* map, const FusedArgs& a, dim3 grid,
                       cudaStream_t st) {
  constexpr int NW = MHD ? 2 + 2 * NDIM : 2 + NDIM;
  int l0 = a.ph.lim[0];
  bool uniform = a.ph.typefull != VACGPU_TVDLF1;
  for (int v = 1; v < NW; v++) uniform = uniform && a.ph.lim[v] == l0;
  if (uniform && l0 == VACGPU_LIM_WOODWARD)
    launch_lim<NDIM, D, MHD, LIMC_WOODWARD>(map, a, grid, st);
  else if (uniform && l0 == VACGPU_LIM_MINMOD)
    launch_lim<NDIM, D, MHD, LIMC_MINMOD>(map, a, grid, st);
  else
    launch_lim<NDIM, D, MHD, LIMC_RUNTIME>(map, a, grid, st);
}

bool launch_sweep_fused(const SweepArgs& s, const void* tmap, const float* win, float* wout,
                        const float* const* idxf, int nzc, cudaStream_t st) {
  const int nd = s.g.ndim;
  if (s.d0 != s.d1 || s.ndir != nd || (nd != 2 && nd != 3)) return false;
  for (int d = 0; d < nd; d++)
    if (s.ph.gmap[d][0] == GMAP_MIXED || s.ph.gmap[d][1] == GMAP_MIXED)
      return false;
  FusedArgs a;
  memset(&a, 0, sizeof(a));
  a.g = s.g;
  a.ph = s.ph;
  for (int d = 0; d < 3; d++) {
    a.dxf[d] = s.a.dxf[d];
    a.idxf[d] = idxf[d];
  }
  a.ctrl = s.ctrl;
  a.wout = wout;
  a.nzc = nzc;
  for (int d = 0; d < 3; d++) a.gravf[d] = (float)s.ph.src_par[d];
  a.cfl = s.ph.courantpar > 0.0;
  const int nw = s.mhd ? 2 + 2 * s.ndir : 2 + s.ndir;
  for (int d = 0; d < 3; d++)
    for (int v = 0; v < nw; v++) {
      if (s.ph.typeB[2 * d][v] == VACGPU_BC_PERIODIC) a.periodic_mask[d] |= 1 << v;
      if (s.ph.typeB[2 * d][v] == VACGPU_BC_ASYMM) a.asymm_lo[d] |= 1 << v;
      if (s.ph.typeB[2 * d + 1][v] == VACGPU_BC_ASYMM) a.asymm_hi[d] |= 1 << v;
    }
  // tiles over x and the row axis, z chunks along the marching axis
  const int kind = fused_kind(nd, s.d0);
  const int tx = kind == 0 ? TileCfg<0>::TX : TileCfg<1>::TX;
  const int ty = kind == 1 ? TileCfg<1>::TY : TileCfg<0>::TY;
  const int ar = kind == 2 && s.d0 == 1 ? 2 : 1;
  const int am = kind == 2 ? s.d0 : 2;
  dim3 grid((s.g.nx[0] + tx - 1) / tx, (s.g.nx[ar] + ty - 1) / ty,
            nd == 3 ? (s.g.nx[am] + nzc - 1) / nzc : 1);
  a.zchunks = grid.z;
  // 3-D grids: the two-cells-per-thread kernel (packed FP32) where it
  // applies; VACGPU_PAIR=0 keeps the one-cell kernel
  if (nd == 3 && launch_sweep_pair(a, s.d0, s.mhd, tmap, nzc, st))
    return true;
  // 2-D grids: the warp-marching two-cells-per-thread kernel where it applies
  if (nd == 2 && launch_sweep_line2(a, win, s.d0, s.mhd, st)) return true;
  const CUtensorMap* map = (const CUtensorMap*)tmap;
  const int D = s.d0;
#define L1(ND, DD)                                              \
  if (nd == ND && D == DD) {                                    \
    if (s.mhd)                                                  \
      launch_one<ND, DD, true>(map, a, grid, st);               \
    else                                                        \
      launch_one<ND, DD, false>(map, a, grid, st);              \
    return true;                                                \
  }
  L1(2, 0) L1(2, 1) L1(3, 0) L1(3, 1) L1(3, 2)
#undef L1
  return false;
}

}  // namespace vacgpu

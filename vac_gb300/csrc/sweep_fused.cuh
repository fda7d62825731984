// sweep_fused.cuh - one split sweep of VAC's twostep Hancock/TVDLF scheme
// (src/vac.t:363-572, src/vactvdlf.t:5-299) as a single kernel for the
// mixed-precision path.
//
// A CTA of 256 threads owns a column tile of the mesh and marches along z
// through a chunk of planes.  Each plane of the state (tile + 2-cell halo,
// all variables) arrives in shared memory with one TMA tensor copy
// (cp.async.bulk.tensor, mbarrier completion), two planes ahead of use.  The
// Hancock predictor w1 is evaluated for the tile + 1-cell halo into shared
// memory (never written to HBM), every face flux of the TVDLF corrector is
// computed once, and the corrected plane goes straight to HBM: HBM traffic
// per sweep is one read and one write of the state plus halo re-reads that
// mostly hit L2.
//
// Geometry kinds: K=0 (x sweep) and K=1 (y sweep of 2-D grids) keep the
// sweep direction inside the tile plane and march along z; K=2 marches along
// the sweep direction itself (z sweep, and y sweep of 3-D grids with tile
// rows along z), so its faces are evaluated in registers plane by plane.
// The tile shape depends on the kind so that each phase is one work item
// per thread: the predictor is needed in full on (TX+2) x TY cells for K=0,
// TX x (TY+2) for K=1 and TX x TY for K=2 -- 256 cells each with 30x8, 32x6
// and 32x8 tiles -- and the in-plane faces number at most 256.  The
// remaining halo cells feed only the div B of the Powell source, so there
// only the transverse B component is predicted.  With
// typelimited='original' the corrector limits the same state w that the
// predictor limits (src/vactvdlf.t:150-157), so the predictor's limited
// slopes are kept in shared memory and reused by the faces.
//
// Ghost semantics follow getboundary applied to w1 after the predictor
// (src/vac.t:567): at a 'periodic' face the predictor is evaluated at the
// ghost position from the (periodic copy) ghost values of w; at 'cont',
// 'symm' and 'asymm' faces w1 in the first ghost layer is the adjacent mesh
// value (sign-flipped for 'asymm').
#pragma once
#include <cuda.h>

#include "physics_mixed.cuh"
#include "vacgpu_internal.h"

namespace vacgpu {

constexpr int FT_NT = 256;  // threads per CTA
constexpr int FB_X = 40;    // TMA box width
constexpr int FWRING = 4;   // state planes resident (j-1, j, j+1, j+2)

// geometry kind of the sweep in direction d of an ndim-D grid
__host__ __device__ constexpr int fused_kind(int ndim, int d) {
  return ndim == 3 && d >= 1 ? 2 : d;
}

template <int K>
struct TileCfg {
  static constexpr int TX = K == 0 ? 30 : 32;   // output tile
  static constexpr int TY = K == 1 ? 6 : 8;
  static constexpr int RX = TX + 2, RY = TY + 2;  // predictor region
  static constexpr int RN = RX * RY;
  static constexpr int BY = TY + 4;              // TMA box rows
  static constexpr int BPL = FB_X * BY;          // floats / variable / plane
  static constexpr int NF = K == 0 ? (TX + 1) * TY : K == 1 ? TX * (TY + 1) : 0;
  static constexpr int NOUT = TX * TY;
  // halo cells where only a transverse B component is predicted
  static constexpr int NB = K == 0 ? 2 * TX : K == 1 ? 2 * TY : 2 * TX + 2 * TY;
};

// floats of one state-plane slot (multiple of 32: 128-byte aligned slots)
__host__ __device__ constexpr int fused_slot_floats(int nw, int K) {
  return (nw * FB_X * (K == 1 ? TileCfg<1>::BY : TileCfg<0>::BY) + 31) / 32 * 32;
}

// shared-memory floats of a sweep of kind K for nw variables: state ring,
// two predictor planes, two face-flux planes, slopes
__host__ __device__ constexpr int fused_smem_floats(int nw, int K) {
  return FWRING * fused_slot_floats(nw, K) +
         2 * nw * (K == 0 ? TileCfg<0>::RN : K == 1 ? TileCfg<1>::RN : TileCfg<2>::RN) +
         (K == 2 ? 0 : 2 * nw * (K == 0 ? TileCfg<0>::NF : TileCfg<1>::NF) + nw * 256);
}

// rows of the TMA box of kind K (one tensor map per box shape)
__host__ __device__ constexpr int fused_box_rows(int K) {
  return K == 1 ? TileCfg<1>::BY : TileCfg<0>::BY;
}

static_assert(fused_box_rows(0) == FUSED_BOX_ROWS[0] &&
                  fused_box_rows(1) == FUSED_BOX_ROWS[1] &&
                  fused_box_rows(2) == FUSED_BOX_ROWS[0],
              "tensor-map box rows");

struct FusedArgs {
  DevGrid g;
  DevPhys ph;
  const float* dxf[3];   // dx over the ghost range (FP32)
  const float* idxf[3];  // 1/dx over the ghost range
  Ctrl* ctrl;
  float* wout;
  int nzc;               // planes per CTA (3-D)
  int zchunks;
  int periodic_mask[3];  // bit iw set: variable iw periodic in dimension d
  int asymm_lo[3], asymm_hi[3];  // bit iw set: 'asymm' at that face
  float gravf[3];        // gravity source parameters (FP32)
  int cfl;               // evaluate the CFL maximum (courantpar > 0)
};

// ------------------------------------------------------------ TMA/mbarrier

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* b, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)),
               "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* b,
                                               unsigned bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_u32(b)),
      "r"(bytes)
      : "memory");
}

// Bounded wait for the phase with the given parity; false on timeout
// (limit cycles; by default about 2^31, > 1 s).
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, int parity,
                                          long long limit = 1LL << 31) {
  const unsigned a = smem_u32(b);
  const long long t0 = clock64();
  while (true) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > limit) return false;
  }
}

// One state plane: box {FB_X, rows, 1, nw} at (x, y, z, 0).
__device__ __forceinline__ void tma_load_plane(const CUtensorMap* map,
                                               float* dst,
                                               unsigned long long* bar, int x,
                                               int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::"
      "bytes [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(0), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void init_bars(unsigned long long* bars) {
  if (threadIdx.x == 0) {
    for (int i = 0; i < FWRING; i++) mbar_init(&bars[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
}

// ---------------------------------------------------------------- kernel

// Limiter of all variables, fixed at compile time when uniform
// (LIMC_RUNTIME: per variable from DevPhys).
enum { LIMC_RUNTIME = 0, LIMC_MINMOD = 1, LIMC_WOODWARD = 2 };

// PM: pressure recovery of the wave speeds; PMF: of the fluxes.
template <int NDIM, int D, bool MHD, int PM, int LIMC, int PMF = PM>
struct Fused {
  static constexpr int K = fused_kind(NDIM, D);  // geometry kind
  static constexpr int AM = K == 2 ? D : 2;       // marching axis (3-D)
  static constexpr int AR = K == 2 && D == 1 ? 2 : 1;  // tile-row axis
  typedef TileCfg<K> C;
  static constexpr int NDIR = NDIM;
  static constexpr int NW = MHD ? 2 + 2 * NDIR : 2 + NDIR;
  static constexpr int E = NDIR + 1;
  static constexpr int SLOT = fused_slot_floats(NW, K);
  // Pressure recovery: PM in the wave speeds, PMF in the four flux
  // evaluations per cell (the same double-float recovery by default; FP32
  // in the fluxes is the opt-in variant -- p enters a flux only through
  // p + B^2/2 and v(e + p), whose FP32 error is set by the energy scale).
  typedef PHMixed<PM> PH;
  typedef PHMixed<PMF> PHF;

  // shared memory: state ring | w1 slot 0 | w1 slot 1 | faces 0 | faces 1
  // | slopes (predictor plane p in w1 slot p & 1; the faces of plane p in
  // face slot (p + 1) & 1)
  static __device__ __forceinline__ float* w1slot(float* sm, int p) {
    return sm + FWRING * SLOT + (p & 1) * NW * C::RN;
  }
  static __device__ __forceinline__ float* fbuf(float* sm, int p) {
    return sm + FWRING * SLOT + 2 * NW * C::RN + ((p + 1) & 1) * NW * C::NF;
  }
  static __device__ __forceinline__ float* ldbuf(float* sm) {
    return sm + FWRING * SLOT + 2 * NW * C::RN + 2 * NW * C::NF;
  }
  // state plane slot: [v][sy][sx]
  static __device__ __forceinline__ float W(const float* s, int v, int sy,
                                            int sx) {
    return s[v * C::BPL + sy * FB_X + sx];
  }

  static __device__ __forceinline__ float lim(const FusedArgs& a, int v,
                                              float x, float y) {
    if (LIMC == LIMC_MINMOD) {
      const float sg = copysignf(1.0f, x);
      return sg * fmaxf(0.0f, fminf(fabsf(x), sg * y));
    }
    if (LIMC == LIMC_WOODWARD) {
      const float sg = copysignf(1.0f, x);
      const float m = fminf(fminf(fabsf(x), sg * y), sg * 0.25f * (y + x));
      return 2.0f * sg * fmaxf(0.0f, m);
    }
    return PH::limiter(a.ph.lim[v], x, y);
  }

  // central-difference div B of the state w at (sy, sx) of plane p0
  static __device__ __forceinline__ float divb_w(const FusedArgs& a,
                                                 const float* pm,
                                                 const float* p0,
                                                 const float* pp, int sy,
                                                 int sx, const int* gc) {
    const int o = sy * FB_X + sx;
    const int bx = (E + 1) * C::BPL, by = (E + 1 + AR) * C::BPL;
    float divb = 0.5f * (p0[bx + o + 1] - p0[bx + o - 1]) * a.idxf[0][gc[0]];
    if (NDIM > 1)
      divb = fmaf(0.5f * (p0[by + o + FB_X] - p0[by + o - FB_X]), a.idxf[AR][gc[AR]], divb);
    if (NDIM > 2) {
      const int bz = (E + 1 + AM) * C::BPL;
      divb = fmaf(0.5f * (pp[bz + o] - pm[bz + o]), a.idxf[AM][gc[AM]], divb);
    }
    return divb;
  }

  // addsource2 on acc with wCT = wc: gravity (specialsource) then the Powell
  // terms (addsource) for qs * div B = qdivb.
  static __device__ __forceinline__ void add_sources(const FusedArgs& a,
                                                     float qs, const float* wc,
                                                     float qdivb, float* acc) {
    if (a.ph.src_id == VACGPU_SRC_GRAVITY) {
#pragma unroll
      for (int d = 1; d <= NDIM; d++) {
        const float gr = a.gravf[d - 1];
        if (gr != 0.0f) acc[d] = acc[d] + (qs * gr) * wc[0];
      }
#pragma unroll
      for (int d = 1; d <= NDIM; d++) {
        const float gr = a.gravf[d - 1];
        if (gr != 0.0f) acc[E] = acc[E] + (qs * gr) * wc[d];
      }
    }
    if (MHD && a.ph.divbfix) {
      const float ri = 1.0f / wc[0];
      float mb = wc[1] * wc[E + 1];
#pragma unroll
      for (int k = 2; k <= NDIR; k++) mb = fmaf(wc[k], wc[E + k], mb);
#pragma unroll
      for (int k = 1; k <= NDIR; k++) {
        acc[k] = acc[k] - wc[E + k] * qdivb;
        acc[E + k] = acc[E + k] - wc[k] * ri * qdivb;
      }
      acc[E] = acc[E] - mb * ri * qdivb;
    }
  }

  // Hancock predictor at the cell (sy, sx) of plane p0; ld receives the
  // limited slopes along D (also the corrector's slopes).
  static __device__ __forceinline__ void predict_cell(
      const FusedArgs& a, const float* pm, const float* p0, const float* pp,
      int sy, int sx, const int* gc, float qdt, float qs, float smallp,
      float* out, float* ld) {
    float u[NW], uL[NW], uR[NW];
#pragma unroll
    for (int v = 0; v < NW; v++) {
      float um, up;
      u[v] = W(p0, v, sy, sx);
      if (K == 0) {
        um = W(p0, v, sy, sx - 1);
        up = W(p0, v, sy, sx + 1);
      } else if (K == 1) {
        um = W(p0, v, sy - 1, sx);
        up = W(p0, v, sy + 1, sx);
      } else {
        um = W(pm, v, sy, sx);
        up = W(pp, v, sy, sx);
      }
      const float l = lim(a, v, up - u[v], u[v] - um);
      ld[v] = l;
      uR[v] = u[v] - 0.5f * l;
      uL[v] = u[v] + 0.5f * l;
    }
    float fL[NW], fR[NW];
    PHF::template flux<NDIR, MHD>(uR, D, a.ph, smallp, fR);
    PHF::template flux<NDIR, MHD>(uL, D, a.ph, smallp, fL);
    const float cq = qdt * a.idxf[D][gc[D]];
#pragma unroll
    for (int v = 0; v < NW; v++) out[v] = u[v] - cq * (fL[v] - fR[v]);
    if (a.ph.sourceunsplit) {
      const float qdivb =
          MHD && a.ph.divbfix ? qs * divb_w(a, pm, p0, pp, sy, sx, gc) : 0.0f;
      add_sources(a, qs, u, qdivb, out);
    }
  }

  // Predictor of the magnetic component b_k alone (k != D): the arithmetic
  // of predict_cell restricted to F_D[b_k] = v_D b_k - m_k/rho b_D and the
  // Powell term of b_k.
  static __device__ __forceinline__ float predict_b(
      const FusedArgs& a, const float* pm, const float* p0, const float* pp,
      int sy, int sx, const int* gc, float qdt, float qs, int k) {
    const int iv[5] = {0, 1 + D, 1 + k, E + 1 + D, E + 1 + k};
    float u[5], uL[5], uR[5];
#pragma unroll
    for (int i = 0; i < 5; i++) {
      const int v = iv[i];
      const float c = W(p0, v, sy, sx);
      float m, p;
      if (K == 0) {
        m = W(p0, v, sy, sx - 1);
        p = W(p0, v, sy, sx + 1);
      } else if (K == 1) {
        m = W(p0, v, sy - 1, sx);
        p = W(p0, v, sy + 1, sx);
      } else {
        m = W(pm, v, sy, sx);
        p = W(pp, v, sy, sx);
      }
      const float l = lim(a, v, p - c, c - m);
      u[i] = c;
      uR[i] = c - 0.5f * l;
      uL[i] = c + 0.5f * l;
    }
    const float riR = 1.0f / uR[0], riL = 1.0f / uL[0];
    const float fR = fmaf(uR[1] * riR, uR[4], -(uR[2] * riR * uR[3]));
    const float fL = fmaf(uL[1] * riL, uL[4], -(uL[2] * riL * uL[3]));
    float out = u[4] - qdt * a.idxf[D][gc[D]] * (fL - fR);
    if (a.ph.sourceunsplit && a.ph.divbfix)
      out = out - u[2] / u[0] * (qs * divb_w(a, pm, p0, pp, sy, sx, gc));
    return out;
  }

  // TVDLF flux at the face between wl and wr (predictor values) with the
  // limited slopes ldl, ldr of the base state; returns cmax.
  static __device__ __forceinline__ float face(const FusedArgs& a,
                                               const float* wl,
                                               const float* wr,
                                               const float* ldl,
                                               const float* ldr, float smallp,
                                               float* F) {
    float L[NW], R[NW], M[NW];
#pragma unroll
    for (int v = 0; v < NW; v++) {
      L[v] = wl[v] + 0.5f * ldl[v];
      R[v] = wr[v] - 0.5f * ldr[v];
      M[v] = 0.5f * (L[v] + R[v]);
    }
#pragma unroll
    for (int v = 0; v < NW; v++) L[v] = 2.0f * M[v] - R[v];
    float fL[NW], fR[NW];
    float cmax;
    if constexpr (PM == PMF) {
      // the mean's pressure from the two recovered face-state pressures
      float pL, pR, riL, riR;
      PHF::template flux_p<NDIR, MHD>(L, D, a.ph, smallp, fL, pL, riL);
      PHF::template flux_p<NDIR, MHD>(R, D, a.ph, smallp, fR, pR, riR);
      cmax = PH::template cmax_mean<NDIR, MHD>(L, R, M, pL, pR, riL, riR, D,
                                                a.ph, smallp);
    } else {
      cmax = PH::template cmax<NDIR, MHD>(M, D, a.ph, smallp);
      PHF::template flux<NDIR, MHD>(L, D, a.ph, smallp, fL);
      PHF::template flux<NDIR, MHD>(R, D, a.ph, smallp, fR);
    }
#pragma unroll
    for (int v = 0; v < NW; v++)
      F[v] = fmaf(-cmax * 0.5f, R[v] - L[v], 0.5f * (fL[v] + fR[v]));
    return cmax;
  }

  // getboundary on w1: region cells in the first ghost layer of a
  // non-periodic x or tile-row face take the adjacent mesh value (when xy
  // is set); at a face of the marching axis the whole plane does (-1 from
  // 0, n from n-1).
  static __device__ void fix_w1_ghosts(const FusedArgs& a, float* sm, int j,
                                       int x0, int y0, bool xy, bool z) {
    const DevGrid& g = a.g;
    float* w1j = w1slot(sm, j);
    if (xy) {
      for (int c = threadIdx.x; c < C::RN; c += FT_NT) {
        const int rx = c % C::RX, ry = c / C::RX;
        const int ix = x0 + rx - 1, iy = y0 + ry - 1;
        int d = -1, src = c, lo = 0;
        if ((ix == -1 || ix == g.nx[0]) && (NDIM < 2 || (iy >= 0 && iy < g.nx[AR]))) {
          d = 0;
          lo = ix == -1;
          src = c + (lo ? 1 : -1);
        } else if (NDIM >= 2 && (iy == -1 || iy == g.nx[AR]) && ix >= 0 && ix < g.nx[0]) {
          d = AR;
          lo = iy == -1;
          src = c + (lo ? C::RX : -C::RX);
        }
        if (d < 0) continue;
        const int asy = lo ? a.asymm_lo[d] : a.asymm_hi[d];
#pragma unroll
        for (int v = 0; v < NW; v++) {
          if ((a.periodic_mask[d] >> v) & 1) continue;
          const float s = w1j[v * C::RN + src];
          w1j[v * C::RN + c] = ((asy >> v) & 1) ? -s : s;
        }
      }
    }
    if (NDIM == 3 && z) {
      const int dst = j == 0 ? -1 : j, srcp = j == 0 ? 0 : j - 1;
      const int asy = j == 0 ? a.asymm_lo[AM] : a.asymm_hi[AM];
      if (xy) __syncthreads();  // the in-plane fix of the source plane is complete
      float* dp = w1slot(sm, dst);
      const float* sp = w1slot(sm, srcp);
      for (int c = threadIdx.x; c < C::RN; c += FT_NT) {
#pragma unroll
        for (int v = 0; v < NW; v++) {
          if ((a.periodic_mask[AM] >> v) & 1) continue;
          const float s = sp[v * C::RN + c];
          dp[v * C::RN + c] = ((asy >> v) & 1) ? -s : s;
        }
      }
    }
  }

  // The TVDLF faces along D (0 or 1) of plane jo into its face slot: one
  // face per thread, each warp one row of faces (x: 31 faces, lane 31
  // idle; y: 32).  The slopes are the predictor's: the thread that predicted
  // the left/lower cell of the face had this thread's index.
  static __device__ __forceinline__ void in_plane_faces(
      const FusedArgs& a, float* sm, int jo, int x0, int y0, float smallp,
      float& qmax) {
    const int tid = threadIdx.x;
    const DevGrid& g = a.g;
    int rx, ry, f;  // left / lower cell of the face (region), face index
    if (K == 0) {
      rx = tid % 32;
      ry = tid / 32 + 1;
      if (rx > C::TX) return;
      f = (ry - 1) * (C::TX + 1) + rx;
    } else {
      if (tid >= C::NF) return;
      rx = tid % 32 + 1;
      ry = tid / 32;
      f = tid;
    }
    const int ix = x0 + rx - 1, iy = y0 + ry - 1;
    const bool valid = K == 0 ? (ix >= -1 && ix < g.nx[0] && (NDIM < 2 || iy < g.nx[AR]))
                              : (iy >= -1 && iy < g.nx[AR] && ix < g.nx[0]);
    if (!valid) return;
    const float* w1o = w1slot(sm, jo);
    const float* lb = ldbuf(sm);
    const int fr = K == 0 ? tid + 1 : tid + 32;
    const int rl = ry * C::RX + rx;
    const int rr = K == 0 ? rl + 1 : rl + C::RX;
    float wl[NW], wr[NW], ldl[NW], ldr[NW], F[NW];
#pragma unroll
    for (int v = 0; v < NW; v++) {
      wl[v] = w1o[v * C::RN + rl];
      wr[v] = w1o[v * C::RN + rr];
      ldl[v] = lb[v * 256 + tid];
      ldr[v] = lb[v * 256 + fr];
    }
    const float cm = face(a, wl, wr, ldl, ldr, smallp, F);
    float* fb = fbuf(sm, jo);
#pragma unroll
    for (int v = 0; v < NW; v++) fb[v * C::NF + f] = F[v];
    if (a.cfl) {
      const int gi = (K == 0 ? ix : iy) + 2;
      const float q = cm * 2.0f / (a.dxf[D][gi] + a.dxf[D][gi + 1]);
      qmax = (q > qmax || q != q) ? q : qmax;  // a NaN sticks
    }
  }

  // mesh coordinates (x, tile row, plane) -> ghost-range indices (x, y, z)
  static __device__ __forceinline__ void gcoords(const DevGrid& g, int ix,
                                                 int iy, int jp, int* gc) {
    gc[0] = ix + 2;
    gc[AR] = iy + g.gh[AR];
    if (NDIM == 3) gc[AM] = jp + g.gh[AM];
    else gc[2] = 0;
  }

  // Corrected state of the output cell (lx, ly) of plane jo:
  // w - qdt/dx (F+ - F-) + sources(w1), written to HBM.  bpl: the state
  // plane jo; bzm: the marching-axis B component of w1 at plane jo-1 (3-D).
  static __device__ __forceinline__ void update(const FusedArgs& a,
                                                float* sm, const float* bpl,
                                                int jo, int ix, int iy,
                                                int lx, int ly, int sh,
                                                float qdt, float qs,
                                                const float* Fm,
                                                const float* Fp, float bzm) {
    const DevGrid& g = a.g;
    const float* c0 = w1slot(sm, jo);
    const int r = (ly + 1) * C::RX + lx + 1;
    int gc[3];
    gcoords(g, ix, iy, jo, gc);
    float acc[NW], wc[NW];
#pragma unroll
    for (int v = 0; v < NW; v++) {
      acc[v] = W(bpl, v, ly + 2, lx + 4 + sh);
      wc[v] = c0[v * C::RN + r];
    }
    const float cq = qdt * a.idxf[D][gc[D]];
#pragma unroll
    for (int v = 0; v < NW; v++) acc[v] = acc[v] - cq * (Fp[v] - Fm[v]);
    if (a.ph.sourceunsplit) {
      float qdivb = 0.0f;
      if (MHD && a.ph.divbfix) {
        const int bxo = (E + 1) * C::RN + r, byo = (E + 1 + AR) * C::RN + r;
        float divb = 0.5f * (c0[bxo + 1] - c0[bxo - 1]) * a.idxf[0][gc[0]];
        if (NDIM > 1)
          divb = fmaf(0.5f * (c0[byo + C::RX] - c0[byo - C::RX]), a.idxf[AR][gc[AR]], divb);
        if (NDIM > 2) {
          const float bzp = w1slot(sm, jo + 1)[(E + 1 + AM) * C::RN + r];
          divb = fmaf(0.5f * (bzp - bzm), a.idxf[AM][gc[AM]], divb);
        }
        qdivb = qs * divb;
      }
      add_sources(a, qs, wc, qdivb, acc);
    }
    const long long off = gidx(g, gc[0], gc[1], gc[2]);
#pragma unroll
    for (int v = 0; v < NW; v++) a.wout[off + v * g.vs] = acc[v];
    if (near_bnd(g, gc)) ghost_images(a, gc, off, acc);
  }

  // Within two cells of a mesh face: the cell is the source of ghost cells.
  static __device__ __forceinline__ bool near_bnd(const DevGrid& g,
                                                  const int* gc) {
    bool b = false;
#pragma unroll
    for (int d = 0; d < NDIM; d++) b = b || gc[d] < 4 || gc[d] >= g.nx[d];
    return b;
  }

  // Ghost-cell preimages of the mesh index gi along one dimension (n cells,
  // ghost-range indices 0..n+3, n >= 4): up to two ghost positions p1, p2
  // whose boundary map lands on gi, and the 'asymm' sign mask of each.
  // periodic: gi-n for gi >= n, gi+n for gi < 4; cont: 0 and 1 for gi = 2,
  // n+2 and n+3 for gi = n+1; symm/asymm: 3-gi for gi < 4, 2n+3-gi for
  // gi >= n (negated for 'asymm' variables).
  static __device__ __forceinline__ int preimages(const FusedArgs& a, int d,
                                                  int gi, int& p1, int& f1,
                                                  int& p2) {
    const int n = a.g.nx[d];
    const int mlo = a.ph.gmap[d][0], mhi = a.ph.gmap[d][1];
    p1 = p2 = gi;
    f1 = 0;
    if (gi < 4) {
      if (mlo == GMAP_CONT && gi == 2) {
        p1 = 0;
        p2 = 1;
        return 2;
      }
      if (mlo == GMAP_MIRROR) {
        p1 = 3 - gi;
        f1 = a.ph.asym[d][0];
        return 1;
      }
      if (mhi == GMAP_PERIODIC) {
        p1 = gi + n;
        return 1;
      }
    }
    if (gi >= n) {
      if (mhi == GMAP_CONT && gi == n + 1) {
        p1 = n + 2;
        p2 = n + 3;
        return 2;
      }
      if (mhi == GMAP_MIRROR) {
        p1 = 2 * n + 3 - gi;
        f1 = a.ph.asym[d][1];
        return 1;
      }
      if (mlo == GMAP_PERIODIC) {
        p1 = gi - n;
        return 1;
      }
    }
    return 0;
  }

  // getboundary of the new state, done by its sources: every ghost cell
  // (gx, gy, gz) holds sign * w(map_x(gx), map_y(gy), map_z(gz)) (the
  // region-by-region copies of src/vacgrid.t:195-413 composed), so the cell
  // gc writes its value to each position whose coordinates are gc's own or
  // preimages in every dimension, at least one of them a preimage.
  // off: the cell's own index in the state buffer (images are offsets
  // from it).  The common case -- an x-boundary cell with interior y and z
  // -- writes its one or two images in its own row without the general
  // loop.
  static __device__ __forceinline__ void ghost_images(const FusedArgs& a,
                                                      const int* gc,
                                                      long long off,
                                                      const float (&acc)[NW]) {
    const DevGrid& g = a.g;
    int x1, x2, fx;
    const int nx_ = 1 + preimages(a, 0, gc[0], x1, fx, x2);
    const bool yin = NDIM < 2 || (gc[1] >= 4 && gc[1] < g.nx[1]);
    const bool zin = NDIM < 3 || (gc[2] >= 4 && gc[2] < g.nx[2]);
    if (yin && zin) {
      for (int i = 1; i < nx_; i++) {
        const long long o = off + ((i == 1 ? x1 : x2) - gc[0]);
        const int fl = i == 1 ? fx : 0;
#pragma unroll
        for (int v = 0; v < NW; v++)
          a.wout[o + v * g.vs] = ((fl >> v) & 1) ? -acc[v] : acc[v];
      }
      return;
    }
    int y1 = 0, y2 = 0, fy = 0, z1 = 0, z2 = 0, fz = 0;
    const int ny_ = NDIM > 1 ? 1 + preimages(a, 1, gc[1], y1, fy, y2) : 1;
    const int nz_ = NDIM > 2 ? 1 + preimages(a, 2, gc[2], z1, fz, z2) : 1;
#pragma unroll 1
    for (int k = 0; k < nz_; k++) {
      const int pz = k == 0 ? gc[2] : (k == 1 ? z1 : z2);
      const int sz = k == 1 ? fz : 0;
#pragma unroll 1
      for (int jj = 0; jj < ny_; jj++) {
        const int py = jj == 0 ? gc[1] : (jj == 1 ? y1 : y2);
        const int sy = jj == 1 ? fy : 0;
        const long long orow = off + (long long)(pz - gc[2]) * g.plane +
                               (long long)(py - gc[1]) * g.P;
#pragma unroll 1
        for (int i = 0; i < nx_; i++) {
          if ((i | jj | k) == 0) continue;
          const int px = i == 0 ? gc[0] : (i == 1 ? x1 : x2);
          const int fl = (i == 1 ? fx : 0) ^ sy ^ sz;
          const long long o = orow + (px - gc[0]);
#pragma unroll
          for (int v = 0; v < NW; v++)
            a.wout[o + v * g.vs] = ((fl >> v) & 1) ? -acc[v] : acc[v];
        }
      }
    }
  }

  // One tile (bx, by) and z chunk bz of one grid.  bars: the CTA's FWRING
  // mbarriers (initialised once); uses[s]: loads completed on slot s before
  // this tile (kept identically by every thread: the phase parity).
  // Returns false when a TMA wait timed out.  The caller synchronises the
  // CTA before reusing the shared memory.
  //
  // 3-D plane loop, iteration j (predictor plane j, corrected plane j-1):
  //   faces of j-1 (x/y sweeps)            reads w1(j-1), slopes(j-1)
  //   wait for state plane j+1; barrier A  (also: nobody is still in j-1)
  //   TMA of state plane j+2 into the slot of j-2
  //   predictor of plane j                 writes w1(j), slopes(j)
  //   barrier B [ghost fix of w1(j); barrier]
  //   corrector of plane j-1               reads faces(j-1), w1(j-1), w1(j)
  static __device__ bool run(const CUtensorMap* map, const FusedArgs& a,
                             float* sm, int bx, int by, int bz,
                             unsigned long long* bars, int* uses,
                             unsigned slotid) {
    Ctrl* ctrl = a.ctrl;
    if (ctrl->done) return true;
    __shared__ float shq[FT_NT / 32];
    const int tid = threadIdx.x;
    const DevGrid& g = a.g;
    // x0: first column; y0: first tile row (axis AR); planes along AM
    const int x0 = bx * C::TX, y0 = by * C::TY;
    const int z0 = NDIM == 3 ? bz * a.nzc : 0;
    const int z1 = NDIM == 3 ? min(z0 + a.nzc, g.nx[AM]) : 1;  // exclusive
    const double dtd = ctrl->dt;
    const float qdt = (float)dtd;               // corrector
    const float qdt2 = (float)(dtd / 2);        // predictor
    const float qs1 = (float)(dtd / 2 / NDIM);  // predictor source
    const float qs2 = (float)(dtd / NDIM);      // corrector source
    const float smallp = (float)ctrl->smallp;
    // The box starts at the column of ix = x0-2 rounded down to a multiple
    // of 4 floats (16 bytes); the state of ix sits at box column
    // ix - x0 + 4 + sh (region column rx at rx + 3 + sh).
    const int cstart = x0 + g.xpad - 2;
    const int colx = cstart & ~3;
    const int sh = cstart - colx;
    const unsigned plane_bytes = NW * C::BPL * 4;
    const bool need_bz = MHD && a.ph.divbfix && a.ph.sourceunsplit;
    // ghost fix of w1 needed: a non-periodic x or row face inside the
    // region, or (per plane) a non-periodic face of the marching axis
    const int all = (1 << NW) - 1;
    const bool fix_xy =
        (a.periodic_mask[0] != all && (x0 == 0 || x0 + C::TX >= g.nx[0])) ||
        (NDIM >= 2 && a.periodic_mask[AR] != all && (y0 == 0 || y0 + C::TY >= g.nx[AR]));
    const bool fix_zb = NDIM == 3 && a.periodic_mask[AM] != all;

    const int pbase = NDIM == 3 ? z0 - 2 : 0;
    auto slot = [&](int p) -> float* { return sm + ((p - pbase) % FWRING) * SLOT; };
    auto issue = [&](int p) {
      const int q = p - pbase;
      fence_proxy_async();
      mbar_expect_tx(&bars[q % FWRING], plane_bytes);
      tma_load_plane(map, slot(p), &bars[q % FWRING], colx, y0, p + g.gh[AM]);
    };
    auto wait_plane = [&](int p) -> bool {
      const int q = p - pbase;
      return mbar_wait(&bars[q % FWRING], (uses[q % FWRING] + q / FWRING) & 1);
    };

    // this thread's full-predictor cell (region coordinates)
    const int frx = K == 0 ? tid % 32 : tid % 32 + 1;
    const int fry = K == 1 ? tid / 32 : tid / 32 + 1;
    // this thread's output cell: warp ly, lane lx
    const int lx = tid % 32, ly = tid / 32;
    const bool has_out = lx < C::TX && ly < C::TY;
    const int oix = x0 + lx, oiy = y0 + ly;
    const bool out_ok = has_out && oix < g.nx[0] && (NDIM < 2 || oiy < g.nx[AR]);

    float qmax = 0.0f;  // CFL: max cmax*2/(dx_i+dx_i+1) over this thread's faces
    const int pfirst = NDIM == 3 ? z0 - 1 : 0;
    const int plast = NDIM == 3 ? z1 : 0;
    if (tid == 0) {
      if (NDIM == 3) {
        issue(z0 - 2);
        issue(z0 - 1);
        issue(z0);
      } else {
        issue(0);
      }
    }
    float Lprev[NW], Fprev[NW];  // marching sweeps: carried along the march
#pragma unroll
    for (int v = 0; v < NW; v++) Lprev[v] = Fprev[v] = 0.0f;

    for (int j = pfirst; j <= plast; j++) {
      const int jo = NDIM == 3 ? j - 1 : 0;  // plane corrected this iteration
      const bool out_plane = NDIM == 3 ? (jo >= z0 && jo < z1) : true;
      // in-plane sweeps: planes outside the chunk feed only b_z of div B
      const bool edge = NDIM == 3 && K < 2 && (j == z0 - 1 || j == z1);

      // marching-axis B of w1(j-2): its slot takes the predictor of plane j
      float bzm = 0.0f;
      if (NDIM == 3 && need_bz && out_plane && has_out)
        bzm = w1slot(sm, j - 2)[(E + 1 + AM) * C::RN + (ly + 1) * C::RX + lx + 1];
      if (NDIM == 3 && K < 2 && out_plane)
        in_plane_faces(a, sm, jo, x0, y0, smallp, qmax);

      bool ok = true;
      if (NDIM == 3) {
        if (j == pfirst) ok = wait_plane(j - 1) && wait_plane(j);
        ok = ok && wait_plane(j + 1);
      } else {
        ok = wait_plane(0);
      }
      if (__syncthreads_or(!ok)) {  // barrier A
        if (tid == 0) {
          atomicExch(&ctrl->fault, 1);
          // copies still in flight (3-D: planes j-1 .. j+1; 2-D: the one
          // plane): wait for them, again with a bound, before exiting
          for (int p = NDIM == 3 ? max(j - 1, pbase) : 0; p <= (NDIM == 3 ? j + 1 : 0); p++) {
            const int q = p - pbase;
            mbar_wait(&bars[q % FWRING], (uses[q % FWRING] + q / FWRING) & 1, 1LL << 28);
          }
        }
        return false;
      }
      if (NDIM == 3 && tid == 0 && j + 2 <= z1 + 1) issue(j + 2);
      const float* pm = NDIM == 3 ? slot(j - 1) : nullptr;
      const float* p0 = slot(j);
      const float* pp = NDIM == 3 ? slot(j + 1) : nullptr;

      // predictor of plane j
      float Lcur[NW];
#pragma unroll
      for (int v = 0; v < NW; v++) Lcur[v] = 0.0f;
      if (edge) {
        if (need_bz && has_out && oix <= g.nx[0] && oiy <= g.nx[AR]) {
          int gc[3];
          gcoords(g, oix, oiy, j, gc);
          w1slot(sm, j)[(E + 1 + AM) * C::RN + (ly + 1) * C::RX + lx + 1] =
              predict_b(a, pm, p0, pp, ly + 2, lx + 4 + sh, gc, qdt2, qs1, AM);
        }
      } else {
        const int ix = x0 + frx - 1, iy = y0 + fry - 1;
        const bool need = ix >= -1 && ix <= g.nx[0] &&
                          (NDIM < 2 || (iy >= -1 && iy <= g.nx[AR] &&
                                        !((ix == -1 || ix == g.nx[0]) &&
                                          (iy == -1 || iy == g.nx[AR]))));
        if (need) {
          int gc[3];
          gcoords(g, ix, iy, j, gc);
          float out[NW];
          predict_cell(a, pm, p0, pp, fry + 1, frx + 3 + sh, gc, qdt2, qs1,
                       smallp, out, Lcur);
          float* w1j = w1slot(sm, j);
          const int rc = fry * C::RX + frx;
#pragma unroll
          for (int v = 0; v < NW; v++) w1j[v * C::RN + rc] = out[v];
          if (K < 2) {
            float* lb = ldbuf(sm);
#pragma unroll
            for (int v = 0; v < NW; v++) lb[v * 256 + tid] = Lcur[v];
          }
        }
        if (need_bz && tid < C::NB + (K == 1 ? 0 : 64 - 2 * C::TX)) {
          // transverse B of the halo cells that only div B reads: the
          // row-axis component on the rows above and below (one warp each),
          // b_x on the columns left and right
          int rx, ry, k;
          bool on = true;
          if (K != 1 && tid < 64) {
            rx = tid % 32 + 1;
            ry = tid < 32 ? 0 : C::RY - 1;
            k = AR;
            on = rx <= C::TX;
          } else {
            const int hh = K == 1 ? tid : tid - 64;
            rx = hh < C::TY ? 0 : C::RX - 1;
            ry = hh % C::TY + 1;
            k = 0;
          }
          const int bix = x0 + rx - 1, biy = y0 + ry - 1;
          if (on && bix <= g.nx[0] && (NDIM < 2 || biy <= g.nx[AR])) {
            int gc[3];
            gcoords(g, bix, biy, j, gc);
            w1slot(sm, j)[(E + 1 + k) * C::RN + ry * C::RX + rx] =
                predict_b(a, pm, p0, pp, ry + 1, rx + 3 + sh, gc, qdt2, qs1, k);
          }
        }
      }
      __syncthreads();  // barrier B
      const bool fz = fix_zb && (j == 0 || j == g.nx[AM]);
      if (fix_xy || fz) {
        fix_w1_ghosts(a, sm, j, x0, y0, fix_xy, fz);
        __syncthreads();
      }

      if (K == 2) {
        // the face between planes j-1 and j of this column
        float Fnew[NW];
#pragma unroll
        for (int v = 0; v < NW; v++) Fnew[v] = 0.0f;
        if (j >= z0) {
          float wl[NW], wr[NW];
          const float* a1 = w1slot(sm, j - 1);
          const float* a2 = w1slot(sm, j);
          const int r = (ly + 1) * C::RX + lx + 1;
#pragma unroll
          for (int v = 0; v < NW; v++) {
            wl[v] = a1[v * C::RN + r];
            wr[v] = a2[v * C::RN + r];
          }
          const float cm = face(a, wl, wr, Lprev, Lcur, smallp, Fnew);
          if (a.cfl && out_ok) {
            const int gz = j + 1;  // ghost-range index of plane j-1
            const float q = cm * 2.0f / (a.dxf[D][gz] + a.dxf[D][gz + 1]);
            qmax = (q > qmax || q != q) ? q : qmax;
          }
        }
        if (out_plane && out_ok)
          update(a, sm, pm, jo, oix, oiy, lx, ly, sh, qdt, qs2, Fprev, Fnew, bzm);
#pragma unroll
        for (int v = 0; v < NW; v++) {
          Lprev[v] = Lcur[v];
          Fprev[v] = Fnew[v];
        }
      } else {
        if (NDIM == 2) {
          in_plane_faces(a, sm, 0, x0, y0, smallp, qmax);
          __syncthreads();
        }
        if (out_plane && out_ok) {
          const float* fb = fbuf(sm, jo);
          float Fm[NW], Fp[NW];
          const int fm = K == 0 ? ly * (C::TX + 1) + lx : ly * C::TX + lx;
          const int fp = K == 0 ? fm + 1 : fm + C::TX;
#pragma unroll
          for (int v = 0; v < NW; v++) {
            Fm[v] = fb[v * C::NF + fm];
            Fp[v] = fb[v * C::NF + fp];
          }
          update(a, sm, NDIM == 3 ? pm : p0, jo, oix, oiy, lx, ly, sh, qdt, qs2,
                 Fm, Fp, bzm);
        }
      }
    }
    {  // phase bookkeeping: planes pbase .. (NDIM==3 ? z1+1 : 0) were loaded
      const int np = NDIM == 3 ? z1 + 2 - pbase : 1;
#pragma unroll
      for (int s2 = 0; s2 < FWRING; s2++) uses[s2] += (np - s2 + FWRING - 1) / FWRING;
    }
    if (a.cfl) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float v = __shfl_xor_sync(0xffffffffu, qmax, o);
        qmax = (v > qmax || v != v) ? v : qmax;
      }
      if ((tid & 31) == 0) shq[tid >> 5] = qmax;
      __syncthreads();
      if (tid == 0) {
        for (int i = 1; i < FT_NT / 32; i++)
          qmax = (shq[i] > qmax || shq[i] != shq[i]) ? shq[i] : qmax;
        const unsigned long long key = dkey((double)qmax);
        if (qmax != 0.0f) atomicMax(&ctrl->face_cmax[D][slotid % NSLOT], key);
      }
    }
    return true;
  }
};

template <int NDIM, int D, bool MHD, int PM, int LIMC, int PMF>
__global__ void __launch_bounds__(FT_NT, 2)
    k_sweep_fused(const __grid_constant__ CUtensorMap map, FusedArgs a) {
  extern __shared__ __align__(128) float dsm[];
  __shared__ __align__(8) unsigned long long bars[FWRING];
  init_bars(bars);
  int uses[FWRING] = {0, 0, 0, 0};
  const unsigned slotid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  Fused<NDIM, D, MHD, PM, LIMC, PMF>::run(&map, a, dsm, blockIdx.x, blockIdx.y,
                                          blockIdx.z, bars, uses, slotid);
}

}  // namespace vacgpu

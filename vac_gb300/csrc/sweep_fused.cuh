// sweep_fused.cuh - one split sweep of VAC's twostep Hancock/TVDLF scheme
// (src/vac.t:363-572, src/vactvdlf.t:5-299) as a single kernel for the
// mixed-precision path.
//
// A CTA owns a 32x8 column tile of the mesh and marches along z through a
// chunk of planes.  Each plane of the state (tile + 2-cell halo, all
// variables) arrives in shared memory with one TMA tensor copy
// (cp.async.bulk.tensor, mbarrier completion), one plane ahead of use.  The
// Hancock predictor w1 is evaluated for the tile + 1-cell halo into a
// 3-plane shared ring (never written to HBM), every face flux of the TVDLF
// corrector is computed once, and the corrected plane goes straight to HBM.
// HBM traffic per sweep is one read and one write of the state (plus halo
// re-reads that mostly hit L2).
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

constexpr int FT_X = 32;               // tile width (x)
constexpr int FT_Y = 8;                // tile height (y)
constexpr int FT_NT = FT_X * FT_Y;     // threads per CTA
constexpr int FB_X = 40;               // TMA box width (16-byte aligned)
constexpr int FB_Y = FT_Y + 4;         // TMA box height
constexpr int FB_PLANE = FB_X * FB_Y;  // floats per variable per plane
constexpr int FR_X = FT_X + 2;         // predictor region width
constexpr int FR_Y = FT_Y + 2;         // predictor region height
constexpr int FR_N = FR_X * FR_Y;
constexpr int FWRING = 4;              // state planes resident
constexpr int FW1RING = 3;             // predictor planes resident
constexpr int FFACE = 9 * 32;          // >= (FT_X+1)*FT_Y, FT_X*(FT_Y+1)

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
};

__host__ __device__ constexpr int fused_smem_floats(int nw) {
  return FWRING * nw * FB_PLANE + FW1RING * nw * FR_N + nw * FFACE;
}

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
// (about 2^31 cycles, > 1 s).
__device__ __forceinline__ bool mbar_wait(unsigned long long* b, int parity) {
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
    if (clock64() - t0 > (1LL << 31)) return false;
  }
}

// One state plane: box {FB_X, FB_Y, 1, nw} at (x, y, z, 0).
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

// ---------------------------------------------------------------- kernel

// Limiter of all variables, fixed at compile time when uniform
// (LIMC_RUNTIME: per variable from DevPhys).
enum { LIMC_RUNTIME = 0, LIMC_MINMOD = 1, LIMC_WOODWARD = 2 };

template <int NDIM, int D, bool MHD, int PM, int LIMC>
struct Fused {
  static constexpr int NDIR = NDIM;
  static constexpr int NW = MHD ? 2 + 2 * NDIR : 2 + NDIR;
  static constexpr int E = NDIR + 1;
  typedef PHMixed<PM> PH;

  // state plane slot: [v][sy][sx]; predictor slot: [v][ry][rx]
  static __device__ __forceinline__ float W(const float* s, int v, int sy,
                                            int sx) {
    return s[v * FB_PLANE + sy * FB_X + sx];
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

  // Predictor of one magnetic component b_k only (k != D): the value the
  // corrector's div B reads in the transverse halo.  Same arithmetic as
  // predict_cell restricted to F_D[b_k] = v_D b_k - m_k/rho b_D and the
  // Powell term of b_k.
  static __device__ __forceinline__ float predict_b(
      const FusedArgs& a, const float* pm, const float* p0, const float* pp,
      int sy, int sx, int gd, const int* gc, float qdt, float qs, int k) {
    const int iv[5] = {0, 1 + D, 1 + k, E + 1 + D, E + 1 + k};
    float u[5], uL[5], uR[5];
#pragma unroll
    for (int i = 0; i < 5; i++) {
      const int v = iv[i];
      float c = W(p0, v, sy, sx), m, p;
      if (D == 0) {
        m = W(p0, v, sy, sx - 1);
        p = W(p0, v, sy, sx + 1);
      } else if (D == 1) {
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
    const float fR = uR[1] * riR * uR[4] - uR[2] * riR * uR[3];
    const float fL = uL[1] * riL * uL[4] - uL[2] * riL * uL[3];
    float out = u[4] - qdt * a.idxf[D][gd] * (fL - fR);
    if (a.ph.sourceunsplit && a.ph.divbfix) {
      const int o = sy * FB_X + sx;
      const int bx = (E + 1) * FB_PLANE, by = (E + 2) * FB_PLANE;
      float divb = 0.5f * (p0[bx + o + 1] - p0[bx + o - 1]) * a.idxf[0][gc[0]];
      if (NDIM > 1)
        divb += 0.5f * (p0[by + o + FB_X] - p0[by + o - FB_X]) * a.idxf[1][gc[1]];
      if (NDIM > 2) {
        const int bz = (E + 3) * FB_PLANE;
        divb += 0.5f * (pp[bz + o] - pm[bz + o]) * a.idxf[2][gc[2]];
      }
      out = out - u[2] / u[0] * (qs * divb);
    }
    return out;
  }

  // Hancock predictor at one cell; u = center, m/p = neighbours along D,
  // divB from the b components of the cross neighbours.
  static __device__ __forceinline__ void predict_cell(
      const FusedArgs& a, const float* pm, const float* p0, const float* pp,
      int sy, int sx, int gd, const int* gc, float qdt, float qs,
      float smallp, float* out) {
    float u[NW], um[NW], up[NW];
#pragma unroll
    for (int v = 0; v < NW; v++) {
      u[v] = W(p0, v, sy, sx);
      if (D == 0) {
        um[v] = W(p0, v, sy, sx - 1);
        up[v] = W(p0, v, sy, sx + 1);
      } else if (D == 1) {
        um[v] = W(p0, v, sy - 1, sx);
        up[v] = W(p0, v, sy + 1, sx);
      } else {
        um[v] = W(pm, v, sy, sx);
        up[v] = W(pp, v, sy, sx);
      }
    }
    float uL[NW], uR[NW];
#pragma unroll
    for (int v = 0; v < NW; v++) {
      float l = lim(a, v, up[v] - u[v], u[v] - um[v]);
      uR[v] = u[v] - 0.5f * l;
      uL[v] = u[v] + 0.5f * l;
    }
    float fL[NW], fR[NW];
    PH::template flux<NDIR, MHD>(uR, D, a.ph, smallp, fR);
    PH::template flux<NDIR, MHD>(uL, D, a.ph, smallp, fL);
    const float cq = qdt * a.idxf[D][gd];
#pragma unroll
    for (int v = 0; v < NW; v++) out[v] = u[v] - cq * (fL[v] - fR[v]);
    add_sources(a, qs, u, pm, p0, pp, sy, sx, gc, out, true);
  }

  // addsource2: gravity (specialsource) then Powell divB (addsource).
  // For the predictor the cross neighbours come from the state planes
  // (w-layout), for the corrector from the predictor planes (r-layout).
  static __device__ __forceinline__ void add_sources(
      const FusedArgs& a, float qs, const float* wc, const float* cm,
      const float* c0, const float* cp, int yy, int xx, const int* gc,
      float* acc, bool wlayout) {
    if (a.ph.src_id == VACGPU_SRC_GRAVITY) {
#pragma unroll
      for (int d = 1; d <= NDIM; d++) {
        float gr = (float)a.ph.src_par[d - 1];
        if (gr != 0.0f) acc[d] = acc[d] + (qs * gr) * wc[0];
      }
#pragma unroll
      for (int d = 1; d <= NDIM; d++) {
        float gr = (float)a.ph.src_par[d - 1];
        if (gr != 0.0f) acc[E] = acc[E] + (qs * gr) * wc[d];
      }
    }
    if (MHD && a.ph.divbfix) {
      const int ps = wlayout ? FB_PLANE : FR_N;
      const int rs = wlayout ? FB_X : FR_X;
      const int o = yy * rs + xx;
      const int bx = (E + 1) * ps, by = (E + 2) * ps;
      float divb = 0.5f * (c0[bx + o + 1] - c0[bx + o - 1]) * a.idxf[0][gc[0]];
      if (NDIM > 1)
        divb += 0.5f * (c0[by + o + rs] - c0[by + o - rs]) * a.idxf[1][gc[1]];
      if (NDIM > 2) {
        const int bz = (E + 3) * ps;
        divb += 0.5f * (cp[bz + o] - cm[bz + o]) * a.idxf[2][gc[2]];
      }
      divb = qs * divb;
      const float ri = 1.0f / wc[0];
      float mb = wc[1] * wc[E + 1];
#pragma unroll
      for (int k = 2; k <= NDIR; k++) mb = fmaf(wc[k], wc[E + k], mb);
#pragma unroll
      for (int k = 1; k <= NDIR; k++) {
        acc[k] = acc[k] - wc[E + k] * divb;
        acc[E + k] = acc[E + k] - wc[k] * ri * divb;
      }
      acc[E] = acc[E] - mb * ri * divb;
    }
  }

  // TVDLF flux at the face between wl/wr (predictor values) with the limited
  // slopes ldl/ldr of the base state; returns cmax.
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
    const float cmax = PH::template cmax<NDIR, MHD>(M, D, a.ph, smallp);
#pragma unroll
    for (int v = 0; v < NW; v++) L[v] = 2.0f * M[v] - R[v];
    float fL[NW], fR[NW];
    PH::template flux<NDIR, MHD>(L, D, a.ph, smallp, fL);
    PH::template flux<NDIR, MHD>(R, D, a.ph, smallp, fR);
#pragma unroll
    for (int v = 0; v < NW; v++)
      F[v] = 0.5f * (fL[v] + fR[v]) - cmax * 0.5f * (R[v] - L[v]);
    return cmax;
  }

  static __device__ __forceinline__ void ldw3(const FusedArgs& a,
                                              const float* bm,
                                              const float* b0,
                                              const float* bp, float* ld) {
#pragma unroll
    for (int v = 0; v < NW; v++)
      ld[v] = a.ph.typefull == VACGPU_TVDLF1
                  ? 0.0f
                  : lim(a, v, bp[v] - b0[v], b0[v] - bm[v]);
  }

  // One tile (bx, by) and z chunk bz of one grid.  bars: the CTA's
  // FWRING mbarriers (initialised once); uses[s]: loads completed on slot s
  // before this tile (kept identically by every thread, gives the phase
  // parity).  Returns false when a TMA wait timed out.
  static __device__ bool run(const CUtensorMap* map, const FusedArgs& a,
                             float* sm, int bx, int by, int bz,
                             unsigned long long* bars, int* uses,
                             unsigned slotid) {
    Ctrl* ctrl = a.ctrl;
    if (ctrl->done) return true;
    __shared__ unsigned long long shkey[FT_NT / 32];
    float* wring = sm;
    float* w1ring = wring + FWRING * NW * FB_PLANE;
    float* fbuf = w1ring + FW1RING * NW * FR_N;
    const int tid = threadIdx.x;
    const int lx = tid % FT_X, ly = tid / FT_X;
    const DevGrid& g = a.g;
    const int x0 = bx * FT_X, y0 = by * FT_Y;
    const int zc = NDIM == 3 ? bz : 0;
    const int z0 = NDIM == 3 ? zc * a.nzc : 0;
    const int z1 = NDIM == 3 ? min(z0 + a.nzc, g.nx[2]) : 1;  // exclusive
    const double dtd = ctrl->dt;
    const float qdt = (float)dtd;                 // corrector
    const float qdt2 = (float)(dtd / 2);          // predictor
    const float qs1 = (float)(dtd / 2 / NDIM);    // predictor source
    const float qs2 = (float)(dtd / NDIM);        // corrector source
    const float smallp = (float)ctrl->smallp;
    const int colx = x0 + g.xpad - 4 + 2;  // TMA x start (multiple of 4)
    const unsigned plane_bytes = NW * FB_PLANE * 4;

    // plane p of the mesh lives in slot (p - pbase) % FWRING
    const int pbase = NDIM == 3 ? z0 - 2 : 0;
    auto issue = [&](int p) {
      int q = p - pbase;
      float* dst = wring + (q % FWRING) * NW * FB_PLANE;
      fence_proxy_async();
      mbar_expect_tx(&bars[q % FWRING], plane_bytes);
      tma_load_plane(map, dst, &bars[q % FWRING], colx, y0, p + g.gh[2]);
    };
    auto slot = [&](int p) -> float* {
      return wring + ((p - pbase) % FWRING) * NW * FB_PLANE;
    };
    auto w1slot = [&](int p) -> float* {
      return w1ring + (((p % FW1RING) + FW1RING) % FW1RING) * NW * FR_N;
    };
    auto wait_plane = [&](int p) -> bool {
      int q = p - pbase;
      return mbar_wait(&bars[q % FWRING], (uses[q % FWRING] + q / FWRING) & 1);
    };

    unsigned long long key = 0ULL;
    const int pfirst = NDIM == 3 ? z0 - 1 : 0;   // first predictor plane
    const int plast = NDIM == 3 ? z1 : 0;        // last predictor plane
    if (tid == 0) {
      if (NDIM == 3) {
        issue(z0 - 2);
        issue(z0 - 1);
        issue(z0);
      } else {
        issue(0);
      }
    }
    // registers carried along z for D==2
    float Lprev[NW], Fprev[NW];
#pragma unroll
    for (int v = 0; v < NW; v++) Lprev[v] = Fprev[v] = 0.0f;

    for (int j = pfirst; j <= plast; j++) {
      if (NDIM == 3 && tid == 0 && j + 2 <= z1 + 1) issue(j + 2);
      // the state planes j-1, j, j+1 must be resident
      bool ok = true;
      if (NDIM == 3) {
        if (j == pfirst) ok = wait_plane(j - 1) && wait_plane(j);
        ok = ok && wait_plane(j + 1);
      } else {
        ok = wait_plane(0);
      }
      if (__syncthreads_or(!ok)) {
        if (tid == 0) atomicExch(&ctrl->fault, 1);
        return false;
      }
      const float* pm = NDIM == 3 ? slot(j - 1) : nullptr;
      const float* p0 = slot(j);
      const float* pp = NDIM == 3 ? slot(j + 1) : nullptr;
      float* w1j = w1slot(j);

      // (1) predictor of plane j: the 32x8 tile cells (one per thread),
      // then the 80 halo cells -- in full where a face flux reads them, only
      // the transverse b component where only div B reads them (MHD), not at
      // all where nothing reads them (HD).
      for (int c = tid; c < FT_NT + 80; c += FT_NT) {
        int rx, ry, hdir;  // hdir: -1 tile, 0 x-halo column, 1 y-halo row
        if (c < FT_NT) {
          rx = c % FT_X + 1;
          ry = c / FT_X + 1;
          hdir = -1;
        } else {
          const int h = c - FT_NT;
          if (h < 64) {
            rx = h % 32 + 1;
            ry = h < 32 ? 0 : FR_Y - 1;
            hdir = 1;
          } else {
            rx = h < 72 ? 0 : FR_X - 1;
            ry = (h - 64) % 8 + 1;
            hdir = 0;
          }
        }
        const int ix = x0 + rx - 1, iy = y0 + ry - 1;
        if (ix > g.nx[0] || (NDIM >= 2 && iy > g.nx[1])) continue;
        if (NDIM < 2 && hdir == 1) continue;
        const bool full = hdir < 0 || hdir == D;
        if (!full && !MHD) continue;
        const int gc[3] = {ix + 2, iy + g.gh[1], j + g.gh[2]};
        const int rc = ry * FR_X + rx;
        if (full) {
          float out[NW];
          predict_cell(a, pm, p0, pp, ry + 1, rx + 3, gc[D], gc, qdt2, qs1,
                       smallp, out);
#pragma unroll
          for (int v = 0; v < NW; v++) w1j[v * FR_N + rc] = out[v];
        } else if (MHD) {
          w1j[(E + 1 + hdir) * FR_N + rc] =
              predict_b(a, pm, p0, pp, ry + 1, rx + 3, gc[D], gc, qdt2, qs1, hdir);
        }
      }
      // D==2: limited slope of the base state at (tile cell, plane j)
      float Lcur[NW];
      if (D == 2) {
        float bm[NW], b0[NW], bp[NW];
#pragma unroll
        for (int v = 0; v < NW; v++) {
          bm[v] = W(pm, v, ly + 2, lx + 4);
          b0[v] = W(p0, v, ly + 2, lx + 4);
          bp[v] = W(pp, v, ly + 2, lx + 4);
        }
        ldw3(a, bm, b0, bp, Lcur);
      }
      __syncthreads();
      // (1b) getboundary(w1): first ghost layer of non-periodic faces
      fix_w1_ghosts(a, j, x0, y0, tid);
      __syncthreads();

      // (2)+(3): the corrector for plane jo = j-1 (3-D) or 0 (2-D)
      const int jo = NDIM == 3 ? j - 1 : 0;
      const bool out_plane = NDIM == 3 ? (jo >= z0 && jo < z1) : true;
      if (D == 2) {
        float Fnew[NW];
        if (j >= z0) {
          float wl[NW], wr[NW];
          const float* a1 = w1slot(j - 1);
          const int r = (ly + 1) * FR_X + lx + 1;
#pragma unroll
          for (int v = 0; v < NW; v++) {
            wl[v] = a1[v * FR_N + r];
            wr[v] = w1j[v * FR_N + r];
          }
          float cm = face(a, wl, wr, Lprev, Lcur, smallp, Fnew);
          const int ix = x0 + lx, iy = y0 + ly;
          if (a.ph.courantpar > 0.0 && ix < g.nx[0] && iy < g.nx[1]) {
            const int gz = j - 1 + 2;
            float q = cm * 2.0f / (a.dxf[2][gz] + a.dxf[2][gz + 1]);
            unsigned long long k = dkey((double)q);
            key = k > key ? k : key;
          }
        }
        if (out_plane)
          corrector_out(a, jo, x0, y0, lx, ly, qdt, qs2, Fprev, Fnew, pbase);
#pragma unroll
        for (int v = 0; v < NW; v++) {
          Lprev[v] = Lcur[v];
          if (j >= z0) Fprev[v] = Fnew[v];
        }
      } else if (out_plane) {
        // in-plane faces of plane jo into fbuf
        const float* bpl = slot(jo);
        const float* w1o = w1slot(jo);
        const int nf = D == 0 ? (FT_X + 1) * FT_Y : FT_X * (FT_Y + 1);
        for (int f = tid; f < nf; f += FT_NT) {
          int fx, fy;  // face between cell (rx,ry) and its +D neighbour
          if (D == 0) {
            fx = f % (FT_X + 1);
            fy = f / (FT_X + 1);
          } else {
            fx = f % FT_X;
            fy = f / FT_X;
          }
          const int ix = D == 0 ? x0 + fx - 1 : x0 + fx;
          const int iy = D == 1 ? y0 + fy - 1 : y0 + fy;
          const bool valid = (D == 0 ? (ix >= -1 && ix < g.nx[0] && iy < g.nx[1])
                                     : (iy >= -1 && iy < g.nx[1] && ix < g.nx[0]));
          if (!valid) continue;
          const int rx = ix - x0 + 1, ry = iy - y0 + 1;
          const int sx = rx + 3, sy = ry + 1;
          const int dxs = D == 0 ? 1 : 0, dys = D == 1 ? 1 : 0;
          float wl[NW], wr[NW], bm[NW], b0[NW], b1[NW], b2[NW];
#pragma unroll
          for (int v = 0; v < NW; v++) {
            wl[v] = w1o[v * FR_N + ry * FR_X + rx];
            wr[v] = w1o[v * FR_N + (ry + dys) * FR_X + rx + dxs];
            bm[v] = W(bpl, v, sy - dys, sx - dxs);
            b0[v] = W(bpl, v, sy, sx);
            b1[v] = W(bpl, v, sy + dys, sx + dxs);
            b2[v] = W(bpl, v, sy + 2 * dys, sx + 2 * dxs);
          }
          float ldl[NW], ldr[NW], F[NW];
          ldw3(a, bm, b0, b1, ldl);
          ldw3(a, b0, b1, b2, ldr);
          float cm = face(a, wl, wr, ldl, ldr, smallp, F);
#pragma unroll
          for (int v = 0; v < NW; v++) fbuf[v * FFACE + f] = F[v];
          if (a.ph.courantpar > 0.0) {
            const int gi = (D == 0 ? ix : iy) + 2;
            float q = cm * 2.0f / (a.dxf[D][gi] + a.dxf[D][gi + 1]);
            unsigned long long k = dkey((double)q);
            key = k > key ? k : key;
          }
        }
        __syncthreads();
        float Fm[NW], Fp[NW];
        const int fm = D == 0 ? ly * (FT_X + 1) + lx : ly * FT_X + lx;
        const int fp = D == 0 ? fm + 1 : fm + FT_X;
#pragma unroll
        for (int v = 0; v < NW; v++) {
          Fm[v] = fbuf[v * FFACE + fm];
          Fp[v] = fbuf[v * FFACE + fp];
        }
        corrector_out(a, jo, x0, y0, lx, ly, qdt, qs2, Fm, Fp, pbase);
      }
      __syncthreads();  // ring slots of planes j-1 (state) and j-2 reusable
    }
    {  // phase bookkeeping: planes pbase .. (NDIM==3 ? z1+1 : 0) were loaded
      const int np = NDIM == 3 ? z1 + 2 - pbase : 1;
#pragma unroll
      for (int s2 = 0; s2 < FWRING; s2++) uses[s2] += (np - s2 + FWRING - 1) / FWRING;
    }
    // CFL maximum of this CTA's faces
    if (a.ph.courantpar > 0.0) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        unsigned long long v = __shfl_xor_sync(0xffffffffu, key, o);
        key = v > key ? v : key;
      }
      if ((tid & 31) == 0) shkey[tid >> 5] = key;
      __syncthreads();
      if (tid == 0) {
        for (int i = 1; i < FT_NT / 32; i++) key = shkey[i] > key ? shkey[i] : key;
        if (key) atomicMax(&ctrl->face_cmax[D][slotid % NSLOT], key);
      }
      __syncthreads();
    }
    return true;
  }

  // getboundary on w1: cells of the predictor region in the first ghost
  // layer of a non-periodic face take the adjacent mesh value (x/y faces of
  // plane j; at z faces the whole plane).
  static __device__ __forceinline__ void fix_w1_ghosts(const FusedArgs& a,
                                                       int j, int x0, int y0,
                                                       int tid) {
    const DevGrid& g = a.g;
    extern __shared__ __align__(128) float dsm[];
    float* w1ring = dsm + FWRING * NW * FB_PLANE;
    auto w1s = [&](int p) -> float* {
      return w1ring + (((p % FW1RING) + FW1RING) % FW1RING) * NW * FR_N;
    };
    float* w1j = w1s(j);
    // x and y faces of plane j
    for (int c = tid; c < FR_N; c += FT_NT) {
      const int rx = c % FR_X, ry = c / FR_X;
      const int ix = x0 + rx - 1, iy = y0 + ry - 1;
      int d = -1, src = c, lo = 0;
      if ((ix == -1 || ix == g.nx[0]) && (NDIM < 2 || (iy >= 0 && iy < g.nx[1]))) {
        d = 0;
        lo = ix == -1;
        src = c + (lo ? 1 : -1);
      } else if (NDIM >= 2 && (iy == -1 || iy == g.nx[1]) && ix >= 0 && ix < g.nx[0]) {
        d = 1;
        lo = iy == -1;
        src = c + (lo ? FR_X : -FR_X);
      }
      if (d < 0) continue;
#pragma unroll
      for (int v = 0; v < NW; v++) {
        if ((a.periodic_mask[d] >> v) & 1) continue;
        const int asy = lo ? a.asymm_lo[d] : a.asymm_hi[d];
        float s = w1j[v * FR_N + src];
        w1j[v * FR_N + c] = ((asy >> v) & 1) ? -s : s;
      }
    }
    if (NDIM == 3) {
      // z faces: plane -1 from plane 0 (now, at j == 0); plane nz from nz-1
      int dst = 0, srcp = 0, lo = 0;
      bool any = false;
      if (j == 0) { dst = -1; srcp = 0; lo = 1; any = true; }
      if (j == g.nx[2]) { dst = j; srcp = j - 1; lo = 0; any = true; }
      if (any) {
        __syncthreads();  // the x/y ghost fix of the source plane is done
        float* dp = w1s(dst);
        const float* sp = w1s(srcp);
        const int asy = lo ? a.asymm_lo[2] : a.asymm_hi[2];
        for (int c = tid; c < FR_N; c += FT_NT) {
#pragma unroll
          for (int v = 0; v < NW; v++) {
            if ((a.periodic_mask[2] >> v) & 1) continue;
            float s = sp[v * FR_N + c];
            dp[v * FR_N + c] = ((asy >> v) & 1) ? -s : s;
          }
        }
      }
    }
  }

  // Corrected state of one tile cell of plane jo: wnew = w - qdt/dx*(F+ - F-)
  // + sources(w1), written to HBM.
  static __device__ __forceinline__ void corrector_out(
      const FusedArgs& a, int jo, int x0, int y0, int lx, int ly, float qdt,
      float qs, const float* Fm, const float* Fp, int pbase) {
    const DevGrid& g = a.g;
    const int ix = x0 + lx, iy = y0 + ly;
    if (ix >= g.nx[0] || (NDIM >= 2 && iy >= g.nx[1])) return;
    extern __shared__ __align__(128) float dsm[];
    const float* bpl = dsm + ((jo - pbase) % FWRING) * NW * FB_PLANE;
    float* w1ring = dsm + FWRING * NW * FB_PLANE;
    auto w1s = [&](int p) -> const float* {
      return w1ring + (((p % FW1RING) + FW1RING) % FW1RING) * NW * FR_N;
    };
    const float* c0 = w1s(jo);
    const float* cm = NDIM == 3 ? w1s(jo - 1) : nullptr;
    const float* cp = NDIM == 3 ? w1s(jo + 1) : nullptr;
    const int rx = lx + 1, ry = ly + 1;
    const int gc[3] = {ix + 2, iy + g.gh[1], jo + g.gh[2]};
    float acc[NW], wc[NW];
#pragma unroll
    for (int v = 0; v < NW; v++) {
      acc[v] = W(bpl, v, ly + 2, lx + 4);
      wc[v] = c0[v * FR_N + ry * FR_X + rx];
    }
    const float cq = qdt * a.idxf[D][gc[D]];
#pragma unroll
    for (int v = 0; v < NW; v++) acc[v] = acc[v] - cq * (Fp[v] - Fm[v]);
    if (a.ph.sourceunsplit) add_sources(a, qs, wc, cm, c0, cp, ry, rx, gc, acc, false);
    const long long off = gidx(g, gc[0], gc[1], gc[2]);
#pragma unroll
    for (int v = 0; v < NW; v++) a.wout[off + v * g.vs] = acc[v];
  }
};

__device__ __forceinline__ void init_bars(unsigned long long* bars) {
  if (threadIdx.x == 0) {
    for (int i = 0; i < FWRING; i++) mbar_init(&bars[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
}

template <int NDIM, int D, bool MHD, int PM, int LIMC>
__global__ void __launch_bounds__(FT_NT, 2)
    k_sweep_fused(const __grid_constant__ CUtensorMap map, FusedArgs a) {
  extern __shared__ __align__(128) float dsm[];
  __shared__ __align__(8) unsigned long long bars[FWRING];
  init_bars(bars);
  int uses[FWRING] = {0, 0, 0, 0};
  const unsigned slotid = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  Fused<NDIM, D, MHD, PM, LIMC>::run(&map, a, dsm, blockIdx.x, blockIdx.y,
                                     blockIdx.z, bars, uses, slotid);
}

}  // namespace vacgpu

// sweep_line2.cuh - the fused sweep of the mixed-precision path for 2-D
// grids as warp-marching lines, two cells per thread in packed FP32.
//
// One split sweep of VAC's twostep Hancock/TVDLF scheme (src/vac.t:363-572,
// src/vactvdlf.t:5-299): Hancock predictor w1 (src/vactvdlf.t:5-89), TVDLF
// corrector with the limited slopes of the base state
// (src/vactvdlf.t:92-299), Powell and gravity sources, CFL maximum and the
// ghost cells of the new state, in one kernel -- what sweep_pair.cuh does
// for 3-D grids, laid out for 2-D ones.
//
// A warp owns a strip of 64 columns (lane l: columns 2l and 2l+1 of the
// strip, one f2 pair per variable) and marches along y through a chunk of
// rows.  Rows arrive by coalesced 8-byte loads straight into registers, one
// row ahead of use; there is no shared memory and no barrier, so the warps
// of a CTA are independent work items.
//
// x sweep: the sweep direction lies along the strip; neighbours come from
// warp shuffles, so a strip computes 60 output columns (two halo columns on
// either side).  The predictor runs one row ahead of the corrector because
// Powell's div B of w1 at row r needs B_y of w1 at rows r-1 and r+1 (MHD).
// y sweep: the sweep direction is the marching direction; a thread carries
// its columns' state, predictor, slopes and face flux from row to row.  MHD
// strips keep two halo columns (B_x of w and w1 at x+-1 for div B; 60
// outputs), HD strips none (64 outputs).
//
// Ghost semantics follow getboundary applied to w1 after the predictor
// (src/vac.t:567): at a 'periodic' face the predictor is evaluated at the
// ghost position from the (periodic copy) ghost values of w; at 'cont',
// 'symm' and 'asymm' faces w1 in the first ghost layer is the adjacent mesh
// value (sign-flipped for 'asymm').  Each output cell within two cells of a
// mesh face also writes its value to the ghost positions whose boundary
// maps land on it, so the next sweep reads filled ghost cells.
#pragma once

#include "batch_items.cuh"
#include "pack2.cuh"
#include "sweep_pair.cuh"

namespace vacgpu {

constexpr int L2_NT = 128;   // threads per CTA: four independent warps
constexpr int L2_ROWS = 32;  // rows per work item
constexpr int L2_LOOK = 3;   // rows in flight ahead of use
constexpr int L2_RING = L2_LOOK + 1;  // staging slots per warp
// a batched work item's strip is bx & L2_STRIP; bit 30 of bx is its sweep
// direction
constexpr int L2_STRIP = (1 << 30) - 1;

// A staged row holds, per variable, 68 floats: the strip's 64 columns from
// the 16-byte boundary at or below its first one (2 columns earlier when
// the strip has halo columns).
constexpr int L2_ROWF = 68;

// floats of one warp's row-staging ring for nw variables
__host__ __device__ constexpr int line2_ring_floats(int nw) { return L2_RING * nw * L2_ROWF; }

template <int D, bool MHD, int LIMC, bool GEN>
struct Line2 {
  static constexpr int NW = MHD ? 6 : 4;
  static constexpr int E = 3;                  // e
  // B_x, B_y (MHD; index 0 stands in for HD, whose code never reads them)
  static constexpr int BX = MHD ? 4 : 0, BY = MHD ? 5 : 0;
  static constexpr int HALO = (D == 0 || MHD) ? 2 : 0;
  static constexpr int TW = 64 - 2 * HALO;     // output columns per strip
  static constexpr unsigned FULL = 0xffffffffu;
  typedef PairSweep<2, MHD, LIMC, GEN> PS;     // for gfix
  typedef Fused<3, 0, true, PREC_FF, LIMC_MINMOD> FX;  // for preimages

  // Per-warp constants of a work item.
  struct Ctx {
    const float* win;   // element (gx, gy) of variable v: win[v*vs + gy*P + gx]
    float* wout;        // the same layout
    int P;              // row pitch and variable stride (elements; 2-D states
    int vs;             // stay below 2^31 elements)
    const float* idy;   // 1/dy and dy over the ghost range
    const float* dy;
    // boundary variable masks of the x and y faces, 8 bits each: periodic
    // (bits 0-7), 'asymm' at the low face (8-15) and at the high face (16-23)
    int bmx, bmy;
    int c0;             // first column of the pair
    int nX, nY;         // mesh cells
    int gy_hi;          // last row of the ghost range (nY + 3)
    bool ok0, ok1;      // the pair's cells are outputs of this strip
    bool fv0, fv1;      // x sweep: the pair's two faces enter the CFL maximum
    f2 idxx, cflx, qdt2, qs1, qs2, nqs1h, nqs2h;
    float qdt;
    bool powell, srcs, cfl, fix_x, fix_y;
    int cs;             // first staged column (16-byte aligned element)
    int cmax4;          // last 16-byte aligned column a row can be read from
    PairK k;
  };

  // Rows reach registers through a per-warp ring of L2_RING slots in
  // shared memory, fed by cp.async 16-byte copies (.cg: through L2 only, so
  // a kernel that runs several steps never reads a stale L1 line) L2_LOOK
  // rows ahead of use; rows in flight hold no registers.  The lanes copy the
  // row's 16-byte chunks between them (chunk q: variable q / 17, columns
  // 4 (q % 17) .. +3 of the staged row) and each reads back its own pair
  // after a warp barrier.  Rows are issued and pulled strictly in order; a
  // pull waits until at most L2_LOOK-1 copies are outstanding (its own row
  // has landed) and issues the next row, whose slot every lane read one pull
  // earlier (before this pull's warp barrier).
  static constexpr int NCHUNK = NW * (L2_ROWF / 4);
  struct Pipe {
    unsigned sm;  // shared address of this warp's ring
    int issued;   // next row to issue
    int rd;       // byte offset of this lane's pair within a variable's row
  };

  static __device__ __forceinline__ void issue_row(const Ctx& c, Pipe& pp) {
    const int gy = min(pp.issued, c.gy_hi);  // rows past the ghost range are not used
    const float* row = c.win + (long long)gy * c.P;
    const unsigned s = pp.sm + (unsigned)((pp.issued % L2_RING) * NW * L2_ROWF * 4);
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int q0 = 0; q0 < NCHUNK; q0 += 32) {
      const int q = q0 + lane;
      if (q < NCHUNK) {
        const int v = q / (L2_ROWF / 4), col = c.cs + 4 * (q % (L2_ROWF / 4));
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s + q * 16),
                     "l"(row + v * c.vs + min(col, c.cmax4))
                     : "memory");
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    pp.issued++;
  }

  static __device__ __forceinline__ void prime(const Ctx& c, Pipe& pp, int first) {
    pp.issued = first;
#pragma unroll
    for (int i = 0; i < L2_LOOK; i++) issue_row(c, pp);
  }

  static __device__ __forceinline__ void pull(const Ctx& c, Pipe& pp, int gy, f2* u) {
    asm volatile("cp.async.wait_group %0;" ::"n"(L2_LOOK - 1) : "memory");
    __syncwarp();
    const unsigned s = pp.sm + (unsigned)((gy % L2_RING) * NW * L2_ROWF * 4) + pp.rd;
#pragma unroll
    for (int v = 0; v < NW; v++) {
      float lo, hi;
      asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];"
                   : "=f"(lo), "=f"(hi)
                   : "r"(s + v * L2_ROWF * 4));
      u[v] = f2m(lo, hi);
    }
    issue_row(c, pp);
  }

  static __device__ __forceinline__ void drain() {
    asm volatile("cp.async.wait_all;" ::: "memory");
  }

  // getboundary of w1 at the x faces of a strip that reaches them: the
  // first ghost column takes the adjacent mesh value (non-periodic
  // variables, negated where 'asymm')
  static __device__ __forceinline__ void fix_w1_x(const FusedArgs& a, const Ctx& c, f2* w1) {
#pragma unroll
    for (int v = 0; v < NW; v++) {
      float lo, hi;
      f2u(w1[v], lo, hi);
      const float dn = __shfl_down_sync(FULL, lo, 1);
      const float up = __shfl_up_sync(FULL, hi, 1);
      const int pm = c.bmx & 255, al = (c.bmx >> 8) & 255, ah = c.bmx >> 16;
      if (c.c0 + 1 == 1) hi = PS::gfix(hi, dn, v, pm, al);
      if (c.c0 == c.nX + 2) lo = PS::gfix(lo, up, v, pm, ah);
      if (c.c0 + 1 == c.nX + 2) hi = PS::gfix(hi, lo, v, pm, ah);
      w1[v] = f2m(lo, hi);
    }
  }

  // the same along y: value `own` of the ghost row replaced from `src`
  static __device__ __forceinline__ f2 fix_y1(const Ctx& c, f2 own, f2 src, int v, int amask) {
    float ol, oh, sl, sh;
    f2u(own, ol, oh);
    f2u(src, sl, sh);
    return f2m(PS::gfix(ol, sl, v, c.bmy & 255, amask), PS::gfix(oh, sh, v, c.bmy & 255, amask));
  }

  // addsource2 with wCT = wc: gravity, then Powell's terms for
  // nq = -qs div B (as PairSweep::sources, 2-D states)
  static __device__ __forceinline__ void sources(const FusedArgs& a, const Ctx& c, f2 qs,
                                                 const f2* wc, f2 nq, f2* acc) {
    if (GEN && a.ph.src_id == VACGPU_SRC_GRAVITY) {
#pragma unroll
      for (int d = 1; d <= 2; d++)
        if (a.gravf[d - 1] != 0.0f) acc[d] = ffma(qs * f2s(a.gravf[d - 1]), wc[0], acc[d]);
#pragma unroll
      for (int d = 1; d <= 2; d++)
        if (a.gravf[d - 1] != 0.0f) acc[E] = ffma(qs * f2s(a.gravf[d - 1]), wc[d], acc[E]);
    }
    if constexpr (MHD) {
      if (c.powell) {
        const f2 t = vrcp(wc[0]) * nq;
        f2 mb = wc[1] * wc[BX];
        mb = ffma(wc[2], wc[BY], mb);
#pragma unroll
        for (int d = 1; d <= 2; d++) {
          acc[d] = ffma(wc[E + d], nq, acc[d]);
          acc[E + d] = ffma(wc[d], t, acc[E + d]);
        }
        acc[E] = ffma(mb, t, acc[E]);
      }
    }
  }

  // TVDLF face flux 2F = F(L) + F(R) - cmax (R - L) of a pair of faces
  static __device__ __forceinline__ f2 face(const f2* L, const f2* R, const PairK& k, f2* G) {
    f2 fL[NW], fR[NW], pL, pR, riL, riR;
    p_flux<D, MHD, 2>(L, k, fL, pL, riL);
    p_flux<D, MHD, 2>(R, k, fR, pR, riR);
    f2 M[NW];
    M[0] = k.half * (L[0] + R[0]);
    M[1 + D] = k.half * (L[1 + D] + R[1 + D]);
    if (MHD) {
      M[BX] = k.half * (L[BX] + R[BX]);
      M[BY] = k.half * (L[BY] + R[BY]);
    }
    const f2 cm = p_cmax_mean<D, MHD, 2>(L, R, M, pL, pR, riL, riR, k);
#pragma unroll
    for (int v = 0; v < NW; v++) G[v] = ffma(cm, L[v] - R[v], fL[v] + fR[v]);
    return cm;
  }

  // Hancock predictor of a pair from the state u and its half slopes hl;
  // cq = dt/2/dx along D; divb: div B of w at the pair
  static __device__ __forceinline__ void predict(const FusedArgs& a, const Ctx& c,
                                                 const f2* u, const f2* hl, f2 cq, f2 divb,
                                                 f2* w1) {
    f2 uL[NW], uR[NW], fL[NW], fR[NW], pt_, ri_;
#pragma unroll
    for (int v = 0; v < NW; v++) {
      uR[v] = u[v] - hl[v];
      uL[v] = u[v] + hl[v];
    }
    p_flux<D, MHD, 2>(uR, c.k, fR, pt_, ri_);
    p_flux<D, MHD, 2>(uL, c.k, fL, pt_, ri_);
#pragma unroll
    for (int v = 0; v < NW; v++) w1[v] = ffma(cq, fR[v] - fL[v], u[v]);
    if (c.srcs) sources(a, c, c.qs1, u, c.nqs1h * divb, w1);
  }

  // getboundary's ghost images of one new cell value (gx, gy) (one lane):
  // the composition of the region copies of src/vacgrid.t:195-413
  static __device__ __forceinline__ void ghost_images(const FusedArgs& a, const Ctx& c,
                                                      int gx, int gy, const float* s) {
    int x1, x2, fx, y1, y2, fy;
    const int nx_ = 1 + FX::preimages(a, 0, gx, x1, fx, x2);
    const int ny_ = 1 + FX::preimages(a, 1, gy, y1, fy, y2);
#pragma unroll 1
    for (int jj = 0; jj < ny_; jj++) {
      const int py = jj == 0 ? gy : (jj == 1 ? y1 : y2);
      const int sy = jj == 1 ? fy : 0;
#pragma unroll 1
      for (int i = 0; i < nx_; i++) {
        if ((i | jj) == 0) continue;
        const int px = i == 0 ? gx : (i == 1 ? x1 : x2);
        const int fl = (i == 1 ? fx : 0) ^ sy;
        float* o = c.wout + (long long)py * c.P + px;
#pragma unroll
        for (int v = 0; v < NW; v++) o[v * c.vs] = ((fl >> v) & 1) ? -s[v] : s[v];
      }
    }
  }

  // the new state of the pair at row gy, with ghost images near faces
  static __device__ __forceinline__ void store(const FusedArgs& a, const Ctx& c, int gy,
                                               const f2* acc) {
    float* o = c.wout + (long long)gy * c.P + c.c0;
    if (c.ok0 && c.ok1) {
#pragma unroll
      for (int v = 0; v < NW; v++) st2(o + v * c.vs, acc[v]);
    } else {
#pragma unroll
      for (int v = 0; v < NW; v++) {
        float lo, hi;
        f2u(acc[v], lo, hi);
        if (c.ok0) o[v * c.vs] = lo;
        if (c.ok1) o[1 + v * c.vs] = hi;
      }
    }
    const bool neary = gy < 4 || gy >= c.nY;
    if (!(neary || c.c0 < 4 || c.c0 + 1 >= c.nX)) return;
#pragma unroll 1
    for (int h = 0; h < 2; h++) {
      const int gx = c.c0 + h;
      if (!(h ? c.ok1 : c.ok0) || !(neary || gx < 4 || gx >= c.nX)) continue;
      float s[NW];
#pragma unroll
      for (int v = 0; v < NW; v++) s[v] = h ? f2hi(acc[v]) : f2lo(acc[v]);
      ghost_images(a, c, gx, gy, s);
    }
  }

  static __device__ __forceinline__ void cfl_fold(f2 cm, f2 cf, bool v0, bool v1, f2& qmax) {
    float cl, ch, ql, qh;
    f2u(cm * cf, cl, ch);
    f2u(qmax, ql, qh);
    if (v0) ql = (cl > ql || cl != cl) ? cl : ql;
    if (v1) qh = (ch > qh || ch != ch) ? ch : qh;
    qmax = f2m(ql, qh);
  }

  // ------------------------------------------------------------ x sweep

  // predictor of one row; bd, bu: B_y of w at the rows below and above
  static __device__ __forceinline__ void predict_x(const FusedArgs& a, const Ctx& c,
                                                   const f2* u, f2 bd, f2 bu, int gy,
                                                   f2* w1, f2* hl) {
    f2 dbx = f2s(0.0f);
#pragma unroll
    for (int v = 0; v < NW; v++) {
      float cl, ch;
      f2u(u[v], cl, ch);
      const float lft = __shfl_up_sync(FULL, ch, 1), rgt = __shfl_down_sync(FULL, cl, 1);
      const float d1 = ch - cl;
      const f2 dp = f2m(d1, rgt - ch), dm = f2m(cl - lft, d1);
      if (MHD && v == BX) dbx = f2m(ch - lft, rgt - cl);
      hl[v] = p_hlim<LIMC>(dp, dm, c.k);
    }
    f2 divb = f2s(0.0f);
    if (MHD && c.powell) divb = ffma(bu - bd, f2s(c.idy[gy]), dbx * c.idxx);
    predict(a, c, u, hl, c.qdt2 * c.idxx, divb, w1);
    if (GEN && c.fix_x) fix_w1_x(a, c, w1);
  }

  // rows gya .. gyb-1 (ghost-range indices)
  static __device__ void run_x(const FusedArgs& a, const Ctx& c, Pipe& pp, int gya, int gyb,
                               f2& qmax) {
    // carried: w of rows r and r+1 (MHD); w1 and half slopes of row r; B_y
    // of w1 at row r-1 (MHD)
    f2 w0[NW], wp[NW], w1c[NW], hlc[NW];
    f2 by1m = f2s(0.0f);
    if (MHD) {
      f2 wmm[NW], wm[NW], t1[NW], th[NW];
      prime(c, pp, gya - 2);
      pull(c, pp, gya - 2, wmm);
      pull(c, pp, gya - 1, wm);
      pull(c, pp, gya, w0);
      pull(c, pp, gya + 1, wp);
      predict_x(a, c, wm, wmm[BY], w0[BY], gya - 1, t1, th);
      by1m = t1[BY];
      predict_x(a, c, w0, wm[BY], wp[BY], gya, w1c, hlc);
    } else {
      prime(c, pp, gya);
      pull(c, pp, gya, w0);
      predict_x(a, c, w0, w0[0], w0[0], gya, w1c, hlc);
    }
    const f2 ncq = f2s(-0.5f * c.qdt) * c.idxx;
    for (int r = gya; r < gyb; r++) {
      // predictor of row r+1: its state, and B_y of w at rows r and r+2 (MHD)
      f2 w1n[NW], hln[NW], wn[NW];
      if (MHD) {
        pull(c, pp, r + 2, wn);
        predict_x(a, c, wp, w0[BY], wn[BY], r + 1, w1n, hln);
      } else {
        pull(c, pp, r + 1, wn);
        predict_x(a, c, wn, wn[0], wn[0], r + 1, w1n, hln);
      }
      // B_y of w1 at rows r-1 and r+1; ghost rows of non-periodic y faces
      // take the adjacent mesh row's
      f2 byd = by1m, byu = w1n[BY];
      if (MHD && GEN && c.fix_y) {
        if (r == 2) byd = fix_y1(c, byd, w1c[BY], BY, (c.bmy >> 8) & 255);
        if (r == c.nY + 1) byu = fix_y1(c, byu, w1c[BY], BY, c.bmy >> 16);
      }
      // faces (c0|c0+1) and (c0+1|c0+2): the right state of the second from
      // the next lane
      f2 L[NW], R[NW], G[NW];
#pragma unroll
      for (int v = 0; v < NW; v++) {
        float rl, rh;
        f2u(w1c[v] - hlc[v], rl, rh);
        const float nb = __shfl_down_sync(FULL, rl, 1);
        L[v] = w1c[v] + hlc[v];
        R[v] = f2m(rh, nb);
      }
      const f2 cm = face(L, R, c.k, G);
      if (c.cfl) cfl_fold(cm, c.cflx, c.fv0, c.fv1, qmax);
      // flux differences of the pair's cells
#pragma unroll
      for (int v = 0; v < NW; v++) {
        float gl, gh;
        f2u(G[v], gl, gh);
        const float gm = __shfl_up_sync(FULL, gh, 1);
        G[v] = f2m(gl - gm, gh - gl);
      }
      f2 acc[NW];
#pragma unroll
      for (int v = 0; v < NW; v++) acc[v] = ffma(ncq, G[v], w0[v]);
      if (c.srcs) {
        f2 divb = f2s(0.0f);
        if (MHD && c.powell) {
          float bl, bh;
          f2u(w1c[BX], bl, bh);
          const float bm_ = __shfl_up_sync(FULL, bh, 1);
          const float bp_ = __shfl_down_sync(FULL, bl, 1);
          divb = ffma(byu - byd, f2s(c.idy[r]), f2m(bh - bm_, bp_ - bl) * c.idxx);
        }
        sources(a, c, c.qs2, w1c, c.nqs2h * divb, acc);
      }
      if (c.ok0 || c.ok1) store(a, c, r, acc);
      by1m = w1c[BY];
#pragma unroll
      for (int v = 0; v < NW; v++) {
        if (MHD) {
          w0[v] = wp[v];
          wp[v] = wn[v];
        } else {
          w0[v] = wn[v];
        }
        w1c[v] = w1n[v];
        hlc[v] = hln[v];
      }
    }
  }

  // ------------------------------------------------------------ y sweep

  // output rows gya .. gyb-1: iterations r = gya-1 .. gyb predict row r,
  // form the face (r-1|r) and update row r-1
  static __device__ void run_y(const FusedArgs& a, const Ctx& c, Pipe& pp, int gya, int gyb,
                               f2& qmax) {
    f2 wm[NW], w0[NW], wp[NW], w1p[NW], hlp[NW], Gp[NW];
    f2 b1pp = f2s(0.0f);  // B_y of w1 at row r-2
    prime(c, pp, gya - 2);
    pull(c, pp, gya - 2, wm);
    pull(c, pp, gya - 1, w0);
    pull(c, pp, gya, wp);
#pragma unroll
    for (int v = 0; v < NW; v++) w1p[v] = hlp[v] = Gp[v] = f2s(0.0f);
    float idp = c.idy[gya - 2], dyp = c.dy[gya - 2];  // row r-1
    float idc = c.idy[gya - 1], dyc = c.dy[gya - 1];  // row r
    for (int r = gya - 1; r <= gyb; r++) {
      f2 wn[NW];
      pull(c, pp, r + 2, wn);
      const float idn = c.idy[min(r + 1, c.gy_hi)], dyn = c.dy[min(r + 1, c.gy_hi)];
      // predictor of row r
      f2 w1[NW], hl[NW];
#pragma unroll
      for (int v = 0; v < NW; v++) hl[v] = p_hlim<LIMC>(wp[v] - w0[v], w0[v] - wm[v], c.k);
      f2 divb = f2s(0.0f);
      if (MHD && c.powell) {
        float bl, bh;
        f2u(w0[BX], bl, bh);
        const float bm_ = __shfl_up_sync(FULL, bh, 1);
        const float bp_ = __shfl_down_sync(FULL, bl, 1);
        divb = ffma(wp[BY] - wm[BY], f2s(idc), f2m(bh - bm_, bp_ - bl) * c.idxx);
      }
      predict(a, c, w0, hl, c.qdt2 * f2s(idc), divb, w1);
      if (GEN && c.fix_x) fix_w1_x(a, c, w1);
      // ghost rows of non-periodic y faces: w1 of row 1 from row 2, of row
      // nY+2 from row nY+1
      if (GEN && c.fix_y) {
        if (r == 2) {
#pragma unroll
          for (int v = 0; v < NW; v++) w1p[v] = fix_y1(c, w1p[v], w1[v], v, (c.bmy >> 8) & 255);
        }
        if (r == c.nY + 2) {
#pragma unroll
          for (int v = 0; v < NW; v++) w1[v] = fix_y1(c, w1[v], w1p[v], v, c.bmy >> 16);
        }
      }
      // face (r-1|r)
      f2 L[NW], R[NW], G[NW];
#pragma unroll
      for (int v = 0; v < NW; v++) {
        L[v] = w1p[v] + hlp[v];
        R[v] = w1[v] - hl[v];
      }
      const f2 cm = face(L, R, c.k, G);
      if (c.cfl && r >= gya) cfl_fold(cm, f2s(2.0f / (dyp + dyc)), c.ok0, c.ok1, qmax);
      // update of row r-1 (div B of its w1: the x part from the neighbour
      // lanes, formed by every lane before the branch)
      f2 db = f2s(0.0f);
      if (MHD && c.srcs && c.powell) {
        float bl, bh;
        f2u(w1p[BX], bl, bh);
        const float bm_ = __shfl_up_sync(FULL, bh, 1);
        const float bp_ = __shfl_down_sync(FULL, bl, 1);
        db = ffma(w1[BY] - b1pp, f2s(idp), f2m(bh - bm_, bp_ - bl) * c.idxx);
      }
      if (r - 1 >= gya && r - 1 < gyb && (c.ok0 || c.ok1)) {
        const f2 ncq = f2s(-0.5f * c.qdt) * f2s(idp);
        f2 acc[NW];
#pragma unroll
        for (int v = 0; v < NW; v++) acc[v] = ffma(ncq, G[v] - Gp[v], wm[v]);
        if (c.srcs) sources(a, c, c.qs2, w1p, c.nqs2h * db, acc);
        store(a, c, r - 1, acc);
      }
      b1pp = w1p[BY];
#pragma unroll
      for (int v = 0; v < NW; v++) {
        w1p[v] = w1[v];
        hlp[v] = hl[v];
        Gp[v] = G[v];
        wm[v] = w0[v];
        w0[v] = wp[v];
        wp[v] = wn[v];
      }
      idp = idc;
      dyp = dyc;
      idc = idn;
      dyc = dyn;
    }
  }

  // One work item: strip sx, output rows gya .. gyb-1; win/wout: the state
  // buffers (without the row offset); ring: this warp's row-staging area of
  // line2_ring_floats(NW) floats in shared memory.
  static __device__ void run(const FusedArgs& a, const float* win, float* wout, float* ring,
                             int sx, int gya, int gyb, unsigned slot) {
    Ctrl* ctrl = a.ctrl;
    // control fields through L2: a persistent batch kernel sets them on
    // another SM earlier in the same launch
    if (__ldcg(&ctrl->done)) return;
    const DevGrid& g = a.g;
    const int lane = threadIdx.x & 31;
    Ctx c;
    c.win = win + g.xpad;
    c.wout = wout + g.xpad;
    c.vs = (int)g.vs;
    c.idy = a.idxf[1];
    c.dy = a.dxf[1];
    c.bmx = a.periodic_mask[0] | a.asymm_lo[0] << 8 | a.asymm_hi[0] << 16;
    c.bmy = a.periodic_mask[1] | a.asymm_lo[1] << 8 | a.asymm_hi[1] << 16;
    c.P = (int)g.P;
    c.nX = g.nx[0];
    c.nY = g.nx[1];
    c.gy_hi = g.nG[1] - 1;
    const int gxs = 2 - HALO + TW * sx;
    c.c0 = gxs + 2 * lane;
    c.cs = HALO ? gxs - 2 : gxs;
    c.cmax4 = (int)g.P - 4 - g.xpad;
    const int ob = gxs + HALO, oe = min(gxs + HALO + TW, c.nX + 2);
    c.ok0 = c.c0 >= ob && c.c0 < oe;
    c.ok1 = c.c0 + 1 >= ob && c.c0 + 1 < oe;
    // x sweep: faces with valid neighbours on both sides (left cells
    // gxs+1 .. gxs+61) that are mesh faces (left cells 1 .. nX+1)
    c.fv0 = c.c0 >= gxs + 1 && c.c0 <= gxs + 61 && c.c0 >= 1 && c.c0 <= c.nX + 1;
    c.fv1 = c.c0 + 1 >= gxs + 1 && c.c0 + 1 <= gxs + 61 && c.c0 + 1 <= c.nX + 1;
    const int gxa = min(c.c0, g.nG[0] - 1), gxb = min(c.c0 + 1, g.nG[0] - 1),
              gxc = min(c.c0 + 2, g.nG[0] - 1);
    c.idxx = f2m(a.idxf[0][gxa], a.idxf[0][gxb]);
    c.cflx = f2m(2.0f / (a.dxf[0][gxa] + a.dxf[0][gxb]), 2.0f / (a.dxf[0][gxb] + a.dxf[0][gxc]));
    const double dtd = __ldcg(&ctrl->dt);
    c.qdt = (float)dtd;
    c.qdt2 = f2s((float)(dtd / 2));
    c.nqs1h = f2s(-((float)(dtd / 2 / 2) * 0.5f));  // -predictor source x 1/2
    c.qs2 = f2s((float)(dtd / 2));                   // corrector source
    c.nqs2h = f2s(-((float)(dtd / 2) * 0.5f));
    c.qs1 = f2s((float)(dtd / 2 / 2));
    c.k.gm1 = f2s(a.ph.gm1f);
    c.k.gamma = f2s(a.ph.gammaf);
    c.k.half = f2s(0.5f);
    c.k.mhalf = f2s(-0.5f);
    c.k.quarter = f2s(0.25f);
    c.k.eighth = f2s(0.125f);
    c.k.mone = f2s(-1.0f);
    c.k.smallp = (float)__ldcg(&ctrl->smallp);
    c.powell = MHD && (!GEN || (a.ph.divbfix && a.ph.sourceunsplit));
    c.srcs = !GEN || a.ph.sourceunsplit;
    c.cfl = !GEN || a.cfl;
    const int all = (1 << NW) - 1;
    c.fix_x = GEN && (c.bmx & 255) != all && (gxs <= 1 || gxs + 63 >= c.nX + 2);
    c.fix_y = GEN && (c.bmy & 255) != all;
    f2 qmax = f2s(0.0f);
    Pipe pp;
    pp.sm = smem_u32(ring);
    pp.rd = (c.c0 - c.cs) * 4;
    if (D == 0)
      run_x(a, c, pp, gya, gyb, qmax);
    else
      run_y(a, c, pp, gya, gyb, qmax);
    drain();  // the ring's last copies land before the next item reuses it
    if (c.cfl) {
      float q;
      {
        const float l = f2lo(qmax), h = f2hi(qmax);
        q = (h > l || h != h) ? h : l;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float v = __shfl_xor_sync(FULL, q, o);
        q = (v > q || v != v) ? v : q;
      }
      if (lane == 0 && q != 0.0f) atomicMax(&ctrl->face_cmax[D][slot % NSLOT], dkey((double)q));
    }
  }
};

}  // namespace vacgpu

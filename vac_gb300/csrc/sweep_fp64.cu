// sweep_fp64.cu - the plain FP64 path: state, fluxes and every intermediate
// in IEEE double, in the reference's operation order.  Built with
// -fmad=false so no multiply-add is contracted, which keeps each value
// bit-identical to the FP64 CPU restatement of the reference.
#include "physics.cuh"
#include "sweep.cuh"

namespace vacgpu {

struct PH64 {
  typedef double T;
  typedef double R;
  static __device__ __forceinline__ R limiter(int lim, R a, R b) {
    return limiter_fn(lim, a, b);
  }
  template <int NDIR, bool MHD>
  static __device__ __forceinline__ void flux(const R* u, int d,
                                              const DevPhys& k, R smallp,
                                              R* f) {
    flux_fn<NDIR, MHD>(u, d, k, smallp, f);
  }
  template <int NDIR, bool MHD>
  static __device__ __forceinline__ R cmax(const R* u, int d,
                                           const DevPhys& k, R smallp) {
    return cmax_fn<NDIR, MHD>(u, d, k, smallp);
  }
  template <int NDIR, bool MHD>
  static __device__ __forceinline__ double pthermal_raw(const R* u,
                                                        const DevPhys& k) {
    return vacgpu::pthermal_raw<NDIR, MHD>(u, k);
  }
  // dx(ix,idim) (gridsetup1, src/vacgrid.t:527-530)
  static __device__ __forceinline__ R dx(const DevArrays& a, int d, int i) {
    return a.dx[d][i];
  }
  // qdt/dx(ix,idim) of addflux (src/vacgrid.t:676-677)
  static __device__ __forceinline__ R qdx(double qdt, const DevArrays& a,
                                          int d, int i) {
    return qdt / a.dx[d][i];
  }
  // cmaxC*two/(dx(ixC)+dx(jxC)) (src/vactvdlf.t:188-190)
  static __device__ __forceinline__ double cfl(R cm, const DevArrays& a,
                                               int d, int i) {
    return cm * 2.0 / (a.dx[d][i] + a.dx[d][i + 1]);
  }
  // cmax/dx of getdt_courant (src/vac.t:701-702)
  static __device__ __forceinline__ double cell_ratio(R cm,
                                                      const DevArrays& a,
                                                      int d, int i) {
    return cm / a.dx[d][i];
  }
  static __device__ __forceinline__ R mul_qg(double qdt, double g) {
    return qdt * g;
  }
  static __device__ __forceinline__ R qdiv(double q) { return q; }
};

VACGPU_DEFINE_LAUNCHERS(fp64, PH64)

}  // namespace vacgpu

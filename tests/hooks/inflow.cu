// A specialbound test hook for the engine (vacgpu_register_bound): the
// device twin of inflow.c,
//   w(ghost) = 0.5*(w(edge) + (1+0.1*iw)*(1+0.1*qt)) + 0.01*x_idim(ghost),
// computed in double and stored in the state's type.  Build with
// -fmad=false so it rounds as the host hook does.
#include <cuda_runtime.h>

#include "../../include/vacgpu.h"

template <typename T>
__global__ void k_inflow(T* w, vacgpu_region r) {
  const int idim = r.iB / 2, upper = r.iB % 2;
  int ext[3];
  for (int d = 0; d < 3; d++) ext[d] = r.hi[d] - r.lo[d] + 1;
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long tot = (long long)ext[0] * ext[1] * ext[2];
  if (n >= tot) return;
  int c[3];
  c[0] = r.lo[0] + (int)(n % ext[0]);
  c[1] = r.lo[1] + (int)((n / ext[0]) % ext[1]);
  c[2] = r.lo[2] + (int)(n / ((long long)ext[0] * ext[1]));
  const int e = upper ? r.lo[idim] - 1 : r.hi[idim] + 1;
  const double qt = *r.qt;
  const double xc = r.x[idim][c[idim]];
  const long long ix = r.offset0 + c[0] * r.stride[0] + c[1] * r.stride[1] +
                       c[2] * r.stride[2];
  const long long ie = ix + (long long)(e - c[idim]) * r.stride[idim];
  for (int iw = 0; iw < 32; iw++) {
    if (!((r.iw_mask >> iw) & 1u)) continue;
    T* a = w + (long long)iw * r.var_stride;
    const double v = 0.5 * ((double)a[ie] + (1.0 + 0.1 * iw) * (1.0 + 0.1 * qt)) +
                     0.01 * xc;
    a[ix] = (T)v;
  }
}

extern "C" int inflow_bound(void* user, void* w, const vacgpu_region* r,
                            void* stream) {
  (void)user;
  long long tot = 1;
  for (int d = 0; d < 3; d++) tot *= r->hi[d] - r->lo[d] + 1;
  const unsigned nb = (unsigned)((tot + 127) / 128);
  cudaStream_t st = (cudaStream_t)stream;
  if (r->elem == 8)
    k_inflow<double><<<nb, 128, 0, st>>>((double*)w, *r);
  else
    k_inflow<float><<<nb, 128, 0, st>>>((float*)w, *r);
  return cudaGetLastError() != cudaSuccess;
}

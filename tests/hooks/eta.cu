// A specialeta test hook for the engine (vacgpu_register_eta): the device
// twin of eta.c,
//   eta = 0.005*(1+x_1^2) + 0.001*J_3^2,  gradeta = (0.01*x_1, 0, 0).
// Build with -fmad=false so it rounds as the host hook does.
#include <cuda_runtime.h>

#include "../../include/vacgpu.h"

__global__ void k_eta(vacgpu_eta_args e) {
  const vacgpu_region& r = e.box;
  int ext[3];
  for (int d = 0; d < 3; d++) ext[d] = r.hi[d] - r.lo[d] + 1;
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= (long long)ext[0] * ext[1] * ext[2]) return;
  int c[3];
  c[0] = r.lo[0] + (int)(n % ext[0]);
  c[1] = r.lo[1] + (int)((n / ext[0]) % ext[1]);
  c[2] = r.lo[2] + (int)(n / ((long long)ext[0] * ext[1]));
  const long long ix = r.offset0 + c[0] * r.stride[0] + c[1] * r.stride[1] +
                       c[2] * r.stride[2];
  const double x1 = r.x[0][c[0]], j3 = e.current[2][ix];
  e.eta[ix] = 0.005 * (1.0 + x1 * x1) + 0.001 * (j3 * j3);
  if (e.gradeta[0]) {
    e.gradeta[0][ix] = 0.01 * x1;
    if (e.gradeta[1]) e.gradeta[1][ix] = 0.0;
    if (e.gradeta[2]) e.gradeta[2][ix] = 0.0;
  }
}

extern "C" int eta_dev(void* user, const vacgpu_eta_args* e, void* stream) {
  (void)user;
  long long tot = 1;
  for (int d = 0; d < 3; d++) tot *= e->box.hi[d] - e->box.lo[d] + 1;
  k_eta<<<(unsigned)((tot + 127) / 128), 128, 0, (cudaStream_t)stream>>>(*e);
  return cudaGetLastError() != cudaSuccess;
}

// A specialsource + getdt_special test hook for the engine
// (vacgpu_register_source_fn): the device twin of source.c,
//   f = 0.02*(0.5+0.1*x_1)*(1+qtC),
//   m_1 += qdt*(rho*f),  e += qdt*(m_1*f),  m_2 -= qdt*(0.05*m_2),
//   dt_mine = 0.05/(0.001 + max |m_1|/rho).
// e is variable 1 + ndir.  For an FP32 state the same
// formulas run in double on the stored floats.  Build with -fmad=false so
// it rounds as the host hook does.
#include <cuda_runtime.h>

#include "../../include/vacgpu.h"

template <typename T>
__global__ void k_src(vacgpu_source_args s, long long e) {
  const vacgpu_region& r = s.box;
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
  const long long N = r.var_stride;
  const T* wc = (const T*)s.wCT;
  T* w = (T*)s.w;
  const double qdt = *s.qdt, qtc = *s.qtC;
  const double f = 0.02 * (0.5 + 0.1 * r.x[0][c[0]]) * (1.0 + qtc);
  w[ix + N] = (T)((double)w[ix + N] + qdt * ((double)wc[ix] * f));
  w[ix + e * N] = (T)((double)w[ix + e * N] + qdt * ((double)wc[ix + N] * f));
  if (e >= 3) w[ix + 2 * N] = (T)((double)w[ix + 2 * N] - qdt * (0.05 * (double)wc[ix + 2 * N]));
}

// one block: max |m_1|/rho over the box, then dt_mine
template <typename T>
__global__ void k_dt(vacgpu_dtspecial_args a) {
  __shared__ double sm[256];
  const vacgpu_region& r = a.box;
  int ext[3];
  for (int d = 0; d < 3; d++) ext[d] = r.hi[d] - r.lo[d] + 1;
  const long long tot = (long long)ext[0] * ext[1] * ext[2];
  const T* w = (const T*)a.w;
  double m = 0.0;
  for (long long n = threadIdx.x; n < tot; n += blockDim.x) {
    int c[3];
    c[0] = r.lo[0] + (int)(n % ext[0]);
    c[1] = r.lo[1] + (int)((n / ext[0]) % ext[1]);
    c[2] = r.lo[2] + (int)(n / ((long long)ext[0] * ext[1]));
    const long long ix = r.offset0 + c[0] * r.stride[0] + c[1] * r.stride[1] +
                         c[2] * r.stride[2];
    double v = (double)w[ix + r.var_stride] / (double)w[ix];
    v = v < 0.0 ? -v : v;
    if (v > m) m = v;
  }
  sm[threadIdx.x] = m;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o && sm[threadIdx.x + o] > sm[threadIdx.x]) sm[threadIdx.x] = sm[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *a.dt = 0.05 / (0.001 + sm[0]);
}

extern "C" int src_dev(void* user, const vacgpu_source_args* s, void* stream) {
  (void)user;
  long long tot = 1;
  for (int d = 0; d < 3; d++) tot *= s->box.hi[d] - s->box.lo[d] + 1;
  const unsigned nb = (unsigned)((tot + 127) / 128);
  if (s->box.elem == 8)
    k_src<double><<<nb, 128, 0, (cudaStream_t)stream>>>(*s, 1 + s->ndir);
  else
    k_src<float><<<nb, 128, 0, (cudaStream_t)stream>>>(*s, 1 + s->ndir);
  return cudaGetLastError() != cudaSuccess;
}

extern "C" int dt_dev(void* user, const vacgpu_dtspecial_args* a, void* stream) {
  (void)user;
  if (a->box.elem == 8)
    k_dt<double><<<1, 256, 0, (cudaStream_t)stream>>>(*a);
  else
    k_dt<float><<<1, 256, 0, (cudaStream_t)stream>>>(*a);
  return cudaGetLastError() != cudaSuccess;
}

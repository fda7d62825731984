// diag.cu - diagnostics of the GPU itself: the FP64-pipe throughput that
// bounds the plain FP64 path (GB300's FP64 rate is a small fraction of its
// FP32 rate, so the FP64 kernels meet this limit before HBM bandwidth).
#include <cuda_runtime.h>

#include <string>

#include "../../include/vacgpu.h"

int vacgpu_internal_fail(const char* msg);

namespace {

constexpr int DIAG_CHAINS = 8;  // independent FMA chains per thread

// iters x DIAG_CHAINS dependent-free DFMA per thread; the sum is written
// only under a condition the inputs never meet, so nothing is optimised
// away and nothing is stored.
__global__ void k_dfma_rate(double* sink, int iters, double a, double b) {
  double x[DIAG_CHAINS];
#pragma unroll
  for (int c = 0; c < DIAG_CHAINS; c++) x[c] = 1e-3 * (threadIdx.x + c);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int c = 0; c < DIAG_CHAINS; c++) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < DIAG_CHAINS; c++) s += x[c];
  if (s == -1.0) sink[0] = s;
}

}  // namespace

extern "C" int vacgpu_measure_fp64_peak(double* flops_per_s, void* stream) {
  if (!flops_per_s) return vacgpu_internal_fail("null argument");
  cudaStream_t st = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return vacgpu_internal_fail("cudaGetDevice/cudaDeviceGetAttribute failed");
  const int threads = 256, blocks = sms * 8, iters = 2048;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return vacgpu_internal_fail("cudaEventCreate failed");
  // a < 1 keeps the chains finite: x -> b/(1-a)
  const double a = 0.999999, b = 1e-7;
  k_dfma_rate<<<blocks, threads, 0, st>>>(nullptr, iters, a, b);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; r++) {
    cudaEventRecord(e0, st);
    k_dfma_rate<<<blocks, threads, 0, st>>>(nullptr, iters, a, b);
    cudaEventRecord(e1, st);
    if (cudaEventSynchronize(e1) != cudaSuccess) break;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return vacgpu_internal_fail((std::string("fp64 peak kernel: ") + cudaGetErrorString(e)).c_str());
  const double fmas = (double)blocks * threads * iters * DIAG_CHAINS;
  *flops_per_s = 2.0 * fmas / (best * 1e-3);
  return 0;
}

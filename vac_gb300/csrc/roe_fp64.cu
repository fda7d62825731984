// roe_fp64.cu - the TVD-MUSCL/Roe corrector of the FP64 path, built with
// -fmad=false like sweep_fp64.cu so every value is bit-identical to the CPU
// restatement of the reference.
#include "physics.cuh"
#include "roe.cuh"

namespace vacgpu {

void launch_correct_roe_fp64(const SweepArgs& s, const double* w,
                             const double* w1, const double* base,
                             double* wout, cudaStream_t st) {
  launch_correct_roe<PH64>(s, w, w1, base, wout, st);
}

}  // namespace vacgpu

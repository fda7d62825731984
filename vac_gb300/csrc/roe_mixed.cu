// roe_mixed.cu - the TVD-MUSCL/Roe corrector of the mixed-precision path:
// FP32 state, fluxes and Roe solver, the thermal pressure recovered in
// double-float arithmetic (physics_mixed.cuh).
#include "physics_mixed.cuh"
#include "roe.cuh"

namespace vacgpu {

void launch_correct_roe_mixed(const SweepArgs& s, const float* w,
                              const float* w1, const float* base, float* wout,
                              cudaStream_t st) {
  launch_correct_roe<PHMixed<PREC_FF>>(s, w, w1, base, wout, st);
}

}  // namespace vacgpu

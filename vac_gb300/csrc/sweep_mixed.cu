// sweep_mixed.cu - the mixed-precision path: FP32 state and fluxes, the
// thermal-pressure recovery at double precision (double-float arithmetic on
// the FP32 pipes by default, see physics_mixed.cuh).
#include "physics_mixed.cuh"
#include "sweep.cuh"

namespace vacgpu {

typedef PHMixed<PREC_FF> PHff;
typedef PHMixed<PREC_F64> PHf64;
typedef PHMixed<PREC_F32> PHf32;

VACGPU_DEFINE_LAUNCHERS(mixed, PHff)
VACGPU_DEFINE_LAUNCHERS(mixedf64, PHf64)
VACGPU_DEFINE_LAUNCHERS(mixedf32, PHf32)

}  // namespace vacgpu

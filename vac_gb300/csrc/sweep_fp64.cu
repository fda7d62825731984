// sweep_fp64.cu - the plain FP64 path: state, fluxes and every intermediate
// in IEEE double, in the reference's operation order.  Built with
// -fmad=false so no multiply-add is contracted, which keeps each value
// bit-identical to the FP64 CPU restatement of the reference.
#include "physics.cuh"
#include "sweep.cuh"

namespace vacgpu {

VACGPU_DEFINE_LAUNCHERS(fp64, PH64)

}  // namespace vacgpu

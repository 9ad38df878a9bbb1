// step_f64.cu - step kernel instantiations for FP64 state planes (solver path).
#include "launch.cuh"

namespace ast {
template int launch_step_r<double, kSoA>(const StepParams&, int, int, cudaStream_t, bool);
}  // namespace ast

// step_f32.cu - step kernel instantiations for FP32 state planes (precision form).
#include "launch.cuh"

namespace ast {
template int launch_step_r<float, kSoA>(const StepParams&, int, int, cudaStream_t, bool);
}  // namespace ast

// step_raw.cu - step kernel instantiations for reference double2 layout (ast_step_raw).
#include "launch.cuh"

namespace ast {
template int launch_step_r<double, kAoS>(const StepParams&, int, int, cudaStream_t, bool);
}  // namespace ast

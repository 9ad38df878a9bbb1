// batch_f32.cu - batch kernel instantiations for FP32 state planes.
#include "launch.cuh"

namespace ast {
template int launch_batch_r<float>(const StepParams*, const int*, int, int, int, int, cudaStream_t, bool);
}  // namespace ast

// batch_f64.cu - batch kernel instantiations for FP64 state planes.
#include "launch.cuh"

namespace ast {
template int launch_batch_r<double>(const StepParams*, const int*, int, int, int, int, cudaStream_t, bool);
}  // namespace ast

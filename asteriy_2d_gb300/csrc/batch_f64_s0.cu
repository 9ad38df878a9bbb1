// batch_f64_s0.cu - batch kernel instantiations, FP64 state planes, tile shape 0.
#include "launch.cuh"

namespace ast {
template int launch_batch_r<double, kShapeTZ[0], kShapeTR[0]>(const StepParams*, const int*, int, int, int, int,
                                                            cudaStream_t, bool);
}  // namespace ast

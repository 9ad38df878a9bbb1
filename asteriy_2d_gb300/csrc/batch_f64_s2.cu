// batch_f64_s2.cu - batch kernel instantiations, FP64 state planes, tile shape 2.
#include "launch.cuh"

namespace ast {
template int launch_batch_r<double, kShapeTZ[2], kShapeTR[2]>(const StepParams*, const int*, int, int, int, int,
                                                            cudaStream_t, bool);
}  // namespace ast

// batch_f32_s1.cu - batch kernel instantiations, FP32 state planes, tile shape 1.
#include "launch.cuh"

namespace ast {
template int launch_batch_r<float, kShapeTZ[1], kShapeTR[1]>(const StepParams*, const int*, int, int, int, int,
                                                            cudaStream_t, bool);
}  // namespace ast

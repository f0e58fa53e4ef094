// lop_square_f32.cu -- square local-operator kernels for f32 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQUARE(float, float)
}  // namespace hgb

// lop_line_f32.cu -- line local-operator kernels for f32 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_LINE(float, float)
}  // namespace hgb

// lop_square_f16.cu -- square local-operator kernels for f16 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQUARE(__half, __half)
}  // namespace hgb

// lop_line_f16.cu -- line local-operator kernels for f16 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_LINE(__half, __half)
}  // namespace hgb

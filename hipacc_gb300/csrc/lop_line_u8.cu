// lop_line_u8.cu -- line local-operator kernels for u8 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_LINE(uint8_t, uint8_t)
}  // namespace hgb

// lop_sq_c_u8.cu -- square local-operator kernels (13x13) for u8 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQ(uint8_t, uint8_t, 13)
}  // namespace hgb

// lop_sq_b_u8.cu -- square local-operator kernels (9x9, 11x11) for u8 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQ(uint8_t, uint8_t, 9)
HGB_INSTANTIATE_SQ(uint8_t, uint8_t, 11)
}  // namespace hgb

// lop_sq_a_u8.cu -- square local-operator kernels (3x3, 5x5, 7x7) for u8 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQ(uint8_t, uint8_t, 3)
HGB_INSTANTIATE_SQ(uint8_t, uint8_t, 5)
HGB_INSTANTIATE_SQ(uint8_t, uint8_t, 7)
template int launch_generic<uint8_t, uint8_t>(const GenParams &, int, cudaStream_t);
}  // namespace hgb

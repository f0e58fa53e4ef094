// lop_sq_b_f32.cu -- square local-operator kernels (9x9, 11x11) for f32 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQ(float, float, 9)
HGB_INSTANTIATE_SQ(float, float, 11)
}  // namespace hgb

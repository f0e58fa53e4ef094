// lop_sq_c_f32.cu -- square local-operator kernels (13x13) for f32 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQ(float, float, 13)
}  // namespace hgb

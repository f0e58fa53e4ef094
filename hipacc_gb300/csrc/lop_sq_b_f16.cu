// lop_sq_b_f16.cu -- square local-operator kernels (9x9, 11x11) for f16 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQ(__half, __half, 9)
HGB_INSTANTIATE_SQ(__half, __half, 11)
}  // namespace hgb

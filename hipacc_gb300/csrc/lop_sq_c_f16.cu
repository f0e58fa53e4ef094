// lop_sq_c_f16.cu -- square local-operator kernels (13x13) for f16 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQ(__half, __half, 13)
}  // namespace hgb

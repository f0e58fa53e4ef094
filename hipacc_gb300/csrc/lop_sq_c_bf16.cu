// lop_sq_c_bf16.cu -- square local-operator kernels (13x13) for bf16 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQ(__nv_bfloat16, __nv_bfloat16, 13)
}  // namespace hgb

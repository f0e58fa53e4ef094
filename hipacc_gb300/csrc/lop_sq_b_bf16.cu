// lop_sq_b_bf16.cu -- square local-operator kernels (9x9, 11x11) for bf16 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQ(__nv_bfloat16, __nv_bfloat16, 9)
HGB_INSTANTIATE_SQ(__nv_bfloat16, __nv_bfloat16, 11)
}  // namespace hgb

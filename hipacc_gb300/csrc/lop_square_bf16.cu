// lop_square_bf16.cu -- square local-operator kernels for bf16 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQUARE(__nv_bfloat16, __nv_bfloat16)
}  // namespace hgb

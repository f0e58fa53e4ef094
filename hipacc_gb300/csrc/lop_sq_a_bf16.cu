// lop_sq_a_bf16.cu -- square local-operator kernels (3x3, 5x5, 7x7) for bf16 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQ(__nv_bfloat16, __nv_bfloat16, 3)
HGB_INSTANTIATE_SQ(__nv_bfloat16, __nv_bfloat16, 5)
HGB_INSTANTIATE_SQ(__nv_bfloat16, __nv_bfloat16, 7)
template int launch_generic<__nv_bfloat16, __nv_bfloat16>(const GenParams &, int, cudaStream_t);
}  // namespace hgb

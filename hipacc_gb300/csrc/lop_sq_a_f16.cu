// lop_sq_a_f16.cu -- square local-operator kernels (3x3, 5x5, 7x7) for f16 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQ(__half, __half, 3)
HGB_INSTANTIATE_SQ(__half, __half, 5)
HGB_INSTANTIATE_SQ(__half, __half, 7)
template int launch_generic<__half, __half>(const GenParams &, int, cudaStream_t);
}  // namespace hgb

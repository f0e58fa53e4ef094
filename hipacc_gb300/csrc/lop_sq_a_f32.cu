// lop_sq_a_f32.cu -- square local-operator kernels (3x3, 5x5, 7x7) for f32 storage (local_op.cuh).
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_SQ(float, float, 3)
HGB_INSTANTIATE_SQ(float, float, 5)
HGB_INSTANTIATE_SQ(float, float, 7)
template int launch_generic<float, float>(const GenParams &, int, cudaStream_t);
}  // namespace hgb

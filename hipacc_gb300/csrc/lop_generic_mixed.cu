// lop_generic_mixed.cu -- general local-operator kernels between storage types
// (local_op.cuh); the same-type ones live in lop_sq_a_*.cu.
#include "local_op_kernels.cuh"

namespace hgb {
HGB_INSTANTIATE_GENERIC(float, __nv_bfloat16)
HGB_INSTANTIATE_GENERIC(float, __half)
HGB_INSTANTIATE_GENERIC(__nv_bfloat16, float)
HGB_INSTANTIATE_GENERIC(__half, float)
HGB_INSTANTIATE_GENERIC(uint8_t, float)
}  // namespace hgb

// pending.cu -- entry points declared in hipacc_gb300.h whose kernels are not
// in this build yet: they validate nothing and report HGB_ERR_UNSUPPORTED.
#include "hgb_internal.cuh"

using namespace hgb;

extern "C" {

int hgb_local_op_adjoint(const hgb_view *, const hgb_view *, const hgb_view *, const float *, const float *, int, int,
                         int, float *, void *) {
  return set_error(HGB_ERR_UNSUPPORTED, "hgb_local_op_adjoint: not built");
}

}  // extern "C"

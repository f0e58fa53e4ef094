// pending.cu -- entry points declared in hipacc_gb300.h whose kernels are not
// in this build yet: they validate nothing and report HGB_ERR_UNSUPPORTED.
#include "hgb_internal.cuh"

using namespace hgb;

extern "C" {

int hgb_pyramid_plan_create(int, const int *, const int *, int, const float *, int, hgb_pyramid_plan **) {
  return set_error(HGB_ERR_UNSUPPORTED, "hgb_pyramid_plan_create: not built");
}
int hgb_pyramid_plan_destroy(hgb_pyramid_plan *) { return HGB_OK; }
int hgb_pyramid_level_view(const hgb_pyramid_plan *, int, int, hgb_view *, hgb_view *) {
  return set_error(HGB_ERR_UNSUPPORTED, "hgb_pyramid_level_view: not built");
}
int hgb_pyramid_decompose(hgb_pyramid_plan *, int, void *) {
  return set_error(HGB_ERR_UNSUPPORTED, "hgb_pyramid_decompose: not built");
}
int hgb_pyramid_collapse(hgb_pyramid_plan *, void *) {
  return set_error(HGB_ERR_UNSUPPORTED, "hgb_pyramid_collapse: not built");
}

int hgb_local_op_adjoint(const hgb_view *, const hgb_view *, const hgb_view *, const float *, const float *, int, int,
                         int, float *, void *) {
  return set_error(HGB_ERR_UNSUPPORTED, "hgb_local_op_adjoint: not built");
}

int hgb_conv_bilateral_mse(const hgb_view *, const hgb_view *, const float *, int, const float *, int, const float *,
                           int, int, double *, const hgb_view *, float *, float *, void *) {
  return set_error(HGB_ERR_UNSUPPORTED, "hgb_conv_bilateral_mse: not built");
}

}  // extern "C"

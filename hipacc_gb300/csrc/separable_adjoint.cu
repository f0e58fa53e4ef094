// separable_adjoint.cu -- hgb_separable_adjoint: the adjoint of hgb_separable
// (FP32 storage), composed from the local-operator kernels.
//
// The forward is the reference's two-operator program: t = rows(in) with the
// 1 x K row taps and the boundary on x, then out = cols(t) with the K x 1
// column taps and the boundary on y (rows of t outside the image are the row
// pass of the remapped input row, or the constant for CONSTANT; that is
// cols(t) with t's own boundary).  Its adjoint is the two transposes in the
// other order:
//   g_t     = cols^T(grad_out)          grad_col(k) = sum grad_out(j) t(r(j + o_k))
//   grad_in = rows^T(g_t)               grad_row(k) = sum g_t(j) in(r(j + o_k))
// Each transpose is hgb_local_op_adjoint with the 1-D mask; t is recomputed
// with hgb_local_op.  t and g_t live in the library workspace behind the
// space the local-operator adjoint uses for its per-tap partials, so its own
// workspace request never moves them.
#include <cstring>

#include "hgb_internal.cuh"

using namespace hgb;

extern "C" int hgb_separable_adjoint(const hgb_view *in, const hgb_view *grad_out, const float *row_taps,
                                     const float *col_taps, int k, int boundary, float const_val,
                                     const hgb_view *grad_in, float *grad_row_dev, float *grad_col_dev,
                                     void *stream) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  rc = check_view(grad_out, "grad_out");
  if (rc) return rc;
  if (grad_in) {
    rc = check_view(grad_in, "grad_in");
    if (rc) return rc;
  }
  HGB_REQUIRE(in->dtype == HGB_F32 && grad_out->dtype == HGB_F32 && (!grad_in || grad_in->dtype == HGB_F32),
              "hgb_separable_adjoint: f32 storage expected");
  HGB_REQUIRE(in->width == grad_out->width && in->height == grad_out->height && in->batch == grad_out->batch &&
                  (!grad_in || (grad_in->width == in->width && grad_in->height == in->height &&
                                grad_in->batch == in->batch)),
              "hgb_separable_adjoint: size mismatch");
  HGB_REQUIRE(row_taps && col_taps, "hgb_separable_adjoint: null taps");
  HGB_REQUIRE(k >= 1 && k <= 15, "hgb_separable_adjoint: K must be 1..15");
  HGB_REQUIRE(boundary >= 0 && boundary <= 4, "hgb_separable_adjoint: bad boundary");
  HGB_REQUIRE(grad_in || grad_row_dev || grad_col_dev, "hgb_separable_adjoint: nothing to compute");
  // workspace: [partials of the local-operator adjoint][t][g_t], dense FP32 images
  const int64_t w = in->width, h = in->height, nb = in->batch;
  const size_t img = (size_t)(w * h * nb) * sizeof(float);
  const size_t parts = ((size_t)15 * 64 * nb * sizeof(float) + 64 + 255) / 256 * 256;
  const size_t timg = (img + 255) / 256 * 256;
  Workspace ws;
  rc = workspace_get(parts + 2 * timg, &ws);
  if (rc) return rc;
  hgb_view t, gt;
  memset(&t, 0, sizeof(t));
  t.data = (char *)ws.base + parts;
  t.dtype = HGB_F32;
  t.width = in->width;
  t.height = in->height;
  t.batch = in->batch;
  t.pitch = w * (int64_t)sizeof(float);
  t.batch_stride = t.pitch * h;
  gt = t;
  gt.data = (char *)ws.base + parts + timg;
  const bool want_gt = grad_in || grad_row_dev;
  // t = rows(in): needed for grad_col
  if (grad_col_dev) {
    rc = hgb_local_op(in, nullptr, &t, nullptr, row_taps, nullptr, nullptr, k, 1, HGB_REDUCE_SUM, boundary, const_val,
                      stream);
    if (rc) return rc;
  }
  // g_t = cols^T(grad_out), grad_col from t
  rc = hgb_local_op_adjoint(grad_col_dev ? &t : nullptr, grad_out, want_gt ? &gt : nullptr, col_taps, nullptr, 1, k,
                            boundary, grad_col_dev, stream);
  if (rc) return rc;
  if (!want_gt) return HGB_OK;
  // grad_in = rows^T(g_t), grad_row from in
  return hgb_local_op_adjoint(grad_row_dev ? in : nullptr, &gt, grad_in, row_taps, nullptr, k, 1, boundary,
                              grad_row_dev, stream);
}

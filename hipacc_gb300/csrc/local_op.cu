// local_op.cu -- hgb_local_op: argument checks, mask padding, dispatch between
// the register-blocked fast kernels and the general kernel, tile autotuning.
#include <cstring>

#include "autotune.h"
// declarations only: the kernels are instantiated in the lop_*.cu units, which
// compile in parallel
#include "local_op.cuh"

namespace hgb {

int num_tile_cfgs() { return 3; }

namespace {

int vec_elems(int dt) { return 16 / dtype_size(dt); }

template <typename TI, typename TO>
int run_conv_typed(const ConvParams &p, int k_w, int k_h, int batch, cudaStream_t st, const char *key) {
  const int n = num_tile_cfgs();
  return autotune_run(key, n, st, [&](int cfg) { return launch_conv<TI, TO>(p, k_w, k_h, batch, st, cfg); });
}

int run_conv(int dti, int dto, const ConvParams &p, int k_w, int k_h, int batch, cudaStream_t st) {
  char key[128];
  // shape class: mask, dtype and image size rounded to a power of two
  int cls = 0;
  while ((1 << cls) < p.is_w * (int64_t)p.is_h / 4096 && cls < 30) ++cls;
  snprintf(key, sizeof(key), "conv/%d/%d/%dx%d/%d/b%d", dti, dto, k_w, k_h, cls, batch > 8 ? 9 : batch);
  if (dti == HGB_F32 && dto == HGB_F32) return run_conv_typed<float, float>(p, k_w, k_h, batch, st, key);
  if (dti == HGB_BF16 && dto == HGB_BF16) return run_conv_typed<__nv_bfloat16, __nv_bfloat16>(p, k_w, k_h, batch, st, key);
  if (dti == HGB_F16 && dto == HGB_F16) return run_conv_typed<__half, __half>(p, k_w, k_h, batch, st, key);
  if (dti == HGB_U8 && dto == HGB_U8) return run_conv_typed<uint8_t, uint8_t>(p, k_w, k_h, batch, st, key);
  return set_error(HGB_ERR_UNSUPPORTED, "conv: storage pair without a fast kernel");
}

int run_generic(int dti, int dto, const GenParams &g, int batch, cudaStream_t st) {
#define HGB_G(A, B, TA, TB) \
  if (dti == A && dto == B) return launch_generic<TA, TB>(g, batch, st);
  HGB_G(HGB_F32, HGB_F32, float, float)
  HGB_G(HGB_BF16, HGB_BF16, __nv_bfloat16, __nv_bfloat16)
  HGB_G(HGB_F16, HGB_F16, __half, __half)
  HGB_G(HGB_F32, HGB_BF16, float, __nv_bfloat16)
  HGB_G(HGB_F32, HGB_F16, float, __half)
  HGB_G(HGB_BF16, HGB_F32, __nv_bfloat16, float)
  HGB_G(HGB_F16, HGB_F32, __half, float)
  HGB_G(HGB_U8, HGB_U8, uint8_t, uint8_t)
  HGB_G(HGB_U8, HGB_F32, uint8_t, float)
#undef HGB_G
  return set_error(HGB_ERR_UNSUPPORTED, "local_op: unsupported storage pair");
}

// smallest fast shape that contains mw x mh with the same tap offsets
bool fast_shape(int mw, int mh, int *kw, int *kh) {
  auto odd_up = [](int v) { return v % 2 ? v : v + 1; };
  if (mh == 1 && mw > 1) {
    *kw = odd_up(mw);
    *kh = 1;
  } else if (mw == 1 && mh > 1) {
    *kw = 1;
    *kh = odd_up(mh);
  } else {
    int s = odd_up(mw > mh ? mw : mh);
    if (s < 3) s = 3;
    *kw = *kh = s;
  }
  return *kw <= 13 && *kh <= 13;
}

}  // namespace

int fill_conv_params(const hgb_view &in, const hgb_window &acc, const hgb_view &out, const hgb_window &is, int boundary,
                     float cval, ConvParams *p) {
  memset(p, 0, sizeof(*p));
  p->in = (const char *)in.data;
  p->in_pitch = in.pitch;
  p->in_bstride = in.batch_stride;
  p->out = (char *)out.data;
  p->out_pitch = out.pitch;
  p->out_bstride = out.batch_stride;
  p->acc_ox = acc.offset_x;
  p->acc_oy = acc.offset_y;
  p->acc_w = acc.width;
  p->acc_h = acc.height;
  p->is_ox = is.offset_x;
  p->is_oy = is.offset_y;
  p->is_w = is.width;
  p->is_h = is.height;
  p->bmode = boundary;
  p->cval = cval;
  p->in_w = in.width;
  p->in_h = in.height;
  p->batch = in.batch;
  p->vec_in = ((uintptr_t)in.data % 16 == 0) && (in.pitch % 16 == 0) && (in.batch_stride % 16 == 0 || in.batch == 1) &&
              (acc.offset_x % vec_elems(in.dtype) == 0);
  p->vec_out = ((uintptr_t)out.data % 16 == 0) && (out.pitch % 16 == 0) &&
               (out.batch_stride % 16 == 0 || out.batch == 1) && (is.offset_x % 4 == 0);
  return HGB_OK;
}

}  // namespace hgb

using namespace hgb;

extern "C" int hgb_local_op(const hgb_view *in, const hgb_window *accw, const hgb_view *out, const hgb_window *isw,
                            const float *mask, const float *mask_dev, const uint8_t *domain, int mask_w, int mask_h,
                            int reduce, int boundary, float const_val, void *stream) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  rc = check_view(out, "out");
  if (rc) return rc;
  HGB_REQUIRE((is_float_storage(in->dtype) || in->dtype == HGB_U8) &&
                  (is_float_storage(out->dtype) || (out->dtype == HGB_U8 && in->dtype == HGB_U8)),
              "hgb_local_op: storage must be f32, bf16, f16 or u8 (u8 output from u8 input)");
  HGB_REQUIRE(in->batch == out->batch, "hgb_local_op: batch mismatch");
  HGB_REQUIRE(mask_w >= 1 && mask_h >= 1 && mask_w <= kMaxMask && mask_h <= kMaxMask,
              "hgb_local_op: mask size must be 1..15");
  HGB_REQUIRE(reduce >= HGB_REDUCE_SUM && reduce <= HGB_REDUCE_PROD, "hgb_local_op: bad reduce mode");
  HGB_REQUIRE(boundary >= HGB_BOUNDARY_UNDEFINED && boundary <= HGB_BOUNDARY_CONSTANT, "hgb_local_op: bad boundary");
  HGB_REQUIRE(mask || mask_dev || domain, "hgb_local_op: a mask or a domain is required");
  HGB_REQUIRE(!(mask && mask_dev), "hgb_local_op: give mask or mask_dev, not both");
  hgb_window acc = window_or_full(accw, *in), is = window_or_full(isw, *out);
  rc = check_window(acc, *in, "accessor window");
  if (rc) return rc;
  rc = check_window(is, *out, "iteration space");
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;

  int kw = 0, kh = 0;
  if (reduce == HGB_REDUCE_SUM && !mask_dev && in->dtype == out->dtype && fast_shape(mask_w, mask_h, &kw, &kh)) {
    ConvParams p;
    fill_conv_params(*in, acc, *out, is, boundary, const_val, &p);
    // embed the mask so that tap offsets are preserved: column c of the
    // original (offset c - mask_w/2) lands at c + kw/2 - mask_w/2.
    const int dx = kw / 2 - mask_w / 2, dy = kh / 2 - mask_h / 2;
    for (int y = 0; y < mask_h; ++y)
      for (int x = 0; x < mask_w; ++x) {
        const bool on = !domain || domain[y * mask_w + x];
        const float m = mask ? mask[y * mask_w + x] : 1.0f;
        p.mask[(y + dy) * kw + (x + dx)] = on ? m : 0.0f;
      }
    for (int i = 0; i < kw * kh; ++i) {
      uint32_t bits;
      memcpy(&bits, &p.mask[i], 4);
      p.mask2[i] = ((f2)bits << 32) | bits;
    }
    return run_conv(in->dtype, out->dtype, p, kw, kh, in->batch, st);
  }
  GenParams g;
  memset(&g, 0, sizeof(g));
  fill_conv_params(*in, acc, *out, is, boundary, const_val, &g.c);
  g.mw = mask_w;
  g.mh = mask_h;
  g.reduce = reduce;
  g.has_mask = (mask || mask_dev) ? 1 : 0;
  g.mask_dev = mask_dev;
  for (int i = 0; i < mask_w * mask_h; ++i) {
    g.c.mask[i] = mask ? mask[i] : 0.0f;
    g.domain[i] = domain ? (domain[i] != 0) : 1;
  }
  return run_generic(in->dtype, out->dtype, g, in->batch, st);
}

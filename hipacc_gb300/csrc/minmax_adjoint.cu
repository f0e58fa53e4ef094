// minmax_adjoint.cu -- hgb_local_op_minmax_adjoint: the adjoint of the MIN /
// MAX local operator, Kernel::reduce(Domain, Reduce::MIN/MAX) and
// Kernel::convolve(mask, Reduce::MIN/MAX) (dsl/kernel.hpp:241-315;
// lib/AST/Convolution.cpp:43-100: acc starts at FLT_MAX / FLT_MIN and takes
// acc = acc < v ? acc : v (MIN) or acc > v ? acc : v (MAX) per tap in
// row-major order, v = m * x for convolve, x for a Domain).
//
// Each output's value came from one tap: the last one whose update replaced
// the running value (on a tie the later tap replaces, as the forward's
// expression does).  Its gradient goes to the pixel that tap read, times the
// mask weight for convolve.  Nothing flows when the initial value was never
// replaced, or when the winning tap read the CONSTANT value outside the image.
//
// Two kernels, deterministic:
//   1. minmax_select_kernel: per output, the winning tap (0 .. taps-1) or 0xFF,
//      into a byte per output in the library workspace;
//   2. minmax_gather_kernel: per input pixel, the sum over every (virtual
//      position that the boundary remap sends to it, tap) of the gradients of
//      the outputs whose winner is that tap, in a fixed order: rows and
//      columns of the pre-images ascending, then taps in row-major order.
#include <algorithm>
#include <cfloat>
#include <cstring>

#include "hgb_internal.cuh"

namespace hgb {
namespace {

constexpr int MM_MAX = 15, MM_T = 256, MM_NONE = 0xFF;

struct MinMaxParams {
  const float *in, *gout;
  float *gin;
  uint8_t *sel;
  int64_t in_p, in_b, gout_p, gout_b, gin_p, gin_b;  // floats
  int w, h, batch;
  int mw, mh, red, bmode;
  float cval;
  int has_mask;
  float mask[MM_MAX * MM_MAX];
  uint8_t dom[MM_MAX * MM_MAX];
};

__global__ void __launch_bounds__(MM_T) minmax_select_kernel(const __grid_constant__ MinMaxParams p) {
  const int64_t n = (int64_t)p.w * p.h;
  const int64_t idx = (int64_t)blockIdx.x * MM_T + threadIdx.x;
  const int b = blockIdx.y;
  if (idx >= n) return;
  const int y = (int)(idx / p.w), x = (int)(idx - (int64_t)y * p.w);
  const int rx = p.mw / 2, ry = p.mh / 2;
  const float *in = p.in + (int64_t)b * p.in_b;
  const bool is_max = p.red == HGB_REDUCE_MAX;
  float acc = is_max ? FLT_MIN : FLT_MAX;
  int win = MM_NONE;
  for (int my = 0; my < p.mh; ++my)
    for (int mx = 0; mx < p.mw; ++mx) {
      const int k = my * p.mw + mx;
      if (!p.dom[k]) continue;
      const int ax = remap(p.bmode, x + mx - rx, 0, p.w), ay = remap(p.bmode, y + my - ry, 0, p.h);
      const bool outside = ax == (int)0x80000000 || ay == (int)0x80000000;
      const float xv = outside ? p.cval : __ldg(in + (int64_t)ay * p.in_p + ax);
      const float v = p.has_mask ? __fmul_rn(p.mask[k], xv) : xv;
      const bool keep = is_max ? acc > v : acc < v;
      if (!keep) {
        acc = v;
        win = outside ? MM_NONE : k;  // a CONSTANT tap outside carries no gradient
      }
    }
  p.sel[(int64_t)b * n + idx] = (uint8_t)win;
}

// virtual positions v in [-reach, n + reach) that the remap sends to i (i itself first)
__device__ __forceinline__ int mm_pre(int mode, int i, int n, int reach, int *out) {
  int k = 0;
  out[k++] = i;
  if (mode == HGB_BOUNDARY_CONSTANT) return k;
  for (int v = -reach; v < 0; ++v)
    if (remap(mode, v, 0, n) == i && k < 2 * MM_MAX + 1) out[k++] = v;
  for (int v = n; v < n + reach; ++v)
    if (remap(mode, v, 0, n) == i && k < 2 * MM_MAX + 1) out[k++] = v;
  return k;
}

__global__ void __launch_bounds__(MM_T) minmax_gather_kernel(const __grid_constant__ MinMaxParams p) {
  const int64_t n = (int64_t)p.w * p.h;
  const int64_t idx = (int64_t)blockIdx.x * MM_T + threadIdx.x;
  const int b = blockIdx.y;
  if (idx >= n) return;
  const int iy = (int)(idx / p.w), ix = (int)(idx - (int64_t)iy * p.w);
  const int rxl = p.mw / 2, ryl = p.mh / 2, rxh = p.mw - 1 - rxl, ryh = p.mh - 1 - ryl;
  const uint8_t *sel = p.sel + (int64_t)b * n;
  const float *gout = p.gout + (int64_t)b * p.gout_b;
  int prx[2 * MM_MAX + 1], pry[2 * MM_MAX + 1];
  const int rx = max(rxl, rxh), ry = max(ryl, ryh);
  const bool inner = ix >= rx && ix < p.w - rx && iy >= ry && iy < p.h - ry;
  int nx = 1, ny = 1;
  prx[0] = ix;
  pry[0] = iy;
  if (!inner) {  // near a border: every virtual position the remap sends here
    nx = mm_pre(p.bmode, ix, p.w, rx + 1, prx);
    ny = mm_pre(p.bmode, iy, p.h, ry + 1, pry);
  }
  float acc = 0.0f;
  for (int a = 0; a < ny; ++a)
    for (int c = 0; c < nx; ++c)
      for (int my = 0; my < p.mh; ++my)
        for (int mx = 0; mx < p.mw; ++mx) {
          const int k = my * p.mw + mx;
          // output j read virtual position v = j + o through tap o
          const int jy = pry[a] - (my - ryl), jx = prx[c] - (mx - rxl);
          if (jx < 0 || jx >= p.w || jy < 0 || jy >= p.h) continue;
          const int64_t j = (int64_t)jy * p.w + jx;
          if (sel[j] != k) continue;
          const float g = __ldg(gout + (int64_t)jy * p.gout_p + jx);
          acc = p.has_mask ? __fmaf_rn(p.mask[k], g, acc) : __fadd_rn(acc, g);
        }
  p.gin[(int64_t)b * p.gin_b + (int64_t)iy * p.gin_p + ix] = acc;
}

}  // namespace
}  // namespace hgb

using namespace hgb;

extern "C" int hgb_local_op_minmax_adjoint(const hgb_view *in, const hgb_view *grad_out, const hgb_view *grad_in,
                                           const float *mask, const uint8_t *domain, int mask_w, int mask_h,
                                           int reduce, int boundary, float const_val, void *stream) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  rc = check_view(grad_out, "grad_out");
  if (rc) return rc;
  rc = check_view(grad_in, "grad_in");
  if (rc) return rc;
  HGB_REQUIRE(in->dtype == HGB_F32 && grad_out->dtype == HGB_F32 && grad_in->dtype == HGB_F32,
              "hgb_local_op_minmax_adjoint: f32 storage expected");
  HGB_REQUIRE(in->width == grad_out->width && in->height == grad_out->height && in->batch == grad_out->batch &&
                  grad_in->width == in->width && grad_in->height == in->height && grad_in->batch == in->batch,
              "hgb_local_op_minmax_adjoint: size mismatch");
  HGB_REQUIRE(mask_w >= 1 && mask_h >= 1 && mask_w <= MM_MAX && mask_h <= MM_MAX,
              "hgb_local_op_minmax_adjoint: mask size must be 1..15");
  HGB_REQUIRE(reduce == HGB_REDUCE_MIN || reduce == HGB_REDUCE_MAX, "hgb_local_op_minmax_adjoint: MIN or MAX");
  HGB_REQUIRE(boundary >= 0 && boundary <= 4, "hgb_local_op_minmax_adjoint: bad boundary");
  HGB_REQUIRE(in->batch <= 65535, "hgb_local_op_minmax_adjoint: at most 65535 images per call");
  MinMaxParams p;
  memset(&p, 0, sizeof(p));
  p.in = (const float *)in->data;
  p.gout = (const float *)grad_out->data;
  p.gin = (float *)grad_in->data;
  HGB_REQUIRE(in->pitch % 4 == 0 && grad_out->pitch % 4 == 0 && grad_in->pitch % 4 == 0 &&
                  in->batch_stride % 4 == 0 && grad_out->batch_stride % 4 == 0 && grad_in->batch_stride % 4 == 0,
              "hgb_local_op_minmax_adjoint: pitches must be whole floats");
  p.in_p = in->pitch / 4;
  p.in_b = in->batch_stride / 4;
  p.gout_p = grad_out->pitch / 4;
  p.gout_b = grad_out->batch_stride / 4;
  p.gin_p = grad_in->pitch / 4;
  p.gin_b = grad_in->batch_stride / 4;
  p.w = in->width;
  p.h = in->height;
  p.batch = in->batch;
  p.mw = mask_w;
  p.mh = mask_h;
  p.red = reduce;
  p.bmode = boundary;
  p.cval = const_val;
  p.has_mask = mask != nullptr;
  for (int k = 0; k < mask_w * mask_h; ++k) {
    p.mask[k] = mask ? mask[k] : 1.0f;
    p.dom[k] = domain ? (domain[k] != 0) : 1;
  }
  const int64_t npx = (int64_t)p.w * p.h;
  const int64_t nblk = (npx + MM_T - 1) / MM_T;
  HGB_REQUIRE(nblk < (int64_t)0x7fffffff, "hgb_local_op_minmax_adjoint: image too large");
  Workspace ws;
  rc = workspace_get((size_t)npx * p.batch + 64, &ws);
  if (rc) return rc;
  p.sel = (uint8_t *)ws.base;
  cudaStream_t st = (cudaStream_t)stream;
  const dim3 grid((unsigned)nblk, (unsigned)p.batch);
  cudaEvent_t ev = before_launch(st);
  minmax_select_kernel<<<grid, MM_T, 0, st>>>(p);
  minmax_gather_kernel<<<grid, MM_T, 0, st>>>(p);
  return after_launch("minmax_gather_kernel", st, ev);
}

// separable.cu -- hgb_separable: a separable K x K filter in one kernel.
//
// The reference has no separable primitive: a program writes two local
// operators, a 1xK mask into an intermediate image and a Kx1 mask over that
// image, each with its boundary condition (lib/AST/Convolution.cpp:397-435,
// lib/AST/BorderHandling.cpp:124-407).  Here one CTA stages its input tile
// (+ halo) once, runs the row pass into an FP32 intermediate tile in shared
// memory and the column pass from it, so the intermediate image never touches
// HBM.  The result equals the two-pass FP32 program bit for bit:
//   * both passes fold their taps in ascending order with fused multiply-add
//     from 0 (the contracted form of `_tmp += mask * in`);
//   * the row pass reads the input through the boundary remap;
//   * intermediate rows outside the image are what the column pass's boundary
//     reads: for CLAMP / MIRROR / REPEAT / UNDEFINED the row pass of the
//     remapped input row (which is what the staged halo rows hold), and for
//     CONSTANT the constant itself.
// Storage f32 / bf16 / f16 in and out (same type), FP32 arithmetic.
#include "stage.cuh"

namespace hgb {
namespace {

constexpr int kSepMaxK = 15;

struct SepParams {
  const char *in;
  int64_t in_pitch, in_bstride;
  char *out;
  int64_t out_pitch, out_bstride;
  int w, h;
  int bmode;
  float cval;
  int vec_in, vec_out;
  float row[kSepMaxK], col[kSepMaxK];
};

constexpr int SP_BX = 32, SP_BY = 8, SP_PX = 4, SP_PY = 4;
constexpr int SP_TW = SP_BX * SP_PX, SP_TH = SP_BY * SP_PY;

template <typename T, int K>
struct SepShape {
  static constexpr int R = K / 2;
  static constexpr int VI = Vec16<T>::N;
  static constexpr int HL = round_up(R, VI);
  static constexpr int SW = HL + SP_TW + round_up(R, VI);
  static constexpr int SH = SP_TH + K - 1;
  static constexpr size_t smem = sizeof(float) * ((size_t)SH * SW + (size_t)SH * SP_TW);
};

template <typename T, int K>
__global__ void __launch_bounds__(SP_BX *SP_BY) separable_kernel(const __grid_constant__ SepParams p) {
  using S = SepShape<T, K>;
  constexpr int R = S::R, HL = S::HL, SW = S::SW, SH = S::SH;
  extern __shared__ __align__(16) float smem[];
  float *tile = smem;
  float *rowb = smem + SH * SW;
  const int b = blockIdx.z;
  const int i0 = blockIdx.x * SP_TW, j0 = blockIdx.y * SP_TH;
  stage_tile<T, SW, SH, SP_BX * SP_BY>(tile, p.in + (int64_t)b * p.in_bstride, p.in_pitch, i0 - HL, j0 - R, 0, p.w,
                                        0, p.h, p.bmode, p.cval, p.vec_in);
  __syncthreads();
  const int tx = threadIdx.x % SP_BX, ty = threadIdx.x / SP_BX;
  // ---- row pass: 4 outputs per thread per staged row
  {
    constexpr int OFF = (HL - R) % 4;
    constexpr int NV = cdiv(OFF + SP_PX + K - 1, 4);
    const int cb = HL - R - OFF + tx * SP_PX;
    for (int r = ty; r < SH; r += SP_BY) {
      float win[NV * 4];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const float4 t = *reinterpret_cast<const float4 *>(&tile[r * SW + cb + 4 * v]);
        win[4 * v] = t.x;
        win[4 * v + 1] = t.y;
        win[4 * v + 2] = t.z;
        win[4 * v + 3] = t.w;
      }
      float acc[SP_PX];
#pragma unroll
      for (int px = 0; px < SP_PX; ++px) {
        acc[px] = 0.0f;
#pragma unroll
        for (int k = 0; k < K; ++k) acc[px] = __fmaf_rn(p.row[k], win[OFF + px + k], acc[px]);
      }
      const int ay = j0 - R + r;
      if (p.bmode == HGB_BOUNDARY_CONSTANT && (ay < 0 || ay >= p.h))
#pragma unroll
        for (int px = 0; px < SP_PX; ++px) acc[px] = p.cval;
      *reinterpret_cast<float4 *>(&rowb[r * SP_TW + tx * SP_PX]) = make_float4(acc[0], acc[1], acc[2], acc[3]);
    }
  }
  __syncthreads();
  // ---- column pass: 4 x 4 outputs per thread
  float acc[SP_PY][SP_PX];
#pragma unroll
  for (int oy = 0; oy < SP_PY; ++oy)
#pragma unroll
    for (int px = 0; px < SP_PX; ++px) acc[oy][px] = 0.0f;
#pragma unroll
  for (int r = 0; r < SP_PY + K - 1; ++r) {
    const float4 t = *reinterpret_cast<const float4 *>(&rowb[(ty * SP_PY + r) * SP_TW + tx * SP_PX]);
    const float v[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
    for (int oy = 0; oy < SP_PY; ++oy) {
      const int k = r - oy;
      if (k < 0 || k >= K) continue;
#pragma unroll
      for (int px = 0; px < SP_PX; ++px) acc[oy][px] = __fmaf_rn(p.col[k], v[px], acc[oy][px]);
    }
  }
  char *out = p.out + (int64_t)b * p.out_bstride;
  const int i = i0 + tx * SP_PX;
#pragma unroll
  for (int oy = 0; oy < SP_PY; ++oy) {
    const int j = j0 + ty * SP_PY + oy;
    if (j >= p.h || i >= p.w) continue;
    store_row<T, SP_PX>(reinterpret_cast<T *>(out + (int64_t)j * p.out_pitch) + i, acc[oy], i, p.w, p.vec_out);
  }
}

template <typename T, int K>
int launch_sep_k(const SepParams &p, int batch, cudaStream_t st) {
  constexpr size_t smem = SepShape<T, K>::smem;
  static bool attr = false;
  if (!attr) {
    HGB_CHECK_CUDA(cudaFuncSetAttribute(separable_kernel<T, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr = true;
  }
  dim3 grid(cdiv(p.w, SP_TW), cdiv(p.h, SP_TH), batch);
  cudaEvent_t ev = before_launch(st);
  separable_kernel<T, K><<<grid, SP_BX * SP_BY, smem, st>>>(p);
  return after_launch("separable_kernel", st, ev);
}

template <typename T>
int launch_sep(const SepParams &p, int k, int batch, cudaStream_t st) {
  switch (k) {
    case 3: return launch_sep_k<T, 3>(p, batch, st);
    case 5: return launch_sep_k<T, 5>(p, batch, st);
    case 7: return launch_sep_k<T, 7>(p, batch, st);
    case 9: return launch_sep_k<T, 9>(p, batch, st);
    case 11: return launch_sep_k<T, 11>(p, batch, st);
    case 13: return launch_sep_k<T, 13>(p, batch, st);
    case 15: return launch_sep_k<T, 15>(p, batch, st);
  }
  return set_error(HGB_ERR_UNSUPPORTED, "hgb_separable: K must be odd, 3..15");
}

}  // namespace
}  // namespace hgb

using namespace hgb;

extern "C" int hgb_separable(const hgb_view *in, const hgb_view *out, const float *row_taps, const float *col_taps,
                             int k, int boundary, float const_val, void *stream) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  rc = check_view(out, "out");
  if (rc) return rc;
  HGB_REQUIRE(in->dtype == out->dtype && is_float_storage(in->dtype), "hgb_separable: same float storage expected");
  HGB_REQUIRE(in->width == out->width && in->height == out->height && in->batch == out->batch,
              "hgb_separable: size mismatch");
  HGB_REQUIRE(row_taps && col_taps, "hgb_separable: null taps");
  HGB_REQUIRE(k >= 3 && k <= kSepMaxK && (k & 1), "hgb_separable: K must be odd, 3..15");
  HGB_REQUIRE(boundary >= 0 && boundary <= 4, "hgb_separable: bad boundary");
  SepParams p;
  memset(&p, 0, sizeof(p));
  p.in = (const char *)in->data;
  p.in_pitch = in->pitch;
  p.in_bstride = in->batch_stride;
  p.out = (char *)out->data;
  p.out_pitch = out->pitch;
  p.out_bstride = out->batch_stride;
  p.w = in->width;
  p.h = in->height;
  p.bmode = boundary;
  p.cval = const_val;
  p.vec_in = ((uintptr_t)in->data % 16 == 0) && in->pitch % 16 == 0 && (in->batch == 1 || in->batch_stride % 16 == 0);
  p.vec_out = ((uintptr_t)out->data % 16 == 0) && out->pitch % 16 == 0 && (out->batch == 1 || out->batch_stride % 16 == 0);
  for (int i = 0; i < k; ++i) {
    p.row[i] = row_taps[i];
    p.col[i] = col_taps[i];
  }
  cudaStream_t st = (cudaStream_t)stream;
  switch (in->dtype) {
    case HGB_F32: return launch_sep<float>(p, k, in->batch, st);
    case HGB_BF16: return launch_sep<__nv_bfloat16>(p, k, in->batch, st);
    default: return launch_sep<__half>(p, k, in->batch, st);
  }
}

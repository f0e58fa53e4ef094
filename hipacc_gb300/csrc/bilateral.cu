// bilateral.cu -- hgb_bilateral: the bilateral filter of
// samples-public/3_Preprocessing/Bilateral_Filter/src/main.cpp:63-77:
//   c_r = 0.5 / sigma_r^2, centre = in(),
//   for every Domain(mask) cell: diff = in(dom) - centre,
//     s = exp(-c_r * diff^2) * mask(dom);  d += s;  p += s * in(dom)
//   out = p / d
// with a float range sigma and a float result.
//
// The filter is bound by the exponential unit (one exponential per tap and
// pixel), not by HBM.  The weight is evaluated as one base-2 exponential with
// the spatial weight folded into the exponent,
//   s = exp2(k2 * diff^2 + log2(mask)),  k2 = -c_r * log2(e),
// (mask cells of 0 give log2 = -inf, i.e. s = 0, which is the Domain's skip).
// The FP32 path uses the ex2.approx instruction through exp2f's fast form.
// For BF16 / F16 storage the fast path (flags bit 0) evaluates two taps'
// weights per instruction with packed half precision (h2exp2) and keeps every
// accumulation in FP32; its error against FP64 is stated by the tests.
#include <cmath>

#include "stage.cuh"

namespace hgb {
namespace {

constexpr int kBilMax = 13;

struct BilParams {
  const char *in;
  int64_t in_pitch, in_bstride;
  char *out;
  int64_t out_pitch, out_bstride;
  int w, h;
  int bmode;
  float cval;
  int vec_in, vec_out;
  float k2;                         // -c_r * log2(e)
  float lmask[kBilMax * kBilMax];   // log2(mask), -inf for zero cells
};

constexpr int BL_BX = 16, BL_BY = 16, BL_PX = 4;
constexpr int BL_TW = BL_BX * BL_PX, BL_TH = BL_BY;

template <typename T, int S>
struct BilShape {
  static constexpr int R = S / 2;
  static constexpr int VI = Vec16<T>::N;
  static constexpr int HL = round_up(R, VI);
  static constexpr int SW = HL + BL_TW + round_up(R, VI);
  static constexpr int SH = BL_TH + S - 1;
};

__device__ __forceinline__ float fast_exp2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

template <typename T, int S, bool FAST>
__global__ void __launch_bounds__(BL_BX *BL_BY) bilateral_kernel(const __grid_constant__ BilParams p) {
  using SH_ = BilShape<T, S>;
  constexpr int R = SH_::R, HL = SH_::HL, SW = SH_::SW, SH = SH_::SH;
  __shared__ __align__(16) float tile[SH * SW];
  const int b = blockIdx.z;
  const int i0 = blockIdx.x * BL_TW, j0 = blockIdx.y * BL_TH;
  stage_tile<T, SW, SH, BL_BX * BL_BY>(tile, p.in + (int64_t)b * p.in_bstride, p.in_pitch, i0 - HL, j0 - R, 0, p.w,
                                        0, p.h, p.bmode, p.cval, p.vec_in);
  __syncthreads();
  const int tx = threadIdx.x % BL_BX, ty = threadIdx.x / BL_BX;
  constexpr int OFF = (HL - R) % 4;
  constexpr int NV = cdiv(OFF + BL_PX + S - 1, 4);
  const int cb = HL - R - OFF + tx * BL_PX;
  float ctr[BL_PX], d[BL_PX], pp[BL_PX];
#pragma unroll
  for (int px = 0; px < BL_PX; ++px) {
    ctr[px] = tile[(ty + R) * SW + HL + tx * BL_PX + px];
    d[px] = 0.0f;
    pp[px] = 0.0f;
  }
#pragma unroll 1
  for (int my = 0; my < S; ++my) {
    float win[NV * 4];
    const float *row = &tile[(ty + my) * SW + cb];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const float4 t = *reinterpret_cast<const float4 *>(row + 4 * v);
      win[4 * v] = t.x;
      win[4 * v + 1] = t.y;
      win[4 * v + 2] = t.z;
      win[4 * v + 3] = t.w;
    }
    if constexpr (!FAST) {
#pragma unroll
      for (int mx = 0; mx < S; ++mx) {
        const float lm = p.lmask[my * S + mx];
#pragma unroll
        for (int px = 0; px < BL_PX; ++px) {
          const float v = win[OFF + px + mx];
          const float df = v - ctr[px];
          const float s = fast_exp2(__fmaf_rn(p.k2 * df, df, lm));
          d[px] += s;
          pp[px] = __fmaf_rn(s, v, pp[px]);
        }
      }
    } else {
      // two outputs per half2: lanes (px, px+1)
      const __half2 k2h = __float2half2_rn(p.k2);
      __half2 c01 = __floats2half2_rn(ctr[0], ctr[1]), c23 = __floats2half2_rn(ctr[2], ctr[3]);
#pragma unroll
      for (int mx = 0; mx < S; ++mx) {
        const __half2 lm = __float2half2_rn(p.lmask[my * S + mx]);
        const __half2 v01 = __floats2half2_rn(win[OFF + mx], win[OFF + mx + 1]);
        const __half2 v23 = __floats2half2_rn(win[OFF + mx + 2], win[OFF + mx + 3]);
        const __half2 df01 = __hsub2(v01, c01), df23 = __hsub2(v23, c23);
        const float2 s01 = __half22float2(h2exp2(__hfma2(__hmul2(k2h, df01), df01, lm)));
        const float2 s23 = __half22float2(h2exp2(__hfma2(__hmul2(k2h, df23), df23, lm)));
        d[0] += s01.x;
        d[1] += s01.y;
        d[2] += s23.x;
        d[3] += s23.y;
        pp[0] = __fmaf_rn(s01.x, win[OFF + mx], pp[0]);
        pp[1] = __fmaf_rn(s01.y, win[OFF + mx + 1], pp[1]);
        pp[2] = __fmaf_rn(s23.x, win[OFF + mx + 2], pp[2]);
        pp[3] = __fmaf_rn(s23.y, win[OFF + mx + 3], pp[3]);
      }
    }
  }
  float res[BL_PX];
#pragma unroll
  for (int px = 0; px < BL_PX; ++px) res[px] = __fdiv_rn(pp[px], d[px]);
  const int i = i0 + tx * BL_PX, j = j0 + ty;
  if (j < p.h && i < p.w)
    store_row<T, BL_PX>(reinterpret_cast<T *>(p.out + (int64_t)b * p.out_bstride + (int64_t)j * p.out_pitch) + i, res, i,
                        p.w, p.vec_out);
}

template <typename T, int S, bool FAST>
int launch_bil_s(const BilParams &p, int batch, cudaStream_t st) {
  dim3 grid(cdiv(p.w, BL_TW), cdiv(p.h, BL_TH), batch);
  cudaEvent_t ev = before_launch(st);
  bilateral_kernel<T, S, FAST><<<grid, BL_BX * BL_BY, 0, st>>>(p);
  return after_launch("bilateral_kernel", st, ev);
}

template <typename T, bool FAST>
int launch_bil(const BilParams &p, int size, int batch, cudaStream_t st) {
  switch (size) {
    case 3: return launch_bil_s<T, 3, FAST>(p, batch, st);
    case 5: return launch_bil_s<T, 5, FAST>(p, batch, st);
    case 7: return launch_bil_s<T, 7, FAST>(p, batch, st);
    case 9: return launch_bil_s<T, 9, FAST>(p, batch, st);
    case 11: return launch_bil_s<T, 11, FAST>(p, batch, st);
    case 13: return launch_bil_s<T, 13, FAST>(p, batch, st);
  }
  return set_error(HGB_ERR_UNSUPPORTED, "hgb_bilateral: size must be odd, 3..13");
}

}  // namespace
}  // namespace hgb

using namespace hgb;

extern "C" int hgb_bilateral(const hgb_view *in, const hgb_view *out, const float *smask, int size, float sigma_r,
                             int boundary, float const_val, int flags, void *stream) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  rc = check_view(out, "out");
  if (rc) return rc;
  HGB_REQUIRE(in->dtype == out->dtype && is_float_storage(in->dtype), "hgb_bilateral: same float storage expected");
  HGB_REQUIRE(in->width == out->width && in->height == out->height && in->batch == out->batch,
              "hgb_bilateral: size mismatch");
  HGB_REQUIRE(smask, "hgb_bilateral: null mask");
  HGB_REQUIRE(size >= 3 && size <= kBilMax && (size & 1), "hgb_bilateral: size must be odd, 3..13");
  HGB_REQUIRE(sigma_r > 0.0f, "hgb_bilateral: sigma_r must be positive");
  HGB_REQUIRE(boundary >= 0 && boundary <= 4, "hgb_bilateral: bad boundary");
  const bool fast = (flags & 1) != 0;
  HGB_REQUIRE(!fast || in->dtype != HGB_F32, "hgb_bilateral: packed half weights need bf16 / f16 storage");
  BilParams p;
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
  const double c_r = 0.5 / ((double)sigma_r * (double)sigma_r);
  p.k2 = (float)(-c_r * 1.4426950408889634);  // log2(e)
  for (int i = 0; i < size * size; ++i)
    p.lmask[i] = smask[i] > 0.0f ? (float)std::log2((double)smask[i]) : -INFINITY;
  for (int i = 0; i < size * size; ++i)
    HGB_REQUIRE(smask[i] >= 0.0f, "hgb_bilateral: spatial weights must be non-negative");
  cudaStream_t st = (cudaStream_t)stream;
  switch (in->dtype) {
    case HGB_F32: return launch_bil<float, false>(p, size, in->batch, st);
    case HGB_BF16:
      return fast ? launch_bil<__nv_bfloat16, true>(p, size, in->batch, st)
                  : launch_bil<__nv_bfloat16, false>(p, size, in->batch, st);
    default:
      return fast ? launch_bil<__half, true>(p, size, in->batch, st) : launch_bil<__half, false>(p, size, in->batch, st);
  }
}

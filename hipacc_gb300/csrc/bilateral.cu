// bilateral.cu -- hgb_bilateral: the bilateral filter of
// samples-public/3_Preprocessing/Bilateral_Filter/src/main.cpp:63-77:
//   c_r = 0.5 / sigma_r^2, centre = in(),
//   for every Domain(mask) cell: diff = in(dom) - centre,
//     s = exp(-c_r * diff^2) * mask(dom);  d += s;  p += s * in(dom)
//   out = p / d
// with a float range sigma and a float result.
//
// The filter is bound by arithmetic (one exponential and four FP32 lane
// operations per tap and pixel), not by HBM.  The weight is one base-2
// exponential with the spatial weight folded into the exponent; the staged
// tile is pre-scaled by q = sqrt(c_r * log2(e)), so that the exponent of a
// tap is a single fused multiply-add of the scaled difference d':
//   s = exp2(-(d'^2 + nl)),  nl = -log2(mask)
// (mask cells of 0 give nl = +inf, i.e. s = 0, which is the Domain's skip),
// and out = (sum s * v') / (sum s) / q.  The FP32 path evaluates the
// differences and the two sums for two pixels per packed f32x2 operation and
// the exponential with ex2.approx (32 per clock and SM on this part).
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
  float q, inv_q;                   // sqrt(-k2) and 1 / q: the FP32 path's tile scale
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
  if constexpr (!FAST) {
    // the FP32 path works on values scaled by q
    for (int c = threadIdx.x; c < SH * SW; c += BL_BX * BL_BY) tile[c] = __fmul_rn(tile[c], p.q);
    __syncthreads();
  }
  const int tx = threadIdx.x % BL_BX, ty = threadIdx.x / BL_BX;
  constexpr int OFF = (HL - R) % 4;
  constexpr int NV = cdiv(OFF + BL_PX + S - 1, 4);
  const int cb = HL - R - OFF + tx * BL_PX;
  float ctr[BL_PX], d[BL_PX], pp[BL_PX];
  // FP32 path: two pixels per f32x2 lane pair
  f2 C2[BL_PX / 2], D2[BL_PX / 2], P2[BL_PX / 2];
#pragma unroll
  for (int px = 0; px < BL_PX; ++px) {
    ctr[px] = tile[(ty + R) * SW + HL + tx * BL_PX + px];
    d[px] = 0.0f;
    pp[px] = 0.0f;
  }
#pragma unroll
  for (int k = 0; k < BL_PX / 2; ++k) {
    C2[k] = f2_pack(ctr[2 * k], ctr[2 * k + 1]);
    D2[k] = 0ull;
    P2[k] = 0ull;
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
      // window pairs starting at even (E) and odd (O) positions
      f2 E[NV * 2], O[NV * 2];
#pragma unroll
      for (int j = 0; j < NV * 2; ++j) {
        E[j] = f2_pack(win[2 * j], win[2 * j + 1]);
        O[j] = f2_pack(win[2 * j + 1], 2 * j + 2 < NV * 4 ? win[2 * j + 2] : 0.0f);
      }
#pragma unroll
      for (int mx = 0; mx < S; ++mx) {
        const float nl = -p.lmask[my * S + mx];
        const f2 NL = f2_pack(nl, nl);
#pragma unroll
        for (int k = 0; k < BL_PX / 2; ++k) {
          const int st = OFF + 2 * k + mx;  // window position of the pair's first pixel
          const f2 V = (st & 1) ? O[st >> 1] : E[st >> 1];
          const f2 df = f2_sub(V, C2[k]);
          const f2 t = f2_fma(df, df, NL);  // d'^2 - lm (measured faster than scalar lm - d'^2)
          const f2 sw = f2_pack(fast_exp2(-f2_lo(t)), fast_exp2(-f2_hi(t)));
          D2[k] = f2_add(D2[k], sw);
          P2[k] = f2_fma(sw, V, P2[k]);
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
  if constexpr (!FAST) {
#pragma unroll
    for (int k = 0; k < BL_PX / 2; ++k) {
      res[2 * k] = __fmul_rn(__fdiv_rn(f2_lo(P2[k]), f2_lo(D2[k])), p.inv_q);
      res[2 * k + 1] = __fmul_rn(__fdiv_rn(f2_hi(P2[k]), f2_hi(D2[k])), p.inv_q);
    }
  } else {
#pragma unroll
    for (int px = 0; px < BL_PX; ++px) res[px] = __fdiv_rn(pp[px], d[px]);
  }
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
  p.q = (float)std::sqrt(c_r * 1.4426950408889634);
  p.inv_q = (float)(1.0 / std::sqrt(c_r * 1.4426950408889634));
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

// stage.cuh -- staging of a halo tile into shared memory as FP32.
//
// Rows [Y0, Y0 + SH) x columns [X0, X0 + SW) of an accessor window
// [ax_lo, ax_hi) x [ay_lo, ay_hi) are copied into `tile` (row pitch SW
// floats).  Chunks of 16 bytes that lie inside the window are loaded with one
// vector load; chunks that leave it are assembled element by element through
// the boundary remap (lib/AST/BorderHandling.cpp:41-120), CONSTANT cells
// reading `cval`.  Vector loads require X0 to be a multiple of the storage's
// 16-byte element count and a 16-byte aligned row base (the caller's `vec`).
#pragma once

#include "hgb_internal.cuh"

namespace hgb {

template <typename TI, int SW, int SH, int NT>
__device__ __forceinline__ void stage_tile(float *tile, const char *in, int64_t pitch, int X0, int Y0, int ax_lo,
                                           int ax_hi, int ay_lo, int ay_hi, int bmode, float cval, bool vec) {
  constexpr int VI = Vec16<TI>::N;
  constexpr int CPR = SW / VI;
  static_assert(SW % VI == 0, "staged row must be whole 16-byte chunks");
  const bool interior = X0 >= ax_lo && X0 + SW <= ax_hi && Y0 >= ay_lo && Y0 + SH <= ay_hi;
  if (interior && vec) {
#pragma unroll 4
    for (int c = threadIdx.x; c < SH * CPR; c += NT) {
      const int r = c / CPR, k = c - r * CPR;
      const TI *src = reinterpret_cast<const TI *>(in + (int64_t)(Y0 + r) * pitch) + X0 + k * VI;
      float f[VI];
      Vec16<TI>::unpack(ldg16(src), f);
      float *dst = &tile[r * SW + k * VI];
#pragma unroll
      for (int q = 0; q < VI; q += 4) *reinterpret_cast<float4 *>(dst + q) = make_float4(f[q], f[q + 1], f[q + 2], f[q + 3]);
    }
    return;
  }
  for (int c = threadIdx.x; c < SH * CPR; c += NT) {
    const int r = c / CPR, k = c - r * CPR;
    const int ay = Y0 + r, ax0 = X0 + k * VI;
    float f[VI];
    if (vec && ay >= ay_lo && ay < ay_hi && ax0 >= ax_lo && ax0 + VI <= ax_hi) {
      const TI *src = reinterpret_cast<const TI *>(in + (int64_t)ay * pitch) + ax0;
      Vec16<TI>::unpack(ldg16(src), f);
    } else {
      const int ry = remap(bmode, ay, ay_lo, ay_hi);
      const TI *row = reinterpret_cast<const TI *>(in + (int64_t)(ry == (int)0x80000000 ? ay_lo : ry) * pitch);
#pragma unroll
      for (int q = 0; q < VI; ++q) {
        const int rx = remap(bmode, ax0 + q, ax_lo, ax_hi);
        f[q] = (rx == (int)0x80000000 || ry == (int)0x80000000) ? cval : Storage<TI>::load(row + rx);
      }
    }
    float *dst = &tile[r * SW + k * VI];
#pragma unroll
    for (int q = 0; q < VI; q += 4) *reinterpret_cast<float4 *>(dst + q) = make_float4(f[q], f[q + 1], f[q + 2], f[q + 3]);
  }
}

// store PX (multiple of 4) consecutive outputs of one row
template <typename TO, int PX>
__device__ __forceinline__ void store_row(TO *dst, const float *v, int i, int is_w, bool vec) {
  if (vec && i + PX <= is_w) {
    if constexpr (sizeof(TO) == 4) {
#pragma unroll
      for (int q = 0; q < PX; q += 4) *reinterpret_cast<float4 *>(dst + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
    } else if constexpr (sizeof(TO) == 1) {
#pragma unroll
      for (int q = 0; q < PX; q += 4)
        *reinterpret_cast<uint32_t *>(dst + q) =
            (uint32_t)Storage<TO>::from_f(v[q]) | ((uint32_t)Storage<TO>::from_f(v[q + 1]) << 8) |
            ((uint32_t)Storage<TO>::from_f(v[q + 2]) << 16) | ((uint32_t)Storage<TO>::from_f(v[q + 3]) << 24);
    } else {
#pragma unroll
      for (int q = 0; q < PX; q += 4) {
        TO t4[4] = {Storage<TO>::from_f(v[q]), Storage<TO>::from_f(v[q + 1]), Storage<TO>::from_f(v[q + 2]),
                    Storage<TO>::from_f(v[q + 3])};
        *reinterpret_cast<uint2 *>(dst + q) = *reinterpret_cast<const uint2 *>(t4);
      }
    }
  } else {
#pragma unroll
    for (int px = 0; px < PX; ++px)
      if (i + px < is_w) dst[px] = Storage<TO>::from_f(v[px]);
  }
}

}  // namespace hgb

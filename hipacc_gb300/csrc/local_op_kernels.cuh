// local_op_kernels.cuh -- launchers and the general-path kernel; included by
// the per-storage-type translation units (lop_sq_*_{f32,bf16,f16,u8}.cu, lop_line_*.cu).
#pragma once

#include "local_op.cuh"

namespace hgb {

// Tile configurations the autotuner chooses from: (BX, BY, PX, PY).
#define HGB_TILE_CFGS(X) \
  X(0, 16, 8, 4, 8)      \
  X(1, 16, 16, 4, 4)     \
  X(2, 32, 4, 4, 8)

template <typename TI, typename TO, int MW, int MH, int BX, int BY, int PX, int PY>
int launch_cfg(const ConvParams &p0, int batch, cudaStream_t st) {
  constexpr int TW = BX * PX, TH = BY * PY;
  constexpr int RX = MW / 2, VI = Vec16<TI>::N;
  constexpr int SW = round_up(RX, VI) + TW + round_up(MW - 1 - RX, VI), SH = TH + MH - 1;
  ConvParams p = p0;
  // FP32 and u8 images read through the whole-image accessor stage their tiles
  // with TMA (the box origin X0 = i0 - round_up(RX, VI) is a multiple of 16 bytes)
  constexpr bool kU8 = std::is_same<TI, uint8_t>::value;
  p.use_tma = 0;
  if ((std::is_same<TI, float>::value || kU8) && p.acc_ox == 0 && p.acc_oy == 0 && p.acc_w == p.in_w &&
      p.acc_h == p.in_h && tma_legal(p.in, p.in_pitch, p.in_bstride, batch) &&
      make_tensor_map_3d(&p.map, kU8 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                         (int)sizeof(TI), p.in, p.in_w, p.in_h, batch, p.in_pitch, p.in_bstride, SW, SH) == HGB_OK) {
    p.use_tma = 1;
    p.status = device_status_word();
  }
  dim3 grid(cdiv(p.is_w, TW), cdiv(p.is_h, TH), batch);
  cudaEvent_t ev = before_launch(st);
  conv_kernel<TI, TO, MW, MH, BX, BY, PX, PY><<<grid, BX * BY, 0, st>>>(p);
  return after_launch("conv_kernel", st, ev);
}

template <typename TI, typename TO, int MW, int MH>
int launch_shape(const ConvParams &p, int batch, cudaStream_t st, int cfg) {
  // masks of 9 x 9 and larger are FMA-bound in every tile shape: one configuration
  if constexpr (MW * MH >= 81) {
    (void)cfg;
    return launch_cfg<TI, TO, MW, MH, 16, 8, 4, 8>(p, batch, st);
  } else {
    switch (cfg) {
#define HGB_CFG_CASE(I, BX, BY, PX, PY) \
  case I: return launch_cfg<TI, TO, MW, MH, BX, BY, PX, PY>(p, batch, st);
      HGB_TILE_CFGS(HGB_CFG_CASE)
#undef HGB_CFG_CASE
    }
    return set_error(HGB_ERR_INVALID, "conv: bad tile configuration");
  }
}

// square masks (translation units per storage type and group of sizes) ...
template <typename TI, typename TO, int K>
int launch_conv_sq(const ConvParams &p, int batch, cudaStream_t st, int cfg) {
  return launch_shape<TI, TO, K, K>(p, batch, st, cfg);
}

// ... and 1xK / Kx1 masks (another one), so that they compile in parallel
template <typename TI, typename TO>
int launch_conv_line(const ConvParams &p, int mw, int mh, int batch, cudaStream_t st, int cfg) {
#define HGB_ROW(K) \
  if (mw == K && mh == 1) return launch_shape<TI, TO, K, 1>(p, batch, st, cfg);
#define HGB_COL(K) \
  if (mw == 1 && mh == K) return launch_shape<TI, TO, 1, K>(p, batch, st, cfg);
  HGB_ROW(3) HGB_ROW(5) HGB_ROW(7) HGB_ROW(9) HGB_ROW(11) HGB_ROW(13)
  HGB_COL(3) HGB_COL(5) HGB_COL(7) HGB_COL(9) HGB_COL(11) HGB_COL(13)
#undef HGB_ROW
#undef HGB_COL
  return set_error(HGB_ERR_UNSUPPORTED, "conv: no fast kernel for this mask shape");
}

// reduce init values: lib/AST/Convolution.cpp:90-100 (MAX starts at FLT_MIN)
__device__ __forceinline__ float reduce_init_f(int red) {
  switch (red) {
    case HGB_REDUCE_MIN: return 3.402823466e+38f;
    case HGB_REDUCE_MAX: return 1.175494351e-38f;
    case HGB_REDUCE_PROD: return 1.0f;
  }
  return 0.0f;
}

template <typename TI, typename TO>
__global__ void __launch_bounds__(256) generic_kernel(const __grid_constant__ GenParams g) {
  constexpr int T = 16;
  constexpr int SMAX = T + kMaxMask - 1;
  __shared__ float tile[SMAX * SMAX];
  __shared__ float smask[kMaxMask * kMaxMask];
  const ConvParams &p = g.c;
  const int mw = g.mw, mh = g.mh, rx = mw / 2, ry = mh / 2;
  const int SW = T + mw - 1, SH = T + mh - 1;
  for (int i = threadIdx.x; i < mw * mh; i += blockDim.x) smask[i] = g.mask_dev ? g.mask_dev[i] : p.mask[i];
  const int b = blockIdx.z;
  const int i0 = blockIdx.x * T, j0 = blockIdx.y * T;
  const char *in = p.in + (int64_t)b * p.in_bstride;
  const int X0 = p.acc_ox + i0 - rx, Y0 = p.acc_oy + j0 - ry;
  const int ax_lo = p.acc_ox, ax_hi = p.acc_ox + p.acc_w, ay_lo = p.acc_oy, ay_hi = p.acc_oy + p.acc_h;
  for (int c = threadIdx.x; c < SW * SH; c += blockDim.x) {
    const int r = c / SW, k = c - r * SW;
    const int ry_ = remap(p.bmode, Y0 + r, ay_lo, ay_hi);
    const int rx_ = remap(p.bmode, X0 + k, ax_lo, ax_hi);
    float v;
    if (ry_ == (int)0x80000000 || rx_ == (int)0x80000000)
      v = p.cval;
    else
      v = Storage<TI>::load(reinterpret_cast<const TI *>(in + (int64_t)ry_ * p.in_pitch) + rx_);
    tile[r * SW + k] = v;
  }
  __syncthreads();
  const int tx = threadIdx.x % T, ty = threadIdx.x / T;
  const int i = i0 + tx, j = j0 + ty;
  if (i >= p.is_w || j >= p.is_h) return;
  const int red = g.reduce;
  float acc = reduce_init_f(red);
  for (int my = 0; my < mh; ++my)
    for (int mx = 0; mx < mw; ++mx) {
      if (!g.domain[my * mw + mx]) continue;
      const float x = tile[(ty + my) * SW + tx + mx];
      const float m = smask[my * mw + mx];
      if (red == HGB_REDUCE_SUM) {
        acc = g.has_mask ? __fmaf_rn(m, x, acc) : __fadd_rn(acc, x);
      } else {
        const float v = g.has_mask ? __fmul_rn(m, x) : x;
        if (red == HGB_REDUCE_MIN)
          acc = acc < v ? acc : v;
        else if (red == HGB_REDUCE_MAX)
          acc = acc > v ? acc : v;
        else
          acc = __fmul_rn(acc, v);
      }
    }
  char *out = p.out + (int64_t)b * p.out_bstride;
  reinterpret_cast<TO *>(out + (int64_t)(p.is_oy + j) * p.out_pitch)[p.is_ox + i] = Storage<TO>::from_f(acc);
}

template <typename TI, typename TO>
int launch_generic(const GenParams &g, int batch, cudaStream_t st) {
  dim3 grid(cdiv(g.c.is_w, 16), cdiv(g.c.is_h, 16), batch);
  cudaEvent_t ev = before_launch(st);
  generic_kernel<TI, TO><<<grid, 256, 0, st>>>(g);
  return after_launch("generic_kernel", st, ev);
}

#define HGB_INSTANTIATE_SQ(TI, TO, K) template int launch_conv_sq<TI, TO, K>(const ConvParams &, int, cudaStream_t, int);
#define HGB_INSTANTIATE_LINE(TI, TO) \
  template int launch_conv_line<TI, TO>(const ConvParams &, int, int, int, cudaStream_t, int);
#define HGB_INSTANTIATE_GENERIC(TI, TO) template int launch_generic<TI, TO>(const GenParams &, int, cudaStream_t);

}  // namespace hgb

// local_op.cuh -- local operator kernels (mask / domain stencils).
//
// Semantics: one output pixel of Hipacc's generated local-operator kernel
// (lib/AST/ASTTranslate.cpp:510-1197): the mask is unrolled row-major
// (lib/AST/Convolution.cpp:397-435) starting from get_init(mode)
// (lib/AST/Convolution.cpp:90-100); every tap reads the accessor through the
// boundary remap (lib/AST/BorderHandling.cpp:124-407).
//
// GB300 design: a CTA computes a TW x TH output tile.  Its input tile plus
// halo is staged once in shared memory as FP32: for FP32 and u8 images read
// through the whole-image accessor by one cp.async.bulk.tensor load (u8 bytes
// are widened in shared memory; cells outside the image, which TMA fills with
// zeros, are then patched with the boundary rule),
// otherwise with 16-byte global loads, remapping element by element only the
// chunks that leave the accessor window.  Each thread keeps a PX x PY block of
// outputs in registers as horizontal pairs and streams the input rows of its
// column window through registers; every tap is one packed f32x2 fused
// multiply-add for two outputs.  SUM keeps the row-major tap order per output,
// the contracted form of the reference's `_tmp += m*x`, bit for bit.
#pragma once

#include <type_traits>

#include "tma.cuh"

namespace hgb {

constexpr int kMaxMask = 15;

struct ConvParams {
  CUtensorMap map;                   // FP32 input, whole image: TMA staging when use_tma
  int use_tma;
  int *status;
  int in_w, in_h, batch;             // input image size (tensor-map extent)
  const char *in;
  int64_t in_pitch, in_bstride;
  char *out;
  int64_t out_pitch, out_bstride;
  int acc_ox, acc_oy, acc_w, acc_h;  // Accessor window (absolute, input)
  int is_ox, is_oy, is_w, is_h;      // IterationSpace window (absolute, output)
  int bmode;
  float cval;
  int vec_in, vec_out;               // 16-byte vector access legal
  float mask[kMaxMask * kMaxMask];   // row-major, padded shape
  f2 mask2[kMaxMask * kMaxMask];     // the same coefficients as (m, m) pairs for f32x2 FMAs
};

struct TileCfg {
  int bx, by, px, py;
};

// fast SUM-convolution kernels exist for these padded shapes
constexpr int kFastSizes[] = {3, 5, 7, 9, 11, 13};

template <typename TI, typename TO, int MW, int MH, int BX, int BY, int PX, int PY>
__global__ void __launch_bounds__(BX *BY) conv_kernel(const __grid_constant__ ConvParams p) {
  constexpr int NT = BX * BY;
  constexpr int RX = MW / 2, RY = MH / 2;
  constexpr int TW = BX * PX, TH = BY * PY;
  constexpr int VI = Vec16<TI>::N;
  constexpr int HL = round_up(RX, VI);
  constexpr int HR = round_up(MW - 1 - RX, VI);
  constexpr int SW = HL + TW + HR;
  constexpr int SH = TH + MH - 1;
  constexpr int CPR = SW / VI;
  static_assert(TW % VI == 0 && SW % 4 == 0 && PX % 4 == 0, "tile shape");
  constexpr bool kTma = std::is_same<TI, float>::value || std::is_same<TI, uint8_t>::value;
  constexpr bool kU8 = std::is_same<TI, uint8_t>::value;
  // The FP32 tile the stencil reads.  u8: only the columns the taps reach
  // (halos rounded to 4), while the byte box keeps 16-byte aligned halos
  // for TMA; the narrower tile leaves room for more CTAs per SM.
  constexpr int HLF = kU8 ? round_up(RX, 4) : HL;
  constexpr int SWF = kU8 ? HLF + TW + round_up(MW - 1 - RX, 4) : SW;
  static_assert(SWF % 4 == 0 && (HL - HLF) % 4 == 0, "u8 tile shape");
  __shared__ __align__(128) float tile[SH * SWF];
  // u8: the TMA box lands here as bytes and is widened into `tile`
  __shared__ __align__(128) uint8_t raw[kU8 ? SH * SW : 16];
  __shared__ __align__(8) uint64_t bar;

  const int b = blockIdx.z;
  const int i0 = blockIdx.x * TW, j0 = blockIdx.y * TH;
  const char *in = p.in + (int64_t)b * p.in_bstride;
  const int X0 = p.acc_ox + i0 - HL;
  const int Y0 = p.acc_oy + j0 - RY;
  const int ax_lo = p.acc_ox, ax_hi = p.acc_ox + p.acc_w;
  const int ay_lo = p.acc_oy, ay_hi = p.acc_oy + p.acc_h;

  // ---- stage input tile + halo as FP32
  const bool interior = X0 >= ax_lo && X0 + SW <= ax_hi && Y0 >= ay_lo && Y0 + SH <= ay_hi;
  if (kTma && p.use_tma) {
    // the accessor window is the whole image: one TMA load of the box
    if (threadIdx.x == 0) {
      mbar_init(&bar, 1);
      mbar_fence_init();
      mbar_expect_tx(&bar, SH * SW * (int)sizeof(TI));
      tma_load_3d(kU8 ? (void *)raw : (void *)tile, &p.map, X0, Y0, b, &bar);
    }
    if (!cta_wait(&bar, 0)) {
      if (threadIdx.x == 0) {
        record_status(p.status, HGB_ERR_TIMEOUT);
        mbar_wait(&bar, 0);  // the load may still land: wait once more (bounded) before leaving
      }
      return;
    }
    if constexpr (kU8) {
      // widen 4 bytes at a time: a byte b placed in the mantissa of 2^23 gives
      // 2^23 + b exactly, and subtracting 2^23 leaves b
      const f2 k23 = f2_pack(8388608.0f, 8388608.0f);
      for (int c = threadIdx.x; c < SH * SWF / 4; c += NT) {
        const int r = c / (SWF / 4), q4 = c - r * (SWF / 4);
        const uint32_t w = reinterpret_cast<const uint32_t *>(raw + r * SW + (HL - HLF))[q4];
        const f2 lo = f2_sub(f2_pack(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440)),
                                     __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7441))), k23);
        const f2 hi = f2_sub(f2_pack(__uint_as_float(__byte_perm(w, 0x4B000000u, 0x7442)),
                                     __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7443))), k23);
        reinterpret_cast<float4 *>(tile)[c] = make_float4(f2_lo(lo), f2_hi(lo), f2_lo(hi), f2_hi(hi));
      }
      if (!interior) __syncthreads();  // the patch below overwrites widened cells
    }
    if (!interior) {
      // cells outside the image (zero-filled by TMA): left / right columns, top
      // / bottom rows of the FP32 tile (its columns start at X0 + HL - HLF)
      const int XF = X0 + (HL - HLF);
      const int nl = max(0, min(SWF, ax_lo - XF)), rs = max(0, min(SWF, ax_hi - XF));
      const int nt = max(0, min(SH, ay_lo - Y0)), bs = max(0, min(SH, ay_hi - Y0));
      const int ncl = nl * SH, ncr = (SWF - rs) * SH, nrt = nt * SWF, nrb = (SH - bs) * SWF;
      for (int c = threadIdx.x; c < ncl + ncr + nrt + nrb; c += NT) {
        int r, q;
        if (c < ncl) {
          r = c / nl;
          q = c - r * nl;
        } else if (c < ncl + ncr) {
          const int d = c - ncl, n = SWF - rs;
          r = d / n;
          q = rs + (d - r * n);
        } else if (c < ncl + ncr + nrt) {
          const int d = c - ncl - ncr;
          r = d / SWF;
          q = d - r * SWF;
        } else {
          const int d = c - ncl - ncr - nrt;
          const int rr = d / SWF;
          r = bs + rr;
          q = d - rr * SWF;
        }
        const int ry = remap(p.bmode, Y0 + r, ay_lo, ay_hi), rx = remap(p.bmode, XF + q, ax_lo, ax_hi);
        tile[r * SWF + q] = (ry == (int)0x80000000 || rx == (int)0x80000000)
                               ? p.cval
                               : Storage<TI>::load(reinterpret_cast<const TI *>(in + (int64_t)ry * p.in_pitch) + rx);
      }
    }
  } else if constexpr (kU8) {
    // u8 without TMA: bytes through the boundary rule straight into the FP32 tile
    const int XF = X0 + (HL - HLF);
    for (int c = threadIdx.x; c < SH * SWF; c += NT) {
      const int r = c / SWF, q = c - r * SWF;
      const int ry = remap(p.bmode, Y0 + r, ay_lo, ay_hi), rx = remap(p.bmode, XF + q, ax_lo, ax_hi);
      tile[c] = (ry == (int)0x80000000 || rx == (int)0x80000000)
                    ? p.cval
                    : Storage<TI>::load(reinterpret_cast<const TI *>(in + (int64_t)ry * p.in_pitch) + rx);
    }
  } else {
    if (interior && p.vec_in) {
#pragma unroll 4
      for (int c = threadIdx.x; c < SH * CPR; c += NT) {
        const int r = c / CPR, k = c - r * CPR;
        const TI *src = reinterpret_cast<const TI *>(in + (int64_t)(Y0 + r) * p.in_pitch) + X0 + k * VI;
        float f[VI];
        Vec16<TI>::unpack(ldg16(src), f);
        float *dst = &tile[r * SW + k * VI];
#pragma unroll
        for (int q = 0; q < VI; q += 4) *reinterpret_cast<float4 *>(dst + q) = make_float4(f[q], f[q + 1], f[q + 2], f[q + 3]);
      }
    } else {
      for (int c = threadIdx.x; c < SH * CPR; c += NT) {
        const int r = c / CPR, k = c - r * CPR;
        const int ay = Y0 + r, ax0 = X0 + k * VI;
        float f[VI];
        if (p.vec_in && ay >= ay_lo && ay < ay_hi && ax0 >= ax_lo && ax0 + VI <= ax_hi) {
          const TI *src = reinterpret_cast<const TI *>(in + (int64_t)ay * p.in_pitch) + ax0;
          Vec16<TI>::unpack(ldg16(src), f);
        } else {
          const int ry = remap(p.bmode, ay, ay_lo, ay_hi);
          const TI *row = reinterpret_cast<const TI *>(in + (int64_t)(ry == (int)0x80000000 ? ay_lo : ry) * p.in_pitch);
#pragma unroll
          for (int q = 0; q < VI; ++q) {
            const int rx = remap(p.bmode, ax0 + q, ax_lo, ax_hi);
            f[q] = (rx == (int)0x80000000 || ry == (int)0x80000000) ? p.cval : Storage<TI>::load(row + rx);
          }
        }
        float *dst = &tile[r * SW + k * VI];
#pragma unroll
        for (int q = 0; q < VI; q += 4) *reinterpret_cast<float4 *>(dst + q) = make_float4(f[q], f[q + 1], f[q + 2], f[q + 3]);
      }
    }
  }
  __syncthreads();

  // ---- register-blocked stencil
  const int tx = threadIdx.x % BX, ty = threadIdx.x / BX;
  constexpr int OFF = (HLF - RX) % 4;
  constexpr int NV = cdiv(OFF + PX + MW - 1, 4);
  const int cbase = HLF - RX - OFF + tx * PX;
  constexpr int NP = PX / 2;
  f2 acc2[PY][NP];
#pragma unroll
  for (int oy = 0; oy < PY; ++oy)
#pragma unroll
    for (int pp = 0; pp < NP; ++pp) acc2[oy][pp] = 0ull;

#pragma unroll
  for (int r = 0; r < PY + MH - 1; ++r) {
    float win[NV * 4];
    const float *row = &tile[(ty * PY + r) * SWF + cbase];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const float4 t = *reinterpret_cast<const float4 *>(row + 4 * v);
      win[4 * v] = t.x;
      win[4 * v + 1] = t.y;
      win[4 * v + 2] = t.z;
      win[4 * v + 3] = t.w;
    }
    // window pairs starting at even (E) and odd (O) positions
    f2 E[NV * 2], O[NV * 2];
#pragma unroll
    for (int j = 0; j < NV * 2; ++j) {
      E[j] = f2_pack(win[2 * j], win[2 * j + 1]);
      O[j] = f2_pack(win[2 * j + 1], 2 * j + 2 < NV * 4 ? win[2 * j + 2] : 0.0f);
    }
#pragma unroll
    for (int oy = 0; oy < PY; ++oy) {
      const int my = r - oy;
      if (my < 0 || my >= MH) continue;
#pragma unroll
      for (int mx = 0; mx < MW; ++mx) {
        const f2 m2 = p.mask2[my * MW + mx];
#pragma unroll
        for (int pp = 0; pp < NP; ++pp) {
          const int st = OFF + 2 * pp + mx;  // window position of the pair's first output
          acc2[oy][pp] = f2_fma(m2, (st & 1) ? O[st >> 1] : E[st >> 1], acc2[oy][pp]);
        }
      }
    }
  }
  float acc[PY][PX];
#pragma unroll
  for (int oy = 0; oy < PY; ++oy)
#pragma unroll
    for (int pp = 0; pp < NP; ++pp) {
      acc[oy][2 * pp] = f2_lo(acc2[oy][pp]);
      acc[oy][2 * pp + 1] = f2_hi(acc2[oy][pp]);
    }

  // ---- store
  char *out = p.out + (int64_t)b * p.out_bstride;
  const int i = i0 + tx * PX;
#pragma unroll
  for (int oy = 0; oy < PY; ++oy) {
    const int j = j0 + ty * PY + oy;
    if (j >= p.is_h || i >= p.is_w) continue;
    TO *dst = reinterpret_cast<TO *>(out + (int64_t)(p.is_oy + j) * p.out_pitch) + p.is_ox + i;
    if (p.vec_out && i + PX <= p.is_w) {
      if constexpr (sizeof(TO) == 4) {
#pragma unroll
        for (int q = 0; q < PX; q += 4)
          *reinterpret_cast<float4 *>(dst + q) = make_float4(acc[oy][q], acc[oy][q + 1], acc[oy][q + 2], acc[oy][q + 3]);
      } else if constexpr (sizeof(TO) == 1) {
#pragma unroll
        for (int q = 0; q < PX; q += 4) {
          const uint32_t wv = (uint32_t)Storage<TO>::from_f(acc[oy][q]) |
                              ((uint32_t)Storage<TO>::from_f(acc[oy][q + 1]) << 8) |
                              ((uint32_t)Storage<TO>::from_f(acc[oy][q + 2]) << 16) |
                              ((uint32_t)Storage<TO>::from_f(acc[oy][q + 3]) << 24);
          *reinterpret_cast<uint32_t *>(dst + q) = wv;
        }
      } else {
#pragma unroll
        for (int q = 0; q < PX; q += 4) {
          TO t4[4] = {Storage<TO>::from_f(acc[oy][q]), Storage<TO>::from_f(acc[oy][q + 1]),
                      Storage<TO>::from_f(acc[oy][q + 2]), Storage<TO>::from_f(acc[oy][q + 3])};
          *reinterpret_cast<uint2 *>(dst + q) = *reinterpret_cast<const uint2 *>(t4);
        }
      }
    } else {
#pragma unroll
      for (int px = 0; px < PX; ++px)
        if (i + px < p.is_w) dst[px] = Storage<TO>::from_f(acc[oy][px]);
    }
  }
}

// General path: any mask shape up to 15x15, any reduce mode, optional domain,
// mask from host parameters or from device memory.  One output per thread.
struct GenParams {
  ConvParams c;
  int mw, mh, reduce;
  int has_mask;
  const float *mask_dev;
  uint8_t domain[kMaxMask * kMaxMask];
};

// square K x K kernels, instantiated per (storage type, K) in the lop_sq_* translation units
template <typename TI, typename TO, int K>
int launch_conv_sq(const ConvParams &p, int batch, cudaStream_t st, int cfg_index);
template <typename TI, typename TO>
int launch_conv_square(const ConvParams &p, int mw, int mh, int batch, cudaStream_t st, int cfg_index) {
  (void)mh;
  switch (mw) {
    case 3: return launch_conv_sq<TI, TO, 3>(p, batch, st, cfg_index);
    case 5: return launch_conv_sq<TI, TO, 5>(p, batch, st, cfg_index);
    case 7: return launch_conv_sq<TI, TO, 7>(p, batch, st, cfg_index);
    case 9: return launch_conv_sq<TI, TO, 9>(p, batch, st, cfg_index);
    case 11: return launch_conv_sq<TI, TO, 11>(p, batch, st, cfg_index);
    case 13: return launch_conv_sq<TI, TO, 13>(p, batch, st, cfg_index);
  }
  return set_error(HGB_ERR_UNSUPPORTED, "conv: no fast kernel for this mask shape");
}
template <typename TI, typename TO>
int launch_conv_line(const ConvParams &p, int mw, int mh, int batch, cudaStream_t st, int cfg_index);
template <typename TI, typename TO>
int launch_conv(const ConvParams &p, int mw, int mh, int batch, cudaStream_t st, int cfg_index) {
  return (mw == mh) ? launch_conv_square<TI, TO>(p, mw, mh, batch, st, cfg_index)
                    : launch_conv_line<TI, TO>(p, mw, mh, batch, st, cfg_index);
}
template <typename TI, typename TO>
int launch_generic(const GenParams &p, int batch, cudaStream_t st);

int num_tile_cfgs();
TileCfg tile_cfg(int i);

}  // namespace hgb

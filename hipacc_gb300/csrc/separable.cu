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
//
// GB300 form: a TMA-legal image (16-byte aligned base, pitch and batch
// stride) is staged by one cp.async.bulk.tensor load per CTA in its storage
// type, and the row pass widens bf16 / f16 as it reads (half the shared memory
// of an FP32 tile, so more CTAs per SM); cells outside the image, which TMA
// fills with zeros, are patched with the boundary rule (a CONSTANT cell holds
// the constant in the storage type).  Other layouts stage an FP32 tile with
// 16-byte global loads.  Both passes run packed f32x2 fused multiply-adds on
// pairs of adjacent outputs, keeping each output's tap order.
#include <algorithm>
#include <type_traits>

#include "stage.cuh"
#include "tma.cuh"

namespace hgb {
namespace {

constexpr int kSepMaxK = 15;

struct SepParams {
  CUtensorMap map;  // storage-type tensor map of the input when use_tma
  int use_tma;
  int *status;
  const char *in;
  int64_t in_pitch, in_bstride;
  char *out;
  int64_t out_pitch, out_bstride;
  int w, h;
  int bmode;
  float cval;
  int vec_in, vec_out;
  float row[kSepMaxK], col[kSepMaxK];
  f2 row2[kSepMaxK], col2[kSepMaxK];  // the same taps as (t, t) pairs
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
  // staged tile: the storage type when TMA stages it, FP32 otherwise; then the row-pass buffer
  static constexpr size_t tile_tma = ((size_t)SH * SW * sizeof(T) + 127) / 128 * 128;
  static constexpr size_t tile_ldg = ((size_t)SH * SW * sizeof(float) + 127) / 128 * 128;
  static constexpr size_t rowbuf = sizeof(float) * (size_t)SH * SP_TW;
  static constexpr size_t smem_tma = tile_tma + rowbuf + 128;
  static constexpr size_t smem_ldg = tile_ldg + rowbuf + 128;
};

// four consecutive staged values as floats (the tile holds the storage type
// or FP32)
template <typename TT>
__device__ __forceinline__ float4 load4(const TT *p) {
  if constexpr (std::is_same<TT, float>::value) {
    return *reinterpret_cast<const float4 *>(p);
  } else {
    const uint2 u = *reinterpret_cast<const uint2 *>(p);
    float f[8];
    Vec16<TT>::unpack(make_uint4(u.x, u.y, 0u, 0u), f);
    return make_float4(f[0], f[1], f[2], f[3]);
  }
}

// row pass over a staged tile: 4 outputs per thread per staged row into the
// FP32 row buffer
template <typename TT, int K, int SW, int SH, int HL>
__device__ __forceinline__ void row_pass(const SepParams &p, const TT *tile, float *rowb, int j0, int tx, int ty) {
  constexpr int R = K / 2;
  constexpr int OFF = (HL - R) % 4;
  constexpr int NV = cdiv(OFF + SP_PX + K - 1, 4);
  const int cb = HL - R - OFF + tx * SP_PX;
  for (int r = ty; r < SH; r += SP_BY) {
    float win[NV * 4];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const float4 t = load4(&tile[r * SW + cb + 4 * v]);
      win[4 * v] = t.x;
      win[4 * v + 1] = t.y;
      win[4 * v + 2] = t.z;
      win[4 * v + 3] = t.w;
    }
    f2 E[NV * 2], O[NV * 2];
#pragma unroll
    for (int j = 0; j < NV * 2; ++j) {
      E[j] = f2_pack(win[2 * j], win[2 * j + 1]);
      O[j] = f2_pack(win[2 * j + 1], 2 * j + 2 < NV * 4 ? win[2 * j + 2] : 0.0f);
    }
    f2 a2[SP_PX / 2];
#pragma unroll
    for (int pp = 0; pp < SP_PX / 2; ++pp) {
      a2[pp] = 0ull;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int st = OFF + 2 * pp + k;
        a2[pp] = f2_fma(p.row2[k], (st & 1) ? O[st >> 1] : E[st >> 1], a2[pp]);
      }
    }
    float acc[SP_PX];
#pragma unroll
    for (int pp = 0; pp < SP_PX / 2; ++pp) {
      acc[2 * pp] = f2_lo(a2[pp]);
      acc[2 * pp + 1] = f2_hi(a2[pp]);
    }
    const int ay = j0 - R + r;
    if (p.bmode == HGB_BOUNDARY_CONSTANT && (ay < 0 || ay >= p.h))
#pragma unroll
      for (int px = 0; px < SP_PX; ++px) acc[px] = p.cval;
    *reinterpret_cast<float4 *>(&rowb[r * SP_TW + tx * SP_PX]) = make_float4(acc[0], acc[1], acc[2], acc[3]);
  }
}

template <typename T, int K>
__global__ void __launch_bounds__(SP_BX *SP_BY) separable_kernel(const __grid_constant__ SepParams p) {
  using S = SepShape<T, K>;
  constexpr int R = S::R, HL = S::HL, SW = S::SW, SH = S::SH;
  constexpr int NT = SP_BX * SP_BY;
  extern __shared__ __align__(128) uint8_t sep_dsm[];
  __shared__ __align__(8) uint64_t bar;
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(sep_dsm) + 127) & ~(uintptr_t)127);
  const int b = blockIdx.z;
  const int i0 = blockIdx.x * SP_TW, j0 = blockIdx.y * SP_TH;
  const int X0 = i0 - HL, Y0 = j0 - R;
  const char *img = p.in + (int64_t)b * p.in_bstride;
  const int tx = threadIdx.x % SP_BX, ty = threadIdx.x / SP_BX;
  float *rowb;
  if (p.use_tma) {
    // the tile stays in the storage type; the row pass widens as it reads
    T *tile = reinterpret_cast<T *>(base);
    rowb = reinterpret_cast<float *>(base + S::tile_tma);
    if (threadIdx.x == 0) {
      mbar_init(&bar, 1);
      mbar_fence_init();
      mbar_expect_tx(&bar, SH * SW * (int)sizeof(T));
      tma_load_3d(tile, &p.map, X0, Y0, b, &bar);
    }
    if (!cta_wait(&bar, 0)) {
      if (threadIdx.x == 0) {
        record_status(p.status, HGB_ERR_TIMEOUT);
        mbar_wait(&bar, 0);  // the load may still land: wait once more (bounded) before leaving
      }
      return;
    }
    if (X0 < 0 || X0 + SW > p.w || Y0 < 0 || Y0 + SH > p.h) {
      // cells outside the image (zero-filled by TMA): left / right columns,
      // top / bottom rows; CONSTANT cells take the constant in the storage type
      const int nl = max(0, min(SW, -X0)), rs = max(0, min(SW, p.w - X0));
      const int nt = max(0, min(SH, -Y0)), bs = max(0, min(SH, p.h - Y0));
      const int ncl = nl * SH, ncr = (SW - rs) * SH, nrt = nt * SW, nrb = (SH - bs) * SW;
      for (int c = threadIdx.x; c < ncl + ncr + nrt + nrb; c += NT) {
        int r, q;
        if (c < ncl) {
          r = c / nl;
          q = c - r * nl;
        } else if (c < ncl + ncr) {
          const int d = c - ncl, n = SW - rs;
          r = d / n;
          q = rs + (d - r * n);
        } else if (c < ncl + ncr + nrt) {
          const int d = c - ncl - ncr;
          r = d / SW;
          q = d - r * SW;
        } else {
          const int d = c - ncl - ncr - nrt;
          const int rr = d / SW;
          r = bs + rr;
          q = d - rr * SW;
        }
        const int ry = remap(p.bmode, Y0 + r, 0, p.h), rx = remap(p.bmode, X0 + q, 0, p.w);
        tile[r * SW + q] = (ry == (int)0x80000000 || rx == (int)0x80000000)
                               ? Storage<T>::from_f(p.cval)
                               : reinterpret_cast<const T *>(img + (int64_t)ry * p.in_pitch)[rx];
      }
    }
    __syncthreads();
    row_pass<T, K, SW, SH, HL>(p, tile, rowb, j0, tx, ty);
  } else {
    float *tile = reinterpret_cast<float *>(base);
    rowb = reinterpret_cast<float *>(base + S::tile_ldg);
    stage_tile<T, SW, SH, NT>(tile, img, p.in_pitch, X0, Y0, 0, p.w, 0, p.h, p.bmode, p.cval, p.vec_in);
    __syncthreads();
    row_pass<float, K, SW, SH, HL>(p, tile, rowb, j0, tx, ty);
  }
  __syncthreads();
  // ---- column pass: 4 x 4 outputs per thread
  f2 c2[SP_PY][SP_PX / 2];
#pragma unroll
  for (int oy = 0; oy < SP_PY; ++oy)
#pragma unroll
    for (int pp = 0; pp < SP_PX / 2; ++pp) c2[oy][pp] = 0ull;
#pragma unroll
  for (int r = 0; r < SP_PY + K - 1; ++r) {
    const float4 t = *reinterpret_cast<const float4 *>(&rowb[(ty * SP_PY + r) * SP_TW + tx * SP_PX]);
    const f2 v01 = f2_pack(t.x, t.y), v23 = f2_pack(t.z, t.w);
#pragma unroll
    for (int oy = 0; oy < SP_PY; ++oy) {
      const int k = r - oy;
      if (k < 0 || k >= K) continue;
      c2[oy][0] = f2_fma(p.col2[k], v01, c2[oy][0]);
      c2[oy][1] = f2_fma(p.col2[k], v23, c2[oy][1]);
    }
  }
  float acc[SP_PY][SP_PX];
#pragma unroll
  for (int oy = 0; oy < SP_PY; ++oy)
#pragma unroll
    for (int pp = 0; pp < SP_PX / 2; ++pp) {
      acc[oy][2 * pp] = f2_lo(c2[oy][pp]);
      acc[oy][2 * pp + 1] = f2_hi(c2[oy][pp]);
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

template <typename T>
constexpr CUtensorMapDataType tma_dtype() {
  return std::is_same<T, float>::value ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
         : std::is_same<T, __half>::value ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                          : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
}

template <typename T, int K>
int launch_sep_k(const SepParams &p0, int batch, cudaStream_t st) {
  using S = SepShape<T, K>;
  SepParams p = p0;
  p.use_tma = 0;
  if (tma_legal(p.in, p.in_pitch, p.in_bstride, batch) &&
      make_tensor_map_3d(&p.map, tma_dtype<T>(), (int)sizeof(T), p.in, p.w, p.h, batch, p.in_pitch, p.in_bstride,
                         S::SW, S::SH) == HGB_OK) {
    p.use_tma = 1;
    p.status = device_status_word();
  }
  const size_t smem = p.use_tma ? S::smem_tma : S::smem_ldg;
  const int rc = ensure_dynamic_smem((const void *)separable_kernel<T, K>, smem);
  if (rc) return rc;
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
    uint32_t rb, cb;
    memcpy(&rb, &p.row[i], 4);
    memcpy(&cb, &p.col[i], 4);
    p.row2[i] = ((f2)rb << 32) | rb;
    p.col2[i] = ((f2)cb << 32) | cb;
  }
  cudaStream_t st = (cudaStream_t)stream;
  switch (in->dtype) {
    case HGB_F32: return launch_sep<float>(p, k, in->batch, st);
    case HGB_BF16: return launch_sep<__nv_bfloat16>(p, k, in->batch, st);
    default: return launch_sep<__half>(p, k, in->batch, st);
  }
}

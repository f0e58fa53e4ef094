// sobel.cu -- u8 Sobel magnitude with the global sum / max of the result fused
// into the same kernel.
//
// Semantics (bit-exact): gx = sum over Domain(mask_x) of mask_x * in,
// gy likewise (samples-public/3_Preprocessing/Sobel/src/main.cpp:56-67 with
// Domain(mask), dsl/mask.hpp:238-250), out = min(|gx| + |gy|, 255); then
// Kernel::reduced_data of the output with a u64 sum and a u8 max
// (dsl/kernel.hpp:121-161).  Integer arithmetic, so every order is exact.
//
// Fast path (the standard 3x3 Sobel masks, TMA-legal layout): sobel3_tma_kernel
// below -- one TMA-staged 128 x 128 tile per CTA, exact fp16x2 arithmetic, the
// sum and max folded into workspace accumulators behind one ticket.  Fallback
// for layouts TMA cannot address (unaligned base or pitch): sobel3_kernel,
// which stages a 128 x 64 tile with 16-byte loads, walks rows with a three-row
// register window and uses the separable form gx = S(x+1) - S(x-1),
// S = top + 2 mid + bottom; gy = D(x-1) + 2 D(x) + D(x+1), D = bottom - top.
// Other masks: sobel_generic_kernel.  The fallbacks reduce sum and max with
// redux.sync across the warp, shared memory across the block and a last-block
// combine of the per-block partials.
#include <algorithm>

#include <cstdio>

#include "autotune.h"
#include "reduce_common.cuh"
#include "tma.cuh"

namespace hgb {

struct SobelParams {
  const uint8_t *in;
  int64_t in_pitch, in_bstride;
  uint8_t *out;
  int64_t out_pitch, out_bstride;
  int w, h;
  int bmode, cval;
  int vec_in, vec_out;
  int size;
  int mx[49], my[49];
  uint64_t *sum_dev;
  uint32_t *max_dev;
  uint2 *partials;  // per block: (sum lo, sum hi) and max in a second array
  uint32_t *partial_max;
  unsigned int *ticket;
};

namespace {

constexpr int SB_BX = 32, SB_BY = 8, SB_PY = 8;
constexpr int SB_TW = SB_BX * 4, SB_TH = SB_BY * SB_PY;
constexpr int SB_HL = 16;
constexpr int SB_SW = SB_HL + SB_TW + 16;  // bytes per staged row
constexpr int SB_SH = SB_TH + 2;

__device__ __forceinline__ void block_reduce_store(const SobelParams &p, uint32_t sum, uint32_t mx) {
  __shared__ uint32_t s_sum[32], s_max[32];
  sum = __reduce_add_sync(0xffffffffu, sum);
  mx = __reduce_max_sync(0xffffffffu, mx);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) {
    s_sum[warp] = sum;
    s_max[warp] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint64_t bs = 0;
    uint32_t bm = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      bs += s_sum[i];
      bm = bm > s_max[i] ? bm : s_max[i];
    }
    const unsigned int r = block_rank();
    p.partials[r] = make_uint2((uint32_t)bs, (uint32_t)(bs >> 32));
    p.partial_max[r] = bm;
  }
  if (take_last_ticket(p.ticket)) {
    // the last block combines all partials in block order
    const unsigned int n = grid_blocks();
    uint64_t ts = 0;
    uint32_t tm = 0;
    for (unsigned int i = threadIdx.x; i < n; i += blockDim.x) {
      const uint2 v = __ldcg(&p.partials[i]);
      ts += (uint64_t)v.x | ((uint64_t)v.y << 32);
      const uint32_t m = __ldcg(&p.partial_max[i]);
      tm = tm > m ? tm : m;
    }
    // 64-bit sums of the per-thread values, then across warps
    for (int d = 16; d > 0; d >>= 1) {
      ts += __shfl_down_sync(0xffffffffu, ts, d);
      const uint32_t o = __shfl_down_sync(0xffffffffu, tm, d);
      tm = tm > o ? tm : o;
    }
    __shared__ uint64_t f_sum[32];
    __shared__ uint32_t f_max[32];
    if (lane == 0) {
      f_sum[warp] = ts;
      f_max[warp] = tm;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      uint64_t s = 0;
      uint32_t m = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
        s += f_sum[i];
        m = m > f_max[i] ? m : f_max[i];
      }
      if (p.sum_dev) *p.sum_dev = s;
      if (p.max_dev) *p.max_dev = m;
    }
    release_ticket(p.ticket);
  }
}

__device__ __forceinline__ int sb_load_px(const SobelParams &p, const uint8_t *img, int x, int y) {
  const int rx = remap(p.bmode, x, 0, p.w), ry = remap(p.bmode, y, 0, p.h);
  if (rx == (int)0x80000000 || ry == (int)0x80000000) return p.cval;
  return img[(int64_t)ry * p.in_pitch + rx];
}

__global__ void __launch_bounds__(SB_BX *SB_BY) sobel3_kernel(const __grid_constant__ SobelParams p) {
  __shared__ __align__(16) uint8_t tile[SB_SH * SB_SW];
  const int b = blockIdx.z;
  const uint8_t *img = p.in + (int64_t)b * p.in_bstride;
  const int i0 = blockIdx.x * SB_TW, j0 = blockIdx.y * SB_TH;
  const int X0 = i0 - SB_HL, Y0 = j0 - 1;
  constexpr int CPR = SB_SW / 16;
  const bool interior = X0 >= 0 && X0 + SB_SW <= p.w && Y0 >= 0 && Y0 + SB_SH <= p.h;
  for (int c = threadIdx.x; c < SB_SH * CPR; c += SB_BX * SB_BY) {
    const int r = c / CPR, k = c - r * CPR;
    const int y = Y0 + r, x = X0 + k * 16;
    uint4 v;
    if (p.vec_in && (interior || (y >= 0 && y < p.h && x >= 0 && x + 16 <= p.w))) {
      v = ldg16(img + (int64_t)y * p.in_pitch + x);
    } else {
      uint32_t wv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        uint32_t wq = 0;
#pragma unroll
        for (int e = 0; e < 4; ++e) wq |= (uint32_t)sb_load_px(p, img, x + 4 * q + e, y) << (8 * e);
        wv[q] = wq;
      }
      v = make_uint4(wv[0], wv[1], wv[2], wv[3]);
    }
    *reinterpret_cast<uint4 *>(&tile[r * SB_SW + k * 16]) = v;
  }
  __syncthreads();

  const int tx = threadIdx.x % SB_BX, ty = threadIdx.x / SB_BX;
  const int xs = SB_HL + 4 * tx;  // staged column of the thread's first pixel
  int top[6], mid[6], bot[6];
  auto load_row = [&](int r, int *v) {
    const uint8_t *row = &tile[r * SB_SW];
    const uint32_t w0 = *reinterpret_cast<const uint32_t *>(row + xs - 4);
    const uint32_t w1 = *reinterpret_cast<const uint32_t *>(row + xs);
    const uint32_t w2 = *reinterpret_cast<const uint32_t *>(row + xs + 4);
    v[0] = w0 >> 24;
    v[1] = w1 & 0xff;
    v[2] = (w1 >> 8) & 0xff;
    v[3] = (w1 >> 16) & 0xff;
    v[4] = w1 >> 24;
    v[5] = w2 & 0xff;
  };
  const int r0 = ty * SB_PY;
  load_row(r0, top);
  load_row(r0 + 1, mid);
  uint32_t tsum = 0, tmax = 0;
  uint8_t *out = p.out + (int64_t)b * p.out_bstride;
  const int xo = i0 + 4 * tx;
#pragma unroll
  for (int oy = 0; oy < SB_PY; ++oy) {
    load_row(r0 + oy + 2, bot);
    int S[6], D[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      S[c] = top[c] + 2 * mid[c] + bot[c];
      D[c] = bot[c] - top[c];
    }
    uint32_t word = 0;
    const int yo = j0 + ty * SB_PY + oy;
    const bool row_ok = yo < p.h;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int gx = S[q + 2] - S[q];
      const int gy = D[q] + 2 * D[q + 1] + D[q + 2];
      int m = abs(gx) + abs(gy);
      m = m < 255 ? m : 255;
      word |= (uint32_t)m << (8 * q);
      if (row_ok && xo + q < p.w) {
        tsum += m;
        tmax = tmax > (uint32_t)m ? tmax : (uint32_t)m;
      }
    }
    if (row_ok) {
      uint8_t *dst = out + (int64_t)yo * p.out_pitch + xo;
      if (p.vec_out && xo + 4 <= p.w) {
        *reinterpret_cast<uint32_t *>(dst) = word;
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (xo + q < p.w) dst[q] = (uint8_t)(word >> (8 * q));
      }
    }
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      top[c] = mid[c];
      mid[c] = bot[c];
    }
  }
  if (p.sum_dev || p.max_dev) block_reduce_store(p, tsum, tmax);
}


// ---------------------------------------------------------------------------
// TMA path for the standard 3x3 masks.  One CTA per 128 x 128 output tile:
// thread 0 loads the tile's 160 x 130 byte halo region with one
// cp.async.bulk.tensor (completion on an mbarrier, bounded wait), and each of
// the four warps runs 32 output rows of it, a lane owning four columns.  A CTA
// holds 21 KB of shared memory and 128 threads, so an SM keeps up to ten tiles
// in flight without a software pipeline, and independent kernels of the same
// step can share the SMs.  Cells outside the image (TMA fills them with 0)
// are patched with the boundary rule before use.
//
// Arithmetic is fp16x2 on exact integers: every intermediate (|gx|, |gy| <=
// 1020, their sum <= 2040) is an integer below 2048 and therefore exact in
// half precision, so results are the integer results bit for bit.  Bytes
// become halves by placing them under the exponent byte 0x64 (1024 + v) with
// one byte permute per pair.
struct SobelTmaParams {
  CUtensorMap map;
  SobelParams p;
  int tiles_x, tiles_y, ntiles;
  int *status;
  unsigned long long *acc;  // workspace accumulators (sum, max), zero at rest
  unsigned int *ticket;
  unsigned int *claim;      // tile counter of the streaming form, zero at rest
};

// The tile is 128 x 128 outputs in every configuration.  The autotuner picks
// the rows per warp (32 rows for 4 warps, or 16 rows for 8 warps: a shorter
// serial stencil per warp after the tile lands, twice the warps per SM) and the
// launch form:
//   one-shot (kSobelStream 0): one CTA per tile, every tile's copy issued at
//     launch;
//   streaming (kSobelStream = CTAs per SM): a few CTAs per SM claim tiles from
//     a counter, each with two stage buffers, so that the next tile's copy
//     lands while the current one is computed.  Tiles go to the CTAs that are
//     free, and the SMs keep room for an independent kernel of the same step.
constexpr int T_TW = 128, T_TH = 128;
constexpr int kSobelWarps[] = {4, 8, 4, 4, 8};
constexpr int kSobelStream[] = {0, 0, 2, 3, 2};
constexpr int kSobelCfgs = 5;
constexpr int T_SW = 160, T_SH = T_TH + 2, T_STAGE = T_SW * T_SH;
constexpr int T_STAGE_PAD = (T_STAGE + 127) / 128 * 128;

__device__ __forceinline__ __half2 u2h(uint32_t u) {
  __half2 h;
  memcpy(&h, &u, 4);
  return h;
}
__device__ __forceinline__ uint32_t h2u(__half2 h) {
  uint32_t u;
  memcpy(&u, &h, 4);
  return u;
}

// One staged tile through the stencil, R output rows per lane.  FULL: every
// output of the tile is inside the image and 4-byte stores are legal (no
// masks, no edge branches).  Rows stream through a three-row window of biased
// pairs P = 1024 + v: row differences H = P(x+1) - P(x-1) and vertical
// differences V = P(bottom) - P(top) cancel the bias exactly, so
// gx = H_top + 2 H_mid + H_bottom and gy = V(x-1) + 2 V(x) + V(x+1).
template <bool FULL, int R>
__device__ __forceinline__ void sobel_tile(const SobelParams &p, const uint8_t *tile, uint8_t *out_row, int xo, int yo,
                                           int xs, uint32_t &tsum, __half2 &tmax) {
  const uint32_t K = 0x64646464u;
  const __half2 c1024 = __float2half2_rn(1024.0f), c255 = __float2half2_rn(255.0f), two = __float2half2_rn(2.0f);
  __half2 P[3][5], H01[3], H23[3];
  __half2 v01, v23;
  if constexpr (!FULL) {
    v01 = __halves2half2(__float2half(xo < p.w ? 1.f : 0.f), __float2half(xo + 1 < p.w ? 1.f : 0.f));
    v23 = __halves2half2(__float2half(xo + 2 < p.w ? 1.f : 0.f), __float2half(xo + 3 < p.w ? 1.f : 0.f));
  }
#pragma unroll
  for (int r = 0; r < R + 2; ++r) {
    const int c = r % 3;
    const uint8_t *row = tile + r * T_SW + xs;
    const uint32_t w0 = *reinterpret_cast<const uint32_t *>(row - 4);
    const uint32_t w1 = *reinterpret_cast<const uint32_t *>(row);
    const uint32_t w2 = *reinterpret_cast<const uint32_t *>(row + 4);
    const uint32_t f1 = __funnelshift_r(w0, w1, 24);  // x-1 .. x+2
    const uint32_t f2 = __funnelshift_r(w1, w2, 24);  // x+3 .. x+6
    P[c][0] = u2h(__byte_perm(f1, K, 0x4140));  // (x-1, x)
    P[c][1] = u2h(__byte_perm(w1, K, 0x4140));  // (x, x+1)
    P[c][2] = u2h(__byte_perm(f1, K, 0x4342));  // (x+1, x+2)
    P[c][3] = u2h(__byte_perm(w1, K, 0x4342));  // (x+2, x+3)
    P[c][4] = u2h(__byte_perm(f2, K, 0x4140));  // (x+3, x+4)
    H01[c] = __hsub2(P[c][2], P[c][0]);
    H23[c] = __hsub2(P[c][4], P[c][2]);
    if (r < 2) continue;
    const int o = r - 2, ct = (r - 2) % 3, cm = (r - 1) % 3;  // top, middle; c is the bottom row
    const __half2 gx01 = __hfma2(two, H01[cm], __hadd2(H01[ct], H01[c]));
    const __half2 gx23 = __hfma2(two, H23[cm], __hadd2(H23[ct], H23[c]));
    __half2 V[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) V[q] = __hsub2(P[c][q], P[ct][q]);
    const __half2 gy01 = __hfma2(two, V[1], __hadd2(V[0], V[2]));
    const __half2 gy23 = __hfma2(two, V[3], __hadd2(V[2], V[4]));
    __half2 m01 = __hmin2(__hadd2(__habs2(gx01), __habs2(gy01)), c255);
    __half2 m23 = __hmin2(__hadd2(__habs2(gx23), __habs2(gy23)), c255);
    bool row_ok = true;
    if constexpr (!FULL) {
      row_ok = yo + o < p.h;
      m01 = row_ok ? __hmul2(m01, v01) : __float2half2_rn(0.0f);
      m23 = row_ok ? __hmul2(m23, v23) : __float2half2_rn(0.0f);
    }
    const uint32_t word = __byte_perm(h2u(__hadd2(m01, c1024)), h2u(__hadd2(m23, c1024)), 0x6420);
    tsum = __dp4a(word, 0x01010101u, tsum);
    tmax = __hmax2(tmax, __hmax2(m01, m23));
    uint8_t *dst = out_row + (int64_t)o * p.out_pitch;
    if constexpr (FULL) {
      *reinterpret_cast<uint32_t *>(dst) = word;
    } else if (row_ok) {
      if (p.vec_out && xo + 4 <= p.w) {
        *reinterpret_cast<uint32_t *>(dst) = word;
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (xo + q < p.w) dst[q] = (uint8_t)(word >> (8 * q));
      }
    }
  }
}

// Staged cells outside the image that the stencil reads (columns 15..144, all
// rows of a tile whose first staged cell is image (X0, Y0)) get the boundary
// rule; TMA filled them with zeros.  Regions: left columns, right columns, top
// row, bottom rows.  Every thread of the CTA takes part.
__device__ __forceinline__ void sobel_patch(const SobelParams &p, const uint8_t *img, uint8_t *tile, int X0, int Y0) {
  constexpr int qa = 15, qb = 145, ncol = qb - qa;
  const int nl = max(0, min(qb, -X0) - qa);
  const int rs = max(qa, p.w - X0), nr = max(0, qb - rs);
  const int ntop = max(0, -Y0);
  const int bs = max(0, p.h - Y0), nb = max(0, T_SH - bs);
  const int n1 = nl * T_SH, n2 = n1 + nr * T_SH, n3 = n2 + ntop * ncol, n4 = n3 + nb * ncol;
  for (int cc = threadIdx.x; cc < n4; cc += blockDim.x) {
    int r, q;
    if (cc < n1) {
      r = cc / nl;
      q = qa + (cc - r * nl);
    } else if (cc < n2) {
      const int d = cc - n1;
      r = d / nr;
      q = rs + (d - r * nr);
    } else if (cc < n3) {
      const int d = cc - n2;
      r = d / ncol;
      q = qa + (d - r * ncol);
    } else {
      const int d = cc - n3;
      const int rr = d / ncol;
      r = bs + rr;
      q = qa + (d - rr * ncol);
    }
    tile[r * T_SW + q] = (uint8_t)sb_load_px(p, img, X0 + q, Y0 + r);
  }
}

template <int T_WARPS>
__global__ void __launch_bounds__(T_WARPS * 32) sobel3_tma_kernel(const __grid_constant__ SobelTmaParams P) {
  constexpr int T_R = T_TH / T_WARPS;
  __shared__ __align__(128) uint8_t tile[T_STAGE_PAD];
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t s_sum[T_WARPS], s_max[T_WARPS];
  const SobelParams &p = P.p;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = blockIdx.x;
  const int tx_ = t % P.tiles_x, r_ = t / P.tiles_x;
  const int i0 = tx_ * T_TW, j0 = (r_ % P.tiles_y) * T_TH, b = r_ / P.tiles_y;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
    mbar_expect_tx(&bar, T_STAGE);
    tma_load_3d(tile, &P.map, i0 - 16, j0 - 1, b, &bar);
  }
  if (!cta_wait(&bar, 0)) {
    if (threadIdx.x == 0) {
      record_status(P.status, HGB_ERR_TIMEOUT);
      mbar_wait(&bar, 0);  // the load may still land: wait once more (bounded) before leaving
    }
    // this CTA's partials are missing; the status word reports the launch as failed
    if (p.sum_dev || p.max_dev)
      if (threadIdx.x == 0) accumulate_and_publish(P.acc, P.acc + 1, P.ticket, 0, 0, p.sum_dev, p.max_dev);
    return;
  }
  const int X0 = i0 - 16, Y0 = j0 - 1;
  if (X0 + 15 < 0 || X0 + 145 > p.w || Y0 < 0 || Y0 + T_SH > p.h) {
    sobel_patch(p, p.in + (int64_t)b * p.in_bstride, tile, X0, Y0);
    __syncthreads();
  }
  uint32_t tsum = 0;
  __half2 tmax = __float2half2_rn(0.0f);
  const int xo = i0 + 4 * lane, jw = j0 + warp * T_R;
  if (jw < p.h) {
    uint8_t *out_row = p.out + (int64_t)b * p.out_bstride + (int64_t)jw * p.out_pitch + xo;
    const uint8_t *wt = tile + warp * T_R * T_SW;
    if (p.vec_out && i0 + T_TW <= p.w && jw + T_R <= p.h)
      sobel_tile<true, T_R>(p, wt, out_row, xo, jw, 16 + 4 * lane, tsum, tmax);
    else
      sobel_tile<false, T_R>(p, wt, out_row, xo, jw, 16 + 4 * lane, tsum, tmax);
  }
  if (p.sum_dev || p.max_dev) {
    const float2 mf = __half22float2(tmax);
    const uint32_t bsum = __reduce_add_sync(0xffffffffu, tsum);
    const uint32_t bmax = __reduce_max_sync(0xffffffffu, (uint32_t)fmaxf(mf.x, mf.y));
    if (lane == 0) {
      s_sum[warp] = bsum;
      s_max[warp] = bmax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long S = 0, M = 0;
#pragma unroll
      for (int i = 0; i < T_WARPS; ++i) {
        S += s_sum[i];
        M = M > s_max[i] ? M : s_max[i];
      }
      accumulate_and_publish(P.acc, P.acc + 1, P.ticket, S, M, p.sum_dev, p.max_dev);
    }
  }
}

// Streaming form: gridDim.x CTAs (a few per SM) claim tiles from P.claim.
// Thread 0 keeps two tiles' copies in flight, one per stage buffer; after a
// tile is computed and every thread's reads of its buffer are done (CTA
// barrier, then a proxy fence), the buffer takes the next claimed tile.  The
// tile numbers travel through shared memory: slot k & 1 is rewritten only
// after the barrier that follows its use, and read only after the barrier
// that follows its rewrite.  Every CTA ends by taking one ticket; the last one
// publishes the sum and maximum and returns the counters to zero.
template <int T_WARPS>
__global__ void __launch_bounds__(T_WARPS * 32) sobel3_stream_kernel(const __grid_constant__ SobelTmaParams P) {
  constexpr int T_R = T_TH / T_WARPS;
  __shared__ __align__(128) uint8_t tile[2][T_STAGE_PAD];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ int s_tile[2];
  __shared__ unsigned long long s_sum[T_WARPS];
  __shared__ uint32_t s_max[T_WARPS];
  const SobelParams &p = P.p;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  auto issue = [&](int k, int t) {  // thread 0: tile t into buffer k
    const int tx_ = t % P.tiles_x, r_ = t / P.tiles_x;
    mbar_expect_tx(&bar[k], T_STAGE);
    tma_load_3d(tile[k], &P.map, tx_ * T_TW - 16, (r_ % P.tiles_y) * T_TH - 1, r_ / P.tiles_y, &bar[k]);
  };
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
    for (int k = 0; k < 2; ++k) {
      const int t = (int)atomicAdd(P.claim, 1u);
      s_tile[k] = t;
      if (t < P.ntiles) issue(k, t);
    }
  }
  __syncthreads();
  unsigned long long tsum64 = 0;
  __half2 tmax = __float2half2_rn(0.0f);
  for (int k = 0;; ++k) {
    const int buf = k & 1;
    const int t = s_tile[buf];
    if (t >= P.ntiles) break;  // the same value in every thread: the CTA leaves together
    if (!cta_wait(&bar[buf], (k >> 1) & 1)) {
      if (threadIdx.x == 0) {
        record_status(P.status, HGB_ERR_TIMEOUT);
        // both copies may still land: wait once more (bounded) for each
        mbar_wait(&bar[buf], (k >> 1) & 1);
        if (s_tile[buf ^ 1] < P.ntiles) mbar_wait(&bar[buf ^ 1], ((k + 1) >> 1) & 1);
      }
      break;  // this CTA's remaining tiles are missing; the status word reports the launch as failed
    }
    const int tx_ = t % P.tiles_x, r_ = t / P.tiles_x;
    const int i0 = tx_ * T_TW, j0 = (r_ % P.tiles_y) * T_TH, b = r_ / P.tiles_y;
    const int X0 = i0 - 16, Y0 = j0 - 1;
    if (X0 + 15 < 0 || X0 + 145 > p.w || Y0 < 0 || Y0 + T_SH > p.h) {
      sobel_patch(p, p.in + (int64_t)b * p.in_bstride, tile[buf], X0, Y0);
      __syncthreads();
    }
    const int xo = i0 + 4 * lane, jw = j0 + warp * T_R;
    if (jw < p.h) {
      uint32_t tsum = 0;
      uint8_t *out_row = p.out + (int64_t)b * p.out_bstride + (int64_t)jw * p.out_pitch + xo;
      const uint8_t *wt = tile[buf] + warp * T_R * T_SW;
      if (p.vec_out && i0 + T_TW <= p.w && jw + T_R <= p.h)
        sobel_tile<true, T_R>(p, wt, out_row, xo, jw, 16 + 4 * lane, tsum, tmax);
      else
        sobel_tile<false, T_R>(p, wt, out_row, xo, jw, 16 + 4 * lane, tsum, tmax);
      tsum64 += tsum;
    }
    __syncthreads();  // every read of tile[buf] and of s_tile is done
    if (threadIdx.x == 0) {
      const int tn = (int)atomicAdd(P.claim, 1u);
      s_tile[buf] = tn;
      if (tn < P.ntiles) {
        fence_proxy_async_smem();
        issue(buf, tn);
      }
    }
  }
  const float2 mf = __half22float2(tmax);
  for (int d = 16; d > 0; d >>= 1) tsum64 += __shfl_xor_sync(0xffffffffu, tsum64, d);
  const uint32_t bmax = __reduce_max_sync(0xffffffffu, (uint32_t)fmaxf(mf.x, mf.y));
  if (lane == 0) {
    s_sum[warp] = tsum64;
    s_max[warp] = bmax;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long S = 0, M = 0;
#pragma unroll
    for (int i = 0; i < T_WARPS; ++i) {
      S += s_sum[i];
      M = M > s_max[i] ? M : s_max[i];
    }
    if (S) atomicAdd(P.acc, S);
    if (M) atomicMax(P.acc + 1, M);
    if (ticket_acq_rel(P.ticket) == gridDim.x - 1) {
      // every CTA has made its last claim and added its partials
      const unsigned long long sum = ld_relaxed_u64(P.acc), mx = ld_relaxed_u64(P.acc + 1);
      if (p.sum_dev) *p.sum_dev = sum;
      if (p.max_dev) *p.max_dev = (uint32_t)mx;
      P.acc[0] = 0ull;
      P.acc[1] = 0ull;
      *P.claim = 0u;
      *P.ticket = 0u;
    }
  }
}

// Any integer masks of size 3, 5 or 7: one pixel per thread, runtime
// coefficients, zero cells skipped (Domain semantics).
__global__ void __launch_bounds__(256) sobel_generic_kernel(const __grid_constant__ SobelParams p) {
  constexpr int T = 16;
  __shared__ uint8_t tile[(T + 6) * (T + 6)];
  const int b = blockIdx.z;
  const uint8_t *img = p.in + (int64_t)b * p.in_bstride;
  const int s = p.size, r = s / 2, SW = T + s - 1;
  const int i0 = blockIdx.x * T, j0 = blockIdx.y * T;
  for (int c = threadIdx.x; c < SW * SW; c += blockDim.x) {
    const int yy = c / SW, xx = c - yy * SW;
    tile[yy * SW + xx] = (uint8_t)sb_load_px(p, img, i0 - r + xx, j0 - r + yy);
  }
  __syncthreads();
  const int tx = threadIdx.x % T, ty = threadIdx.x / T;
  const int x = i0 + tx, y = j0 + ty;
  uint32_t m = 0;
  const bool ok = x < p.w && y < p.h;
  if (ok) {
    int gx = 0, gy = 0;
    for (int yy = 0; yy < s; ++yy)
      for (int xx = 0; xx < s; ++xx) {
        const int v = tile[(ty + yy) * SW + tx + xx];
        gx += p.mx[yy * s + xx] * v;
        gy += p.my[yy * s + xx] * v;
      }
    const int g = abs(gx) + abs(gy);
    m = g < 255 ? g : 255;
    p.out[(int64_t)b * p.out_bstride + (int64_t)y * p.out_pitch + x] = (uint8_t)m;
  }
  if (p.sum_dev || p.max_dev) block_reduce_store(p, ok ? m : 0u, ok ? m : 0u);
}

const int kSobelX3[9] = {-1, 0, 1, -2, 0, 2, -1, 0, 1};
const int kSobelY3[9] = {-1, -2, -1, 0, 0, 0, 1, 2, 1};

}  // namespace
}  // namespace hgb

using namespace hgb;

extern "C" int hgb_sobel_mag(const hgb_view *in, const hgb_view *out, const int *mask_x, const int *mask_y, int size,
                             int boundary, int const_val, uint64_t *sum_dev, uint32_t *max_dev, void *stream) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  rc = check_view(out, "out");
  if (rc) return rc;
  HGB_REQUIRE(in->dtype == HGB_U8 && out->dtype == HGB_U8, "hgb_sobel_mag: u8 images expected");
  HGB_REQUIRE(in->width == out->width && in->height == out->height && in->batch == out->batch,
              "hgb_sobel_mag: size mismatch");
  HGB_REQUIRE(mask_x && mask_y, "hgb_sobel_mag: null mask");
  HGB_REQUIRE(size == 3 || size == 5 || size == 7, "hgb_sobel_mag: size must be 3, 5 or 7");
  HGB_REQUIRE(boundary >= 0 && boundary <= 4, "hgb_sobel_mag: bad boundary");
  HGB_REQUIRE(const_val >= 0 && const_val <= 255, "hgb_sobel_mag: constant must fit u8");
  // with in->batch > 1 the fused sum / max cover every image of the batch
  SobelParams p;
  memset(&p, 0, sizeof(p));
  p.in = (const uint8_t *)in->data;
  p.in_pitch = in->pitch;
  p.in_bstride = in->batch_stride;
  p.out = (uint8_t *)out->data;
  p.out_pitch = out->pitch;
  p.out_bstride = out->batch_stride;
  p.w = in->width;
  p.h = in->height;
  p.bmode = boundary;
  p.cval = const_val;
  p.size = size;
  for (int i = 0; i < size * size; ++i) {
    p.mx[i] = mask_x[i];
    p.my[i] = mask_y[i];
  }
  p.vec_in = ((uintptr_t)in->data % 16 == 0) && in->pitch % 16 == 0 && (in->batch == 1 || in->batch_stride % 16 == 0);
  p.vec_out = ((uintptr_t)out->data % 4 == 0) && out->pitch % 4 == 0 && (out->batch == 1 || out->batch_stride % 4 == 0);
  p.sum_dev = sum_dev;
  p.max_dev = max_dev;
  bool fast = size == 3;
  for (int i = 0; fast && i < 9; ++i) fast = mask_x[i] == kSobelX3[i] && mask_y[i] == kSobelY3[i];
  dim3 grid = fast ? dim3(cdiv(p.w, SB_TW), cdiv(p.h, SB_TH), in->batch) : dim3(cdiv(p.w, 16), cdiv(p.h, 16), in->batch);
  if (sum_dev || max_dev) {
    const size_t nb = (size_t)grid.x * grid.y * grid.z;
    Workspace ws;
    rc = workspace_get(nb * 12 + 256, &ws);
    if (rc) return rc;
    p.partials = (uint2 *)ws.base;
    p.partial_max = (uint32_t *)((char *)ws.base + nb * 8);
    p.ticket = ws.tickets + 0;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (fast && tma_legal(in->data, in->pitch, in->batch_stride, in->batch)) {
    SobelTmaParams P;
    memset(&P, 0, sizeof(P));
    P.p = p;
    P.tiles_x = cdiv(p.w, T_TW);
    P.tiles_y = cdiv(p.h, T_TH);
    P.ntiles = P.tiles_x * P.tiles_y * in->batch;
    P.status = device_status_word();
    rc = make_tensor_map_3d(&P.map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, in->data, p.w, p.h, in->batch, in->pitch,
                            in->batch_stride, T_SW, T_SH);
    if (rc == HGB_OK) {
      // the streaming form always takes a ticket (it resets its tile counter)
      Workspace ws;
      rc = workspace_get(0, &ws);
      if (rc) return rc;
      P.acc = ws.acc + kSlotSobel;
      P.ticket = ws.tickets + 0;
      P.claim = ws.tickets + kTicketSobelClaim;
      char key[96];
      snprintf(key, sizeof(key), "sobel3:%dx%dx%d", 1 << (32 - __builtin_clz((unsigned)p.w)),
               1 << (32 - __builtin_clz((unsigned)p.h)), in->batch);
      return autotune_run(key, kSobelCfgs, st, [&](int cfg) {
        const int per_sm = kSobelStream[cfg], warps = kSobelWarps[cfg];
        if (per_sm > 0) {
          const void *fn = warps == 8 ? (const void *)sobel3_stream_kernel<8> : (const void *)sobel3_stream_kernel<4>;
          const int fit = resident_ctas(fn, warps * 32, 0);
          const int grid = std::max(1, std::min(P.ntiles, num_sms() * std::max(1, std::min(per_sm, fit))));
          cudaEvent_t ev = before_launch(st);
          if (warps == 8)
            sobel3_stream_kernel<8><<<grid, 256, 0, st>>>(P);
          else
            sobel3_stream_kernel<4><<<grid, 128, 0, st>>>(P);
          return after_launch("sobel3_stream_kernel", st, ev);
        }
        cudaEvent_t ev = before_launch(st);
        if (warps == 8)
          sobel3_tma_kernel<8><<<P.ntiles, 256, 0, st>>>(P);
        else
          sobel3_tma_kernel<4><<<P.ntiles, 128, 0, st>>>(P);
        return after_launch("sobel3_tma_kernel", st, ev);
      });
    }
  }
  cudaEvent_t ev = before_launch(st);
  if (fast)
    sobel3_kernel<<<grid, SB_BX * SB_BY, 0, st>>>(p);
  else
    sobel_generic_kernel<<<grid, 256, 0, st>>>(p);
  return after_launch("sobel", st, ev);
}

// sobel.cu -- u8 Sobel magnitude with the global sum / max of the result fused
// into the same kernel.
//
// Semantics (bit-exact): gx = sum over Domain(mask_x) of mask_x * in,
// gy likewise (samples-public/3_Preprocessing/Sobel/src/main.cpp:56-67 with
// Domain(mask), dsl/mask.hpp:238-250), out = min(|gx| + |gy|, 255); then
// Kernel::reduced_data of the output with a u64 sum and a u8 max
// (dsl/kernel.hpp:121-161).  Integer arithmetic, so every order is exact.
//
// Fast path (the standard 3x3 Sobel masks): a CTA stages a 128 x 64 output
// tile plus a one-pixel halo as bytes in shared memory (16-byte loads, remap
// only on border tiles).  A thread owns 4 adjacent columns x 8 rows, walks the
// rows with a three-row register window and uses the separable form
// gx = S(x+1) - S(x-1), S = top + 2 mid + bottom; gy = D(x-1) + 2 D(x) + D(x+1),
// D = bottom - top.  The result is written as one 32-bit word per row; sum and
// max are reduced with redux.sync across the warp, shared memory across the
// block and a last-block combine of the per-block partials.
#include "reduce_common.cuh"

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
  cudaEvent_t ev = before_launch(st);
  if (fast)
    sobel3_kernel<<<grid, SB_BX * SB_BY, 0, st>>>(p);
  else
    sobel_generic_kernel<<<grid, 256, 0, st>>>(p);
  return after_launch("sobel", st, ev);
}

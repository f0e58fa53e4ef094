// local_adjoint.cu -- hgb_local_op_adjoint: the adjoint of the SUM local
// operator out(j) = sum_o m_o in(r(j + o)) (r = boundary remap,
// lib/AST/BorderHandling.cpp:41-120; tap offsets o = (mx - mw/2, my - mh/2)).
//   grad_in(i)  = sum over (j, o) with r(j + o) = i of m_o grad_out(j)
//   grad_m(o)   = sum_j grad_out(j) in(r(j + o))
// CONSTANT taps read the constant, which carries no gradient.  The boundary is
// transposed by gathering over the pre-images of i under r: for pixels far
// from the border the only pre-image is i itself (grad_in is the correlation
// with the flipped mask, staged in shared memory); near the border every
// virtual position within the mask radius that r sends to i contributes
// (CLAMP: all positions beyond the edge, MIRROR: the reflected one, REPEAT: the
// wrapped ones).  grad_m is reduced per tap over row blocks and combined in
// FP64 in a fixed order, so it is deterministic.  FP32 storage.
//
// Both gradients of a square 3x3, 5x5 or 7x7 mask on TMA-legal images of at
// least 8 x 8 go through one fused persistent kernel (adj_fused_kernel): the
// CTA walks 64 x 16 tiles, stages grad_out and in with TMA into two buffers
// (the next tile's boxes land while this one computes), reads twelve-value
// register windows per row, and accumulates the mask gradient per pair of taps
// in packed f32x2 registers; pixels within the mask radius of an edge go
// through the pre-images from a flat band list after the tiles.
#include <algorithm>
#include <cstring>

#include "band.cuh"
#include "reduce_common.cuh"
#include "tma.cuh"

namespace hgb {
namespace {

constexpr int LA_TW = 32, LA_TH = 16, LA_T = 256, LA_MAX = 15;
constexpr int LA_SW = LA_TW + 2 * LA_MAX, LA_SH = LA_TH + 2 * LA_MAX;
constexpr int LA_ROWBLOCKS = 64;
constexpr int LM_TW = 64, LM_TH = 16, LM_PX = 4;  // tiles of the square-mask kernels

struct AdjParams {
  const float *in, *gout;
  float *gin;
  int64_t in_p, gout_p, gin_p, in_b, gout_b, gin_b;  // floats
  int w, h, batch;
  int mw, mh, bmode;
  const float *mask_dev;
  float mask[LA_MAX * LA_MAX];
  float *part;          // [taps][batch * LA_ROWBLOCKS]
  float *grad_mask_dev;
};

__device__ __forceinline__ int pre_list(int mode, int i, int n, int lo_off, int hi_off, int *out) {
  // virtual v with r(v) == i among [-hi_off, n + lo_off): the positions a tap
  // can reach from inside the image
  int k = 0;
  out[k++] = i;
  if (mode == HGB_BOUNDARY_CONSTANT) return k;
  for (int v = -hi_off; v < 0; ++v)
    if (remap(mode, v, 0, n) == i && k < 2 * LA_MAX + 1) out[k++] = v;
  for (int v = n; v < n + lo_off; ++v)
    if (remap(mode, v, 0, n) == i && k < 2 * LA_MAX + 1) out[k++] = v;
  return k;
}

__global__ void __launch_bounds__(LA_T) adj_in_kernel(const __grid_constant__ AdjParams p) {
  __shared__ float sg[LA_SW * LA_SH];
  __shared__ float msk[LA_MAX * LA_MAX];
  const int b = blockIdx.z;
  const int X0 = blockIdx.x * LA_TW, Y0 = blockIdx.y * LA_TH;
  const int mw = p.mw, mh = p.mh, rxl = mw / 2, ryl = mh / 2, rxh = mw - 1 - rxl, ryh = mh - 1 - ryl;
  const float *gout = p.gout + (int64_t)b * p.gout_b;
  for (int k = threadIdx.x; k < mw * mh; k += LA_T) msk[k] = p.mask_dev ? __ldg(p.mask_dev + k) : p.mask[k];
  // grad_out over [X0 - rxh, X0 + TW + rxl) x [Y0 - ryh, Y0 + TH + ryl), zero outside the image
  const int sw = LA_TW + mw - 1, sh = LA_TH + mh - 1;
  for (int c = threadIdx.x; c < sw * sh; c += LA_T) {
    const int r = c / sw, q = c - r * sw;
    const int gy = Y0 - ryh + r, gx = X0 - rxh + q;
    sg[r * LA_SW + q] = (gx >= 0 && gx < p.w && gy >= 0 && gy < p.h) ? __ldg(gout + (int64_t)gy * p.gout_p + gx) : 0.0f;
  }
  __syncthreads();
  const int tx = threadIdx.x % LA_TW, ty = threadIdx.x / LA_TW;
  for (int py = ty; py < LA_TH; py += LA_T / LA_TW) {
    const int ix = X0 + tx, iy = Y0 + py;
    if (ix >= p.w || iy >= p.h) continue;
    float acc = 0.0f;
    // pixels with no pre-image besides themselves: farther than the larger
    // reach of the mask from every border
    const int rx = max(rxl, rxh), ry = max(ryl, ryh);
    const bool inner = ix >= rx && ix < p.w - rx && iy >= ry && iy < p.h - ry;
    if (inner) {
      // j = i - o for every tap (mask flipped), rows and columns ascending in o
      for (int my = 0; my < mh; ++my)
        for (int mx = 0; mx < mw; ++mx) {
          const int jy = iy - (my - ryl), jx = ix - (mx - rxl);
          acc = __fmaf_rn(msk[my * mw + mx], sg[(jy - Y0 + ryh) * LA_SW + (jx - X0 + rxh)], acc);
        }
    } else {
      int prx[2 * LA_MAX + 1], pry[2 * LA_MAX + 1];
      const int nx = pre_list(p.bmode, ix, p.w, rxl + 1, rxh + 1, prx);
      const int ny = pre_list(p.bmode, iy, p.h, ryl + 1, ryh + 1, pry);
      for (int a = 0; a < ny; ++a)
        for (int c = 0; c < nx; ++c)
          for (int my = 0; my < mh; ++my)
            for (int mx = 0; mx < mw; ++mx) {
              const int jy = pry[a] - (my - ryl), jx = prx[c] - (mx - rxl);
              if (jx < 0 || jx >= p.w || jy < 0 || jy >= p.h) continue;
              acc = __fmaf_rn(msk[my * mw + mx], __ldg(gout + (int64_t)jy * p.gout_p + jx), acc);
            }
    }
    p.gin[(int64_t)b * p.gin_b + (int64_t)iy * p.gin_p + ix] = acc;
  }
}

// Square K x K masks: grad_in on a 64 x 16 tile, a thread per four
// consecutive pixels of a row.  Inside the image (every pixel at least the
// radius from the border) grad_in(i) = sum_o m_o grad_out(i - o): each staged
// row value serves all taps that read it.  Pixels near the border gather over
// their pre-images as adj_in_kernel does.
template <int K>
__global__ void __launch_bounds__(LA_T) adj_in_tile_kernel(const __grid_constant__ AdjParams p) {
  constexpr int R = K / 2, SW = LM_TW + 2 * R, SH = LM_TH + 2 * R;
  __shared__ float sg[SH * SW];
  __shared__ float msk[K * K];
  const int b = blockIdx.z, X0 = blockIdx.x * LM_TW, Y0 = blockIdx.y * LM_TH;
  const float *gout = p.gout + (int64_t)b * p.gout_b;
  for (int k = threadIdx.x; k < K * K; k += LA_T) msk[k] = p.mask_dev ? __ldg(p.mask_dev + k) : p.mask[k];
  for (int c = threadIdx.x; c < SH * SW; c += LA_T) {
    const int r = c / SW, q = c - r * SW;
    const int gy = Y0 - R + r, gx = X0 - R + q;
    sg[c] = (gx >= 0 && gx < p.w && gy >= 0 && gy < p.h) ? __ldg(gout + (int64_t)gy * p.gout_p + gx) : 0.0f;
  }
  __syncthreads();
  const int tx = threadIdx.x % (LM_TW / LM_PX), ty = threadIdx.x / (LM_TW / LM_PX);
  const int x = X0 + tx * LM_PX, y = Y0 + ty;
  if (y >= p.h || x >= p.w) return;
  float acc[LM_PX];
#pragma unroll
  for (int q = 0; q < LM_PX; ++q) acc[q] = 0.0f;
  const bool inner = x >= R && x + LM_PX - 1 < p.w - R && y >= R && y < p.h - R;
  if (inner) {
    // taps in the order of adj_in_kernel: my, then mx ascending; j = i - o
#pragma unroll
    for (int my = 0; my < K; ++my) {
      const float *row = &sg[(ty + 2 * R - my) * SW + tx * LM_PX];  // grad_out row y - (my - R)
      float v[LM_PX + K - 1];
#pragma unroll
      for (int i = 0; i < LM_PX + K - 1; ++i) v[i] = row[i];
#pragma unroll
      for (int mx = 0; mx < K; ++mx)
#pragma unroll
        for (int q = 0; q < LM_PX; ++q)  // column x + q - (mx - R): v[q + 2R - mx]
          acc[q] = __fmaf_rn(msk[my * K + mx], v[q + 2 * R - mx], acc[q]);
    }
  } else {
    for (int q = 0; q < LM_PX; ++q) {
      const int ix = x + q;
      if (ix >= p.w) break;
      int prx[2 * LA_MAX + 1], pry[2 * LA_MAX + 1];
      const int nx = pre_list(p.bmode, ix, p.w, R + 1, R + 1, prx);
      const int ny = pre_list(p.bmode, y, p.h, R + 1, R + 1, pry);
      float a = 0.0f;
      for (int ia = 0; ia < ny; ++ia)
        for (int ic = 0; ic < nx; ++ic)
          for (int my = 0; my < K; ++my)
            for (int mx = 0; mx < K; ++mx) {
              const int jy = pry[ia] - (my - R), jx = prx[ic] - (mx - R);
              if (jx < 0 || jx >= p.w || jy < 0 || jy >= p.h) continue;
              a = __fmaf_rn(msk[my * K + mx], __ldg(gout + (int64_t)jy * p.gout_p + jx), a);
            }
      acc[q] = a;
    }
  }
  float *gin = p.gin + (int64_t)b * p.gin_b + (int64_t)y * p.gin_p;
#pragma unroll
  for (int q = 0; q < LM_PX; ++q)
    if (x + q < p.w) gin[x + q] = acc[q];
}

// grid (taps, LA_ROWBLOCKS, batch): partial of grad_m(o) over a band of rows
__global__ void __launch_bounds__(LA_T) adj_mask_kernel(const __grid_constant__ AdjParams p) {
  const int o = blockIdx.x, b = blockIdx.z;
  const int my = o / p.mw, mx = o - my * p.mw;
  const int oy = my - p.mh / 2, ox = mx - p.mw / 2;
  const float *in = p.in + (int64_t)b * p.in_b;
  const float *gout = p.gout + (int64_t)b * p.gout_b;
  float s = 0.0f;
  for (int y = blockIdx.y; y < p.h; y += gridDim.y) {
    const int ry = remap(p.bmode, y + oy, 0, p.h);
    if (ry == (int)0x80000000) continue;
    for (int x = threadIdx.x; x < p.w; x += LA_T) {
      const int rx = remap(p.bmode, x + ox, 0, p.w);
      if (rx == (int)0x80000000) continue;
      s = __fmaf_rn(__ldg(gout + (int64_t)y * p.gout_p + x), __ldg(in + (int64_t)ry * p.in_p + rx), s);
    }
  }
  __shared__ float sb[LA_T / 32];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) s += __shfl_down_sync(0xffffffffu, s, d);
  if ((threadIdx.x & 31) == 0) sb[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int i = 0; i < LA_T / 32; ++i) t += sb[i];
    p.part[(size_t)o * gridDim.y * gridDim.z + (size_t)b * gridDim.y + blockIdx.y] = t;
  }
}

// Square K x K masks: one CTA per 64 x 16 tile of grad_out accumulates every
// tap's partial at once.  The input region the tile's taps read is staged once
// (through the boundary remap; CONSTANT taps read 0, which adds nothing), a
// thread owns four consecutive pixels of a row and keeps the K * K partials in
// registers, reusing each staged value for all taps that read it.  Per-CTA
// partials [cta][tap] are combined in FP64 in a fixed order.
template <int K>
__global__ void __launch_bounds__(LA_T) adj_mask_tile_kernel(const __grid_constant__ AdjParams p) {
  constexpr int R = K / 2, SW = LM_TW + 2 * R, SH = LM_TH + 2 * R;
  __shared__ float s_in[SH * SW];
  __shared__ float s_red[LA_T / 32][K * K];
  const int b = blockIdx.z, X0 = blockIdx.x * LM_TW, Y0 = blockIdx.y * LM_TH;
  const float *in = p.in + (int64_t)b * p.in_b;
  const float *gout = p.gout + (int64_t)b * p.gout_b;
  for (int c = threadIdx.x; c < SH * SW; c += LA_T) {
    const int r = c / SW, q = c - r * SW;
    const int ry = remap(p.bmode, Y0 - R + r, 0, p.h), rx = remap(p.bmode, X0 - R + q, 0, p.w);
    s_in[c] = (ry == (int)0x80000000 || rx == (int)0x80000000) ? 0.0f : __ldg(in + (int64_t)ry * p.in_p + rx);
  }
  const int tx = threadIdx.x % (LM_TW / LM_PX), ty = threadIdx.x / (LM_TW / LM_PX);
  const int x = X0 + tx * LM_PX, y = Y0 + ty;
  float g[LM_PX];
#pragma unroll
  for (int q = 0; q < LM_PX; ++q)
    g[q] = (y < p.h && x + q < p.w) ? __ldg(gout + (int64_t)y * p.gout_p + x + q) : 0.0f;
  __syncthreads();
  float dm[K * K];
#pragma unroll
  for (int i = 0; i < K * K; ++i) dm[i] = 0.0f;
#pragma unroll
  for (int my = 0; my < K; ++my) {
    const float *row = &s_in[(ty + my) * SW + tx * LM_PX];
    float v[LM_PX + K - 1];
#pragma unroll
    for (int i = 0; i < LM_PX + K - 1; ++i) v[i] = row[i];
#pragma unroll
    for (int mx = 0; mx < K; ++mx)
#pragma unroll
      for (int q = 0; q < LM_PX; ++q) dm[my * K + mx] = __fmaf_rn(g[q], v[q + mx], dm[my * K + mx]);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < K * K; ++i) {
    float t = dm[i];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) t += __shfl_down_sync(0xffffffffu, t, d);
    if (lane == 0) s_red[warp][i] = t;
  }
  __syncthreads();
  const unsigned cta = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
  const unsigned ncta = gridDim.x * gridDim.y * gridDim.z;
  for (int i = threadIdx.x; i < K * K; i += LA_T) {
    float t = 0.0f;
    for (int w = 0; w < LA_T / 32; ++w) t += s_red[w][i];
    p.part[(size_t)i * ncta + cta] = t;
  }
}

// ---------------------------------------------------------------- fused form
constexpr int AF_TW = 64, AF_TH = 16, AF_GX = AF_TW / 4, AF_W = AF_TW + 8;  // staged columns X0-4 ..

struct AdjFusedParams {
  CUtensorMap map_g;  // grad_out, box AF_W x (AF_TH + 2R)
  CUtensorMap map_x;  // in, same box
  AdjParams p;
  int *status;
  int tiles_x, tiles_y, ntiles;
  int vec_gin;        // grad_in rows allow aligned 16-byte stores
};

template <int K>
struct AfShape {
  static constexpr int R = K / 2, H = AF_TH + 2 * R, NP = (K + 1) / 2;  // staged rows, tap pairs per mask row
  static constexpr int N = (AF_W * H + 31) / 32 * 32;                   // floats per staged array (128-byte multiple)
};

__device__ __forceinline__ void af_window12(const float *row, float (&w)[12]) {
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    const float4 t4 = reinterpret_cast<const float4 *>(row)[v];
    w[4 * v] = t4.x;
    w[4 * v + 1] = t4.y;
    w[4 * v + 2] = t4.z;
    w[4 * v + 3] = t4.w;
  }
}

template <int K>
__global__ void __launch_bounds__(LA_T, 2) adj_fused_kernel(const __grid_constant__ AdjFusedParams P) {
  using S = AfShape<K>;
  constexpr int R = S::R, FH = S::H, NP = S::NP, FN = S::N;
  static_assert(R <= 3, "the twelve-value windows cover radius 3");
  __shared__ __align__(128) float stg[2][2][FN];  // [buffer][grad_out, in]
  __shared__ __align__(16) f2 m2[K][2 * NP];     // mask pairs (m, m), padded to an even count per row
  __shared__ float msk[K * K];
  __shared__ float red[LA_T / 32][K * K];
  __shared__ __align__(8) uint64_t bars[2];
  const AdjParams &p = P.p;
  const int W = p.w, H = p.h, bm = p.bmode;
  for (int i = threadIdx.x; i < K * 2 * NP; i += LA_T) {
    const int oy = i / (2 * NP), ox = i - oy * (2 * NP);
    const float m = ox < K ? (p.mask_dev ? __ldg(p.mask_dev + oy * K + ox) : p.mask[oy * K + ox]) : 0.0f;
    m2[oy][ox] = f2_pack(m, m);
    if (ox < K) msk[oy * K + ox] = m;
  }
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  auto origin = [&](int t, int &b, int &X0, int &Y0) {
    const int per = P.tiles_x * P.tiles_y, bz = t / per, r = t - bz * per, by = r / P.tiles_x;
    b = bz;
    X0 = (r - by * P.tiles_x) * AF_TW;
    Y0 = by * AF_TH;
  };
  auto issue = [&](int t, int s) {
    int b, X0, Y0;
    origin(t, b, X0, Y0);
    mbar_expect_tx(&bars[s], 2 * AF_W * FH * 4);
    tma_load_3d(stg[s][0], &P.map_g, X0 - 4, Y0 - R, b, &bars[s]);
    tma_load_3d(stg[s][1], &P.map_x, X0 - 4, Y0 - R, b, &bars[s]);
  };
  // the first tile's boxes land while the band's grad_in runs
  if (threadIdx.x == 0) issue(blockIdx.x, 0);
  const int band_per = band_size(W, H, R);
  int64_t k0, k1;
  cta_share((int64_t)band_per * p.batch, k0, k1);
  for (int64_t k = k0 + threadIdx.x; k < k1; k += LA_T) {
    const int b = (int)(k / band_per);
    int jy, jx;
    band_pos((int)(k - (int64_t)b * band_per), W, H, R, jy, jx);
    const float *g = p.gout + (int64_t)b * p.gout_b;
    int prx[1 + R], pry[1 + R];
    const int nx = preimages(bm, jx, W, R, prx), ny = preimages(bm, jy, H, R, pry);
    float acc = 0.0f;
    for (int iy = 0; iy < ny; ++iy)
      for (int oy = 0; oy < K; ++oy) {
        const int sy = pry[iy] - (oy - R);
        if (sy < 0 || sy >= H) continue;
        const float *grow = g + (int64_t)sy * p.gout_p;
        for (int ix = 0; ix < nx; ++ix)
#pragma unroll
          for (int ox = 0; ox < K; ++ox) {  // the row's loads in flight together
            const int sxp = prx[ix] - (ox - R);
            if (sxp < 0 || sxp >= W) continue;
            acc = __fmaf_rn(msk[oy * K + ox], grow[sxp], acc);
          }
      }
    p.gin[(int64_t)b * p.gin_b + (int64_t)jy * p.gin_p + jx] = acc;
  }
  const int tx = threadIdx.x % AF_GX, ty = threadIdx.x / AF_GX;
  f2 DM[K][NP];  // dL/dmask per pair of taps (oy, 2 op), (oy, 2 op + 1)
#pragma unroll
  for (int i = 0; i < K; ++i)
#pragma unroll
    for (int j = 0; j < NP; ++j) DM[i][j] = 0ull;
  int it = 0;
  for (int t = blockIdx.x; t < P.ntiles; t += gridDim.x, ++it) {
    int b, X0, Y0;
    origin(t, b, X0, Y0);
    const int s = it & 1;
    // the next tile's boxes land while this one computes
    const bool next = t + (int)gridDim.x < P.ntiles;
    if (next && threadIdx.x == 0) {
      fence_proxy_async_smem();
      issue(t + gridDim.x, s ^ 1);
    }
    if (!cta_wait(&bars[s], (it >> 1) & 1)) {
      if (threadIdx.x == 0) {
        record_status(P.status, HGB_ERR_TIMEOUT);
        mbar_wait(&bars[s], (it >> 1) & 1);
        if (next) mbar_wait(&bars[s ^ 1], ((it + 1) >> 1) & 1);
      }
      break;
    }
    const float *sg = stg[s][0], *sx = stg[s][1];
    const int jx0 = X0 + 4 * tx, jy = Y0 + ty;
    if (jx0 >= 4 && jx0 + 3 < W - R && jy >= R && jy < H - R) {
      // grad_in: pixel pair pp (staged column 4 tx + 4 + 2 pp) gathers
      // grad_out at columns 4 tx + 4 + 2 pp + R - ox of row ty + 2R - oy
      f2 GI0 = 0ull, GI1 = 0ull;
#pragma unroll
      for (int oy = 0; oy < K; ++oy) {
        float w[12];
        af_window12(&sg[(ty + 2 * R - oy) * AF_W + 4 * tx], w);
        const float4 *mr = reinterpret_cast<const float4 *>(&m2[oy][0]);
#pragma unroll
        for (int o2 = 0; o2 < NP; ++o2) {
          const float4 mm = mr[o2];  // taps 2 o2, 2 o2 + 1 as pairs (m, m)
#pragma unroll
          for (int l = 0; l < 2; ++l) {
            const int ox = 2 * o2 + l;
            if (ox >= K) continue;
            const f2 M = l ? f2_pack(mm.z, mm.w) : f2_pack(mm.x, mm.y);
            GI0 = f2_fma(M, f2_pack(w[4 + R - ox], w[5 + R - ox]), GI0);
            GI1 = f2_fma(M, f2_pack(w[6 + R - ox], w[7 + R - ox]), GI1);
          }
        }
      }
      float *dxr = p.gin + (int64_t)b * p.gin_b + (int64_t)jy * p.gin_p + jx0;
      if (P.vec_gin) {
        *reinterpret_cast<float4 *>(dxr) = make_float4(f2_lo(GI0), f2_hi(GI0), f2_lo(GI1), f2_hi(GI1));
      } else {
        dxr[0] = f2_lo(GI0);
        dxr[1] = f2_hi(GI0);
        dxr[2] = f2_lo(GI1);
        dxr[3] = f2_hi(GI1);
      }
      // mask gradient: pixel i (column 4 tx + 4 + i) with in at columns
      // 4 tx + 4 + i - R + ox of row ty + oy
      const float4 gc = *reinterpret_cast<const float4 *>(&sg[(ty + R) * AF_W + 4 * tx + 4]);
      const f2 GG[4] = {f2_pack(gc.x, gc.x), f2_pack(gc.y, gc.y), f2_pack(gc.z, gc.z), f2_pack(gc.w, gc.w)};
#pragma unroll
      for (int oy = 0; oy < K; ++oy) {
        float xw[12];
        af_window12(&sx[(ty + oy) * AF_W + 4 * tx], xw);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int op = 0; op < NP; ++op)
            DM[oy][op] = f2_fma(GG[i], f2_pack(xw[4 - R + i + 2 * op], xw[5 - R + i + 2 * op]), DM[oy][op]);
      }
    }
    __syncthreads();  // every thread is done with this buffer before it is reloaded
  }
  // band pixels, second part: their mask-gradient terms (in through the boundary;
  // CONSTANT taps outside carry none)
  for (int64_t k = k0 + threadIdx.x; k < k1; k += LA_T) {
    const int b = (int)(k / band_per);
    int jy, jx;
    band_pos((int)(k - (int64_t)b * band_per), W, H, R, jy, jx);
    const float gj = p.gout[(int64_t)b * p.gout_b + (int64_t)jy * p.gout_p + jx];
    const float *x = p.in + (int64_t)b * p.in_b;
    const f2 GJ = f2_pack(gj, gj);
    int rx[2 * NP];
#pragma unroll
    for (int o = 0; o < 2 * NP; ++o) rx[o] = o < K ? remap(bm, jx + o - R, 0, W) : (int)0x80000000;
#pragma unroll
    for (int oy = 0; oy < K; ++oy) {
      const int ry = remap(bm, jy + oy - R, 0, H);
#pragma unroll
      for (int op = 0; op < NP; ++op) {
        const float x0 = (ry == (int)0x80000000 || rx[2 * op] == (int)0x80000000)
                             ? 0.0f
                             : __ldg(x + (int64_t)ry * p.in_p + rx[2 * op]);
        const float x1 = (ry == (int)0x80000000 || rx[2 * op + 1] == (int)0x80000000)
                             ? 0.0f
                             : __ldg(x + (int64_t)ry * p.in_p + rx[2 * op + 1]);
        DM[oy][op] = f2_fma(GJ, f2_pack(x0, x1), DM[oy][op]);
      }
    }
  }
  // per-CTA partial of every tap: warp sums, then the warps in order
#pragma unroll
  for (int oy = 0; oy < K; ++oy)
#pragma unroll
    for (int ox = 0; ox < K; ++ox) {
      float v = (ox & 1) ? f2_hi(DM[oy][ox >> 1]) : f2_lo(DM[oy][ox >> 1]);
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][oy * K + ox] = v;
    }
  __syncthreads();
  for (int o = threadIdx.x; o < K * K; o += LA_T) {
    float sum = 0.0f;
    for (int wv = 0; wv < LA_T / 32; ++wv) sum += red[wv][o];
    p.part[(size_t)o * gridDim.x + blockIdx.x] = sum;
  }
}

// one CTA per tap: thread t folds partials t, t + LA_T, ... in FP64, then a
// fixed tree over the threads (the same order on every run)
__global__ void __launch_bounds__(LA_T) adj_mask_combine(const __grid_constant__ AdjParams p, int nparts) {
  __shared__ double sh[LA_T];
  const int o = blockIdx.x;
  double s = 0.0;
  for (int k = threadIdx.x; k < nparts; k += LA_T) s += (double)p.part[(size_t)o * nparts + k];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int d = LA_T / 2; d > 0; d >>= 1) {
    if (threadIdx.x < d) sh[threadIdx.x] += sh[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) p.grad_mask_dev[o] = (float)sh[0];
}

}  // namespace
}  // namespace hgb

using namespace hgb;

extern "C" int hgb_local_op_adjoint(const hgb_view *in, const hgb_view *grad_out, const hgb_view *grad_in,
                                    const float *mask, const float *mask_dev, int mask_w, int mask_h, int boundary,
                                    float *grad_mask_dev, void *stream) {
  int rc = check_view(grad_out, "grad_out");
  if (rc) return rc;
  HGB_REQUIRE(grad_out->dtype == HGB_F32, "hgb_local_op_adjoint: f32 storage expected");
  HGB_REQUIRE(mask_w >= 1 && mask_h >= 1 && mask_w <= LA_MAX && mask_h <= LA_MAX,
              "hgb_local_op_adjoint: mask size must be 1..15");
  HGB_REQUIRE((mask != nullptr) != (mask_dev != nullptr), "hgb_local_op_adjoint: give exactly one of mask, mask_dev");
  HGB_REQUIRE(boundary >= 0 && boundary <= 4, "hgb_local_op_adjoint: bad boundary");
  HGB_REQUIRE(grad_in || grad_mask_dev, "hgb_local_op_adjoint: nothing to compute");
  if (grad_in) {
    rc = check_view(grad_in, "grad_in");
    if (rc) return rc;
    HGB_REQUIRE(grad_in->dtype == HGB_F32 && grad_in->width == grad_out->width &&
                    grad_in->height == grad_out->height && grad_in->batch == grad_out->batch,
                "hgb_local_op_adjoint: grad_in must match grad_out");
  }
  if (grad_mask_dev) {
    rc = check_view(in, "in");
    if (rc) return rc;
    HGB_REQUIRE(in->dtype == HGB_F32 && in->width == grad_out->width && in->height == grad_out->height &&
                    in->batch == grad_out->batch,
                "hgb_local_op_adjoint: in must match grad_out");
  }
  AdjParams p;
  memset(&p, 0, sizeof(p));
  p.gout = (const float *)grad_out->data;
  p.gout_p = grad_out->pitch / 4;
  p.gout_b = grad_out->batch_stride / 4;
  if (in) {
    p.in = (const float *)in->data;
    p.in_p = in->pitch / 4;
    p.in_b = in->batch_stride / 4;
  }
  if (grad_in) {
    p.gin = (float *)grad_in->data;
    p.gin_p = grad_in->pitch / 4;
    p.gin_b = grad_in->batch_stride / 4;
  }
  p.w = grad_out->width;
  p.h = grad_out->height;
  p.batch = grad_out->batch;
  p.mw = mask_w;
  p.mh = mask_h;
  p.bmode = boundary;
  p.mask_dev = mask_dev;
  if (mask)
    for (int i = 0; i < mask_w * mask_h; ++i) p.mask[i] = mask[i];
  p.grad_mask_dev = grad_mask_dev;
  cudaStream_t st = (cudaStream_t)stream;
  const int K = mask_w;
  if (grad_in && grad_mask_dev && mask_w == mask_h && (K == 3 || K == 5 || K == 7) && p.w >= 8 && p.h >= 8 &&
      tma_legal(p.gout, grad_out->pitch, grad_out->batch_stride, p.batch) &&
      tma_legal(p.in, in->pitch, in->batch_stride, p.batch)) {
    AdjFusedParams P;
    memset(&P, 0, sizeof(P));
    const int fh = AF_TH + 2 * (K / 2);
    if (make_tensor_map_3d(&P.map_g, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, p.gout, p.w, p.h, p.batch, grad_out->pitch,
                           grad_out->batch_stride, AF_W, fh) == HGB_OK &&
        make_tensor_map_3d(&P.map_x, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, p.in, p.w, p.h, p.batch, in->pitch,
                           in->batch_stride, AF_W, fh) == HGB_OK) {
      P.p = p;
      P.status = device_status_word();
      P.tiles_x = cdiv(p.w, AF_TW);
      P.tiles_y = cdiv(p.h, AF_TH);
      P.ntiles = P.tiles_x * P.tiles_y * p.batch;
      P.vec_gin = ((uintptr_t)grad_in->data % 16 == 0 && grad_in->pitch % 16 == 0 &&
                   (p.batch == 1 || grad_in->batch_stride % 16 == 0))
                      ? 1
                      : 0;
      const void *kern = K == 3 ? (const void *)adj_fused_kernel<3>
                                : (K == 5 ? (const void *)adj_fused_kernel<5> : (const void *)adj_fused_kernel<7>);
      const int grid = std::max(1, std::min(P.ntiles, num_sms() * resident_ctas(kern, LA_T, 0)));
      Workspace ws;
      rc = workspace_get((size_t)K * K * grid * 4 + 64, &ws);
      if (rc) return rc;
      P.p.part = (float *)ws.base;
      cudaEvent_t ev = before_launch(st);
      if (K == 3)
        adj_fused_kernel<3><<<grid, LA_T, 0, st>>>(P);
      else if (K == 5)
        adj_fused_kernel<5><<<grid, LA_T, 0, st>>>(P);
      else
        adj_fused_kernel<7><<<grid, LA_T, 0, st>>>(P);
      adj_mask_combine<<<K * K, LA_T, 0, st>>>(P.p, grid);
      return after_launch("local_op_adjoint fused", st, ev);
    }
  }
  cudaEvent_t ev = before_launch(st);
  if (grad_in) {
    const dim3 tg(cdiv(p.w, LM_TW), cdiv(p.h, LM_TH), p.batch);
    if (mask_w == mask_h && mask_w == 3)
      adj_in_tile_kernel<3><<<tg, LA_T, 0, st>>>(p);
    else if (mask_w == mask_h && mask_w == 5)
      adj_in_tile_kernel<5><<<tg, LA_T, 0, st>>>(p);
    else if (mask_w == mask_h && mask_w == 7)
      adj_in_tile_kernel<7><<<tg, LA_T, 0, st>>>(p);
    else
      adj_in_kernel<<<dim3(cdiv(p.w, LA_TW), cdiv(p.h, LA_TH), p.batch), LA_T, 0, st>>>(p);
  }
  if (grad_mask_dev) {
    const int taps = mask_w * mask_h;
    const bool tiled = mask_w == mask_h && (mask_w == 3 || mask_w == 5 || mask_w == 7);
    const dim3 tg(cdiv(p.w, LM_TW), cdiv(p.h, LM_TH), p.batch);
    const int nparts = tiled ? (int)(tg.x * tg.y * tg.z) : LA_ROWBLOCKS * p.batch;
    Workspace ws;
    rc = workspace_get((size_t)taps * nparts * 4 + 64, &ws);
    if (rc) return rc;
    p.part = (float *)ws.base;
    if (!tiled)
      adj_mask_kernel<<<dim3(taps, LA_ROWBLOCKS, p.batch), LA_T, 0, st>>>(p);
    else if (mask_w == 3)
      adj_mask_tile_kernel<3><<<tg, LA_T, 0, st>>>(p);
    else if (mask_w == 5)
      adj_mask_tile_kernel<5><<<tg, LA_T, 0, st>>>(p);
    else
      adj_mask_tile_kernel<7><<<tg, LA_T, 0, st>>>(p);
    adj_mask_combine<<<taps, LA_T, 0, st>>>(p, nparts);
  }
  return after_launch("local_op_adjoint", st, ev);
}

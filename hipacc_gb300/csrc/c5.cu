// c5.cu -- forward + adjoint of  y1 = conv(x, mask), y = bilateral(y1; smask,
// sigma_r), loss = mean((y - t)^2)  over a batch of FP32 images, with the
// gradients of the loss with respect to x, the mask and sigma_r.
//
// Forward semantics: conv as hgb_local_op (row-major taps, fused
// multiply-add); bilateral as samples-public/3_Preprocessing/Bilateral_Filter
// (w = smask * exp(-c (y1_q - y1_p)^2), c = 1/(2 sigma_r^2), y = sum w y1_q /
// sum w) reading y1 through the same boundary mode.  Adjoint (hand-derived,
// checked against FP64 central differences by the tests):
//   g_p = 2 (y_p - t_p) / n,  a_p = g_p / W_p
//   dL/dy1_q += a_p w_po (1 - 2c (y1_q - y_p)(y1_q - y1_p))      (q = r(p+o))
//   dL/dy1_p += a_p sum_o w_po (y1_q - y_p) 2c (y1_q - y1_p)
//   dL/dc     = sum_p a_p sum_o w_po (y1_q - y_p) (-(y1_q - y1_p)^2)
//   dL/dsigma = dL/dc * (-1/sigma^3)
//   dL/dx_{r(j+o)} += m_o dL/dy1_j,   dL/dm_o = sum_j dL/dy1_j x_{r(j+o)}
// The boundary is transposed by gathering over pre-images: pixel q collects
// from every (p, o) with r(p + o) = q, found per axis among the virtual
// positions within the radius of the border (CLAMP and MIRROR send several
// virtual positions to an edge pixel; CONSTANT taps carry no gradient).  The
// bilateral weights are recomputed in the adjoint, never stored.
//
// The bilateral works on values scaled by q = sqrt(c log2 e): with u = q y1 a
// tap's weight is exp2(lsm_o - (u_q - u_p)^2) (lsm = log2 smask), and with
// u_y = q y the factor 2c (y1_q - y_p)(y1_q - y1_p) is C2S (u_q - u_yp)(u_q -
// u_p) with C2S = 2 ln 2.
//
// Fused form (mode 0): three persistent kernels over 64 x 16 tiles, 16 x 16
// threads with four horizontally adjacent pixels each, two pixels per packed
// f32x2 operation (every lane rounded like the scalar instruction):
//  1. forward: x staged with a radius of 7 through the boundary; y1 on the
//     tile plus the bilateral radius, eight cells per thread; the bilateral on
//     u (one ex2 and four packed lane operations per tap and pixel pair); the
//     loss and its gradient.  It writes per pixel the float4
//     (u, a, -a u_y, u_y).
//  2. bilateral adjoint: away from the band of radius 4 along the image edges,
//     pixel j gathers from its neighbours p = j - o with the weight of tap o
//     at p, which by the spatial mask's point symmetry is also the weight of
//     j's own tap -o: one ex2 and ten packed operations per tap serve the
//     neighbour term, the centre term and dL/dc.  Band pixels, whose taps
//     cross the edge, go through the pre-images one pixel per thread, as an
//     equal contiguous share of the batch's band list per CTA after its tiles,
//     so the tiles cost the same and the walk has no tail of border tiles.
//  3. convolution adjoint: grad_in as the transposed convolution away from the
//     band of radius 3, and the mask gradient accumulated per pair of taps in
//     packed registers; band pixels again from a flat list.
// Every CTA walks tiles blockIdx.x, blockIdx.x + gridDim.x, ...; the
// reductions (loss, dL/dc, dL/dmask) keep per-thread and per-CTA partials in
// a fixed assignment and are combined in FP64 in block order by the CTA that
// takes the last ticket, so results do not change from run to run.
//
// Unfused form (mode 1): the chain per image as a kernel-per-operator
// framework launches it (conv, bilateral forward, loss gradient, bilateral
// adjoint without the symmetry reuse, conv adjoint, mask gradient), one pixel
// per thread, for comparison.
// Boundary CLAMP, MIRROR or CONSTANT(0); images at least 8 x 8.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "band.cuh"
#include "reduce_common.cuh"
#include "tma.cuh"

namespace hgb {
namespace {

constexpr int C5_T = 256;
constexpr int C5_MK = 7, C5_MR = 3;  // conv mask
constexpr int C5_BK = 9, C5_BR = 4;  // bilateral
constexpr int C5_OUT = (int)0x80000000;  // remap result of a CONSTANT tap outside the image
constexpr float C2S = 1.3862943611198906f;  // 2 ln 2
// unfused kernels: 32 x 16 tiles, one pixel per thread
constexpr int U_TW = 32, U_TH = 16;
constexpr int UY_W = U_TW + 2 * C5_BR, UY_H = U_TH + 2 * C5_BR;  // y1 / a / y (radius 4)
constexpr int UD_W = U_TW + 2 * C5_MR, UD_H = U_TH + 2 * C5_MR;  // dy1 / x (radius 3)
// fused kernels: 64 x 16 tiles, four pixels per thread
constexpr int F_TW = 64, F_TH = 16, F_GX = F_TW / 4;
constexpr int FX_R = C5_MR + C5_BR;                          // radius of the staged x
// x: columns X0-8 .. X0+75 (the convolution reads up to X0+70; a row of 84
// floats puts eight consecutive rows on distinct 16-byte bank groups), rows Y0-7 ..
constexpr int FX_W = F_TW + 20, FX_H = F_TH + 2 * FX_R;
constexpr int FY_W = F_TW + 2 * C5_BR, FY_H = F_TH + 2 * C5_BR;  // u / staged pairs: columns X0-4 .., rows Y0-4 ..
constexpr int FC_W = F_TW + 8, FC_H = F_TH + 2 * C5_MR;      // dy1 / x: columns X0-4 .., rows Y0-3 ..
constexpr int NL_W = C5_BK + 1;  // range-weight pairs per mask row, padded for 16-byte loads
constexpr int US_W = FY_W + 4;  // row stride of the forward's u (eight consecutive rows on distinct bank groups)
constexpr int FX_N = 2528, FC_N = 1600;  // floats per staged array (128-byte multiples)
static_assert(FX_W * FX_H <= FX_N && FX_N % 32 == 0 && FC_W * FC_H <= FC_N && FC_N % 32 == 0,
              "TMA destinations stay 128-byte aligned");
static_assert(F_GX * F_TH == C5_T, "16 x 16 threads");
// Staged rows of pairs are skewed by one element every 8 (16-byte elements)
// or every 16 (8-byte elements): a thread reads positions 4 tx + s, and
// without the skew the 8 (16) lanes of one shared-memory phase would fall on
// 2 (4) bank groups.
constexpr int SQ_W = FY_W + FY_W / 8;   // float4 pairs (u, a)
constexpr int SB_W = FY_W + FY_W / 16;  // float2 pairs (B)
__host__ __device__ constexpr int skew8(int k) { return k + (k >> 3); }
__host__ __device__ constexpr int skew16(int k) { return k + (k >> 4); }
static_assert(skew8(FY_W - 1) < SQ_W && skew16(FY_W - 1) < SB_W, "skewed rows");
static_assert(FY_H * (FY_W / 8) <= C5_T, "one group of eight y1 cells per thread");

struct C5Params {
  CUtensorMap map_xf;      // x, box FX_W x FX_H (forward)
  CUtensorMap map_xc;      // x, box FC_W x FC_H (conv adjoint)
  CUtensorMap map_g;       // dy1, box FC_W x FC_H (conv adjoint)
  int use_tma;             // the maps are valid (x TMA-legal); else plain loads
  int *status;             // device status word (bounded waits)
  const float *x, *t;
  int64_t xp, tp, xb, tb;  // pitches / batch strides in floats
  float4 *pk;              // fused: per pixel (u, a, -a u_y, u_y)
  float *y1, *y, *a;       // unfused intermediates
  float *dy1, *dx;
  int64_t ip, ib;          // pitch / batch stride of the intermediates, in elements
  int64_t dxp, dxb;
  int w, h, batch;
  int bmode;
  int vec_x, vec_dx;       // rows of x / grad_x allow aligned float4 accesses
  const float *mask_dev;   // 49
  const float *sigma_dev;  // 1
  float lsm[C5_BK * C5_BK];  // log2(smask), -inf for zero cells
  double inv_n;            // 1 / (batch * w * h)
  float2 *loss_part;       // per block Kahan (s, c)
  float *dc_part;          // per block
  float *dm_part;          // per block x 49
  unsigned int *tickets;   // [0] forward, [1] bilateral adjoint, [2] conv adjoint
  double *loss_dev;
  float *grad_mask_dev, *grad_sigma_dev;
  int img_offset;          // image of the launch (per-image launches; 0 otherwise)
  int tiles_x, tiles_y, ntiles;  // tile grid of the launch (all images, or one image)
};

// tile t of the launch: image, origin
template <int TW, int TH>
__device__ __forceinline__ void tile_origin(const C5Params &p, int t, int &b, int &X0, int &Y0) {
  const int per = p.tiles_x * p.tiles_y;
  const int bz = t / per, r = t - bz * per;
  const int by = r / p.tiles_x;
  b = bz + p.img_offset;
  X0 = (r - by * p.tiles_x) * TW;
  Y0 = by * TH;
}

// Deterministic block-wide FP64 sum of item(0..n-1): thread t folds items
// t, t + C5_T, ... in order, then a fixed tree over the threads.  Every thread
// of the block calls it; every thread gets the sum.
template <class F>
__device__ __forceinline__ double block_sum_fixed(int n, F item, double *sh) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += C5_T) s += item(i);
  sh[threadIdx.x] = s;
  __syncthreads();
#pragma unroll
  for (int d = C5_T / 2; d > 0; d >>= 1) {
    if (threadIdx.x < d) sh[threadIdx.x] += sh[threadIdx.x + d];
    __syncthreads();
  }
  const double r = sh[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ float ex2f(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ int remap_c5(int mode, int v, int n) { return remap(mode, v, 0, n); }

__device__ __forceinline__ void sigma_consts(const C5Params &p, float &c, float &k2) {
  const float s = __ldg(p.sigma_dev);
  c = 0.5f / (s * s);
  k2 = -c * 1.4426950408889634f;
}

// block-wide sum of a float (thread 0 returns the value)
__device__ __forceinline__ float block_sum_f(float v, float *sbuf) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
  if ((threadIdx.x & 31) == 0) sbuf[threadIdx.x >> 5] = v;
  __syncthreads();
  float r = 0.0f;
  if (threadIdx.x == 0)
    for (int i = 0; i < C5_T / 32; ++i) r += sbuf[i];
  __syncthreads();
  return r;
}

// per-CTA Kahan partial of the squared error, FP64 combine by the last CTA
__device__ __forceinline__ void loss_publish(const C5Params &p, Kahan lsum, double *dsh) {
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    Kahan o;
    o.s = __shfl_down_sync(0xffffffffu, lsum.s, d);
    o.c = __shfl_down_sync(0xffffffffu, lsum.c, d);
    lsum = kahan_merge(lsum, o);
  }
  __shared__ float2 kp[C5_T / 32];
  if ((threadIdx.x & 31) == 0) kp[threadIdx.x >> 5] = make_float2(lsum.s, lsum.c);
  __syncthreads();
  const unsigned int nb = grid_blocks();
  if (threadIdx.x == 0) {
    Kahan k{0.0f, 0.0f};
    for (int i = 0; i < C5_T / 32; ++i) k = kahan_merge(k, Kahan{kp[i].x, kp[i].y});
    p.loss_part[block_rank()] = make_float2(k.s, k.c);
  }
  if (take_last_ticket(p.tickets + 0)) {
    const double s = block_sum_fixed(
        (int)nb,
        [&](int i) {
          const float2 v = __ldcg(p.loss_part + i);
          return (double)v.x - (double)v.y;
        },
        dsh);
    if (threadIdx.x == 0) {
      *p.loss_dev = s * p.inv_n;
      p.tickets[0] = 0u;
    }
  }
}

// ================================================================== fused form

// a mask row of range-weight pairs, two per 16-byte load
__device__ __forceinline__ void nl_row(const f2 *row, f2 (&o)[NL_W]) {
#pragma unroll
  for (int i = 0; i < NL_W / 2; ++i) {
    const ulonglong2 v = reinterpret_cast<const ulonglong2 *>(row)[i];
    o[2 * i] = v.x;
    o[2 * i + 1] = v.y;
  }
}

// one bilateral tap for a pixel pair: weight e = exp2(-(d'^2 + nl))
__device__ __forceinline__ void bil_tap(f2 V, f2 C, f2 NL, f2 &Ws, f2 &Ns) {
  const f2 d = f2_sub(V, C);
  const f2 t = f2_fma(d, d, NL);
  const f2 e = f2_pack(ex2f(-f2_lo(t)), ex2f(-f2_hi(t)));
  Ws = f2_add(Ws, e);
  Ns = f2_fma(e, V, Ns);
}

// One thread issues the TMA loads of a tile's staged boxes on the stage's
// barrier.
__device__ __forceinline__ void c5_issue(uint64_t *bar, unsigned bytes, void *d0, const CUtensorMap *m0, void *d1,
                                         const CUtensorMap *m1, int x, int y, int b) {
  mbar_expect_tx(bar, bytes);
  tma_load_3d(d0, m0, x, y, b, bar);
  if (d1) tma_load_3d(d1, m1, x, y, b, bar);
}

// Bounded wait for stage s of tile iteration i; on expiry records the status
// and waits (bounded) for the loads still in flight, the next tile's included.
__device__ __forceinline__ bool c5_wait(const C5Params &p, uint64_t *bars, int i, bool next_issued) {
  const int s = i & 1;
  if (cta_wait(&bars[s], (i >> 1) & 1)) return true;
  if (threadIdx.x == 0) {
    record_status(p.status, HGB_ERR_TIMEOUT);
    mbar_wait(&bars[s], (i >> 1) & 1);
    if (next_issued) mbar_wait(&bars[s ^ 1], ((i + 1) >> 1) & 1);
  }
  return false;
}

__global__ void __launch_bounds__(C5_T, 5) c5_forward_kernel(const __grid_constant__ C5Params p) {
  __shared__ __align__(128) float xst[2][FX_N];  // x: double-buffered TMA stages
  __shared__ __align__(16) float us[FY_H * US_W];
  __shared__ f2 m2[C5_MK * C5_MK];
  __shared__ __align__(16) f2 nl2[C5_BK * NL_W];
  __shared__ __align__(8) uint64_t bars[2];
  double *dsh = reinterpret_cast<double *>(&xst[0][0]);  // the final combine, after the tiles
  const int W = p.w, H = p.h, bm = p.bmode;
  if (p.use_tma && threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_fence_init();
  }
  for (int i = threadIdx.x; i < C5_MK * C5_MK; i += C5_T) {
    const float m = __ldg(p.mask_dev + i);
    m2[i] = f2_pack(m, m);
  }
  for (int i = threadIdx.x; i < C5_BK * NL_W; i += C5_T) {
    const int oy = i / NL_W, ox = i - oy * NL_W;
    const float n = ox < C5_BK ? -p.lsm[oy * C5_BK + ox] : 0.0f;
    nl2[i] = f2_pack(n, n);
  }
  float c, k2;
  sigma_consts(p, c, k2);
  const float q = sqrtf(-k2), inv_q = 1.0f / q;
  const float g_scale = (float)(2.0 * p.inv_n);
  const int tx = threadIdx.x % F_GX, ty = threadIdx.x / F_GX;
  Kahan lsum{0.0f, 0.0f};
  __syncthreads();  // barriers initialised
  auto issue = [&](int tile, int s) {
    int b, X0, Y0;
    tile_origin<F_TW, F_TH>(p, tile, b, X0, Y0);
    c5_issue(&bars[s], FX_W * FX_H * 4, xst[s], &p.map_xf, nullptr, nullptr, X0 - 8, Y0 - FX_R, b);
  };
  if (p.use_tma && threadIdx.x == 0) issue(blockIdx.x, 0);
  int it = 0;
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x, ++it) {
    int b, X0, Y0;
    tile_origin<F_TW, F_TH>(p, tile, b, X0, Y0);
    const float *x = p.x + (int64_t)b * p.xb;
    const bool edge = !(X0 >= 8 && X0 - 8 + FX_W <= W && Y0 >= FX_R && Y0 + F_TH + FX_R <= H);
    float *xs = xst[p.use_tma ? (it & 1) : 0];
    // x on rows Y0-7 .., columns X0-8 .. through the boundary
    if (p.use_tma) {
      // the next tile's box lands while this one computes (its stage was last
      // read by the convolution of the previous tile, before a CTA barrier)
      const bool next = tile + (int)gridDim.x < p.ntiles;
      if (next && threadIdx.x == 0) {
        fence_proxy_async_smem();
        issue(tile + gridDim.x, (it & 1) ^ 1);
      }
      if (!c5_wait(p, bars, it, next)) break;
      if (edge) {  // cells outside the image (zero-filled) through the boundary
        for (int cc = threadIdx.x; cc < FX_W * FX_H; cc += C5_T) {
          const int r = cc / FX_W, k = cc - r * FX_W;
          const int vy = Y0 - FX_R + r, vx = X0 - 8 + k;
          if (vy >= 0 && vy < H && vx >= 0 && vx < W) continue;
          const int ry = remap_c5(bm, vy, H), rx = remap_c5(bm, vx, W);
          xs[cc] = (ry == C5_OUT || rx == C5_OUT) ? 0.0f : __ldg(x + (int64_t)ry * p.xp + rx);
        }
        __syncthreads();
      }
    } else {
      __syncthreads();  // the previous tile's reads of xs are done
      if (p.vec_x && !edge) {
        for (int c4 = threadIdx.x; c4 < FX_H * (FX_W / 4); c4 += C5_T) {
          const int r = c4 / (FX_W / 4), k4 = c4 - r * (FX_W / 4);
          reinterpret_cast<float4 *>(xs)[c4] =
              __ldg(reinterpret_cast<const float4 *>(x + (int64_t)(Y0 - FX_R + r) * p.xp + X0 - 8) + k4);
        }
      } else {
        for (int cc = threadIdx.x; cc < FX_W * FX_H; cc += C5_T) {
          const int r = cc / FX_W, k = cc - r * FX_W;
          const int ry = remap_c5(bm, Y0 - FX_R + r, H), rx = remap_c5(bm, X0 - 8 + k, W);
          xs[cc] = (ry == C5_OUT || rx == C5_OUT) ? 0.0f : __ldg(x + (int64_t)ry * p.xp + rx);
        }
      }
      __syncthreads();
    }
    // u = q y1 on rows Y0-4 .., columns X0-4 ..: eight cells per thread from
    // one 16-value row window of x per mask row, taps row-major (y1 exactly as
    // hgb_local_op computes it)
    if (threadIdx.x < FY_H * (FY_W / 8)) {
      // consecutive threads take consecutive rows (distinct bank groups)
      const int g = threadIdx.x / FY_H, r = threadIdx.x - g * FY_H, k0 = 8 * g;
      f2 acc[4] = {0ull, 0ull, 0ull, 0ull};
#pragma unroll
      for (int my = 0; my < C5_MK; ++my) {
        const float4 *row = reinterpret_cast<const float4 *>(&xs[(r + my) * FX_W + k0]);
        float w[16];
#pragma unroll
        for (int v = 0; v < 4; ++v) {
          const float4 t4 = row[v];
          w[4 * v] = t4.x;
          w[4 * v + 1] = t4.y;
          w[4 * v + 2] = t4.z;
          w[4 * v + 3] = t4.w;
        }
#pragma unroll
        for (int mx = 0; mx < C5_MK; ++mx) {
          const f2 M = m2[my * C5_MK + mx];
#pragma unroll
          for (int i = 0; i < 4; ++i) acc[i] = f2_fma(M, f2_pack(w[2 * i + 1 + mx], w[2 * i + 2 + mx]), acc[i]);
        }
      }
      float4 *o = reinterpret_cast<float4 *>(&us[r * US_W + k0]);
      o[0] = make_float4(q * f2_lo(acc[0]), q * f2_hi(acc[0]), q * f2_lo(acc[1]), q * f2_hi(acc[1]));
      o[1] = make_float4(q * f2_lo(acc[2]), q * f2_hi(acc[2]), q * f2_lo(acc[3]), q * f2_hi(acc[3]));
    }
    __syncthreads();
    // a cell outside the image is u at the remapped position (the bilateral
    // reads y1 through the boundary); cells beyond the radius of the image
    // are read by no pixel of it
    if (!(X0 >= C5_BR && X0 + F_TW + C5_BR <= W && Y0 >= C5_BR && Y0 + F_TH + C5_BR <= H)) {
      for (int cc = threadIdx.x; cc < FY_H * FY_W; cc += C5_T) {
        const int r = cc / FY_W, k = cc - r * FY_W;
        const int vy = Y0 - C5_BR + r, vx = X0 - C5_BR + k;
        if (vy >= 0 && vy < H && vx >= 0 && vx < W) continue;
        if (vy < -C5_BR || vy >= H + C5_BR || vx < -C5_BR || vx >= W + C5_BR) continue;
        const int ry = remap_c5(bm, vy, H), rx = remap_c5(bm, vx, W);
        us[r * US_W + k] = (ry == C5_OUT || rx == C5_OUT) ? 0.0f : us[(ry - Y0 + C5_BR) * US_W + rx - X0 + C5_BR];
      }
      __syncthreads();
    }
    // the targets of the four pixels, loaded before the bilateral hides their latency
    const int gy = Y0 + ty, gx0 = X0 + 4 * tx;
    float tv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    if (gy < H) {
      const float *trow = p.t + (int64_t)b * p.tb + (int64_t)gy * p.tp;
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (gx0 + i < W) tv[i] = __ldg(trow + gx0 + i);
    }
    // bilateral: pixels 4 tx .. 4 tx + 3 of row ty, pairs (0, 1) and (2, 3)
    const float4 cv = *reinterpret_cast<const float4 *>(&us[(ty + C5_BR) * US_W + 4 * tx + C5_BR]);
    const f2 C0 = f2_pack(cv.x, cv.y), C1 = f2_pack(cv.z, cv.w);
    f2 Ws0 = 0ull, Ws1 = 0ull, Ns0 = 0ull, Ns1 = 0ull;
#pragma unroll 3
    for (int oy = 0; oy < C5_BK; ++oy) {
      const float4 *row = reinterpret_cast<const float4 *>(&us[(ty + oy) * US_W + 4 * tx]);
      float w[12];
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        const float4 t4 = row[v];
        w[4 * v] = t4.x;
        w[4 * v + 1] = t4.y;
        w[4 * v + 2] = t4.z;
        w[4 * v + 3] = t4.w;
      }
      f2 NLr[NL_W];
      nl_row(&nl2[oy * NL_W], NLr);
#pragma unroll
      for (int ox = 0; ox < C5_BK; ++ox) {
        const f2 NL = NLr[ox];
        bil_tap(f2_pack(w[ox], w[ox + 1]), C0, NL, Ws0, Ns0);
        bil_tap(f2_pack(w[ox + 2], w[ox + 3]), C1, NL, Ws1, Ns1);
      }
    }
    if (gy < H && gx0 < W) {
      const float Wv[4] = {f2_lo(Ws0), f2_hi(Ws0), f2_lo(Ws1), f2_hi(Ws1)};
      const float Nv[4] = {f2_lo(Ns0), f2_hi(Ns0), f2_lo(Ns1), f2_hi(Ns1)};
      const float Uv[4] = {cv.x, cv.y, cv.z, cv.w};
      float4 *orow = p.pk + (int64_t)b * p.ib + (int64_t)gy * p.ip;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int gx = gx0 + i;
        if (gx >= W) break;
        const float uy = Nv[i] / Wv[i];
        const float e = uy * inv_q - tv[i];
        lsum = kahan_add(lsum, e * e);
        const float a = (g_scale * e) / Wv[i];
        orow[gx] = make_float4(Uv[i], a, -a * uy, uy);
      }
    }
  }  // tiles
  loss_publish(p, lsum, dsh);
}

// one symmetric tap of the bilateral adjoint for a pixel pair j (centre U, A =
// a_j, B = -a_j u_yj) and its neighbour pair p = j - o (Pu, Pa, PB = -a_p
// u_yp); s = {sum e a_p, sum e d (u_j a_p - a_p u_yp), sum e d a_j (u_p -
// u_yj), the same times d} with d = u_j - u_p
__device__ __forceinline__ void adj_tap(f2 Pu, f2 Pa, f2 PB, f2 U, f2 A, f2 B, f2 NL, f2 (&s)[4]) {
  const f2 d = f2_sub(U, Pu);
  const f2 t = f2_fma(d, d, NL);
  const f2 e = f2_pack(ex2f(-f2_lo(t)), ex2f(-f2_hi(t)));
  const f2 h = f2_mul(e, d);
  s[0] = f2_fma(e, Pa, s[0]);
  s[1] = f2_fma(h, f2_fma(U, Pa, PB), s[1]);
  const f2 wd = f2_mul(h, f2_fma(A, Pu, B));
  s[2] = f2_add(s[2], wd);
  s[3] = f2_fma(wd, d, s[3]);
}

// dL/dy1 of a band pixel j through the pre-images, from the forward's packed
// values; adds j's dL/dc share (times -q^3) to dc
__device__ float bil_adj_band(const C5Params &p, const float4 *pk, int jy, int jx, const float *lsm, float inv_q3,
                              float &dc) {
  const int W = p.w, H = p.h, bm = p.bmode;
  const float4 J = __ldg(pk + (int64_t)jy * p.ip + jx);
  // centre term and dL/dc over j's own taps, read through the boundary
  int rx[C5_BK];
#pragma unroll
  for (int o = 0; o < C5_BK; ++o) rx[o] = remap_c5(bm, jx + o - C5_BR, W);
  float ctr = 0.0f, s2 = 0.0f;
  for (int oy = 0; oy < C5_BK; ++oy) {
    const int ry = remap_c5(bm, jy + oy - C5_BR, H);
#pragma unroll
    for (int ox = 0; ox < C5_BK; ++ox) {
      const float uq = (ry == C5_OUT || rx[ox] == C5_OUT) ? 0.0f : __ldg(pk + (int64_t)ry * p.ip + rx[ox]).x;
      const float d = uq - J.x;
      const float e = ex2f(__fmaf_rn(-d, d, lsm[oy * C5_BK + ox]));
      const float wd = e * __fmaf_rn(J.y, uq, J.z) * d;
      ctr += wd;
      s2 = __fmaf_rn(wd, d, s2);
    }
  }
  dc = __fmaf_rn(-inv_q3, s2, dc);
  // neighbour term gathered over the pre-images of j
  int prx[1 + C5_BR], pry[1 + C5_BR];
  const int nx = preimages(bm, jx, W, C5_BR, prx), ny = preimages(bm, jy, H, C5_BR, pry);
  float dn = 0.0f;
  for (int iy = 0; iy < ny; ++iy)
    for (int oy = 0; oy < C5_BK; ++oy) {
      const int py = pry[iy] - (oy - C5_BR);
      if (py < 0 || py >= H) continue;
      const float4 *prow = pk + (int64_t)py * p.ip;
      for (int ix = 0; ix < nx; ++ix)
#pragma unroll
        for (int ox = 0; ox < C5_BK; ++ox) {  // the row's loads in flight together
          const int px = prx[ix] - (ox - C5_BR);
          if (px < 0 || px >= W) continue;
          const float4 P = __ldg(prow + px);
          const float d = J.x - P.x;
          const float e = ex2f(__fmaf_rn(-d, d, lsm[oy * C5_BK + ox]));
          dn = __fmaf_rn(e, __fmaf_rn(-C2S * d, __fmaf_rn(J.x, P.y, P.z), P.y), dn);
        }
    }
  return __fmaf_rn(C2S, ctr, dn);
}

__global__ void __launch_bounds__(C5_T, 4) c5_bilateral_adjoint_kernel(const __grid_constant__ C5Params p) {
  // per staged position k of a row: (u_k, u_k+1, a_k, a_k+1) and (B_k, B_k+1),
  // so that a pixel pair's neighbours at any offset are one aligned load each
  __shared__ __align__(16) float4 sq[FY_H * SQ_W];
  __shared__ __align__(16) f2 sb[FY_H * SB_W];
  __shared__ __align__(16) f2 nl2[C5_BK * NL_W];
  __shared__ float lsm[C5_BK * C5_BK];
  __shared__ float sbuf[32];
  double *dsh = reinterpret_cast<double *>(sq);  // the final combine, after the tiles
  const int W = p.w, H = p.h;
  for (int i = threadIdx.x; i < C5_BK * NL_W; i += C5_T) {
    const int oy = i / NL_W, ox = i - oy * NL_W;
    const float n = ox < C5_BK ? -p.lsm[oy * C5_BK + ox] : 0.0f;
    nl2[i] = f2_pack(n, n);
    if (ox < C5_BK) lsm[oy * C5_BK + ox] = p.lsm[oy * C5_BK + ox];
  }
  float c, k2;
  sigma_consts(p, c, k2);
  const float q = sqrtf(-k2), inv_q = 1.0f / q;
  const float inv_q3 = inv_q * inv_q * inv_q;
  const int tx = threadIdx.x % F_GX, ty = threadIdx.x / F_GX;
  float dc = 0.0f;
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
    int b, X0, Y0;
    tile_origin<F_TW, F_TH>(p, tile, b, X0, Y0);
    const float4 *pk = p.pk + (int64_t)b * p.ib;
    __syncthreads();  // the previous tile's reads are done
    // in-image cells of rows Y0-4 .., columns X0-4 ..: two positions per item
    for (int it = threadIdx.x; it < FY_H * (FY_W / 2); it += C5_T) {
      const int r = it / (FY_W / 2), k = (it - r * (FY_W / 2)) * 2;
      const int gy = Y0 - C5_BR + r, gx = X0 - C5_BR + k;
      if (gy < 0 || gy >= H) continue;
      const float4 *src = pk + (int64_t)gy * p.ip;
      const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      const float4 v0 = (gx >= 0 && gx < W) ? __ldg(src + gx) : z;
      const float4 v1 = (gx + 1 >= 0 && gx + 1 < W) ? __ldg(src + gx + 1) : z;
      const float4 v2 = (gx + 2 >= 0 && gx + 2 < W) ? __ldg(src + gx + 2) : z;
      sq[r * SQ_W + skew8(k)] = make_float4(v0.x, v1.x, v0.y, v1.y);
      sq[r * SQ_W + skew8(k + 1)] = make_float4(v1.x, v2.x, v1.y, v2.y);
      sb[r * SB_W + skew16(k)] = f2_pack(v0.z, v1.z);
      sb[r * SB_W + skew16(k + 1)] = f2_pack(v1.z, v2.z);
    }
    __syncthreads();
    const int jx0 = X0 + 4 * tx, jy = Y0 + ty;
    if (jx0 >= C5_BR && jx0 + 3 < W - C5_BR && jy >= C5_BR && jy < H - C5_BR) {
      // skewed position 4 tx + s of a row = base + s + (s < 4 ? 0 : s < 8 ? k1 : k2)
      const int q1 = tx & 1, b1 = (tx & 3) == 3, b2 = (tx & 3) >= 2;
      const int qbase = 4 * tx + (tx >> 1), bbase = 4 * tx + (tx >> 2);
      const int ce_q = (ty + C5_BR) * SQ_W + qbase + q1, ce_b = (ty + C5_BR) * SB_W + bbase + b1;
      const float4 J0 = sq[ce_q + 4], J1 = sq[ce_q + 6];
      const f2 U0 = f2_pack(J0.x, J0.y), U1 = f2_pack(J1.x, J1.y);
      const f2 A0 = f2_pack(J0.z, J0.w), A1 = f2_pack(J1.z, J1.w);
      const f2 B0 = sb[ce_b + 4], B1 = sb[ce_b + 6];
      f2 s0[4] = {0ull, 0ull, 0ull, 0ull}, s1[4] = {0ull, 0ull, 0ull, 0ull};
#pragma unroll 3
      for (int oy = 0; oy < C5_BK; ++oy) {
        // neighbours p = j - o: row ty + 8 - oy, positions 4 tx + s, s = 0 .. 10;
        // pair 0 takes tap ox = 8 - s, pair 1 tap ox = 10 - s
        const int row = ty + 2 * C5_BR - oy;
        const float4 *qr = &sq[row * SQ_W + qbase];
        const f2 *br = &sb[row * SB_W + bbase];
        f2 NL[NL_W];
        nl_row(&nl2[oy * NL_W], NL);
#pragma unroll
        for (int s = 0; s <= 2 * C5_BR + 2; ++s) {
          const float4 P = qr[s + (s < 4 ? 0 : s < 8 ? q1 : 1)];
          const f2 Pu = f2_pack(P.x, P.y), Pa = f2_pack(P.z, P.w), PB = br[s + (s < 4 ? 0 : s < 8 ? b1 : b2)];
          if (s <= 2 * C5_BR) adj_tap(Pu, Pa, PB, U0, A0, B0, NL[2 * C5_BR - s], s0);
          if (s >= 2) adj_tap(Pu, Pa, PB, U1, A1, B1, NL[2 * C5_BR + 2 - s], s1);
        }
      }
      // dL/dy1 = sum e a_p - C2S (neighbour sum + centre sum); dL/dc share -s3 / q^3
      const float4 o = make_float4(f2_lo(s0[0]) - C2S * (f2_lo(s0[1]) + f2_lo(s0[2])),
                                   f2_hi(s0[0]) - C2S * (f2_hi(s0[1]) + f2_hi(s0[2])),
                                   f2_lo(s1[0]) - C2S * (f2_lo(s1[1]) + f2_lo(s1[2])),
                                   f2_hi(s1[0]) - C2S * (f2_hi(s1[1]) + f2_hi(s1[2])));
      *reinterpret_cast<float4 *>(p.dy1 + (int64_t)b * p.ib + (int64_t)jy * p.ip + jx0) = o;
      dc = __fmaf_rn(-inv_q3, (f2_lo(s0[3]) + f2_hi(s0[3])) + (f2_lo(s1[3]) + f2_hi(s1[3])), dc);
    }
  }  // tiles
  // band pixels of every image of the batch: an equal contiguous share per CTA
  {
    const int per = band_size(W, H, C5_BR);
    int64_t k0, k1;
    cta_share((int64_t)per * p.batch, k0, k1);
    for (int64_t k = k0 + threadIdx.x; k < k1; k += C5_T) {
      const int b = (int)(k / per);
      int jy, jx;
      band_pos((int)(k - (int64_t)b * per), W, H, C5_BR, jy, jx);
      const float g = bil_adj_band(p, p.pk + (int64_t)b * p.ib, jy, jx, lsm, inv_q3, dc);
      p.dy1[(int64_t)b * p.ib + (int64_t)jy * p.ip + jx] = g;
    }
  }
  const float bdc = block_sum_f(dc, sbuf);
  const unsigned int nb = grid_blocks();
  if (threadIdx.x == 0) p.dc_part[block_rank()] = bdc;
  if (take_last_ticket(p.tickets + 1)) {
    const double s = block_sum_fixed((int)nb, [&](int i) { return (double)__ldcg(p.dc_part + i); }, dsh);
    if (threadIdx.x == 0) {
      const double sg = (double)__ldg(p.sigma_dev);
      *p.grad_sigma_dev = (float)(s * (-1.0 / (sg * sg * sg)));
      p.tickets[1] = 0u;
    }
  }
}

// stage rows Y0-3 .., columns X0-4 .. of one image plane without TMA (zero
// outside the image)
__device__ __forceinline__ void c5_stage_plain(float *dst, const float *src, int64_t pitch, int X0, int Y0, int W,
                                               int H, bool vec) {
  for (int it = threadIdx.x; it < FC_H * (FC_W / 4); it += C5_T) {
    const int r = it / (FC_W / 4), k = (it - r * (FC_W / 4)) * 4;
    const int gy = Y0 - C5_MR + r, gx = X0 - 4 + k;
    float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (gy >= 0 && gy < H) {
      const float *row = src + (int64_t)gy * pitch;
      if (vec && gx >= 0 && gx + 3 < W) {
        v = __ldg(reinterpret_cast<const float4 *>(row + gx));
      } else {
        v.x = (gx >= 0 && gx < W) ? __ldg(row + gx) : 0.0f;
        v.y = (gx + 1 >= 0 && gx + 1 < W) ? __ldg(row + gx + 1) : 0.0f;
        v.z = (gx + 2 >= 0 && gx + 2 < W) ? __ldg(row + gx + 2) : 0.0f;
        v.w = (gx + 3 >= 0 && gx + 3 < W) ? __ldg(row + gx + 3) : 0.0f;
      }
    }
    *reinterpret_cast<float4 *>(&dst[r * FC_W + k]) = v;
  }
}

// a row window of twelve staged values (three aligned 16-byte loads)
__device__ __forceinline__ void c5_window12(const float *row, float (&w)[12]) {
#pragma unroll
  for (int v = 0; v < 3; ++v) {
    const float4 t4 = reinterpret_cast<const float4 *>(row)[v];
    w[4 * v] = t4.x;
    w[4 * v + 1] = t4.y;
    w[4 * v + 2] = t4.z;
    w[4 * v + 3] = t4.w;
  }
}

__global__ void __launch_bounds__(C5_T, 2) c5_conv_adjoint_kernel(const __grid_constant__ C5Params p) {
  __shared__ __align__(128) float stg[2][2][FC_N];  // [stage][dy1, x]: TMA double buffer
  __shared__ __align__(16) f2 m2[C5_MK][8];        // mask pairs (m, m); the eighth is padding
  __shared__ float msk[C5_MK * C5_MK];
  __shared__ float red[C5_T / 32][C5_MK * C5_MK];
  __shared__ __align__(8) uint64_t bars[2];
  const int W = p.w, H = p.h, bm = p.bmode;
  for (int i = threadIdx.x; i < C5_MK * 8; i += C5_T) {
    const int oy = i / 8, ox = i - oy * 8;
    const float m = ox < C5_MK ? __ldg(p.mask_dev + oy * C5_MK + ox) : 0.0f;
    m2[oy][ox] = f2_pack(m, m);
    if (ox < C5_MK) msk[oy * C5_MK + ox] = m;
  }
  if (p.use_tma && threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  auto issue = [&](int tile, int s) {
    int b, X0, Y0;
    tile_origin<F_TW, F_TH>(p, tile, b, X0, Y0);
    c5_issue(&bars[s], 2 * FC_W * FC_H * 4, stg[s][0], &p.map_g, stg[s][1], &p.map_xc, X0 - 4, Y0 - C5_MR, b);
  };
  // the first tile's boxes land while the band's grad_in runs
  if (p.use_tma && threadIdx.x == 0) issue(blockIdx.x, 0);
  // band pixels of every image of the batch, an equal contiguous share per
  // CTA; first part (before the mask-gradient registers are live): grad_in
  // through the pre-images
  const int band_per = band_size(W, H, C5_MR);
  int64_t k0, k1;
  cta_share((int64_t)band_per * p.batch, k0, k1);
  for (int64_t k = k0 + threadIdx.x; k < k1; k += C5_T) {
    const int b = (int)(k / band_per);
    int jy, jx;
    band_pos((int)(k - (int64_t)b * band_per), W, H, C5_MR, jy, jx);
    const float *g = p.dy1 + (int64_t)b * p.ib;
    int prx[1 + C5_MR], pry[1 + C5_MR];
    const int nx = preimages(bm, jx, W, C5_MR, prx), ny = preimages(bm, jy, H, C5_MR, pry);
    float acc = 0.0f;
    for (int iy = 0; iy < ny; ++iy)
      for (int oy = 0; oy < C5_MK; ++oy) {
        const int sy = pry[iy] - (oy - C5_MR);
        if (sy < 0 || sy >= H) continue;
        const float *grow = g + (int64_t)sy * p.ip;
        for (int ix = 0; ix < nx; ++ix)
#pragma unroll
          for (int ox = 0; ox < C5_MK; ++ox) {  // the row's loads in flight together
            const int sxp = prx[ix] - (ox - C5_MR);
            if (sxp < 0 || sxp >= W) continue;
            acc = __fmaf_rn(msk[oy * C5_MK + ox], grow[sxp], acc);
          }
      }
    p.dx[(int64_t)b * p.dxb + (int64_t)jy * p.dxp + jx] = acc;
  }
  const int tx = threadIdx.x % F_GX, ty = threadIdx.x / F_GX;
  // dL/dmask per pair of taps (oy, 2 op), (oy, 2 op + 1); the eighth tap of a
  // row is padding
  f2 DM[C5_MK][4];
#pragma unroll
  for (int i = 0; i < C5_MK; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) DM[i][j] = 0ull;
  int it = 0;
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x, ++it) {
    int b, X0, Y0;
    tile_origin<F_TW, F_TH>(p, tile, b, X0, Y0);
    const int s = p.use_tma ? (it & 1) : 0;
    if (p.use_tma) {
      // the next tile's boxes land while this one computes
      const bool next = tile + (int)gridDim.x < p.ntiles;
      if (next && threadIdx.x == 0) {
        fence_proxy_async_smem();
        issue(tile + gridDim.x, s ^ 1);
      }
      if (!c5_wait(p, bars, it, next)) break;
    } else {
      c5_stage_plain(stg[0][0], p.dy1 + (int64_t)b * p.ib, p.ip, X0, Y0, W, H, true);
      c5_stage_plain(stg[0][1], p.x + (int64_t)b * p.xb, p.xp, X0, Y0, W, H, p.vec_x);
      __syncthreads();
    }
    const float *sg = stg[s][0], *sx = stg[s][1];
    const int jx0 = X0 + 4 * tx, jy = Y0 + ty;
    if (jx0 >= 4 && jx0 + 3 < W - C5_MR && jy >= C5_MR && jy < H - C5_MR) {
      // grad_in: pixel pair pp (columns 4 tx + 4 + 2 pp ..) gathers dy1 at
      // columns 4 tx + 7 + 2 pp - ox of row ty + 6 - oy
      f2 GI0 = 0ull, GI1 = 0ull;
#pragma unroll
      for (int oy = 0; oy < C5_MK; ++oy) {
        float w[12];
        c5_window12(&sg[(ty + 2 * C5_MR - oy) * FC_W + 4 * tx], w);
        const float4 *mr = reinterpret_cast<const float4 *>(&m2[oy][0]);
#pragma unroll
        for (int o2 = 0; o2 < 4; ++o2) {
          const float4 mm = mr[o2];  // taps 2 o2, 2 o2 + 1 as pairs (m, m)
#pragma unroll
          for (int l = 0; l < 2; ++l) {
            const int ox = 2 * o2 + l;
            if (ox >= C5_MK) continue;
            const f2 M = l ? f2_pack(mm.z, mm.w) : f2_pack(mm.x, mm.y);
            GI0 = f2_fma(M, f2_pack(w[7 - ox], w[8 - ox]), GI0);
            GI1 = f2_fma(M, f2_pack(w[9 - ox], w[10 - ox]), GI1);
          }
        }
      }
      float *dxr = p.dx + (int64_t)b * p.dxb + (int64_t)jy * p.dxp + jx0;
      if (p.vec_dx) {
        *reinterpret_cast<float4 *>(dxr) = make_float4(f2_lo(GI0), f2_hi(GI0), f2_lo(GI1), f2_hi(GI1));
      } else {
        dxr[0] = f2_lo(GI0);
        dxr[1] = f2_hi(GI0);
        dxr[2] = f2_lo(GI1);
        dxr[3] = f2_hi(GI1);
      }
      // mask gradient: pixel i (column 4 tx + 4 + i) with x at columns
      // 4 tx + 1 + i + ox of row ty + oy
      const float4 gc = *reinterpret_cast<const float4 *>(&sg[(ty + C5_MR) * FC_W + 4 * tx + 4]);
      const f2 GG[4] = {f2_pack(gc.x, gc.x), f2_pack(gc.y, gc.y), f2_pack(gc.z, gc.z), f2_pack(gc.w, gc.w)};
#pragma unroll
      for (int oy = 0; oy < C5_MK; ++oy) {
        float xw[12];
        c5_window12(&sx[(ty + oy) * FC_W + 4 * tx], xw);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int op = 0; op < 4; ++op)
            DM[oy][op] = f2_fma(GG[i], f2_pack(xw[1 + i + 2 * op], xw[2 + i + 2 * op]), DM[oy][op]);
      }
    }
    __syncthreads();  // every thread is done with this stage before it is reloaded
  }  // tiles
  // band pixels, second part: their mask-gradient terms
  for (int64_t k = k0 + threadIdx.x; k < k1; k += C5_T) {
    const int b = (int)(k / band_per);
    int jy, jx;
    band_pos((int)(k - (int64_t)b * band_per), W, H, C5_MR, jy, jx);
    const float *g = p.dy1 + (int64_t)b * p.ib;
    const float *x = p.x + (int64_t)b * p.xb;
    // x through the boundary (CONSTANT taps outside carry none)
    const float gj = g[(int64_t)jy * p.ip + jx];
    const f2 GJ = f2_pack(gj, gj);
    int rx[2 * 4];
#pragma unroll
    for (int o = 0; o < 8; ++o) rx[o] = o < C5_MK ? remap_c5(bm, jx + o - C5_MR, W) : C5_OUT;
#pragma unroll
    for (int oy = 0; oy < C5_MK; ++oy) {
      const int ry = remap_c5(bm, jy + oy - C5_MR, H);
#pragma unroll
      for (int op = 0; op < 4; ++op) {
        const float x0 =
            (ry == C5_OUT || rx[2 * op] == C5_OUT) ? 0.0f : __ldg(x + (int64_t)ry * p.xp + rx[2 * op]);
        const float x1 =
            (ry == C5_OUT || rx[2 * op + 1] == C5_OUT) ? 0.0f : __ldg(x + (int64_t)ry * p.xp + rx[2 * op + 1]);
        DM[oy][op] = f2_fma(GJ, f2_pack(x0, x1), DM[oy][op]);
      }
    }
  }
  // block partials of dL/dmask (49 values), FP64 combine by the last block
#pragma unroll
  for (int oy = 0; oy < C5_MK; ++oy)
#pragma unroll
    for (int ox = 0; ox < C5_MK; ++ox) {
      float v = (ox & 1) ? f2_hi(DM[oy][ox >> 1]) : f2_lo(DM[oy][ox >> 1]);
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][oy * C5_MK + ox] = v;
    }
  __syncthreads();
  const unsigned int nb = grid_blocks();
  if (threadIdx.x < C5_MK * C5_MK) {
    float sum = 0.0f;
    for (int wv = 0; wv < C5_T / 32; ++wv) sum += red[wv][threadIdx.x];
    p.dm_part[(size_t)block_rank() * C5_MK * C5_MK + threadIdx.x] = sum;
    __threadfence();
  }
  if (take_last_ticket(p.tickets + 2)) {
    // a warp per tap: lanes fold the partials i = lane, lane + 32, ... in
    // order, then a fixed shuffle tree (the same sum on every run)
    const int wv = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int o = wv; o < C5_MK * C5_MK; o += C5_T / 32) {
      double sum = 0.0;
      for (int i = lane; i < (int)nb; i += 32) sum += (double)__ldcg(p.dm_part + (size_t)i * C5_MK * C5_MK + o);
#pragma unroll
      for (int d = 16; d > 0; d >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, d);
      if (lane == 0) p.grad_mask_dev[o] = (float)sum;
    }
    if (threadIdx.x == 0) p.tickets[2] = 0u;
  }
}

// ================================================================== unfused form

// bilateral forward of one image from y1 (computed by hgb_local_op): writes y
// and W (into a); the loss gradient follows in its own pass
__global__ void __launch_bounds__(C5_T) c5u_forward_kernel(const __grid_constant__ C5Params p) {
  __shared__ float ys[UY_W * UY_H];
  const int W = p.w, H = p.h, bm = p.bmode;
  float c, k2;
  sigma_consts(p, c, k2);
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
    int b, X0, Y0;
    tile_origin<U_TW, U_TH>(p, tile, b, X0, Y0);
    const float *y1 = p.y1 + (int64_t)b * p.ib;
    __syncthreads();  // the previous tile's reads of ys are done
    for (int cc = threadIdx.x; cc < UY_W * UY_H; cc += C5_T) {
      const int r = cc / UY_W, k = cc - r * UY_W;
      const int ry = remap_c5(bm, Y0 - C5_BR + r, H), rx = remap_c5(bm, X0 - C5_BR + k, W);
      ys[cc] = (ry == C5_OUT || rx == C5_OUT) ? 0.0f : __ldg(y1 + (int64_t)ry * p.ip + rx);
    }
    __syncthreads();
    const int tx = threadIdx.x % U_TW, ty = threadIdx.x / U_TW;
    for (int py = ty; py < U_TH; py += C5_T / U_TW) {
      const int gx = X0 + tx, gy = Y0 + py;
      if (gx >= W || gy >= H) continue;
      const float ctr = ys[(py + C5_BR) * UY_W + tx + C5_BR];
      float N = 0.0f, Wt = 0.0f;
#pragma unroll 3
      for (int oy = 0; oy < C5_BK; ++oy)
#pragma unroll
        for (int ox = 0; ox < C5_BK; ++ox) {
          const float v = ys[(py + oy) * UY_W + tx + ox];
          const float d = v - ctr;
          const float wt = ex2f(__fmaf_rn(k2 * d, d, p.lsm[oy * C5_BK + ox]));
          N = __fmaf_rn(wt, v, N);
          Wt += wt;
        }
      const int64_t o = (int64_t)b * p.ib + (int64_t)gy * p.ip + gx;
      p.y[o] = N / Wt;
      p.a[o] = Wt;
    }
  }
}

// a = 2 (y - t) / (n W) and the loss partials, one image
__global__ void __launch_bounds__(C5_T) c5_alpha_kernel(const __grid_constant__ C5Params p) {
  const int b = blockIdx.z + p.img_offset;
  const int gx = blockIdx.x * U_TW + threadIdx.x % U_TW;
  Kahan lsum{0.0f, 0.0f};
  for (int py = threadIdx.x / U_TW; py < U_TH; py += C5_T / U_TW) {
    const int gy = blockIdx.y * U_TH + py;
    if (gx >= p.w || gy >= p.h) continue;
    const int64_t o = (int64_t)b * p.ib + (int64_t)gy * p.ip + gx;
    const float e = p.y[o] - __ldg(p.t + (int64_t)b * p.tb + (int64_t)gy * p.tp + gx);
    lsum = kahan_add(lsum, e * e);
    p.a[o] = (float)(2.0 * (double)e * p.inv_n) / p.a[o];
  }
  __shared__ float sbuf[32];
  const float v = block_sum_f(lsum.s - lsum.c, sbuf);
  if (threadIdx.x == 0) p.loss_part[block_rank() + (unsigned)p.img_offset * grid_blocks()] = make_float2(v, 0.0f);
}

// bilateral adjoint of one image, every pixel through the pre-images (no
// weight reuse between the centre and the neighbour terms)
__global__ void __launch_bounds__(C5_T) c5u_bilateral_adjoint_kernel(const __grid_constant__ C5Params p) {
  __shared__ float y1s[UY_W * UY_H], as[UY_W * UY_H], yss[UY_W * UY_H];
  __shared__ float sbuf[32];
  const int W = p.w, H = p.h, bm = p.bmode;
  float c, k2;
  sigma_consts(p, c, k2);
  const float c2 = 2.0f * c;
  float dc = 0.0f;
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
    int b, X0, Y0;
    tile_origin<U_TW, U_TH>(p, tile, b, X0, Y0);
    const int64_t base = (int64_t)b * p.ib;
    __syncthreads();  // the previous tile's reads are done
    // in-image cells of [X0-4, X0+TW+4) x [Y0-4, Y0+TH+4); others are never read
    for (int cc = threadIdx.x; cc < UY_W * UY_H; cc += C5_T) {
      const int r = cc / UY_W, k = cc - r * UY_W;
      const int gy = Y0 - C5_BR + r, gx = X0 - C5_BR + k;
      if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
        const int64_t o = base + (int64_t)gy * p.ip + gx;
        y1s[cc] = p.y1[o];
        as[cc] = p.a[o];
        yss[cc] = p.y[o];
      }
    }
    __syncthreads();
    auto S = [&](int gy, int gx) { return (gy - Y0 + C5_BR) * UY_W + gx - X0 + C5_BR; };
    const int tx = threadIdx.x % U_TW, ty = threadIdx.x / U_TW;
    for (int py = ty; py < U_TH; py += C5_T / U_TW) {
      const int jx = X0 + tx, jy = Y0 + py;
      if (jx >= W || jy >= H) continue;
      const int sj = S(jy, jx);
      const float y1j = y1s[sj], aj = as[sj], yj = yss[sj];
      float ctr = 0.0f;
      // centre term and dL/dc over j's own taps
      for (int oy = 0; oy < C5_BK; ++oy)
        for (int ox = 0; ox < C5_BK; ++ox) {
          const int qy = remap_c5(bm, jy + oy - C5_BR, H), qx = remap_c5(bm, jx + ox - C5_BR, W);
          const float v = (qy == C5_OUT || qx == C5_OUT) ? 0.0f : y1s[S(qy, qx)];
          const float d = v - y1j;
          const float e = ex2f(__fmaf_rn(k2 * d, d, p.lsm[oy * C5_BK + ox]));
          const float u = e * (v - yj);
          ctr = __fmaf_rn(u, c2 * d, ctr);
          dc = __fmaf_rn(aj * u, -(d * d), dc);
        }
      // neighbour term gathered over the pre-images of j
      int prx[1 + C5_BR], pry[1 + C5_BR];
      const int nx = preimages(bm, jx, W, C5_BR, prx), ny = preimages(bm, jy, H, C5_BR, pry);
      float dn = 0.0f;
      for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix)
          for (int oy = 0; oy < C5_BK; ++oy)
            for (int ox = 0; ox < C5_BK; ++ox) {
              const int qy = pry[iy] - (oy - C5_BR), qx = prx[ix] - (ox - C5_BR);
              if (qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
              const int sp = S(qy, qx);
              const float d = y1j - y1s[sp];
              const float e = ex2f(__fmaf_rn(k2 * d, d, p.lsm[oy * C5_BK + ox]));
              dn = __fmaf_rn(as[sp] * e, 1.0f - c2 * (y1j - yss[sp]) * d, dn);
            }
      p.dy1[base + (int64_t)jy * p.ip + jx] = __fmaf_rn(aj, ctr, dn);
    }
  }  // tiles
  const float bdc = block_sum_f(dc, sbuf);
  if (threadIdx.x == 0) p.dc_part[block_rank() + (unsigned)p.img_offset * grid_blocks()] = bdc;
}

// convolution adjoint of one image (grad_in only), every pixel through the
// pre-images
__global__ void __launch_bounds__(C5_T) c5u_conv_adjoint_kernel(const __grid_constant__ C5Params p) {
  __shared__ float sd[UD_W * UD_H];
  __shared__ float msk[C5_MK * C5_MK];
  const int W = p.w, H = p.h, bm = p.bmode;
  for (int i = threadIdx.x; i < C5_MK * C5_MK; i += C5_T) msk[i] = __ldg(p.mask_dev + i);
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
    int b, X0, Y0;
    tile_origin<U_TW, U_TH>(p, tile, b, X0, Y0);
    const int64_t base = (int64_t)b * p.ib;
    __syncthreads();  // the previous tile's reads are done
    for (int cc = threadIdx.x; cc < UD_W * UD_H; cc += C5_T) {
      const int r = cc / UD_W, k = cc - r * UD_W;
      const int gy = Y0 - C5_MR + r, gx = X0 - C5_MR + k;
      sd[cc] = (gx >= 0 && gx < W && gy >= 0 && gy < H) ? p.dy1[base + (int64_t)gy * p.ip + gx] : 0.0f;
    }
    __syncthreads();
    const int tx = threadIdx.x % U_TW, ty = threadIdx.x / U_TW;
    for (int py = ty; py < U_TH; py += C5_T / U_TW) {
      const int ix = X0 + tx, iy = Y0 + py;
      if (ix >= W || iy >= H) continue;
      int prx[1 + C5_MR], pry[1 + C5_MR];
      const int nx = preimages(bm, ix, W, C5_MR, prx), ny = preimages(bm, iy, H, C5_MR, pry);
      float acc = 0.0f;
      for (int aa = 0; aa < ny; ++aa)
        for (int cx = 0; cx < nx; ++cx)
          for (int oy = 0; oy < C5_MK; ++oy)
            for (int ox = 0; ox < C5_MK; ++ox) {
              const int jy = pry[aa] - (oy - C5_MR), jx = prx[cx] - (ox - C5_MR);
              if (jx < 0 || jx >= W || jy < 0 || jy >= H) continue;
              acc = __fmaf_rn(msk[oy * C5_MK + ox], sd[(jy - Y0 + C5_MR) * UD_W + jx - X0 + C5_MR], acc);
            }
      p.dx[(int64_t)b * p.dxb + (int64_t)iy * p.dxp + ix] = acc;
    }
  }
}

// the mask gradient as its own pass over one image
__global__ void __launch_bounds__(C5_T) c5_dmask_kernel(const __grid_constant__ C5Params p) {
  const int b = blockIdx.z + p.img_offset;
  const int o = blockIdx.x;  // one mask tap per block row of the grid
  const int oy = o / C5_MK, ox = o % C5_MK;
  const int64_t base = (int64_t)b * p.ib;
  const float *x = p.x + (int64_t)b * p.xb;
  float s = 0.0f;
  for (int64_t i = (int64_t)blockIdx.y * C5_T + threadIdx.x; i < (int64_t)p.w * p.h; i += (int64_t)gridDim.y * C5_T) {
    const int jx = (int)(i % p.w), jy = (int)(i / p.w);
    const int ry = remap_c5(p.bmode, jy + oy - C5_MR, p.h), rx = remap_c5(p.bmode, jx + ox - C5_MR, p.w);
    if (ry == C5_OUT || rx == C5_OUT) continue;
    s = __fmaf_rn(p.dy1[base + (int64_t)jy * p.ip + jx], __ldg(x + (int64_t)ry * p.xp + rx), s);
  }
  __shared__ float sbuf[32];
  const float v = block_sum_f(s, sbuf);
  if (threadIdx.x == 0) p.dm_part[((size_t)p.img_offset * gridDim.y + blockIdx.y) * C5_MK * C5_MK + o] = v;
}

// final FP64 combines of the per-image partials (one CTA, fixed order)
__global__ void __launch_bounds__(C5_T) c5_combine_kernel(const __grid_constant__ C5Params p, int loss_parts,
                                                          int dc_parts, int dm_parts) {
  __shared__ double dsh[C5_T];
  for (int o = 0; o < C5_MK * C5_MK; ++o) {
    const double s =
        block_sum_fixed(dm_parts, [&](int k) { return (double)p.dm_part[(size_t)k * C5_MK * C5_MK + o]; }, dsh);
    if (threadIdx.x == 0) p.grad_mask_dev[o] = (float)s;
  }
  const double l = block_sum_fixed(loss_parts, [&](int k) { return (double)p.loss_part[k].x; }, dsh);
  const double dc = block_sum_fixed(dc_parts, [&](int k) { return (double)p.dc_part[k]; }, dsh);
  if (threadIdx.x == 0) {
    *p.loss_dev = l * p.inv_n;
    const double sg = (double)p.sigma_dev[0];
    *p.grad_sigma_dev = (float)(dc * (-1.0 / (sg * sg * sg)));
  }
}

}  // namespace
}  // namespace hgb

using namespace hgb;

extern "C" int hgb_conv_bilateral_mse(const hgb_view *x, const hgb_view *t, const float *mask_dev, int mask_k,
                                      const float *smask, int smask_k, const float *sigma_dev, int boundary, int mode,
                                      double *loss_dev, const hgb_view *grad_x, float *grad_mask_dev,
                                      float *grad_sigma_dev, void *stream) {
  int rc = check_view(x, "x");
  if (rc) return rc;
  rc = check_view(t, "t");
  if (rc) return rc;
  rc = check_view(grad_x, "grad_x");
  if (rc) return rc;
  HGB_REQUIRE(x->dtype == HGB_F32 && t->dtype == HGB_F32 && grad_x->dtype == HGB_F32,
              "hgb_conv_bilateral_mse: f32 images expected");
  HGB_REQUIRE(t->width == x->width && t->height == x->height && t->batch == x->batch && grad_x->width == x->width &&
                  grad_x->height == x->height && grad_x->batch == x->batch,
              "hgb_conv_bilateral_mse: size mismatch");
  HGB_REQUIRE(mask_k == C5_MK && smask_k == C5_BK, "hgb_conv_bilateral_mse: built for a 7x7 mask and a 9x9 bilateral");
  HGB_REQUIRE(mask_dev && smask && sigma_dev && loss_dev && grad_mask_dev && grad_sigma_dev,
              "hgb_conv_bilateral_mse: null argument");
  HGB_REQUIRE(boundary == HGB_BOUNDARY_CLAMP || boundary == HGB_BOUNDARY_MIRROR || boundary == HGB_BOUNDARY_CONSTANT,
              "hgb_conv_bilateral_mse: boundary must be CLAMP, MIRROR or CONSTANT");
  HGB_REQUIRE(x->width >= 8 && x->height >= 8, "hgb_conv_bilateral_mse: images must be at least 8 x 8");
  HGB_REQUIRE(mode == 0 || mode == 1, "hgb_conv_bilateral_mse: mode must be 0 (fused) or 1 (unfused)");
  HGB_REQUIRE(x->pitch % 4 == 0 && t->pitch % 4 == 0 && grad_x->pitch % 4 == 0, "hgb_conv_bilateral_mse: pitches");
  for (int i = 0; i < C5_BK; ++i)
    for (int j = 0; j < C5_BK; ++j) {
      HGB_REQUIRE(smask[i * C5_BK + j] >= 0.0f, "hgb_conv_bilateral_mse: spatial weights must be non-negative");
      HGB_REQUIRE(smask[i * C5_BK + j] == smask[(C5_BK - 1 - i) * C5_BK + (C5_BK - 1 - j)],
                  "hgb_conv_bilateral_mse: spatial weights must be point-symmetric");
    }
  const int W = x->width, H = x->height, B = x->batch;
  const int64_t ip = (W + 3) / 4 * 4, ib = ip * H;  // intermediates, elements
  const dim3 ugrid(cdiv(W, U_TW), cdiv(H, U_TH), B);
  const size_t nblk = (size_t)ugrid.x * ugrid.y * B;  // at least the CTAs of any launch below
  const int red_rows = 64;  // row blocks of the unfused mask-gradient pass
  const size_t nparts = std::max(nblk, (size_t)B * red_rows);
  // workspace: the fused form's packed float4 per pixel (or the unfused
  // form's y1, y, a), then dy1, then the partials
  const size_t img_bytes = (size_t)ib * B * 4;
  const size_t part_bytes = nparts * (8 + 4 + 4 * C5_MK * C5_MK) + 1024;
  Workspace ws;
  rc = workspace_get(5 * img_bytes + part_bytes, &ws);
  if (rc) return rc;
  C5Params p;
  memset(&p, 0, sizeof(p));
  p.x = (const float *)x->data;
  p.t = (const float *)t->data;
  p.xp = x->pitch / 4;
  p.tp = t->pitch / 4;
  p.xb = x->batch_stride / 4;
  p.tb = t->batch_stride / 4;
  char *wsb = (char *)ws.base;
  p.pk = (float4 *)wsb;
  p.y1 = (float *)wsb;
  p.y = (float *)(wsb + img_bytes);
  p.a = (float *)(wsb + 2 * img_bytes);
  p.dy1 = (float *)(wsb + 4 * img_bytes);
  char *parts = wsb + 5 * img_bytes;
  p.loss_part = (float2 *)parts;
  p.dc_part = (float *)(parts + nparts * 8);
  p.dm_part = (float *)(parts + nparts * 12);
  p.ip = ip;
  p.ib = ib;
  p.dx = (float *)grad_x->data;
  p.dxp = grad_x->pitch / 4;
  p.dxb = grad_x->batch_stride / 4;
  p.w = W;
  p.h = H;
  p.batch = B;
  p.bmode = boundary;
  p.vec_x = ((uintptr_t)x->data % 16 == 0 && x->pitch % 16 == 0 && x->batch_stride % 16 == 0) ? 1 : 0;
  p.vec_dx = ((uintptr_t)grad_x->data % 16 == 0 && grad_x->pitch % 16 == 0 && grad_x->batch_stride % 16 == 0) ? 1 : 0;
  p.mask_dev = mask_dev;
  p.sigma_dev = sigma_dev;
  for (int i = 0; i < C5_BK * C5_BK; ++i)
    p.lsm[i] = smask[i] > 0.0f ? (float)std::log2((double)smask[i]) : -INFINITY;
  p.inv_n = 1.0 / ((double)B * W * H);
  p.tickets = ws.tickets + 8;
  p.loss_dev = loss_dev;
  p.grad_mask_dev = grad_mask_dev;
  p.grad_sigma_dev = grad_sigma_dev;
  if (mode == 0 && tma_legal(x->data, x->pitch, x->batch_stride, B) &&
      make_tensor_map_3d(&p.map_xf, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, x->data, W, H, B, x->pitch, x->batch_stride,
                         FX_W, FX_H) == HGB_OK &&
      make_tensor_map_3d(&p.map_xc, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, x->data, W, H, B, x->pitch, x->batch_stride,
                         FC_W, FC_H) == HGB_OK &&
      make_tensor_map_3d(&p.map_g, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, p.dy1, W, H, B, ip * 4, ib * 4, FC_W, FC_H) ==
          HGB_OK) {
    p.use_tma = 1;
    p.status = device_status_word();
  }
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t ev = before_launch(st);
  if (mode == 0) {
    // persistent grids: one wave of resident CTAs walking the tiles
    p.tiles_x = cdiv(W, F_TW);
    p.tiles_y = cdiv(H, F_TH);
    p.ntiles = p.tiles_x * p.tiles_y * B;
    auto wave = [&](const void *k) { return std::max(1, std::min(p.ntiles, num_sms() * resident_ctas(k, C5_T, 0))); };
    c5_forward_kernel<<<wave((const void *)c5_forward_kernel), C5_T, 0, st>>>(p);
    c5_bilateral_adjoint_kernel<<<wave((const void *)c5_bilateral_adjoint_kernel), C5_T, 0, st>>>(p);
    c5_conv_adjoint_kernel<<<wave((const void *)c5_conv_adjoint_kernel), C5_T, 0, st>>>(p);
    return after_launch("c5 fused", st, ev);
  }
  // unfused chain, one image at a time
  p.tiles_x = (int)ugrid.x;
  p.tiles_y = (int)ugrid.y;
  const dim3 g1(ugrid.x, ugrid.y, 1);
  const int per_image = (int)(ugrid.x * ugrid.y);
  auto wave = [&](const void *k) { return std::max(1, std::min(per_image, num_sms() * resident_ctas(k, C5_T, 0))); };
  const int g_bil = wave((const void *)c5u_bilateral_adjoint_kernel);
  for (int b = 0; b < B; ++b) {
    hgb_view xv{(void *)(p.x + (int64_t)b * p.xb), HGB_F32, W, H, 1, x->pitch, x->pitch * H};
    hgb_view yv{p.y1 + (int64_t)b * ib, HGB_F32, W, H, 1, ip * 4, ib * 4};
    rc = hgb_local_op(&xv, nullptr, &yv, nullptr, nullptr, mask_dev, nullptr, C5_MK, C5_MK, HGB_REDUCE_SUM, boundary,
                      0.0f, stream);
    if (rc) return rc;
    C5Params q = p;
    q.img_offset = b;
    q.ntiles = per_image;
    c5u_forward_kernel<<<wave((const void *)c5u_forward_kernel), C5_T, 0, st>>>(q);
    c5_alpha_kernel<<<g1, C5_T, 0, st>>>(q);
    c5u_bilateral_adjoint_kernel<<<g_bil, C5_T, 0, st>>>(q);
    c5u_conv_adjoint_kernel<<<wave((const void *)c5u_conv_adjoint_kernel), C5_T, 0, st>>>(q);
    c5_dmask_kernel<<<dim3(C5_MK * C5_MK, red_rows, 1), C5_T, 0, st>>>(q);
  }
  c5_combine_kernel<<<1, C5_T, 0, st>>>(p, (int)nblk, B * g_bil, B * red_rows);
  return after_launch("c5 unfused", st, ev);
}

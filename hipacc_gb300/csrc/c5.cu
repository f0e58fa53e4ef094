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
// bilateral weights are recomputed in the adjoint, never stored.  Inside the
// image the spatial mask's symmetry makes one exponential serve both the
// neighbour term (weight of tap o at p = j - o) and the centre term (tap -o
// at j).  Reductions (loss, dL/dc, dL/dmask) use per-block partials combined
// in FP64 in block order by the block that takes the last ticket.
//
// Launch forms: mode 0 = three batched kernels (forward with the conv
// recomputed on its halo and the loss gradient in the epilogue, bilateral
// adjoint, conv adjoint with the mask gradient); mode 1 = the unfused chain
// per image (conv, bilateral forward, loss gradient, bilateral adjoint without
// the symmetry reuse, conv adjoint, mask gradient) for comparison.
// Boundary CLAMP, MIRROR or CONSTANT(0); images at least 8 x 8.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "reduce_common.cuh"

namespace hgb {
namespace {

constexpr int C5_TW = 32, C5_TH = 16, C5_T = 256;
constexpr int C5_MK = 7, C5_MR = 3;  // conv mask
constexpr int C5_BK = 9, C5_BR = 4;  // bilateral
// staged regions
constexpr int XS_W = C5_TW + 2 * (C5_MR + C5_BR), XS_H = C5_TH + 2 * (C5_MR + C5_BR);  // x for the fused forward
constexpr int YS_W = C5_TW + 2 * C5_BR, YS_H = C5_TH + 2 * C5_BR;                      // y1 / a / y (radius 4)
constexpr int DS_W = C5_TW + 2 * C5_MR, DS_H = C5_TH + 2 * C5_MR;                      // dy1 / x (radius 3)

struct C5Params {
  const float *x, *t;
  int64_t xp, tp, xb, tb;  // pitches / batch strides in floats
  float *y1, *y, *a, *dy1, *dx;
  int64_t ip, ib;          // pitch / batch stride of the intermediates and dx (floats)
  int64_t dxp, dxb;
  int w, h, batch;
  int bmode;
  const float *mask_dev;   // 49
  const float *sigma_dev;  // 1
  float lsm[C5_BK * C5_BK];  // log2(smask)
  float sm[C5_BK * C5_BK];
  double inv_n;            // 1 / (batch * w * h)
  float2 *loss_part;       // per block Kahan (s, c)
  float *dc_part;          // per block
  float *dm_part;          // per block x 49
  unsigned int *tickets;   // [0] forward, [1] bilateral adjoint, [2] conv adjoint
  double *loss_dev;
  float *grad_mask_dev, *grad_sigma_dev;
  int fuse_conv;           // forward computes y1 from x (else reads y1)
  int fuse_loss;           // forward writes a (else writes y and W into a)
  int symmetric;           // bilateral adjoint reuses weights
  int fuse_dmask;          // conv adjoint accumulates dL/dmask
  int img_offset;          // image of the launch (per-image launches; 0 otherwise)
  int tiles_x, tiles_y, ntiles;  // tile grid of the launch (all images, or one image)
  int combine;             // the launch covers the batch: its last CTA publishes the sums
};

// tile t of the launch: image, origin
__device__ __forceinline__ void tile_origin(const C5Params &p, int t, int &b, int &X0, int &Y0) {
  const int per = p.tiles_x * p.tiles_y;
  const int bz = t / per, r = t - bz * per;
  const int by = r / p.tiles_x;
  b = bz + p.img_offset;
  X0 = (r - by * p.tiles_x) * C5_TW;
  Y0 = by * C5_TH;
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

// block-wide sum of a float (all threads get nothing; thread 0 returns the value)
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

// ------------------------------------------------------------------ forward
__global__ void __launch_bounds__(C5_T) c5_forward_kernel(const __grid_constant__ C5Params p) {
  __shared__ float xs[XS_W * XS_H];
  __shared__ float ys[YS_W * YS_H];
  __shared__ float msk[C5_MK * C5_MK];
  __shared__ double dsh[C5_T];
  const int W = p.w, H = p.h, bm = p.bmode;
  for (int i = threadIdx.x; i < C5_MK * C5_MK; i += C5_T) msk[i] = __ldg(p.mask_dev + i);
  float c, k2;
  sigma_consts(p, c, k2);
  Kahan lsum{0.0f, 0.0f};
  // persistent: the CTA walks tiles blockIdx.x, blockIdx.x + gridDim.x, ...
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
  int b, X0, Y0;
  tile_origin(p, tile, b, X0, Y0);
  const float *x = p.x + (int64_t)b * p.xb;
  __syncthreads();  // the previous tile's reads of xs / ys are done
  if (p.fuse_conv) {
    constexpr int R = C5_MR + C5_BR;
    for (int c = threadIdx.x; c < XS_W * XS_H; c += C5_T) {
      const int r = c / XS_W, q = c - r * XS_W;
      const int ry = remap_c5(bm, Y0 - R + r, H), rx = remap_c5(bm, X0 - R + q, W);
      xs[c] = (ry == (int)0x80000000 || rx == (int)0x80000000) ? 0.0f : __ldg(x + (int64_t)ry * p.xp + rx);
    }
    __syncthreads();
    // y1 on the tile + bilateral halo, four adjacent cells per thread from one
    // row window of the staged x per mask row (taps row-major, as one cell at a
    // time); a halo cell outside the image is y1 at the remapped position (the
    // bilateral reads y1 through the boundary)
    static_assert(YS_W % 4 == 0 && YS_H * (YS_W / 4) <= C5_T, "one group of four cells per thread");
    for (int g = threadIdx.x; g < YS_H * (YS_W / 4); g += C5_T) {
      const int r = g / (YS_W / 4), q4 = (g - r * (YS_W / 4)) * 4;
      const int vy = Y0 - C5_BR + r, vx = X0 - C5_BR + q4;
      if (vy >= 0 && vy < H && vx >= 0 && vx + 3 < W) {
        // staged rows r .. r + 6, columns q4 .. q4 + 9 (R = MR + BR)
        float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int my = 0; my < C5_MK; ++my) {
          float v[4 + C5_MK - 1];
#pragma unroll
          for (int i = 0; i < 4 + C5_MK - 1; ++i) v[i] = xs[(r + my) * XS_W + q4 + i];
#pragma unroll
          for (int mx = 0; mx < C5_MK; ++mx)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[j] = __fmaf_rn(msk[my * C5_MK + mx], v[j + mx], acc[j]);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) ys[r * YS_W + q4 + j] = acc[j];
        continue;
      }
      for (int j = 0; j < 4; ++j) {
        const int ry = remap_c5(bm, vy, H), rx = remap_c5(bm, vx + j, W);
        float acc = 0.0f;
        if (ry != (int)0x80000000 && rx != (int)0x80000000) {
          // staged x coordinate of (ry - 3, rx - 3)
          const int sy = ry - C5_MR - (Y0 - R), sx = rx - C5_MR - (X0 - R);
#pragma unroll
          for (int my = 0; my < C5_MK; ++my)
#pragma unroll
            for (int mx = 0; mx < C5_MK; ++mx)
              acc = __fmaf_rn(msk[my * C5_MK + mx], xs[(sy + my) * XS_W + sx + mx], acc);
        }
        ys[r * YS_W + q4 + j] = acc;
      }
    }
  } else {
    const float *y1 = p.y1 + (int64_t)b * p.ib;
    for (int c = threadIdx.x; c < YS_W * YS_H; c += C5_T) {
      const int r = c / YS_W, q = c - r * YS_W;
      const int ry = remap_c5(bm, Y0 - C5_BR + r, H), rx = remap_c5(bm, X0 - C5_BR + q, W);
      ys[c] = (ry == (int)0x80000000 || rx == (int)0x80000000) ? 0.0f : __ldg(y1 + (int64_t)ry * p.ip + rx);
    }
  }
  __syncthreads();
  const int tx = threadIdx.x % C5_TW, ty = threadIdx.x / C5_TW;
  for (int py = ty; py < C5_TH; py += C5_T / C5_TW) {
    const int gx = X0 + tx, gy = Y0 + py;
    if (gx >= W || gy >= H) continue;
    const float ctr = ys[(py + C5_BR) * YS_W + tx + C5_BR];
    float N = 0.0f, Wt = 0.0f;
#pragma unroll 3
    for (int oy = 0; oy < C5_BK; ++oy)
#pragma unroll
      for (int ox = 0; ox < C5_BK; ++ox) {
        const float v = ys[(py + oy) * YS_W + tx + ox];
        const float d = v - ctr;
        const float wt = ex2f(__fmaf_rn(k2 * d, d, p.lsm[oy * C5_BK + ox]));
        N = __fmaf_rn(wt, v, N);
        Wt += wt;
      }
    const float yv = N / Wt;
    const int64_t o = (int64_t)b * p.ib + (int64_t)gy * p.ip + gx;
    if (p.fuse_conv) p.y1[o] = ctr;
    if (p.fuse_loss) {
      const float tv = __ldg(p.t + (int64_t)b * p.tb + (int64_t)gy * p.tp + gx);
      const float e = yv - tv;
      lsum = kahan_add(lsum, e * e);
      p.a[o] = (float)(2.0 * (double)e * p.inv_n) / Wt;
      p.y[o] = yv;
    } else {
      p.y[o] = yv;
      p.a[o] = Wt;  // the unfused chain keeps W and forms a in its own pass
    }
  }
  }  // tiles
  if (!p.fuse_loss) return;
  // per-CTA Kahan partial of the squared error, FP64 combine by the last CTA
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

// unfused chain: a = 2 (y - t) / (n W) and the loss partials, one image
__global__ void __launch_bounds__(C5_T) c5_alpha_kernel(const __grid_constant__ C5Params p) {
  const int b = blockIdx.z + p.img_offset;
  const int gx = blockIdx.x * C5_TW + threadIdx.x % C5_TW;
  Kahan lsum{0.0f, 0.0f};
  for (int py = threadIdx.x / C5_TW; py < C5_TH; py += C5_T / C5_TW) {
    const int gy = blockIdx.y * C5_TH + py;
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

// ------------------------------------------------------------------ bilateral adjoint
// per-axis pre-images of index j under the remap, among virtual positions
// within `rad` of the image: at most 1 + rad entries
__device__ __forceinline__ int preimages(int mode, int j, int n, int rad, int *out) {
  int k = 0;
  out[k++] = j;
  if (mode == HGB_BOUNDARY_CONSTANT || (j >= rad && j < n - rad)) return k;
  for (int v = -rad; v < 0; ++v)
    if (remap(mode, v, 0, n) == j) out[k++] = v;
  for (int v = n; v < n + rad; ++v)
    if (remap(mode, v, 0, n) == j) out[k++] = v;
  return k;
}

__global__ void __launch_bounds__(C5_T) c5_bilateral_adjoint_kernel(const __grid_constant__ C5Params p) {
  // staged per pixel of the tile + radius: (q y1, a, a q y, q y) with
  // q = sqrt(c log2 e), so that a tap's weight is exp2(lsm - d'^2) for the
  // scaled difference d' = q (y1_j - y1_p)
  __shared__ float4 s4[YS_W * YS_H];
  __shared__ float sbuf[32];
  __shared__ double dsh[C5_T];
  const int W = p.w, H = p.h, bm = p.bmode;
  float c, k2;
  sigma_consts(p, c, k2);
  const float c2 = 2.0f * c;
  const float q = sqrtf(-k2), inv_q = 1.0f / q;
  // 2c (y1_j - y_p)(y1_j - y1_p) = C2S (q y1_j - q y_p) d' with C2S = 2c / q^2 = 2 ln 2
  constexpr float C2S = 1.3862943611198906f;
  const float inv_q3 = inv_q * inv_q * inv_q;
  float dc = 0.0f;
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
  int b, X0, Y0;
  tile_origin(p, tile, b, X0, Y0);
  const int64_t base = (int64_t)b * p.ib;
  __syncthreads();  // the previous tile's reads are done
  // in-image cells of [X0-4, X0+TW+4) x [Y0-4, Y0+TH+4); others are never read
  for (int cc = threadIdx.x; cc < YS_W * YS_H; cc += C5_T) {
    const int r = cc / YS_W, qx = cc - r * YS_W;
    const int gy = Y0 - C5_BR + r, gx = X0 - C5_BR + qx;
    if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
      const int64_t o = base + (int64_t)gy * p.ip + gx;
      const float a = p.a[o], uy = q * p.y[o];
      s4[cc] = make_float4(q * p.y1[o], a, a * uy, uy);
    }
  }
  __syncthreads();
  const int tx = threadIdx.x % C5_TW, ty = threadIdx.x / C5_TW;
  auto S = [&](int gy, int gx) { return s4[(gy - Y0 + C5_BR) * YS_W + gx - X0 + C5_BR]; };
  for (int py = ty; py < C5_TH; py += C5_T / C5_TW) {
    const int jx = X0 + tx, jy = Y0 + py;
    if (jx >= W || jy >= H) continue;
    const int sj = (py + C5_BR) * YS_W + tx + C5_BR;
    const float4 J = s4[sj];
    const float u1j = J.x, aj = J.y, uyj = J.w;
    float dn = 0.0f, s1 = 0.0f, s2 = 0.0f;
    const bool inner = jx >= C5_BR && jx < W - C5_BR && jy >= C5_BR && jy < H - C5_BR;
    if (inner && p.symmetric) {
#pragma unroll 3
      for (int oy = 0; oy < C5_BK; ++oy)
#pragma unroll
        for (int ox = 0; ox < C5_BK; ++ox) {
          // p = j - o; tap o of p reads j, tap -o of j reads p; one weight
          const float4 P = s4[sj - (oy - C5_BR) * YS_W - (ox - C5_BR)];
          const float d = u1j - P.x;
          const float e = ex2f(__fmaf_rn(-d, d, p.lsm[oy * C5_BK + ox]));
          // neighbour term a_p e (1 - 2c (y1_j - y_p) d)
          const float t = __fmaf_rn(u1j, P.y, -P.z);
          dn = __fmaf_rn(e, __fmaf_rn(-C2S * d, t, P.y), dn);
          // j's own tap -o: e (y1_p - y_j) d' into the centre and dL/dc sums
          const float wd = e * (P.x - uyj) * d;
          s1 += wd;
          s2 = __fmaf_rn(wd, d, s2);
        }
      // centre term a_j sum e (y1_p - y_j) 2c (y1_p - y1_j) = -C2S a_j s1;
      // dL/dc over j's taps: -a_j s2 / q^3
      dc = __fmaf_rn(-aj * inv_q3, s2, dc);
      p.dy1[base + (int64_t)jy * p.ip + jx] = __fmaf_rn(-C2S * aj, s1, dn);
      continue;
    }
    const float y1j = u1j * inv_q, yj = uyj * inv_q;
    float ctr = 0.0f;
    // centre term and dL/dc over j's own taps
    for (int oy = 0; oy < C5_BK; ++oy)
      for (int ox = 0; ox < C5_BK; ++ox) {
        const int qy = remap_c5(bm, jy + oy - C5_BR, H), qx = remap_c5(bm, jx + ox - C5_BR, W);
        const float v = (qy == (int)0x80000000 || qx == (int)0x80000000) ? 0.0f : S(qy, qx).x * inv_q;
        const float d = v - y1j;
        const float e = ex2f(__fmaf_rn(k2 * d, d, p.lsm[oy * C5_BK + ox]));
        const float u = e * (v - yj);
        ctr = __fmaf_rn(u, c2 * d, ctr);
        dc = __fmaf_rn(aj * u, -(d * d), dc);
      }
    // neighbour term gathered over the pre-images of j
    int prx[1 + C5_BR], pry[1 + C5_BR];
    const int nx = preimages(bm, jx, W, C5_BR, prx), ny = preimages(bm, jy, H, C5_BR, pry);
    for (int iy = 0; iy < ny; ++iy)
      for (int ix = 0; ix < nx; ++ix)
        for (int oy = 0; oy < C5_BK; ++oy)
          for (int ox = 0; ox < C5_BK; ++ox) {
            const int qy = pry[iy] - (oy - C5_BR), qx = prx[ix] - (ox - C5_BR);
            if (qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
            const float4 P = S(qy, qx);
            const float y1p = P.x * inv_q, ypp = P.w * inv_q;
            const float d = y1j - y1p;
            const float e = ex2f(__fmaf_rn(k2 * d, d, p.lsm[oy * C5_BK + ox]));
            dn = __fmaf_rn(P.y * e, 1.0f - c2 * (y1j - ypp) * d, dn);
          }
    p.dy1[base + (int64_t)jy * p.ip + jx] = __fmaf_rn(aj, ctr, dn);
  }
  }  // tiles
  const float bdc = block_sum_f(dc, sbuf);
  const unsigned int nb = grid_blocks();
  const unsigned int rank = block_rank() + (unsigned)p.img_offset * nb;
  if (threadIdx.x == 0) p.dc_part[rank] = bdc;
  if (p.combine && take_last_ticket(p.tickets + 1)) {
    const double s = block_sum_fixed((int)nb, [&](int i) { return (double)__ldcg(p.dc_part + i); }, dsh);
    if (threadIdx.x == 0) {
      const double sg = (double)__ldg(p.sigma_dev);
      *p.grad_sigma_dev = (float)(s * (-1.0 / (sg * sg * sg)));
      p.tickets[1] = 0u;
    }
  }
}

// ------------------------------------------------------------------ conv adjoint
__global__ void __launch_bounds__(C5_T) c5_conv_adjoint_kernel(const __grid_constant__ C5Params p) {
  __shared__ float sd[DS_W * DS_H], sx[DS_W * DS_H];
  __shared__ float msk[C5_MK * C5_MK];
  __shared__ float red[C5_T / 32][C5_MK * C5_MK];
  __shared__ double dsh[C5_T];
  const int W = p.w, H = p.h, bm = p.bmode;
  for (int i = threadIdx.x; i < C5_MK * C5_MK; i += C5_T) msk[i] = __ldg(p.mask_dev + i);
  float dm[C5_MK * C5_MK];
#pragma unroll
  for (int i = 0; i < C5_MK * C5_MK; ++i) dm[i] = 0.0f;
  for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
  int b, X0, Y0;
  tile_origin(p, tile, b, X0, Y0);
  const int64_t base = (int64_t)b * p.ib;
  const float *x = p.x + (int64_t)b * p.xb;
  __syncthreads();  // the previous tile's reads are done
  for (int c = threadIdx.x; c < DS_W * DS_H; c += C5_T) {
    const int r = c / DS_W, q = c - r * DS_W;
    const int gy = Y0 - C5_MR + r, gx = X0 - C5_MR + q;
    sd[c] = (gx >= 0 && gx < W && gy >= 0 && gy < H) ? p.dy1[base + (int64_t)gy * p.ip + gx] : 0.0f;
    const int ry = remap_c5(bm, gy, H), rx = remap_c5(bm, gx, W);
    sx[c] = (ry == (int)0x80000000 || rx == (int)0x80000000) ? 0.0f : __ldg(x + (int64_t)ry * p.xp + rx);
  }
  __syncthreads();
  auto D = [&](int gy, int gx) { return sd[(gy - Y0 + C5_MR) * DS_W + gx - X0 + C5_MR]; };
  // a thread per pair of horizontally adjacent pixels: each staged row window
  // serves both pixels' taps (taps in the same row-major order per pixel)
  static_assert(C5_TW * C5_TH == 2 * C5_T, "two pixels per thread");
  const int tx2 = threadIdx.x % (C5_TW / 2), py = threadIdx.x / (C5_TW / 2);
  const int ix0 = X0 + 2 * tx2, iy = Y0 + py;
  const bool cst = bm == HGB_BOUNDARY_CONSTANT;
  if (iy < H && ix0 < W) {
    const bool inner2 = ix0 >= C5_MR && ix0 + 1 < W - C5_MR && iy >= C5_MR && iy < H - C5_MR;
    if (inner2) {
      float acc0 = 0.0f, acc1 = 0.0f;
#pragma unroll
      for (int oy = 0; oy < C5_MK; ++oy) {
        // grad_out row iy - (oy - 3), columns ix0 - 3 .. ix0 + 4
        const float *row = &sd[(py + 2 * C5_MR - oy) * DS_W + 2 * tx2];
        float v[2 + C5_MK - 1];
#pragma unroll
        for (int i = 0; i < 2 + C5_MK - 1; ++i) v[i] = row[i];
#pragma unroll
        for (int ox = 0; ox < C5_MK; ++ox) {
          acc0 = __fmaf_rn(msk[oy * C5_MK + ox], v[2 * C5_MR - ox], acc0);
          acc1 = __fmaf_rn(msk[oy * C5_MK + ox], v[2 * C5_MR - ox + 1], acc1);
        }
      }
      float *dx = p.dx + (int64_t)b * p.dxb + (int64_t)iy * p.dxp + ix0;
      dx[0] = acc0;
      dx[1] = acc1;
    } else {
      for (int j = 0; j < 2; ++j) {
        const int ix = ix0 + j;
        if (ix >= W) break;
        float acc = 0.0f;
        int prx[1 + C5_MR], pry[1 + C5_MR];
        const int nx = preimages(bm, ix, W, C5_MR, prx), ny = preimages(bm, iy, H, C5_MR, pry);
        for (int aa = 0; aa < ny; ++aa)
          for (int c = 0; c < nx; ++c)
            for (int oy = 0; oy < C5_MK; ++oy)
              for (int ox = 0; ox < C5_MK; ++ox) {
                const int jy = pry[aa] - (oy - C5_MR), jx = prx[c] - (ox - C5_MR);
                if (jx < 0 || jx >= W || jy < 0 || jy >= H) continue;
                acc = __fmaf_rn(msk[oy * C5_MK + ox], D(jy, jx), acc);
              }
        p.dx[(int64_t)b * p.dxb + (int64_t)iy * p.dxp + ix] = acc;
      }
    }
    if (p.fuse_dmask) {
      const float dj0 = D(iy, ix0), dj1 = ix0 + 1 < W ? D(iy, ix0 + 1) : 0.0f;
      const bool inner_taps = ix0 >= C5_MR && ix0 + 1 < W - C5_MR && iy >= C5_MR && iy < H - C5_MR;
#pragma unroll
      for (int oy = 0; oy < C5_MK; ++oy) {
        // x through the boundary, row iy + oy - 3, columns ix0 - 3 .. ix0 + 4
        const float *row = &sx[(py + oy) * DS_W + 2 * tx2];
        float v[2 + C5_MK - 1];
#pragma unroll
        for (int i = 0; i < 2 + C5_MK - 1; ++i) v[i] = row[i];
        const int vy = iy + oy - C5_MR;
#pragma unroll
        for (int ox = 0; ox < C5_MK; ++ox) {
          float t0 = v[ox], t1 = v[ox + 1];
          if (cst && !inner_taps) {  // CONSTANT taps outside the image carry no gradient
            const int vx = ix0 + ox - C5_MR;
            const bool yo = vy < 0 || vy >= H;
            if (yo || vx < 0 || vx >= W) t0 = 0.0f;
            if (yo || vx + 1 < 0 || vx + 1 >= W) t1 = 0.0f;
          }
          dm[oy * C5_MK + ox] = __fmaf_rn(dj1, t1, __fmaf_rn(dj0, t0, dm[oy * C5_MK + ox]));
        }
      }
    }
  }
  }  // tiles
  if (!p.fuse_dmask) return;
  // block partials of dL/dmask (49 values), FP64 combine by the last block
#pragma unroll
  for (int i = 0; i < C5_MK * C5_MK; ++i) {
    float v = dm[i];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][i] = v;
  }
  __syncthreads();
  const unsigned int nb = grid_blocks();
  const unsigned int rank = block_rank() + (unsigned)p.img_offset * nb;
  if (threadIdx.x < C5_MK * C5_MK) {
    float s = 0.0f;
    for (int wv = 0; wv < C5_T / 32; ++wv) s += red[wv][threadIdx.x];
    p.dm_part[(size_t)rank * C5_MK * C5_MK + threadIdx.x] = s;
    __threadfence();
  }
  if (p.combine && take_last_ticket(p.tickets + 2)) {
    for (int o = 0; o < C5_MK * C5_MK; ++o) {
      const double s = block_sum_fixed(
          (int)nb, [&](int i) { return (double)__ldcg(p.dm_part + (size_t)i * C5_MK * C5_MK + o); }, dsh);
      if (threadIdx.x == 0) p.grad_mask_dev[o] = (float)s;
    }
    if (threadIdx.x == 0) p.tickets[2] = 0u;
  }
}

// unfused chain: the mask gradient as its own pass over one image
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
    if (ry == (int)0x80000000 || rx == (int)0x80000000) continue;
    s = __fmaf_rn(p.dy1[base + (int64_t)jy * p.ip + jx], __ldg(x + (int64_t)ry * p.xp + rx), s);
  }
  __shared__ float sbuf[32];
  const float v = block_sum_f(s, sbuf);
  if (threadIdx.x == 0) p.dm_part[((size_t)p.img_offset * gridDim.y + blockIdx.y) * C5_MK * C5_MK + o] = v;
}

// unfused chain: final FP64 combines of the per-image partials (one CTA,
// fixed order)
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
  const int64_t ip = (W + 3) / 4 * 4, ib = ip * H;  // intermediates, floats
  const dim3 grid(cdiv(W, C5_TW), cdiv(H, C5_TH), B);
  const size_t nblk = (size_t)grid.x * grid.y * B;
  const int red_rows = 64;  // row blocks of the unfused mask-gradient pass
  const size_t nparts = std::max(nblk, (size_t)B * red_rows);
  // workspace: y1, y, a, dy1 images + partials
  const size_t img_bytes = (size_t)ib * B * 4;
  const size_t part_bytes = nparts * (8 + 4 + 4 * C5_MK * C5_MK) + 1024;
  Workspace ws;
  rc = workspace_get(4 * img_bytes + part_bytes, &ws);
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
  p.y1 = (float *)wsb;
  p.y = (float *)(wsb + img_bytes);
  p.a = (float *)(wsb + 2 * img_bytes);
  p.dy1 = (float *)(wsb + 3 * img_bytes);
  char *parts = wsb + 4 * img_bytes;
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
  p.mask_dev = mask_dev;
  p.sigma_dev = sigma_dev;
  for (int i = 0; i < C5_BK * C5_BK; ++i) {
    p.sm[i] = smask[i];
    p.lsm[i] = smask[i] > 0.0f ? (float)std::log2((double)smask[i]) : -INFINITY;
  }
  p.inv_n = 1.0 / ((double)B * W * H);
  p.tickets = ws.tickets + 8;
  p.loss_dev = loss_dev;
  p.grad_mask_dev = grad_mask_dev;
  p.grad_sigma_dev = grad_sigma_dev;
  p.tiles_x = (int)grid.x;
  p.tiles_y = (int)grid.y;
  cudaStream_t st = (cudaStream_t)stream;
  // persistent grids: one wave of resident CTAs walking the tiles
  const int occ[3] = {resident_ctas((const void *)c5_forward_kernel, C5_T, 0),
                      resident_ctas((const void *)c5_bilateral_adjoint_kernel, C5_T, 0),
                      resident_ctas((const void *)c5_conv_adjoint_kernel, C5_T, 0)};
  auto wave = [&](int k, int ntiles) { return std::max(1, std::min(ntiles, num_sms() * occ[k])); };
  cudaEvent_t ev = before_launch(st);
  if (mode == 0) {
    p.fuse_conv = 1;
    p.fuse_loss = 1;
    p.symmetric = 1;
    p.fuse_dmask = 1;
    p.combine = 1;
    p.ntiles = (int)nblk;
    c5_forward_kernel<<<wave(0, p.ntiles), C5_T, 0, st>>>(p);
    c5_bilateral_adjoint_kernel<<<wave(1, p.ntiles), C5_T, 0, st>>>(p);
    c5_conv_adjoint_kernel<<<wave(2, p.ntiles), C5_T, 0, st>>>(p);
    return after_launch("c5 fused", st, ev);
  }
  // unfused chain, one image at a time
  const dim3 g1(grid.x, grid.y, 1);
  const int per_image = (int)(grid.x * grid.y);
  const int g_bil = wave(1, per_image);
  for (int b = 0; b < B; ++b) {
    hgb_view xv{(void *)(p.x + (int64_t)b * p.xb), HGB_F32, W, H, 1, x->pitch, x->pitch * H};
    hgb_view yv{p.y1 + (int64_t)b * ib, HGB_F32, W, H, 1, ip * 4, ib * 4};
    rc = hgb_local_op(&xv, nullptr, &yv, nullptr, nullptr, mask_dev, nullptr, C5_MK, C5_MK, HGB_REDUCE_SUM, boundary,
                      0.0f, stream);
    if (rc) return rc;
    C5Params q = p;
    q.img_offset = b;
    q.fuse_conv = 0;
    q.fuse_loss = 0;
    q.symmetric = 0;
    q.fuse_dmask = 0;
    q.combine = 0;
    q.ntiles = per_image;
    c5_forward_kernel<<<wave(0, per_image), C5_T, 0, st>>>(q);
    c5_alpha_kernel<<<g1, C5_T, 0, st>>>(q);
    c5_bilateral_adjoint_kernel<<<g_bil, C5_T, 0, st>>>(q);
    c5_conv_adjoint_kernel<<<wave(2, per_image), C5_T, 0, st>>>(q);
    c5_dmask_kernel<<<dim3(C5_MK * C5_MK, red_rows, 1), C5_T, 0, st>>>(q);
  }
  c5_combine_kernel<<<1, C5_T, 0, st>>>(p, (int)nblk, B * g_bil, B * red_rows);
  return after_launch("c5 unfused", st, ev);
}

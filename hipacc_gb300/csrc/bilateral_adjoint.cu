// bilateral_adjoint.cu -- hgb_bilateral_adjoint: the adjoint of the bilateral
// filter of samples-public/3_Preprocessing/Bilateral_Filter/src/main.cpp:63-77
// (hgb_bilateral's forward, FP32 storage):
//   y_p = N_p / W_p,  N_p = sum_o w_po v_q,  W_p = sum_o w_po,
//   w_po = smask_o exp(-c (v_q - in_p)^2),  c = 1 / (2 sigma_r^2),
//   v_q = in(r(p + o)) through the boundary remap, or the constant.
// For g = dL/dy it returns dL/din and dL/dsigma_r:
//   a_p = g_p / W_p
//   dL/din_q += a_p w_po (1 - 2c (v_q - y_p)(v_q - in_p))      (tap o of p reads q)
//   dL/din_p += a_p sum_o w_po (v_q - y_p) 2c (v_q - in_p)     (p's own weights)
//   dL/dc     = sum_p a_p sum_o w_po (v_q - y_p) (-(v_q - in_p)^2),  dL/dsigma_r = -dL/dc / sigma_r^3
// Taps that read the constant carry no gradient to any pixel.
//
// Three launches.  The weights are recomputed, never stored:
//  1. bil_stats_kernel: W_p and y_p of every pixel (the forward over a staged
//     tile), written as a_p = g_p / W_p and y_p into the library workspace.
//  2. bil_adjoint_kernel: per pixel j the gather of every (p, o) whose tap
//     reads j.  Inside the image (j at least the radius from every edge) the
//     readers are p = j - o, and with a point-symmetric spatial mask one
//     exponential gives both the weight of tap o at p and of tap -o at j.  Near
//     an edge the boundary is transposed: the virtual positions within the
//     radius that the remap sends to j (CLAMP: all positions beyond the edge,
//     MIRROR: the reflected ones, REPEAT: the wrapped ones) are listed per
//     axis and every real pixel p = v - o is visited.  Per-CTA partials of
//     dL/dc go to the workspace.
//  3. bil_adjoint_combine_kernel: one CTA sums the partials in FP64 in block
//     order (deterministic) and writes dL/dsigma_r.
//
// Point-symmetric masks on images of at least 32 x 32 take the packed form
// instead (the structure of the differentiation kernels): on values scaled by
// q = sqrt(c log2 e), so that a weight is exp2(lsm - d'^2),
//  1. bpk_forward_kernel: the bilateral over 64 x 16 tiles, four pixels per
//     thread, two per packed f32x2 operation; it writes per pixel the float4
//     (u, a, -a u_y, u_y) with u = q in, u_y = q y, a = g / W;
//  2. bpk_adjoint_kernel: persistent CTAs over the tiles; staged rows hold
//     pairs (u_k, u_k+1, a_k, a_k+1) and (B_k, B_k+1), skewed against bank
//     conflicts; one ex2 and ten packed lane operations per tap serve the
//     neighbour term, the centre term and dL/dc; pixels within the radius of
//     an edge take the pre-image path from a flat band list (band.cuh), an
//     equal share per CTA after its tiles;
//  3. the same combine.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "band.cuh"
#include "stage.cuh"

namespace hgb {
namespace {

constexpr int BA_TW = 32, BA_TH = 16, BA_T = 256, BA_MAX = 13;

struct BilAdjParams {
  const float *in, *gout;
  float *gin;
  int64_t in_p, in_b, g_p, g_b, gi_p, gi_b;  // floats
  float *a, *y;                              // workspace: a_p and y_p, dense w x h per image
  double *dc_part;                           // per CTA of the adjoint launch
  float *grad_sigma;
  int w, h, batch;
  int bmode, sym;
  float cval;
  float k2, c2;                              // -c log2(e), 2c
  double sigma;
  float lm[BA_MAX * BA_MAX];                 // log2(smask), -inf for zero cells
  // packed form
  float4 *pk;                                // per pixel (u, a, -a u_y, u_y), dense w x h per image
  float q, inv_q, inv_q3;                    // sqrt(-k2), 1 / q, 1 / q^3
  int vec_in;                                // 16-byte loads of `in` rows are legal
  int tiles_x, tiles_y, ntiles;
};

__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// input at virtual position (vx, vy) through the boundary remap (the constant
// for CONSTANT taps outside the image)
__device__ __forceinline__ float ba_load(const BilAdjParams &p, const float *img, int vx, int vy) {
  const int rx = remap(p.bmode, vx, 0, p.w), ry = remap(p.bmode, vy, 0, p.h);
  if (rx == (int)0x80000000 || ry == (int)0x80000000) return p.cval;
  return __ldg(img + (int64_t)ry * p.in_p + rx);
}

template <int K>
__global__ void __launch_bounds__(BA_T) bil_stats_kernel(const __grid_constant__ BilAdjParams p) {
  constexpr int R = K / 2, SW = BA_TW + 2 * R, SH = BA_TH + 2 * R;
  __shared__ float s_in[SW * SH];
  const int b = blockIdx.z, X0 = blockIdx.x * BA_TW, Y0 = blockIdx.y * BA_TH;
  const float *img = p.in + (int64_t)b * p.in_b;
  for (int c = threadIdx.x; c < SW * SH; c += BA_T) {
    const int r = c / SW, q = c - r * SW;
    s_in[c] = ba_load(p, img, X0 - R + q, Y0 - R + r);
  }
  __syncthreads();
  const int tx = threadIdx.x % BA_TW;
  for (int py = threadIdx.x / BA_TW; py < BA_TH; py += BA_T / BA_TW) {
    const int x = X0 + tx, y = Y0 + py;
    if (x >= p.w || y >= p.h) continue;
    const float ctr = s_in[(py + R) * SW + tx + R];
    float N = 0.0f, W = 0.0f;
#pragma unroll
    for (int oy = 0; oy < K; ++oy)
#pragma unroll
      for (int ox = 0; ox < K; ++ox) {
        const float v = s_in[(py + oy) * SW + tx + ox];
        const float d = v - ctr;
        const float e = ex2_approx(__fmaf_rn(p.k2 * d, d, p.lm[oy * K + ox]));
        N = __fmaf_rn(e, v, N);
        W += e;
      }
    const int64_t o = ((int64_t)b * p.h + y) * p.w + x;
    p.a[o] = __ldg(p.gout + (int64_t)b * p.g_b + (int64_t)y * p.g_p + x) / W;
    p.y[o] = N / W;
  }
}

// per-axis virtual positions v in [-R, n + R) with r(v) == j, j first
template <int R>
__device__ __forceinline__ int ba_preimages(int mode, int j, int n, int *out) {
  int k = 0;
  out[k++] = j;
  if (mode == HGB_BOUNDARY_CONSTANT || (j >= R && j < n - R)) return k;
  for (int v = -R; v < 0; ++v)
    if (remap(mode, v, 0, n) == j && k < 2 * R + 1) out[k++] = v;
  for (int v = n; v < n + R; ++v)
    if (remap(mode, v, 0, n) == j && k < 2 * R + 1) out[k++] = v;
  return k;
}

template <int K>
__global__ void __launch_bounds__(BA_T) bil_adjoint_kernel(const __grid_constant__ BilAdjParams p) {
  constexpr int R = K / 2, SW = BA_TW + 2 * R, SH = BA_TH + 2 * R;
  __shared__ float s_in[SW * SH], s_a[SW * SH], s_y[SW * SH];
  __shared__ double s_dc[BA_T / 32];
  const int b = blockIdx.z, X0 = blockIdx.x * BA_TW, Y0 = blockIdx.y * BA_TH;
  const float *img = p.in + (int64_t)b * p.in_b;
  const float *A = p.a + (int64_t)b * p.w * p.h, *Y = p.y + (int64_t)b * p.w * p.h;
  for (int c = threadIdx.x; c < SW * SH; c += BA_T) {
    const int r = c / SW, q = c - r * SW;
    const int vx = X0 - R + q, vy = Y0 - R + r;
    s_in[c] = ba_load(p, img, vx, vy);
    const bool real = vx >= 0 && vx < p.w && vy >= 0 && vy < p.h;
    s_a[c] = real ? A[(int64_t)vy * p.w + vx] : 0.0f;
    s_y[c] = real ? Y[(int64_t)vy * p.w + vx] : 0.0f;
  }
  __syncthreads();
  const float k2 = p.k2, c2 = p.c2;
  float dc = 0.0f;
  const int tx = threadIdx.x % BA_TW;
  for (int py = threadIdx.x / BA_TW; py < BA_TH; py += BA_T / BA_TW) {
    const int jx = X0 + tx, jy = Y0 + py;
    if (jx >= p.w || jy >= p.h) continue;
    const int sj = (py + R) * SW + tx + R;
    const float inj = s_in[sj], aj = s_a[sj], yj = s_y[sj];
    float dn = 0.0f, ctr = 0.0f;
    const bool inner = jx >= R && jx < p.w - R && jy >= R && jy < p.h - R;
    if (inner && p.sym) {
#pragma unroll
      for (int oy = 0; oy < K; ++oy)
#pragma unroll
        for (int ox = 0; ox < K; ++ox) {
          // p = j - o: tap o of p reads j; tap -o of j reads p; one weight
          const int sp = sj - (oy - R) * SW - (ox - R);
          const float inp = s_in[sp];
          const float d = inj - inp;
          const float e = ex2_approx(__fmaf_rn(k2 * d, d, p.lm[oy * K + ox]));
          dn = __fmaf_rn(s_a[sp] * e, 1.0f - c2 * (inj - s_y[sp]) * d, dn);
          const float u = e * (inp - yj);
          ctr = __fmaf_rn(u, -c2 * d, ctr);
          dc = __fmaf_rn(aj * u, -(d * d), dc);
        }
    } else {
      // j's own weights: the centre term and dL/dc (taps staged through the remap)
      for (int oy = 0; oy < K; ++oy)
        for (int ox = 0; ox < K; ++ox) {
          const float v = s_in[sj + (oy - R) * SW + (ox - R)];
          const float d = v - inj;
          const float e = ex2_approx(__fmaf_rn(k2 * d, d, p.lm[oy * K + ox]));
          const float u = e * (v - yj);
          ctr = __fmaf_rn(u, c2 * d, ctr);
          dc = __fmaf_rn(aj * u, -(d * d), dc);
        }
      // every tap that reads j: virtual positions v with r(v) = j, readers p = v - o
      int prx[2 * R + 1], pry[2 * R + 1];
      const int nx = ba_preimages<R>(p.bmode, jx, p.w, prx), ny = ba_preimages<R>(p.bmode, jy, p.h, pry);
      for (int iy = 0; iy < ny; ++iy)
        for (int ix = 0; ix < nx; ++ix)
          for (int oy = 0; oy < K; ++oy)
            for (int ox = 0; ox < K; ++ox) {
              const int qy = pry[iy] - (oy - R), qx = prx[ix] - (ox - R);
              if (qx < 0 || qx >= p.w || qy < 0 || qy >= p.h) continue;
              const int64_t o = (int64_t)qy * p.w + qx;
              const float inp = __ldg(img + (int64_t)qy * p.in_p + qx);
              const float d = inj - inp;
              const float e = ex2_approx(__fmaf_rn(k2 * d, d, p.lm[oy * K + ox]));
              dn = __fmaf_rn(A[o] * e, 1.0f - c2 * (inj - Y[o]) * d, dn);
            }
    }
    if (p.gin) p.gin[(int64_t)b * p.gi_b + (int64_t)jy * p.gi_p + jx] = __fmaf_rn(aj, ctr, dn);
  }
  // the CTA's partial of dL/dc: warp sums, then the warps in order (FP64)
  double v = (double)dc;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
  if ((threadIdx.x & 31) == 0) s_dc[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < BA_T / 32; ++i) s += s_dc[i];
    p.dc_part[blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z)] = s;
  }
}

// ---------------------------------------------------------------- packed form
constexpr int BP_TW = 64, BP_TH = 16, BP_GX = BP_TW / 4, BP_SW = BP_TW + 16;  // staged in: columns X0-8 ..
constexpr float BP_C2S = 1.3862943611198906f;                                  // 2 ln 2

__device__ __forceinline__ void bp_tile(const BilAdjParams &p, int t, int &b, int &X0, int &Y0) {
  const int per = p.tiles_x * p.tiles_y, bz = t / per, r = t - bz * per, by = r / p.tiles_x;
  b = bz;
  X0 = (r - by * p.tiles_x) * BP_TW;
  Y0 = by * BP_TH;
}

// a mask row of range-weight pairs (-lsm, -lsm), two per 16-byte load
template <int N>
__device__ __forceinline__ void bp_nl_row(const f2 *row, f2 (&o)[N]) {
#pragma unroll
  for (int i = 0; i < N / 2; ++i) {
    const ulonglong2 v = reinterpret_cast<const ulonglong2 *>(row)[i];
    o[2 * i] = v.x;
    o[2 * i + 1] = v.y;
  }
}

template <int K>
__global__ void __launch_bounds__(BA_T) bpk_forward_kernel(const __grid_constant__ BilAdjParams p) {
  constexpr int R = K / 2, SH = BP_TH + 2 * R, NLW = K + 1;
  constexpr int L = (R + 3) / 4 * 4, OFFW = L - R;  // window starts at column 8 - L of a pixel group
  constexpr int NV = (OFFW + 3 + K + 3) / 4;      // 16-byte loads per window row
  __shared__ __align__(16) float tile[SH * BP_SW];
  __shared__ __align__(16) f2 nl2[K * NLW];
  const int b = blockIdx.z, X0 = blockIdx.x * BP_TW, Y0 = blockIdx.y * BP_TH;
  for (int i = threadIdx.x; i < K * NLW; i += BA_T) {
    const int oy = i / NLW, ox = i - oy * NLW;
    const float n = ox < K ? -p.lm[oy * K + ox] : 0.0f;
    nl2[i] = f2_pack(n, n);
  }
  stage_tile<float, BP_SW, SH, BA_T>(tile, reinterpret_cast<const char *>(p.in + (int64_t)b * p.in_b), p.in_p * 4,
                                     X0 - 8, Y0 - R, 0, p.w, 0, p.h, p.bmode, p.cval, p.vec_in);
  __syncthreads();
  for (int c = threadIdx.x; c < SH * BP_SW; c += BA_T) tile[c] *= p.q;
  __syncthreads();
  const int tx = threadIdx.x % BP_GX, ty = threadIdx.x / BP_GX;
  const float4 cv = *reinterpret_cast<const float4 *>(&tile[(ty + R) * BP_SW + 8 + 4 * tx]);
  const f2 C0 = f2_pack(cv.x, cv.y), C1 = f2_pack(cv.z, cv.w);
  f2 Ws0 = 0ull, Ws1 = 0ull, Ns0 = 0ull, Ns1 = 0ull;
#pragma unroll 1
  for (int oy = 0; oy < K; ++oy) {
    const float4 *row = reinterpret_cast<const float4 *>(&tile[(ty + oy) * BP_SW + 4 * tx + 8 - L]);
    float w[NV * 4];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      const float4 t4 = row[v];
      w[4 * v] = t4.x;
      w[4 * v + 1] = t4.y;
      w[4 * v + 2] = t4.z;
      w[4 * v + 3] = t4.w;
    }
    f2 NL[NLW];
    bp_nl_row(&nl2[oy * NLW], NL);
#pragma unroll
    for (int ox = 0; ox < K; ++ox) {
#pragma unroll
      for (int pp = 0; pp < 2; ++pp) {
        const f2 V = f2_pack(w[OFFW + 2 * pp + ox], w[OFFW + 2 * pp + ox + 1]);
        const f2 d = f2_sub(V, pp ? C1 : C0);
        const f2 tt = f2_fma(d, d, NL[ox]);
        const f2 e = f2_pack(ex2_approx(-f2_lo(tt)), ex2_approx(-f2_hi(tt)));
        if (pp) {
          Ws1 = f2_add(Ws1, e);
          Ns1 = f2_fma(e, V, Ns1);
        } else {
          Ws0 = f2_add(Ws0, e);
          Ns0 = f2_fma(e, V, Ns0);
        }
      }
    }
  }
  const int gy = Y0 + ty, gx0 = X0 + 4 * tx;
  if (gy >= p.h) return;
  const float Wv[4] = {f2_lo(Ws0), f2_hi(Ws0), f2_lo(Ws1), f2_hi(Ws1)};
  const float Nv[4] = {f2_lo(Ns0), f2_hi(Ns0), f2_lo(Ns1), f2_hi(Ns1)};
  const float Uv[4] = {cv.x, cv.y, cv.z, cv.w};
  const float *grow = p.gout + (int64_t)b * p.g_b + (int64_t)gy * p.g_p;
  float4 *orow = p.pk + ((int64_t)b * p.h + gy) * p.w;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gx = gx0 + i;
    if (gx >= p.w) break;
    const float uy = Nv[i] / Wv[i];
    const float a = __ldg(grow + gx) / Wv[i];
    orow[gx] = make_float4(Uv[i], a, -a * uy, uy);
  }
}

// one symmetric tap for a pixel pair: centre (U, A = a_j, B = -a_j u_yj),
// neighbour pair (Pu, Pa, PB); s = {sum e a_p, sum e d (u_j a_p - a_p u_yp),
// sum e d a_j (u_p - u_yj), the same times d}, d = u_j - u_p
__device__ __forceinline__ void bpk_tap(f2 Pu, f2 Pa, f2 PB, f2 U, f2 A, f2 B, f2 NL, f2 (&s)[4]) {
  const f2 d = f2_sub(U, Pu);
  const f2 t = f2_fma(d, d, NL);
  const f2 e = f2_pack(ex2_approx(-f2_lo(t)), ex2_approx(-f2_hi(t)));
  const f2 h = f2_mul(e, d);
  s[0] = f2_fma(e, Pa, s[0]);
  s[1] = f2_fma(h, f2_fma(U, Pa, PB), s[1]);
  const f2 wd = f2_mul(h, f2_fma(A, Pu, B));
  s[2] = f2_add(s[2], wd);
  s[3] = f2_fma(wd, d, s[3]);
}

// dL/din of a band pixel j through the pre-images, from the packed values;
// adds j's dL/dc share (times -q^3) to dc
template <int K>
__device__ float bpk_band(const BilAdjParams &p, const float4 *pk, const float *lm, int jy, int jx, float &dc) {
  constexpr int R = K / 2;
  const int W = p.w, H = p.h, bm = p.bmode;
  const float4 J = pk[(int64_t)jy * W + jx];
  const float ucst = p.q * p.cval;
  int rx[K];
#pragma unroll
  for (int o = 0; o < K; ++o) rx[o] = remap(bm, jx + o - R, 0, W);
  float ctr = 0.0f, s2 = 0.0f;
  for (int oy = 0; oy < K; ++oy) {
    const int ry = remap(bm, jy + oy - R, 0, H);
#pragma unroll
    for (int ox = 0; ox < K; ++ox) {
      const float uq = (ry == (int)0x80000000 || rx[ox] == (int)0x80000000) ? ucst : pk[(int64_t)ry * W + rx[ox]].x;
      const float d = uq - J.x;
      const float e = ex2_approx(__fmaf_rn(-d, d, lm[oy * K + ox]));
      const float wd = e * __fmaf_rn(J.y, uq, J.z) * d;
      ctr += wd;
      s2 = __fmaf_rn(wd, d, s2);
    }
  }
  dc = __fmaf_rn(-p.inv_q3, s2, dc);
  int prx[1 + R], pry[1 + R];
  const int nx = preimages(bm, jx, W, R, prx), ny = preimages(bm, jy, H, R, pry);
  float dn = 0.0f;
  for (int iy = 0; iy < ny; ++iy)
    for (int oy = 0; oy < K; ++oy) {
      const int py = pry[iy] - (oy - R);
      if (py < 0 || py >= H) continue;
      const float4 *prow = pk + (int64_t)py * W;
      for (int ix = 0; ix < nx; ++ix)
#pragma unroll
        for (int ox = 0; ox < K; ++ox) {  // the row's loads in flight together
          const int px = prx[ix] - (ox - R);
          if (px < 0 || px >= W) continue;
          const float4 P = prow[px];
          const float d = J.x - P.x;
          const float e = ex2_approx(__fmaf_rn(-d, d, lm[oy * K + ox]));
          dn = __fmaf_rn(e, __fmaf_rn(-BP_C2S * d, __fmaf_rn(J.x, P.y, P.z), P.y), dn);
        }
    }
  return __fmaf_rn(BP_C2S, ctr, dn);
}

template <int K>
struct BpkShape {
  static constexpr int R = K / 2, FW = BP_TW + 2 * R, FH = BP_TH + 2 * R;  // staged positions: columns X0-R ..
  static constexpr int SQW = FW + FW / 8, SBW = FW + FW / 16;               // skewed row strides
  static constexpr size_t smem = (size_t)FH * SQW * 16 + (size_t)FH * SBW * 8 + 128;
};
__device__ __forceinline__ int bp_sk8(int k) { return k + (k >> 3); }
__device__ __forceinline__ int bp_sk16(int k) { return k + (k >> 4); }

template <int K>
__global__ void __launch_bounds__(BA_T) bpk_adjoint_kernel(const __grid_constant__ BilAdjParams p) {
  using S = BpkShape<K>;
  constexpr int R = S::R, FW = S::FW, FH = S::FH, SQW = S::SQW, SBW = S::SBW, NLW = K + 1;
  extern __shared__ __align__(16) uint8_t bpk_dsm[];
  float4 *sq = reinterpret_cast<float4 *>(bpk_dsm);                    // (u_k, u_k+1, a_k, a_k+1)
  f2 *sb = reinterpret_cast<f2 *>(bpk_dsm + (size_t)FH * SQW * 16);  // (B_k, B_k+1)
  __shared__ __align__(16) f2 nl2[K * NLW];
  __shared__ float lm[K * K];
  __shared__ double s_dc[BA_T / 32];
  const int W = p.w, H = p.h;
  for (int i = threadIdx.x; i < K * NLW; i += BA_T) {
    const int oy = i / NLW, ox = i - oy * NLW;
    const float n = ox < K ? -p.lm[oy * K + ox] : 0.0f;
    nl2[i] = f2_pack(n, n);
    if (ox < K) lm[oy * K + ox] = p.lm[oy * K + ox];
  }
  const int tx = threadIdx.x % BP_GX, ty = threadIdx.x / BP_GX;
  float dc = 0.0f;
  for (int t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
    int b, X0, Y0;
    bp_tile(p, t, b, X0, Y0);
    const float4 *pk = p.pk + (int64_t)b * W * H;
    __syncthreads();  // the previous tile's reads are done (and nl2 / lm written)
    // in-image cells of rows Y0-R .., columns X0-R ..: two positions per item
    for (int it = threadIdx.x; it < FH * (FW / 2); it += BA_T) {
      const int r = it / (FW / 2), k = (it - r * (FW / 2)) * 2;
      const int gy = Y0 - R + r, gx = X0 - R + k;
      if (gy < 0 || gy >= H) continue;
      const float4 *src = pk + (int64_t)gy * W;
      const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      const float4 v0 = (gx >= 0 && gx < W) ? src[gx] : z;
      const float4 v1 = (gx + 1 >= 0 && gx + 1 < W) ? src[gx + 1] : z;
      const float4 v2 = (gx + 2 >= 0 && gx + 2 < W) ? src[gx + 2] : z;
      sq[r * SQW + bp_sk8(k)] = make_float4(v0.x, v1.x, v0.y, v1.y);
      sq[r * SQW + bp_sk8(k + 1)] = make_float4(v1.x, v2.x, v1.y, v2.y);
      sb[r * SBW + bp_sk16(k)] = f2_pack(v0.z, v1.z);
      sb[r * SBW + bp_sk16(k + 1)] = f2_pack(v1.z, v2.z);
    }
    __syncthreads();
    const int jx0 = X0 + 4 * tx, jy = Y0 + ty;
    if (jx0 >= band_left(R) && jx0 + 3 < W - R && jy >= R && jy < H - R) {
      // positions 4 tx + s of a row: pair pp's centre at s = R + 2 pp, its
      // neighbours for tap ox at s = 2R + 2 pp - ox
      const int cq = (ty + R) * SQW, cb = (ty + R) * SBW;
      const float4 J0 = sq[cq + bp_sk8(4 * tx + R)], J1 = sq[cq + bp_sk8(4 * tx + R + 2)];
      const f2 U0 = f2_pack(J0.x, J0.y), U1 = f2_pack(J1.x, J1.y);
      const f2 A0 = f2_pack(J0.z, J0.w), A1 = f2_pack(J1.z, J1.w);
      const f2 B0 = sb[cb + bp_sk16(4 * tx + R)], B1 = sb[cb + bp_sk16(4 * tx + R + 2)];
      f2 s0[4] = {0ull, 0ull, 0ull, 0ull}, s1[4] = {0ull, 0ull, 0ull, 0ull};
#pragma unroll 1
      for (int oy = 0; oy < K; ++oy) {
        const int row = ty + 2 * R - oy;
        const float4 *qr = sq + row * SQW;
        const f2 *br = sb + row * SBW;
        f2 NL[NLW];
        bp_nl_row(&nl2[oy * NLW], NL);
#pragma unroll
        for (int s = 0; s <= 2 * R + 2; ++s) {
          const int pos = 4 * tx + s;
          const float4 P = qr[bp_sk8(pos)];
          const f2 Pu = f2_pack(P.x, P.y), Pa = f2_pack(P.z, P.w), PB = br[bp_sk16(pos)];
          if (s <= 2 * R) bpk_tap(Pu, Pa, PB, U0, A0, B0, NL[2 * R - s], s0);
          if (s >= 2) bpk_tap(Pu, Pa, PB, U1, A1, B1, NL[2 * R + 2 - s], s1);
        }
      }
      if (p.gin) {
        float *gi = p.gin + (int64_t)b * p.gi_b + (int64_t)jy * p.gi_p + jx0;
        gi[0] = f2_lo(s0[0]) - BP_C2S * (f2_lo(s0[1]) + f2_lo(s0[2]));
        gi[1] = f2_hi(s0[0]) - BP_C2S * (f2_hi(s0[1]) + f2_hi(s0[2]));
        gi[2] = f2_lo(s1[0]) - BP_C2S * (f2_lo(s1[1]) + f2_lo(s1[2]));
        gi[3] = f2_hi(s1[0]) - BP_C2S * (f2_hi(s1[1]) + f2_hi(s1[2]));
      }
      dc = __fmaf_rn(-p.inv_q3, (f2_lo(s0[3]) + f2_hi(s0[3])) + (f2_lo(s1[3]) + f2_hi(s1[3])), dc);
    }
  }
  // band pixels of every image: an equal contiguous share per CTA
  {
    const int per = band_size(W, H, R);
    int64_t k0, k1;
    cta_share((int64_t)per * p.batch, k0, k1);
    for (int64_t k = k0 + threadIdx.x; k < k1; k += BA_T) {
      const int b = (int)(k / per);
      int jy, jx;
      band_pos((int)(k - (int64_t)b * per), W, H, R, jy, jx);
      const float g = bpk_band<K>(p, p.pk + (int64_t)b * W * H, lm, jy, jx, dc);
      if (p.gin) p.gin[(int64_t)b * p.gi_b + (int64_t)jy * p.gi_p + jx] = g;
    }
  }
  // the CTA's partial of dL/dc (FP64, warps in order)
  double v = (double)dc;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_down_sync(0xffffffffu, v, d);
  if ((threadIdx.x & 31) == 0) s_dc[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sum = 0.0;
    for (int i = 0; i < BA_T / 32; ++i) sum += s_dc[i];
    p.dc_part[blockIdx.x] = sum;
  }
}

__global__ void bil_adjoint_combine_kernel(const __grid_constant__ BilAdjParams p, int nparts);

template <int K>
int launch_bpk(const BilAdjParams &p0, cudaStream_t st) {
  BilAdjParams p = p0;
  const dim3 fgrid(cdiv(p.w, BP_TW), cdiv(p.h, BP_TH), p.batch);
  p.tiles_x = (int)fgrid.x;
  p.tiles_y = (int)fgrid.y;
  p.ntiles = (int)(fgrid.x * fgrid.y * fgrid.z);
  const void *kern = (const void *)bpk_adjoint_kernel<K>;
  const size_t smem = BpkShape<K>::smem;
  int rc = ensure_dynamic_smem(kern, smem);
  if (rc) return rc;
  const int grid = std::max(1, std::min(p.ntiles, num_sms() * resident_ctas(kern, BA_T, smem)));
  cudaEvent_t ev = before_launch(st);
  bpk_forward_kernel<K><<<fgrid, BA_T, 0, st>>>(p);
  bpk_adjoint_kernel<K><<<grid, BA_T, smem, st>>>(p);
  if (p.grad_sigma) bil_adjoint_combine_kernel<<<1, BA_T, 0, st>>>(p, grid);
  return after_launch("bpk_adjoint_kernel", st, ev);
}

// one CTA: the partials in a fixed order (thread t folds t, t + 256, ...; then a
// fixed tree), so the result is the same on every run
__global__ void __launch_bounds__(BA_T) bil_adjoint_combine_kernel(const __grid_constant__ BilAdjParams p, int nparts) {
  __shared__ double sh[BA_T];
  double s = 0.0;
  for (int i = threadIdx.x; i < nparts; i += BA_T) s += p.dc_part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int d = BA_T / 2; d > 0; d >>= 1) {
    if (threadIdx.x < d) sh[threadIdx.x] += sh[threadIdx.x + d];
    __syncthreads();
  }
  if (threadIdx.x == 0) *p.grad_sigma = (float)(sh[0] * (-1.0 / (p.sigma * p.sigma * p.sigma)));
}

template <int K>
int launch_bil_adjoint(const BilAdjParams &p, cudaStream_t st) {
  const dim3 grid(cdiv(p.w, BA_TW), cdiv(p.h, BA_TH), p.batch);
  cudaEvent_t ev = before_launch(st);
  bil_stats_kernel<K><<<grid, BA_T, 0, st>>>(p);
  bil_adjoint_kernel<K><<<grid, BA_T, 0, st>>>(p);
  if (p.grad_sigma) bil_adjoint_combine_kernel<<<1, BA_T, 0, st>>>(p, (int)(grid.x * grid.y * grid.z));
  return after_launch("bil_adjoint_kernel", st, ev);
}

}  // namespace
}  // namespace hgb

using namespace hgb;

extern "C" int hgb_bilateral_adjoint(const hgb_view *in, const hgb_view *grad_out, const float *smask, int size,
                                     float sigma_r, int boundary, float const_val, const hgb_view *grad_in,
                                     float *grad_sigma_dev, void *stream) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  rc = check_view(grad_out, "grad_out");
  if (rc) return rc;
  HGB_REQUIRE(grad_in || grad_sigma_dev, "hgb_bilateral_adjoint: no gradient requested");
  if (grad_in) {
    rc = check_view(grad_in, "grad_in");
    if (rc) return rc;
  }
  HGB_REQUIRE(in->dtype == HGB_F32 && grad_out->dtype == HGB_F32 && (!grad_in || grad_in->dtype == HGB_F32),
              "hgb_bilateral_adjoint: f32 images expected");
  HGB_REQUIRE(grad_out->width == in->width && grad_out->height == in->height && grad_out->batch == in->batch &&
                  (!grad_in || (grad_in->width == in->width && grad_in->height == in->height &&
                                grad_in->batch == in->batch)),
              "hgb_bilateral_adjoint: size mismatch");
  HGB_REQUIRE(!grad_in || (grad_in->data != in->data && grad_in->data != grad_out->data),
              "hgb_bilateral_adjoint: grad_in must not alias the inputs");
  HGB_REQUIRE(in->pitch % 4 == 0 && grad_out->pitch % 4 == 0 && (!grad_in || grad_in->pitch % 4 == 0),
              "hgb_bilateral_adjoint: pitches must be whole floats");
  HGB_REQUIRE(smask, "hgb_bilateral_adjoint: null mask");
  HGB_REQUIRE(size >= 3 && size <= BA_MAX && (size & 1), "hgb_bilateral_adjoint: size must be odd, 3..13");
  HGB_REQUIRE(sigma_r > 0.0f, "hgb_bilateral_adjoint: sigma_r must be positive");
  HGB_REQUIRE(boundary >= 0 && boundary <= 4, "hgb_bilateral_adjoint: bad boundary");
  BilAdjParams p;
  memset(&p, 0, sizeof(p));
  p.in = (const float *)in->data;
  p.gout = (const float *)grad_out->data;
  p.gin = grad_in ? (float *)grad_in->data : nullptr;
  p.in_p = in->pitch / 4;
  p.in_b = in->batch_stride / 4;
  p.g_p = grad_out->pitch / 4;
  p.g_b = grad_out->batch_stride / 4;
  p.gi_p = grad_in ? grad_in->pitch / 4 : 0;
  p.gi_b = grad_in ? grad_in->batch_stride / 4 : 0;
  p.w = in->width;
  p.h = in->height;
  p.batch = in->batch;
  // UNDEFINED reads through CLAMP, as the forward
  p.bmode = boundary == HGB_BOUNDARY_UNDEFINED ? HGB_BOUNDARY_CLAMP : boundary;
  p.cval = const_val;
  const double c = 0.5 / ((double)sigma_r * (double)sigma_r);
  p.k2 = (float)(-c * 1.4426950408889634);
  p.c2 = (float)(2.0 * c);
  p.sigma = sigma_r;
  p.sym = 1;
  for (int i = 0; i < size * size; ++i) {
    HGB_REQUIRE(smask[i] >= 0.0f, "hgb_bilateral_adjoint: spatial weights must be non-negative");
    p.lm[i] = smask[i] > 0.0f ? (float)std::log2((double)smask[i]) : -INFINITY;
    if (smask[i] != smask[size * size - 1 - i]) p.sym = 0;
  }
  p.grad_sigma = grad_sigma_dev;
  const size_t px = (size_t)p.w * p.h * p.batch;
  cudaStream_t st = (cudaStream_t)stream;
  if (p.sym && p.w >= 32 && p.h >= 32) {
    // packed form: the float4 per pixel, then per-CTA partials
    p.q = (float)std::sqrt(c * 1.4426950408889634);
    p.inv_q = 1.0f / p.q;
    p.inv_q3 = p.inv_q * p.inv_q * p.inv_q;
    p.vec_in = ((uintptr_t)in->data % 16 == 0 && in->pitch % 16 == 0 && (in->batch == 1 || in->batch_stride % 16 == 0))
                   ? 1
                   : 0;
    const size_t nparts = (size_t)num_sms() * 32;  // at least the CTAs of the persistent adjoint
    Workspace ws;
    rc = workspace_get(px * 16 + nparts * 8 + 256, &ws);
    if (rc) return rc;
    p.dc_part = (double *)ws.base;
    p.pk = (float4 *)((char *)ws.base + (nparts * 8 + 255) / 256 * 256);
    switch (size) {
      case 3: return launch_bpk<3>(p, st);
      case 5: return launch_bpk<5>(p, st);
      case 7: return launch_bpk<7>(p, st);
      case 9: return launch_bpk<9>(p, st);
      case 11: return launch_bpk<11>(p, st);
      default: return launch_bpk<13>(p, st);
    }
  }
  const size_t nparts = (size_t)cdiv(p.w, BA_TW) * cdiv(p.h, BA_TH) * p.batch;
  Workspace ws;
  rc = workspace_get(px * 8 + nparts * 8 + 256, &ws);
  if (rc) return rc;
  p.dc_part = (double *)ws.base;
  p.a = (float *)((char *)ws.base + (nparts * 8 + 255) / 256 * 256);
  p.y = p.a + px;
  switch (size) {
    case 3: return launch_bil_adjoint<3>(p, st);
    case 5: return launch_bil_adjoint<5>(p, st);
    case 7: return launch_bil_adjoint<7>(p, st);
    case 9: return launch_bil_adjoint<9>(p, st);
    case 11: return launch_bil_adjoint<11>(p, st);
    default: return launch_bil_adjoint<13>(p, st);
  }
}

// point_ops.cu -- point operators: RGBA->gray, binary combinations, storage
// conversion and resampling reads.
//
// Point operators in the reference are generated per kernel with one pixel
// per thread and scalar loads (lib/AST/ASTTranslate.cpp:923, pixels per thread
// from include/hipacc/Device/TargetDescription.h:85-91).  Here every thread
// moves 16 pixels with 16-byte vector loads and stores over a grid sized to
// the SM count; dense images are treated as one long row.
#include <algorithm>

#include "tma.cuh"

namespace hgb {
namespace {

struct RowSpace {
  // iteration over (batch, row, chunk-of-16) work items; dense images fold
  // into a single row per image
  int rows_per_img, row_len, chunks_per_row;
  int64_t nitems;
};

RowSpace make_rows(int w, int h, int batch, bool dense) {
  RowSpace r;
  if (dense) {
    r.rows_per_img = 1;
    r.row_len = w * h;
  } else {
    r.rows_per_img = h;
    r.row_len = w;
  }
  r.chunks_per_row = cdiv(r.row_len, 16);
  r.nitems = (int64_t)batch * r.rows_per_img * r.chunks_per_row;
  return r;
}

int grid_for(int64_t items, int threads) {
  const int64_t need = (items + threads - 1) / threads;
  const int64_t cap = (int64_t)num_sms() * 8;
  return (int)(need < cap ? (need > 0 ? need : 1) : cap);
}

struct GrayParams {
  const uint8_t *in;
  int64_t in_pitch, in_bstride;
  uint8_t *out;
  int64_t out_pitch, out_bstride;
  RowSpace rs;
  int vec;
  uint32_t wpack;  // wr | wg << 8 | wb << 16 when every weight fits a byte
  int wr, wg, wb, shift, use_dp4a;
};

__device__ __forceinline__ uint32_t gray_px(const GrayParams &p, uint32_t rgba) {
  uint32_t v;
  if (p.use_dp4a)
    v = __dp4a(rgba, p.wpack, 0u);
  else
    v = (uint32_t)(p.wr * (int)(rgba & 0xff) + p.wg * (int)((rgba >> 8) & 0xff) + p.wb * (int)((rgba >> 16) & 0xff));
  return (v >> p.shift) & 0xffu;
}

__device__ __forceinline__ void gray_chunk_addr(const GrayParams &p, int64_t it, const uint8_t *&src, uint8_t *&dst,
                                                int &x0) {
  const int chunk = (int)(it % p.rs.chunks_per_row);
  const int64_t row_g = it / p.rs.chunks_per_row;
  const int b = (int)(row_g / p.rs.rows_per_img);
  const int row = (int)(row_g - (int64_t)b * p.rs.rows_per_img);
  src = p.in + (int64_t)b * p.in_bstride + (int64_t)row * p.in_pitch + (int64_t)chunk * 64;
  dst = p.out + (int64_t)b * p.out_bstride + (int64_t)row * p.out_pitch + (int64_t)chunk * 16;
  x0 = chunk * 16;
}

__device__ __forceinline__ uint4 gray_16(const GrayParams &p, uint4 a, uint4 bq, uint4 c, uint4 d) {
  const uint32_t px[16] = {a.x, a.y, a.z, a.w, bq.x, bq.y, bq.z, bq.w, c.x, c.y, c.z, c.w, d.x, d.y, d.z, d.w};
  uint32_t o[4];
#pragma unroll
  for (int q = 0; q < 4; ++q)
    o[q] = gray_px(p, px[4 * q]) | (gray_px(p, px[4 * q + 1]) << 8) | (gray_px(p, px[4 * q + 2]) << 16) |
           (gray_px(p, px[4 * q + 3]) << 24);
  return make_uint4(o[0], o[1], o[2], o[3]);
}

__device__ __forceinline__ void gray_scalar(const GrayParams &p, const uint8_t *src, uint8_t *dst, int x0) {
  for (int q = 0; q < 16 && x0 + q < p.rs.row_len; ++q) {
    const uint8_t *s = src + 4 * q;
    const uint32_t rgba = (uint32_t)s[0] | ((uint32_t)s[1] << 8) | ((uint32_t)s[2] << 16) | ((uint32_t)s[3] << 24);
    dst[q] = (uint8_t)gray_px(p, rgba);
  }
}

// Each CTA owns a contiguous range of 16-pixel chunks; a thread keeps two
// chunks (128 bytes of loads) in flight per iteration.
__global__ void __launch_bounds__(256) gray_kernel(const __grid_constant__ GrayParams p) {
  const int64_t per = (p.rs.nitems + gridDim.x - 1) / gridDim.x;
  const int64_t beg = (int64_t)blockIdx.x * per;
  const int64_t end = beg + per < p.rs.nitems ? beg + per : p.rs.nitems;
  for (int64_t it = beg + threadIdx.x; it < end; it += 2 * blockDim.x) {
    const int64_t it2 = it + blockDim.x;
    const uint8_t *s0, *s1 = nullptr;
    uint8_t *d0, *d1 = nullptr;
    int x0, x1 = 0;
    gray_chunk_addr(p, it, s0, d0, x0);
    const bool has2 = it2 < end;
    if (has2) gray_chunk_addr(p, it2, s1, d1, x1);
    const bool v0 = p.vec && x0 + 16 <= p.rs.row_len, v1 = has2 && p.vec && x1 + 16 <= p.rs.row_len;
    uint4 a0, b0, c0, e0, a1, b1, c1, e1;
    if (v0) {
      a0 = ldg16(s0);
      b0 = ldg16(s0 + 16);
      c0 = ldg16(s0 + 32);
      e0 = ldg16(s0 + 48);
    }
    if (v1) {
      a1 = ldg16(s1);
      b1 = ldg16(s1 + 16);
      c1 = ldg16(s1 + 32);
      e1 = ldg16(s1 + 48);
    }
    if (v0)
      stg16(d0, gray_16(p, a0, b0, c0, e0));
    else
      gray_scalar(p, s0, d0, x0);
    if (v1)
      stg16(d1, gray_16(p, a1, b1, c1, e1));
    else if (has2)
      gray_scalar(p, s1, d1, x1);
  }
}

// ---------------------------------------------------------------- binary ops
template <typename T>
struct BinParams {
  const char *a, *b;
  char *out;
  int64_t a_pitch, b_pitch, o_pitch, a_bs, b_bs, o_bs;
  RowSpace rs;
  int op;
  float alpha, beta;
};

template <typename T>
__device__ __forceinline__ float bin_apply(const BinParams<T> &p, float a, float b) {
  switch (p.op) {
    case 0: return __fsub_rn(a, b);
    case 1: return __fadd_rn(a, b);
    default: return __fadd_rn(__fmul_rn(p.alpha, a), __fmul_rn(p.beta, b));
  }
}

template <typename T>
__global__ void __launch_bounds__(256) binary_kernel(const __grid_constant__ BinParams<T> p) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; it < p.rs.nitems; it += stride) {
    const int chunk = (int)(it % p.rs.chunks_per_row);
    const int64_t row_g = it / p.rs.chunks_per_row;
    const int bi = (int)(row_g / p.rs.rows_per_img);
    const int row = (int)(row_g - (int64_t)bi * p.rs.rows_per_img);
    const T *a = reinterpret_cast<const T *>(p.a + bi * p.a_bs + row * p.a_pitch) + chunk * 16;
    const T *b = reinterpret_cast<const T *>(p.b + bi * p.b_bs + row * p.b_pitch) + chunk * 16;
    T *o = reinterpret_cast<T *>(p.out + bi * p.o_bs + row * p.o_pitch) + chunk * 16;
    const int x0 = chunk * 16;
    for (int q = 0; q < 16 && x0 + q < p.rs.row_len; ++q)
      o[q] = Storage<T>::from_f(bin_apply(p, Storage<T>::to_f(a[q]), Storage<T>::to_f(b[q])));
  }
}

// ---------------------------------------------------------------- convert
template <typename TI, typename TO>
__global__ void __launch_bounds__(256) convert_kernel(const char *in, int64_t ip, int64_t ibs, char *out, int64_t op,
                                                      int64_t obs, int w, int h, int batch) {
  const int64_t n = (int64_t)w * h * batch;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    const int x = (int)(i % w);
    const int64_t r = i / w;
    const int y = (int)(r % h), b = (int)(r / h);
    const TI v = reinterpret_cast<const TI *>(in + b * ibs + y * ip)[x];
    float f;
    if constexpr (sizeof(TI) == 1)
      f = (float)v;
    else
      f = Storage<TI>::to_f(v);
    TO *o = reinterpret_cast<TO *>(out + b * obs + y * op) + x;
    if constexpr (sizeof(TO) == 1) {
      // truncation toward zero as a C cast, saturated to [0, 255]
      f = fminf(fmaxf(f, 0.0f), 255.0f);
      *o = (TO)(int)f;
    } else {
      *o = Storage<TO>::from_f(f);
    }
  }
}

// ---------------------------------------------------------------- resample
// lib/AST/Interpolate.cpp:85-113 (mapped = scale/2 + scale*x, contracted to
// one fma as nvcc and aarch64 GCC do) and runtime/hipacc_cu_interpolate.hpp:173-216.
__device__ __forceinline__ float mapped(float s, int x) { return __fmaf_rn(s, (float)x, s * 0.5f); }

// B5 / CF / L3 accessors of the CPU back end (runtime/hipacc_cpu_interpolate.hpp:
// binomial5, bicubic_spline with a = -0.5, lanczos with l = 3), every product
// and sum rounded separately in the macros' order, taps clamped to the image.
// B5: xb = x_mapped, columns x_int-1..x_int+2, weight b5((x_frac + 1) - j);
// CF: xb = x_mapped - 0.5, columns x_int-1..x_int+2, weight cubic((x_frac - 1) + j);
// L3: xb = x_mapped - 0.5, columns x_int-2..x_int+3 and rows y_int-1..y_int+4,
//     weight lanczos((frac - 2) + j); the reference gives the fifth tap of the
//     second row the sixth tap's weight, and so does this kernel.
__device__ __forceinline__ float wt_b5(float d) {
  d = fabsf(d);
  return d < 0.5f ? 0.75f : (d < 1.0f ? 0.5f : (d < 1.5f ? 0.125f : 0.0f));
}
__device__ __forceinline__ float wt_cf(float d) {
  d = fabsf(d);
  const float a = -0.5f;
  if (d < 1.0f) {
    const float t1 = __fmul_rn(__fmul_rn(__fmul_rn(a + 2.0f, d), d), d);
    const float t2 = __fmul_rn(__fmul_rn(a + 3.0f, d), d);
    return __fadd_rn(__fsub_rn(t1, t2), 1.0f);
  }
  if (d < 2.0f) {
    const float t1 = __fmul_rn(__fmul_rn(__fmul_rn(a, d), d), d);
    const float t2 = __fmul_rn(__fmul_rn(5.0f * a, d), d);
    const float t3 = __fmul_rn(8.0f * a, d);
    return __fsub_rn(__fadd_rn(__fsub_rn(t1, t2), t3), 4.0f * a);
  }
  return 0.0f;
}
__device__ __forceinline__ float wt_l3(float d) {
  d = fabsf(d);
  if (d == 0.0f) return 1.0f;
  if (d < 3.0f) {
    // the reference's pi is the double of <cmath>: arguments and denominator in double
    const double pi = 3.14159265358979323846, ad = (double)d;
    const float s1 = sinf((float)(pi * ad / 3.0)), s2 = sinf((float)(pi * ad));
    return (float)((double)__fmul_rn(3.0f, __fmul_rn(s1, s2)) / (pi * pi * ad * ad));
  }
  return 0.0f;
}

// Tap tables of the filtered modes, per output column and per output row: the
// first tap index and the n weights (the weights depend only on the column or
// the row, so each is evaluated once per call instead of once per pixel).
constexpr int RS_MAXT = 6;
struct ResTap {
  int first;
  float w[RS_MAXT];
};

__global__ void __launch_bounds__(256) resample_taps_kernel(ResTap *cols, ResTap *rows, int sw, int sh, int dw,
                                                            int dh, int imode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= dw + dh) return;
  const bool is_col = i < dw;
  const int o = is_col ? i : i - dw;
  const float s = is_col ? (float)sw / (float)dw : (float)sh / (float)dh;
  const bool b5 = imode == 3, l3 = imode == 5;
  const float m = mapped(s, o);
  float b = b5 ? m : m - 0.5f;
  b = b < 0.0f ? 0.0f : b;
  const int bi = (int)b;
  const float f = b - (float)bi;
  const float t = b5 ? f + 1.0f : (l3 ? f - 2.0f : f - 1.0f);
  ResTap tap;
  // columns x_int-2.. for L3, x_int-1.. otherwise; rows y_int-1.. for every mode
  tap.first = (is_col && l3) ? bi - 2 : bi - 1;
#pragma unroll
  for (int j = 0; j < RS_MAXT; ++j) {
    const float d = b5 ? __fsub_rn(t, (float)j) : __fadd_rn(t, (float)j);
    tap.w[j] = b5 ? wt_b5(d) : (l3 ? wt_l3(d) : wt_cf(d));
  }
  (is_col ? cols : rows)[o] = tap;
}

// out(x, y) = sum_k (sum_j src(x_j, y_k) w_j) w_k, every product and sum rounded
// separately in the macros' order; taps clamped to the image.  The reference
// gives the fifth tap of the second row of L3 the sixth tap's weight.
template <int N, bool L3>
__global__ void __launch_bounds__(256) resample_filtered_kernel(const char *in, int64_t ip, int64_t ibs, int sw,
                                                                int sh, char *out, int64_t op, int64_t obs, int dw,
                                                                int dh, const ResTap *cols, const ResTap *rows) {
  const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y, b = blockIdx.z;
  if (x >= dw || y >= dh) return;
  const float *src = reinterpret_cast<const float *>(in + (int64_t)b * ibs);
  const ResTap cx = cols[x], cy = rows[y];
  float acc_out = 0.0f;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    const int yy = min(max(cy.first + k, 0), sh - 1);
    const float *row = reinterpret_cast<const float *>(reinterpret_cast<const char *>(src) + yy * ip);
    float acc = 0.0f;
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const int xx = min(max(cx.first + j, 0), sw - 1);
      const float wj = (L3 && k == 1 && j == 4) ? cx.w[5] : cx.w[j];
      const float p = __fmul_rn(__ldg(row + xx), wj);
      acc = j == 0 ? p : __fadd_rn(acc, p);
    }
    const float q = __fmul_rn(acc, cy.w[k]);
    acc_out = k == 0 ? q : __fadd_rn(acc_out, q);
  }
  reinterpret_cast<float *>(out + (int64_t)b * obs + (int64_t)y * op)[x] = acc_out;
}

// Filtered modes, separable form.  In the order above, the row sum of tap row
// k (the rounded products over j, summed from j = 0) depends only on the
// source row and the output column, so every output row whose taps include
// that source row uses the same number.  A CTA takes a 64 x 32 output tile:
// its 256 threads first compute the row sums of the R source rows the tile
// needs (R <= RF_MAXR, checked by the host from the scale) for the tile's 64
// columns into shared memory, then every output of the tile from them.  Same
// operations in the same order as resample_filtered_kernel, so the same bits.
// L3 also keeps the second row's variant (its fifth tap weighed with the sixth
// weight) for every source row.
constexpr int RF_TW = 64, RF_TH = 32, RF_MAXR = 64;
template <int N, bool L3>
__global__ void __launch_bounds__(256) resample_sep_kernel(const char *in, int64_t ip, int64_t ibs, int sw, int sh,
                                                           char *out, int64_t op, int64_t obs, int dw, int dh,
                                                           const ResTap *cols, const ResTap *rows, int *status) {
  __shared__ float hs[(L3 ? 2 : 1) * RF_MAXR * RF_TW];
  __shared__ int s_first[RF_TH];
  __shared__ float s_w[RF_TH][N];
  const int c = threadIdx.x & (RF_TW - 1), rg = threadIdx.x / RF_TW;
  const int x0 = blockIdx.x * RF_TW, y0 = blockIdx.y * RF_TH, b = blockIdx.z;
  const int x = x0 + c, nrow = min(RF_TH, dh - y0);
  if ((int)threadIdx.x < nrow) {
    const ResTap cy = rows[y0 + threadIdx.x];
    s_first[threadIdx.x] = cy.first;
#pragma unroll
    for (int k = 0; k < N; ++k) s_w[threadIdx.x][k] = cy.w[k];
  }
  const int r0 = rows[y0].first;
  const int R = rows[y0 + nrow - 1].first + N - r0;
  if (R > RF_MAXR) {  // the host keeps the scale in range; never taken
    if (threadIdx.x == 0) record_status(status, HGB_ERR_INTERNAL);
    return;
  }
  const float *src = reinterpret_cast<const float *>(in + (int64_t)b * ibs);
  if (x < dw) {
    const ResTap cx = cols[x];
    int xs[N];
#pragma unroll
    for (int j = 0; j < N; ++j) xs[j] = min(max(cx.first + j, 0), sw - 1);
    for (int r = rg; r < R; r += 256 / RF_TW) {
      const int yy = min(max(r0 + r, 0), sh - 1);
      const float *row = reinterpret_cast<const float *>(reinterpret_cast<const char *>(src) + yy * ip);
      float v[N];
#pragma unroll
      for (int j = 0; j < N; ++j) v[j] = __ldg(row + xs[j]);
      float acc = __fmul_rn(v[0], cx.w[0]);
#pragma unroll
      for (int j = 1; j < N; ++j) acc = __fadd_rn(acc, __fmul_rn(v[j], cx.w[j]));
      hs[r * RF_TW + c] = acc;
      if constexpr (L3) {
        float a2 = __fmul_rn(v[0], cx.w[0]);
#pragma unroll
        for (int j = 1; j < N; ++j) a2 = __fadd_rn(a2, __fmul_rn(v[j], cx.w[j == 4 ? 5 : j]));
        hs[RF_MAXR * RF_TW + r * RF_TW + c] = a2;
      }
    }
  }
  __syncthreads();
  if (x >= dw) return;
  float *dst = reinterpret_cast<float *>(out + (int64_t)b * obs) + x;
  for (int yl = rg; yl < nrow; yl += 256 / RF_TW) {
    const int base = s_first[yl] - r0;
    float acc_out = 0.0f;
#pragma unroll
    for (int k = 0; k < N; ++k) {
      const float h = hs[((L3 && k == 1) ? RF_MAXR * RF_TW : 0) + (base + k) * RF_TW + c];
      const float q = __fmul_rn(h, s_w[yl][k]);
      acc_out = k == 0 ? q : __fadd_rn(acc_out, q);
    }
    *reinterpret_cast<float *>(reinterpret_cast<char *>(dst) + (int64_t)(y0 + yl) * op) = acc_out;
  }
}

// NN and LF: a thread per column and four rows 8 apart (a 32 x 32 block of
// outputs per CTA), so that every thread has four independent reads in flight
constexpr int RS_ROWS = 4;
// Sample positions along one axis, evaluated once per CTA for its 32 columns
// and 32 rows instead of once per pixel.  NN keeps the clamped index of the
// mapped coordinate.  LF keeps, for b = max(mapped - 0.5, 0), the clamped
// indices of floor(b) and floor(b) + 1 and the weights (1 - f, f) of the
// fraction f; the pixel's four weights are the rounded products of a column
// weight and a row weight, and the sum is w00 v00 rounded, then three fused
// multiply-adds in the order (x1, y0), (x0, y1), (x1, y1).
struct RsAxis {
  int i0, i1;
  float w0, w1;
};
__device__ __forceinline__ RsAxis rs_axis(float s, int o, int n, bool lf) {
  const float m = mapped(s, o);
  RsAxis a;
  if (!lf) {
    a.i0 = a.i1 = min(max((int)m, 0), n - 1);
    a.w0 = a.w1 = 0.0f;
    return a;
  }
  float bpos = m - 0.5f;
  bpos = bpos < 0.0f ? 0.0f : bpos;
  const int bi = (int)bpos;
  const float f = bpos - (float)bi;
  a.i0 = min(bi, n - 1);
  a.i1 = min(bi + 1, n - 1);
  a.w0 = 1.0f - f;
  a.w1 = f;
  return a;
}

__global__ void __launch_bounds__(256) resample_kernel(const char *in, int64_t ip, int64_t ibs, int sw, int sh,
                                                       char *out, int64_t op, int64_t obs, int dw, int dh, int imode) {
  __shared__ RsAxis s_col[32], s_row[8 * RS_ROWS];
  const int x = blockIdx.x * 32 + threadIdx.x, b = blockIdx.z, yb = blockIdx.y * 8 * RS_ROWS;
  const bool lf = imode != 1;
  const int t = threadIdx.y * 32 + threadIdx.x;
  if (t < 32) {
    const int xc = blockIdx.x * 32 + t;
    if (xc < dw) s_col[t] = rs_axis((float)sw / (float)dw, xc, sw, lf);
  } else if (t < 32 + 8 * RS_ROWS) {
    const int yr = yb + t - 32;
    if (yr < dh) s_row[t - 32] = rs_axis((float)sh / (float)dh, yr, sh, lf);
  }
  __syncthreads();
  if (x >= dw) return;
  const RsAxis cx = s_col[threadIdx.x];
  const char *src = in + (int64_t)b * ibs;
  float v[RS_ROWS];
#pragma unroll
  for (int k = 0; k < RS_ROWS; ++k) {
    const int yl = threadIdx.y + 8 * k;
    if (yb + yl >= dh) break;
    const RsAxis ry = s_row[yl];
    const float *r0 = reinterpret_cast<const float *>(src + ry.i0 * ip);
    if (!lf) {
      v[k] = __ldg(r0 + cx.i0);
    } else {
      const float *r1 = reinterpret_cast<const float *>(src + ry.i1 * ip);
      const float wa = __fmul_rn(cx.w0, ry.w0), wb = __fmul_rn(cx.w1, ry.w0);
      const float wc = __fmul_rn(cx.w0, ry.w1), wd = __fmul_rn(cx.w1, ry.w1);
      float r = __fmul_rn(wa, __ldg(r0 + cx.i0));
      r = __fmaf_rn(wb, __ldg(r0 + cx.i1), r);
      r = __fmaf_rn(wc, __ldg(r1 + cx.i0), r);
      r = __fmaf_rn(wd, __ldg(r1 + cx.i1), r);
      v[k] = r;
    }
  }
#pragma unroll
  for (int k = 0; k < RS_ROWS; ++k) {
    const int y = yb + threadIdx.y + 8 * k;
    if (y >= dh) break;
    reinterpret_cast<float *>(out + (int64_t)b * obs + (int64_t)y * op)[x] = v[k];
  }
}

// ---------------------------------------------------------------- gray, bulk copies
// Dense images (rows back to back, the batch contiguous) are one flat array of
// N pixels, cut into units of GB_UNIT pixels (16 KiB of uchar4).  Each CTA
// takes one unit: thread 0 issues one cp.async.bulk of the unit into shared
// memory (completion on an mbarrier) and every thread turns GB_PX / 4 groups
// of four staged pixels, GB_T groups apart, into 4-byte stores.  With 16 KiB
// of shared memory per CTA the SM holds many such CTAs, so many copies are in
// flight without a software pipeline, and an independent kernel of the same
// step can share the SMs.  The last CTA converts the pixels after the last
// whole unit with plain loads.
constexpr int GB_T = 256, GB_PX = 16;
constexpr int GB_UNIT = GB_PX * GB_T;
constexpr int GB_STAGE = GB_UNIT * 4;

struct GrayBulkParams {
  GrayParams p;
  int64_t npx;  // pixels of the flat array
  int64_t nunits;
  int *status;
};

__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__global__ void __launch_bounds__(GB_T) gray_bulk_kernel(const __grid_constant__ GrayBulkParams B) {
  __shared__ __align__(128) uint8_t stage[GB_STAGE];
  __shared__ __align__(8) uint64_t bar;
  const GrayParams &p = B.p;
  const int64_t u = blockIdx.x;
  if (u < B.nunits) {
    if (threadIdx.x == 0) {
      mbar_init(&bar, 1);
      mbar_fence_init();
      mbar_expect_tx(&bar, GB_STAGE);
      bulk_load(stage, p.in + u * GB_STAGE, GB_STAGE, &bar);
    }
    if (!cta_wait(&bar, 0)) {
      if (threadIdx.x == 0) {
        record_status(B.status, HGB_ERR_TIMEOUT);
        mbar_wait(&bar, 0);  // the copy may still land: wait once more (bounded) before leaving
      }
      return;
    }
    // four pixels per 16-byte read, the warp's reads consecutive (no bank
    // conflicts), one 4-byte store per read: a warp writes 128 contiguous bytes
    const uint4 *src = reinterpret_cast<const uint4 *>(stage) + threadIdx.x;
    uint32_t *dst = reinterpret_cast<uint32_t *>(p.out + u * GB_UNIT) + threadIdx.x;
#pragma unroll
    for (int k = 0; k < GB_PX / 4; ++k) {
      const uint4 q = src[k * GB_T];
      dst[k * GB_T] = gray_px(p, q.x) | (gray_px(p, q.y) << 8) | (gray_px(p, q.z) << 16) | (gray_px(p, q.w) << 24);
    }
    return;
  }
  // the pixels after the last whole unit (fewer than GB_UNIT)
  for (int64_t i = B.nunits * GB_UNIT + threadIdx.x; i < B.npx; i += GB_T) {
    const uint8_t *s = p.in + 4 * i;
    const uint32_t rgba = (uint32_t)s[0] | ((uint32_t)s[1] << 8) | ((uint32_t)s[2] << 16) | ((uint32_t)s[3] << 24);
    p.out[i] = (uint8_t)gray_px(p, rgba);
  }
}

bool dense(const hgb_view &v) {
  const int64_t row = (int64_t)v.width * dtype_size(v.dtype);
  return v.pitch == row && (v.batch == 1 || v.batch_stride == row * v.height);
}

}  // namespace
}  // namespace hgb

using namespace hgb;

extern "C" int hgb_point_gray(const hgb_view *in, const hgb_view *out, int wr, int wg, int wb, int shift, void *stream) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  rc = check_view(out, "out");
  if (rc) return rc;
  HGB_REQUIRE(in->dtype == HGB_U8X4 && out->dtype == HGB_U8, "hgb_point_gray: uchar4 -> u8 expected");
  HGB_REQUIRE(in->width == out->width && in->height == out->height && in->batch == out->batch,
              "hgb_point_gray: size mismatch");
  HGB_REQUIRE(wr >= 0 && wg >= 0 && wb >= 0 && shift >= 0 && shift < 32 && wr + wg + wb < (1 << 23),
              "hgb_point_gray: bad weights");
  GrayParams p;
  p.in = (const uint8_t *)in->data;
  p.in_pitch = in->pitch;
  p.in_bstride = in->batch_stride;
  p.out = (uint8_t *)out->data;
  p.out_pitch = out->pitch;
  p.out_bstride = out->batch_stride;
  const bool d = dense(*in) && dense(*out);
  p.rs = make_rows(in->width, in->height, in->batch, d);
  // vector path: every chunk start is 16-byte aligned on both sides
  p.vec = ((uintptr_t)in->data % 16 == 0) && ((uintptr_t)out->data % 16 == 0) &&
          (d || (in->pitch % 16 == 0 && out->pitch % 16 == 0)) &&
          (in->batch == 1 || (in->batch_stride % 16 == 0 && out->batch_stride % 16 == 0));
  p.wr = wr;
  p.wg = wg;
  p.wb = wb;
  p.shift = shift;
  p.use_dp4a = wr < 256 && wg < 256 && wb < 256;
  p.wpack = (uint32_t)wr | ((uint32_t)wg << 8) | ((uint32_t)wb << 16);
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t npx = (int64_t)in->width * in->height * in->batch;
  if (d && p.vec && npx >= (int64_t)GB_UNIT) {
    // dense, 16-byte aligned: one bulk copy per CTA over the flat array
    GrayBulkParams B;
    B.p = p;
    B.npx = npx;
    B.nunits = npx / GB_UNIT;
    B.status = device_status_word();
    const int64_t g = B.nunits + (npx % GB_UNIT ? 1 : 0);
    HGB_REQUIRE(g < (int64_t)0x7fffffff, "hgb_point_gray: image too large");
    cudaEvent_t ev = before_launch(st);
    gray_bulk_kernel<<<(unsigned)g, GB_T, 0, st>>>(B);
    return after_launch("gray_bulk_kernel", st, ev);
  }
  // one resident wave: every CTA owns one contiguous range
  int grid = num_sms() * resident_ctas((const void *)gray_kernel, 256, 0);
  const int64_t need = (p.rs.nitems + 511) / 512;
  if (need < grid) grid = (int)(need > 0 ? need : 1);
  cudaEvent_t ev = before_launch(st);
  gray_kernel<<<grid, 256, 0, st>>>(p);
  return after_launch("gray_kernel", st, ev);
}

extern "C" int hgb_point_binary(int op, const hgb_view *a, const hgb_view *b, const hgb_view *out, float alpha,
                                float beta, void *stream) {
  int rc = check_view(a, "a");
  if (rc) return rc;
  rc = check_view(b, "b");
  if (rc) return rc;
  rc = check_view(out, "out");
  if (rc) return rc;
  HGB_REQUIRE(op >= 0 && op <= 2, "hgb_point_binary: bad op");
  HGB_REQUIRE(a->dtype == b->dtype && a->dtype == out->dtype && is_float_storage(a->dtype),
              "hgb_point_binary: same float storage expected");
  HGB_REQUIRE(a->width == out->width && b->width == out->width && a->height == out->height &&
                  b->height == out->height && a->batch == out->batch && b->batch == out->batch,
              "hgb_point_binary: size mismatch");
  cudaStream_t st = (cudaStream_t)stream;
  const bool d = dense(*a) && dense(*b) && dense(*out);
  cudaEvent_t ev = before_launch(st);
#define HGB_BIN(T)                                                                                              \
  {                                                                                                             \
    BinParams<T> p{(const char *)a->data, (const char *)b->data, (char *)out->data, a->pitch, b->pitch,         \
                   out->pitch, a->batch_stride, b->batch_stride, out->batch_stride,                             \
                   make_rows(a->width, a->height, a->batch, d), op, alpha, beta};                               \
    binary_kernel<T><<<grid_for(p.rs.nitems, 256), 256, 0, st>>>(p);                                           \
  }
  if (a->dtype == HGB_F32) HGB_BIN(float) else if (a->dtype == HGB_BF16) HGB_BIN(__nv_bfloat16) else HGB_BIN(__half)
#undef HGB_BIN
  return after_launch("binary_kernel", st, ev);
}

extern "C" int hgb_convert(const hgb_view *in, const hgb_view *out, void *stream) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  rc = check_view(out, "out");
  if (rc) return rc;
  HGB_REQUIRE(in->width == out->width && in->height == out->height && in->batch == out->batch,
              "hgb_convert: size mismatch");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = (int64_t)in->width * in->height * in->batch;
  const int grid = grid_for(n, 256);
  cudaEvent_t ev = before_launch(st);
#define HGB_CV(TI, TO) \
  convert_kernel<TI, TO><<<grid, 256, 0, st>>>((const char *)in->data, in->pitch, in->batch_stride, (char *)out->data, \
                                               out->pitch, out->batch_stride, in->width, in->height, in->batch)
  const int a = in->dtype, b = out->dtype;
  if (a == HGB_F32 && b == HGB_BF16) HGB_CV(float, __nv_bfloat16);
  else if (a == HGB_F32 && b == HGB_F16) HGB_CV(float, __half);
  else if (a == HGB_BF16 && b == HGB_F32) HGB_CV(__nv_bfloat16, float);
  else if (a == HGB_F16 && b == HGB_F32) HGB_CV(__half, float);
  else if (a == HGB_F32 && b == HGB_F32) HGB_CV(float, float);
  else if (a == HGB_U8 && b == HGB_F32) HGB_CV(uint8_t, float);
  else if (a == HGB_F32 && b == HGB_U8) HGB_CV(float, uint8_t);
  else {
    if (ev) cudaEventDestroy(ev);
    return set_error(HGB_ERR_UNSUPPORTED, "hgb_convert: unsupported dtype pair");
  }
#undef HGB_CV
  return after_launch("convert_kernel", st, ev);
}

extern "C" int hgb_resample(const hgb_view *in, const hgb_view *out, int imode, void *stream) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  rc = check_view(out, "out");
  if (rc) return rc;
  HGB_REQUIRE(in->dtype == HGB_F32 && out->dtype == HGB_F32, "hgb_resample: f32 expected");
  HGB_REQUIRE(imode >= 1 && imode <= 5, "hgb_resample: imode must be 1 (NN), 2 (LF), 3 (B5), 4 (CF) or 5 (L3)");
  HGB_REQUIRE(in->batch == out->batch, "hgb_resample: batch mismatch");
  HGB_REQUIRE(in->pitch % 4 == 0 && out->pitch % 4 == 0, "hgb_resample: pitches must be whole floats");
  HGB_REQUIRE(out->batch <= 65535, "hgb_resample: at most 65535 images per call");
  cudaStream_t st = (cudaStream_t)stream;
  const dim3 grid(cdiv(out->width, 32), cdiv(out->height, 8), out->batch), block(32, 8);
  if (imode <= 2) {
    const dim3 g4(grid.x, cdiv(out->height, 8 * RS_ROWS), out->batch);
    cudaEvent_t ev = before_launch(st);
    resample_kernel<<<g4, block, 0, st>>>((const char *)in->data, in->pitch, in->batch_stride, in->width,
                                            in->height, (char *)out->data, out->pitch, out->batch_stride,
                                            out->width, out->height, imode);
    return after_launch("resample_kernel", st, ev);
  }
  // filtered modes: tap tables in the library workspace (calls sharing it are ordered on one stream)
  Workspace ws;
  rc = workspace_get(((size_t)out->width + out->height) * sizeof(ResTap), &ws);
  if (rc) return rc;
  ResTap *cols = (ResTap *)ws.base, *rows = cols + out->width;
  cudaEvent_t ev = before_launch(st);
  resample_taps_kernel<<<cdiv(out->width + out->height, 256), 256, 0, st>>>(cols, rows, in->width, in->height,
                                                                             out->width, out->height, imode);
  const char *src = (const char *)in->data;
  char *dst = (char *)out->data;
  // the separable form holds the row sums of at most RF_MAXR source rows per
  // 32 output rows: first taps advance by at most ceil(31 * sh / dh) + 1 rows
  const int n = imode == 5 ? 6 : 4;
  if ((double)in->height / out->height * (RF_TH - 1) + 2 + n <= RF_MAXR) {
    const dim3 gs(cdiv(out->width, RF_TW), cdiv(out->height, RF_TH), out->batch);
    int *status = device_status_word();
    if (imode == 5)
      resample_sep_kernel<6, true><<<gs, 256, 0, st>>>(src, in->pitch, in->batch_stride, in->width, in->height, dst,
                                                       out->pitch, out->batch_stride, out->width, out->height, cols,
                                                       rows, status);
    else
      resample_sep_kernel<4, false><<<gs, 256, 0, st>>>(src, in->pitch, in->batch_stride, in->width, in->height,
                                                        dst, out->pitch, out->batch_stride, out->width, out->height,
                                                        cols, rows, status);
    return after_launch("resample_sep_kernel", st, ev);
  }
  if (imode == 5)
    resample_filtered_kernel<6, true><<<grid, block, 0, st>>>(src, in->pitch, in->batch_stride, in->width,
                                                              in->height, dst, out->pitch, out->batch_stride,
                                                              out->width, out->height, cols, rows);
  else
    resample_filtered_kernel<4, false><<<grid, block, 0, st>>>(src, in->pitch, in->batch_stride, in->width,
                                                               in->height, dst, out->pitch, out->batch_stride,
                                                               out->width, out->height, cols, rows);
  return after_launch("resample_filtered_kernel", st, ev);
}

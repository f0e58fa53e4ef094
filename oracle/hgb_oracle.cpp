// hgb_oracle.cpp -- TEST INFRASTRUCTURE ONLY (see hgb_oracle.h).
//
// CPU restatement of the code Hipacc's CPU back end emits for the image
// hot path.  Loop shape follows lib/Backend/CPU_x86.cpp:2973-2992,3682-3689
// (OpenMP over output rows, scalar body); interior pixels read directly and
// border pixels go through the boundary remap, as the generated border
// variants do (lib/AST/ASTTranslate.cpp:787-917).
//
// Deliberate definitions where the reference is undefined, shared with the
// CUDA library so that results agree everywhere:
//   * UNDEFINED boundary: the reference reads outside the image (undefined
//     behaviour); here out-of-range taps are clamped.  Tests compare only
//     pixels whose taps are all in range for this mode.
//   * MIRROR with a radius larger than the window: the reference reflects once
//     and may still be out of range; here the reflection (upper side first,
//     then lower side, as lib/AST/BorderHandling.cpp:124-407 orders them) is
//     repeated until the index is in range.  It is identical to the reference
//     whenever one reflection suffices.
#include "hgb_oracle.h"

#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <type_traits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int kConstIdx = INT_MIN;

// lib/AST/BorderHandling.cpp:41-120 (clamp_/repeat_/mirror_/constant_{lower,upper})
inline int remap_idx(int mode, int idx, int lo, int hi) {
  if (idx >= lo && idx < hi) return idx;
  switch (mode) {
    case ORC_REPEAT: {
      // while (idx >= upper) idx -= w; while (idx < lower) idx += w;
      const int w = hi - lo;
      int r = (idx - lo) % w;
      if (r < 0) r += w;
      return lo + r;
    }
    case ORC_MIRROR:
      // if (idx >= upper) idx = upper - (idx+1 - upper);
      // if (idx <  lower) idx = lower + (lower - idx-1);
      while (idx < lo || idx >= hi) {
        if (idx >= hi) idx = hi - (idx + 1 - hi);
        if (idx < lo) idx = lo + (lo - idx - 1);
      }
      return idx;
    case ORC_CONSTANT:
      return kConstIdx;
    case ORC_CLAMP:
    default:  // UNDEFINED is defined as CLAMP (see file header)
      return idx < lo ? lo : hi - 1;
  }
}

// lib/AST/Convolution.cpp:90-100 get_init<T>(mode)
template <typename T>
T reduce_init(int red) {
  switch (red) {
    case ORC_SUM: return T(0);
    case ORC_MIN: return std::numeric_limits<T>::max();
    case ORC_MAX: return std::numeric_limits<T>::min();  // FLT_MIN for float (sic)
    case ORC_PROD: return T(1);
  }
  return T(0);
}

template <typename T>
inline T fma_t(T a, T b, T c) {
  return std::fma(a, b, c);
}

// lib/AST/Convolution.cpp:43-87 getConvolutionStmt: red += v; red = min(red, v);
// red = max(red, v); red *= v.  hipacc::math::min/max are (a<b?a:b)/(a>b?a:b)
// (dsl/math_functions.hpp:347-376).
template <typename T>
inline void accumulate(T &acc, int red, bool has_mask, T m, T x, int contract) {
  if (red == ORC_SUM) {
    if (has_mask) {
      if (contract)
        acc = fma_t(m, x, acc);
      else {
        T p = m * x;
        acc = acc + p;
      }
    } else {
      acc = acc + x;
    }
    return;
  }
  T v = has_mask ? T(m * x) : x;
  switch (red) {
    case ORC_MIN: acc = acc < v ? acc : v; break;
    case ORC_MAX: acc = acc > v ? acc : v; break;
    case ORC_PROD: acc = acc * v; break;
  }
}

template <typename T>
void local_op(const T *in, long in_stride, int aox, int aoy, int aw, int ah, T *out, long out_stride,
              int iox, int ioy, int iw, int ih, const T *mask, const uint8_t *domain, int mw,
              int mh, int red, int bmode, T cval, int contract, int nthreads) {
  const int rx = mw / 2, ry = mh / 2;
  const T init = reduce_init<T>(red);
  const bool has_mask = mask != nullptr;
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int j = 0; j < ih; ++j) {
    for (int i = 0; i < iw; ++i) {
      const int cx = aox + i, cy = aoy + j;
      const bool interior = (cx - rx >= aox) && (cx + (mw - 1 - rx) < aox + aw) && (cy - ry >= aoy) &&
                            (cy + (mh - 1 - ry) < aoy + ah);
      T acc = init;
      for (int my = 0; my < mh; ++my) {
        for (int mx = 0; mx < mw; ++mx) {
          if (domain && !domain[my * mw + mx]) continue;  // dsl/mask.hpp:112-126
          const int ax = cx + mx - rx, ay = cy + my - ry;
          T x;
          if (interior) {
            x = in[(long)ay * in_stride + ax];
          } else {
            const int rxi = remap_idx(bmode, ax, aox, aox + aw);
            const int ryi = remap_idx(bmode, ay, aoy, aoy + ah);
            if (rxi == kConstIdx || ryi == kConstIdx)
              x = cval;
            else
              x = in[(long)ryi * in_stride + rxi];
          }
          accumulate<T>(acc, red, has_mask, has_mask ? mask[my * mw + mx] : T(0), x, contract);
        }
      }
      out[(long)(ioy + j) * out_stride + (iox + i)] = acc;
    }
  }
}

// Sampling position of the mapped (cell-centred) coordinate used by NN and LF
// accessors: acc_scale/2 + acc_scale*x (lib/AST/Interpolate.cpp:85-113) with
// acc_scale = (float)acc_width/is_width (lib/AST/ASTTranslate.cpp:586-605).
inline float mapped_coord(float scale, int x, int contract) {
  if (contract) return std::fma(scale, (float)x, scale / 2);
  float a = scale / 2;
  float b = scale * (float)x;
  return a + b;
}

// runtime/hipacc_cpu_interpolate.hpp:157-197 with CLAMP taps on [0,sw)x[0,sh).
template <typename T>
inline T interp_lf(const T *src, int sw, int sh, float xm, float ym, int contract) {
  float xb = xm - 0.5f;
  float yb = ym - 0.5f;
  if (xb < 0.0f) xb = 0.0f;
  if (yb < 0.0f) yb = 0.0f;
  int xi = (int)xb;
  int yi = (int)yb;
  float xf = xb - (float)xi;
  float yf = yb - (float)yi;
  auto cl = [](int v, int hi) { return v >= hi ? hi - 1 : (v < 0 ? 0 : v); };
  const int x0 = cl(xi, sw), x1 = cl(xi + 1, sw), y0 = cl(yi, sh), y1 = cl(yi + 1, sh);
  const T a = src[(long)y0 * sw + x0], b = src[(long)y0 * sw + x1];
  const T c = src[(long)y1 * sw + x0], d = src[(long)y1 * sw + x1];
  const float wa = (1.0f - xf) * (1.0f - yf);
  const float wb = xf * (1.0f - yf);
  const float wc = (1.0f - xf) * yf;
  const float wd = xf * yf;
  if (std::is_same<T, float>::value) {
    if (contract) {
      float r = wa * (float)a;
      r = std::fma(wb, (float)b, r);
      r = std::fma(wc, (float)c, r);
      r = std::fma(wd, (float)d, r);
      return (T)r;
    }
    float r = wa * (float)a;
    float t = wb * (float)b;
    r = r + t;
    t = wc * (float)c;
    r = r + t;
    t = wd * (float)d;
    r = r + t;
    return (T)r;
  }
  return (T)((double)wa * (double)a + (double)wb * (double)b + (double)wc * (double)c +
             (double)wd * (double)d);
}

template <typename T>
void resample_nn(const T *src, int sw, int sh, T *dst, int dw, int dh, int contract) {
  const float sx = (float)sw / (float)dw, sy = (float)sh / (float)dh;
  for (int y = 0; y < dh; ++y) {
    int yy = (int)mapped_coord(sy, y, contract);
    yy = std::min(std::max(yy, 0), sh - 1);
    for (int x = 0; x < dw; ++x) {
      int xx = (int)mapped_coord(sx, x, contract);
      xx = std::min(std::max(xx, 0), sw - 1);
      dst[(long)y * dw + x] = src[(long)yy * sw + xx];
    }
  }
}

template <typename T>
void resample_lf(const T *src, int sw, int sh, T *dst, int dw, int dh, int contract) {
  const float sx = (float)sw / (float)dw, sy = (float)sh / (float)dh;
  for (int y = 0; y < dh; ++y) {
    const float ym = mapped_coord(sy, y, contract);
    for (int x = 0; x < dw; ++x) {
      dst[(long)y * dw + x] = interp_lf<T>(src, sw, sh, mapped_coord(sx, x, contract), ym, contract);
    }
  }
}

// Pyramid decomposition: per level the sample runs blur (Gaussian, full level
// size) -> Subsample (NN accessor) -> DifferenceOfGaussian (G_l - LF(G_{l+1}))
// (samples-public/5_Other/Gaussian_Laplacian_Pyramid/src/main.cpp:199-231).
template <typename T>
void pyramid_decompose(T **gauss, T **lap, int w, int h, int levels, const T *mask, int msize,
                       int bmode, int contract, int nthreads) {
  int lw = w, lh = h;
  std::vector<T> tmp;
  for (int l = 0; l + 1 < levels; ++l) {
    const int nw = lw / 2, nh = lh / 2;
    tmp.assign((size_t)lw * lh, T(0));
    local_op<T>(gauss[l], lw, 0, 0, lw, lh, tmp.data(), lw, 0, 0, lw, lh, mask, nullptr, msize, msize,
                ORC_SUM, bmode, T(0), contract, nthreads);
    resample_nn<T>(tmp.data(), lw, lh, gauss[l + 1], nw, nh, contract);
    std::vector<T> up((size_t)lw * lh);
    resample_lf<T>(gauss[l + 1], nw, nh, up.data(), lw, lh, contract);
    for (long p = 0; p < (long)lw * lh; ++p) lap[l][p] = gauss[l][p] - up[p];
    lw = nw;
    lh = nh;
  }
}

// Bilateral filter body (samples-public/3_Preprocessing/Bilateral_Filter/src/main.cpp:63-77).
template <typename T>
void bilateral(const T *in, int w, int h, long stride, T *out, long out_stride, const T *smask,
               int size, T sigma_r, int bmode, T cval, int contract, int nthreads) {
  const int r = size / 2;
  const T c_r = T(0.5) / (sigma_r * sigma_r);
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      const T center = in[(long)y * stride + x];
      T d = T(0), p = T(0);
      const bool interior = x - r >= 0 && x + r < w && y - r >= 0 && y + r < h;
      for (int my = 0; my < size; ++my) {
        for (int mx = 0; mx < size; ++mx) {
          const T m = smask[my * size + mx];
          if (m == T(0)) continue;  // Domain(mask) skips zero cells
          const int ax = x + mx - r, ay = y + my - r;
          T v;
          if (interior) {
            v = in[(long)ay * stride + ax];
          } else {
            const int rxi = remap_idx(bmode, ax, 0, w), ryi = remap_idx(bmode, ay, 0, h);
            v = (rxi == kConstIdx || ryi == kConstIdx) ? cval : in[(long)ryi * stride + rxi];
          }
          const T diff = v - center;
          const T e = (-c_r * diff) * diff;
          const T s = std::exp(e) * m;
          d = d + s;
          if (contract)
            p = std::fma(s, v, p);
          else {
            T t = s * v;
            p = p + t;
          }
        }
      }
      out[(long)y * out_stride + x] = p / d;
    }
  }
}

}  // namespace

extern "C" {

int orc_remap(int mode, int idx, int lower, int upper) { return remap_idx(mode, idx, lower, upper); }

void orc_local_op_f32(const float *in, long in_stride, int acc_ox, int acc_oy, int acc_w, int acc_h,
                      float *out, long out_stride, int is_ox, int is_oy, int is_w, int is_h,
                      const float *mask, const uint8_t *domain, int mw, int mh, int reduce, int bmode,
                      float cval, int contract, int nthreads) {
  local_op<float>(in, in_stride, acc_ox, acc_oy, acc_w, acc_h, out, out_stride, is_ox, is_oy, is_w, is_h,
                  mask, domain, mw, mh, reduce, bmode, cval, contract, nthreads);
}

void orc_local_op_f64(const double *in, long in_stride, int acc_ox, int acc_oy, int acc_w, int acc_h,
                      double *out, long out_stride, int is_ox, int is_oy, int is_w, int is_h,
                      const double *mask, const uint8_t *domain, int mw, int mh, int reduce, int bmode,
                      double cval, int contract, int nthreads) {
  local_op<double>(in, in_stride, acc_ox, acc_oy, acc_w, acc_h, out, out_stride, is_ox, is_oy, is_w,
                   is_h, mask, domain, mw, mh, reduce, bmode, cval, contract, nthreads);
}

void orc_separable_f32(const float *in, int w, int h, float *out, const float *row_taps,
                       const float *col_taps, int k, int bmode, float cval, int contract, int nthreads) {
  std::vector<float> tmp((size_t)w * h);
  local_op<float>(in, w, 0, 0, w, h, tmp.data(), w, 0, 0, w, h, row_taps, nullptr, k, 1, ORC_SUM, bmode,
                  cval, contract, nthreads);
  local_op<float>(tmp.data(), w, 0, 0, w, h, out, w, 0, 0, w, h, col_taps, nullptr, 1, k, ORC_SUM, bmode,
                  cval, contract, nthreads);
}

void orc_separable_f64(const double *in, int w, int h, double *out, const double *row_taps,
                       const double *col_taps, int k, int bmode, double cval, int nthreads) {
  std::vector<double> tmp((size_t)w * h);
  local_op<double>(in, w, 0, 0, w, h, tmp.data(), w, 0, 0, w, h, row_taps, nullptr, k, 1, ORC_SUM,
                   bmode, cval, 0, nthreads);
  local_op<double>(tmp.data(), w, 0, 0, w, h, out, w, 0, 0, w, h, col_taps, nullptr, 1, k, ORC_SUM,
                   bmode, cval, 0, nthreads);
}

void orc_sobel_mag_u8(const uint8_t *in, int w, int h, long in_stride, uint8_t *out, long out_stride,
                      const int *mask_x, const int *mask_y, int size, int bmode, int cval, int nthreads) {
  const int r = size / 2;
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int y = 0; y < h; ++y) {
    for (int x = 0; x < w; ++x) {
      const bool interior = x - r >= 0 && x + r < w && y - r >= 0 && y + r < h;
      int gx = 0, gy = 0;
      for (int my = 0; my < size; ++my) {
        for (int mx = 0; mx < size; ++mx) {
          const int cx = mask_x[my * size + mx], cy = mask_y[my * size + mx];
          if (cx == 0 && cy == 0) continue;
          const int ax = x + mx - r, ay = y + my - r;
          int v;
          if (interior) {
            v = in[(long)ay * in_stride + ax];
          } else {
            const int rxi = remap_idx(bmode, ax, 0, w), ryi = remap_idx(bmode, ay, 0, h);
            v = (rxi == kConstIdx || ryi == kConstIdx) ? cval : in[(long)ryi * in_stride + rxi];
          }
          gx += cx * v;  // reduce(dom_x, SUM, mask_x(dom_x) * input(dom_x))
          gy += cy * v;
        }
      }
      int mag = std::abs(gx) + std::abs(gy);
      out[(long)y * out_stride + x] = (uint8_t)(mag > 255 ? 255 : mag);
    }
  }
}

void orc_rgba_to_gray_u8(const uint8_t *in, int w, int h, long in_stride_px, uint8_t *out,
                         long out_stride, int wr, int wg, int wb, int shift, int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int y = 0; y < h; ++y) {
    const uint8_t *row = in + (long)y * in_stride_px * 4;
    for (int x = 0; x < w; ++x) {
      const int v = wr * row[4 * x + 0] + wg * row[4 * x + 1] + wb * row[4 * x + 2];
      out[(long)y * out_stride + x] = (uint8_t)(v >> shift);
    }
  }
}

// ---- REDUCTION_CPU_2D restated (runtime/hipacc_cpu_red.hpp:19-68, PPT = 1) ----
// libgomp's static schedule hands thread t a contiguous block of rows:
// q = h / T rows each, the first h % T threads one more.
}  // extern "C"
template <typename T, typename A, typename F>
static A reduce_2d(const T *in, int w, int h, long stride, int nthreads, F op) {
  if (nthreads < 1) nthreads = 1;
  std::vector<A> part((size_t)nthreads, A(0));
  const int q = h / nthreads, rem = h % nthreads;
#pragma omp parallel for schedule(static, 1) num_threads(nthreads)
  for (int t = 0; t < nthreads; ++t) {
    const int rows = q + (t < rem ? 1 : 0);
    const int y0 = t * q + std::min(t, rem);
    if (rows == 0) continue;
    A acc = (A)in[(long)y0 * stride];
    for (int y = y0; y < y0 + rows; ++y) {
      for (int x = (y == y0 ? 1 : 0); x < w; ++x) acc = op(acc, (A)in[(long)y * stride + x]);
    }
    part[(size_t)t] = acc;
  }
  A r = part[0];
  for (int t = 1; t < nthreads; ++t) r = op(r, part[(size_t)t]);
  return r;
}
extern "C" {

uint64_t orc_reduce_sum_u8_u64(const uint8_t *in, int w, int h, long stride, int nthreads) {
  return reduce_2d<uint8_t, uint64_t>(in, w, h, stride, nthreads,
                                      [](uint64_t a, uint64_t b) { return a + b; });
}

uint32_t orc_reduce_max_u8(const uint8_t *in, int w, int h, long stride, int nthreads) {
  return reduce_2d<uint8_t, uint32_t>(in, w, h, stride, nthreads,
                                      [](uint32_t a, uint32_t b) { return a > b ? a : b; });
}

float orc_reduce_f32(const float *in, int w, int h, long stride, int op, int nthreads) {
  switch (op) {
    case ORC_SUM: return reduce_2d<float, float>(in, w, h, stride, nthreads, [](float a, float b) { return a + b; });
    case ORC_MIN: return reduce_2d<float, float>(in, w, h, stride, nthreads, [](float a, float b) { return a < b ? a : b; });
    case ORC_MAX: return reduce_2d<float, float>(in, w, h, stride, nthreads, [](float a, float b) { return a > b ? a : b; });
    case ORC_PROD: return reduce_2d<float, float>(in, w, h, stride, nthreads, [](float a, float b) { return a * b; });
  }
  return 0.0f;
}

// ------------------------------------------------------------------ binning
static inline uint32_t hist_index(float pixel, unsigned num_bins) {
  const float v = pixel / 255.0f * (float)num_bins;  // two roundings, as the sample
  if (!(v >= 0.0f)) return 0u;
  if (v >= 4294967296.0f) return 0xffffffffu;
  return (uint32_t)v;
}

void orc_histogram_f32(const float *in, int w, int h, long stride, unsigned num_bins, uint32_t *bins) {
  for (unsigned i = 0; i < num_bins; ++i) bins[i] = 0;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const uint32_t idx = hist_index(in[(long)y * stride + x], num_bins);
      if (idx < num_bins) bins[idx] += 1u;
    }
}

void orc_histogram_u8(const uint8_t *in, int w, int h, long stride, unsigned num_bins, uint32_t *bins) {
  for (unsigned i = 0; i < num_bins; ++i) bins[i] = 0;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const uint32_t idx = hist_index((float)in[(long)y * stride + x], num_bins);
      if (idx < num_bins) bins[idx] += 1u;
    }
}

// Exact-as-possible value of the same reduction (FP64, serial); the error
// reference for float sums.
double orc_reduce_f32_exact(const float *in, int w, int h, long stride, int op) {
  double r = in[0];
  for (int y = 0; y < h; ++y)
    for (int x = (y == 0 ? 1 : 0); x < w; ++x) {
      const double v = in[(long)y * stride + x];
      switch (op) {
        case ORC_SUM: r += v; break;
        case ORC_MIN: r = r < v ? r : v; break;
        case ORC_MAX: r = r > v ? r : v; break;
        case ORC_PROD: r *= v; break;
      }
    }
  return r;
}

void orc_bilateral_f32(const float *in, int w, int h, long stride, float *out, long out_stride,
                       const float *smask, int size, float sigma_r, int bmode, float cval, int contract,
                       int nthreads) {
  bilateral<float>(in, w, h, stride, out, out_stride, smask, size, sigma_r, bmode, cval, contract, nthreads);
}

void orc_bilateral_f64(const double *in, int w, int h, long stride, double *out, long out_stride,
                       const double *smask, int size, double sigma_r, int bmode, double cval, int nthreads) {
  bilateral<double>(in, w, h, stride, out, out_stride, smask, size, sigma_r, bmode, cval, 0, nthreads);
}

// ------------------------------------------------------------------ B5 / CF / L3
// The CPU back end's binomial, cubic and Lanczos-3 filtering accessors
// (runtime/hipacc_cpu_interpolate.hpp:199-520: binomial5, bicubic_spline with
// a = -0.5, lanczos with l = 3 and the <cmath> M_PI) with clamped taps over
// the whole image.  Every product and sum is rounded separately, left to
// right, as the macros' expressions; taps and weights per mode:
//   B5: xb = x_mapped,       columns x_int-1..x_int+2, weight b5((x_frac + 1) - j)
//   CF: xb = x_mapped - 0.5, columns x_int-1..x_int+2, weight cubic((x_frac - 1) + j)
//   L3: xb = x_mapped - 0.5, columns x_int-2..x_int+3, weight lanczos((x_frac - 2) + j),
//       rows y_int-1..y_int+4 with weight lanczos((y_frac - 2) + k) (the macro's row offset);
//       the fifth tap of the second row carries the sixth tap's weight
//       lanczos((x_frac - 2) + 5), as in the macro (and the DSL's accessor)
static float wt_binomial5(float d) {
  d = std::fabs(d);
  if (d < 0.5f) return 6.0f / 8.0f;
  if (d < 1.0f) return 4.0f / 8.0f;
  if (d < 1.5f) return 1.0f / 8.0f;
  return 0.0f;
}

static float wt_cubic(float d) {
  d = std::fabs(d);
  const float a = -0.5f;
  if (d < 1.0f) return (a + 2.0f) * d * d * d - (a + 3.0f) * d * d + 1.0f;
  if (d < 2.0f) return a * d * d * d - 5.0f * a * d * d + 8.0f * a * d - 4.0f * a;
  return 0.0f;
}

static float wt_lanczos(float d) {
  d = std::fabs(d);
  const float l = 3.0f;
  if (d == 0.0f) return 1.0f;
  if (d < l) {
    // M_PI is the double of <cmath>: the arguments and the denominator are
    // evaluated in double, the sines in float
    const float s1 = std::sin((float)(M_PI * (double)d / (double)l));
    const float s2 = std::sin((float)(M_PI * (double)d));
    return (float)((double)(l * (s1 * s2)) / (M_PI * M_PI * (double)d * (double)d));
  }
  return 0.0f;
}

static inline float clamp_tap(const float *src, int sw, int sh, int x, int y) {
  x = x < 0 ? 0 : (x >= sw ? sw - 1 : x);
  y = y < 0 ? 0 : (y >= sh ? sh - 1 : y);
  return src[(long)y * sw + x];
}

static float interp_filtered(const float *src, int sw, int sh, float xm, float ym, int mode) {
  const bool b5 = mode == 3, l3 = mode == 5;
  float xb = b5 ? xm : xm - 0.5f, yb = b5 ? ym : ym - 0.5f;
  if (xb < 0.0f) xb = 0.0f;
  if (yb < 0.0f) yb = 0.0f;
  const int xi = (int)xb, yi = (int)yb;
  const float xf = xb - (float)xi, yf = yb - (float)yi;
  const int n = l3 ? 6 : 4;                        // taps per row / rows
  const int cx0 = l3 ? xi - 2 : xi - 1, cy0 = yi - 1;  // first column / row
  auto w = [&](float d) { return b5 ? wt_binomial5(d) : (l3 ? wt_lanczos(d) : wt_cubic(d)); };
  const float tx = b5 ? xf + 1.0f : (l3 ? xf - 2.0f : xf - 1.0f);
  const float ty = b5 ? yf + 1.0f : (l3 ? yf - 2.0f : yf - 1.0f);
  float out = 0.0f;
  for (int k = 0; k < n; ++k) {
    float row = 0.0f;
    for (int j = 0; j < n; ++j) {
      const int jw = (l3 && k == 1 && j == 4) ? 5 : j;  // the macro's weight for this tap
      const float p = clamp_tap(src, sw, sh, cx0 + j, cy0 + k) * w(b5 ? tx - (float)jw : tx + (float)jw);
      row = j == 0 ? p : row + p;
    }
    const float q = row * w(b5 ? ty - (float)k : ty + (float)k);
    out = k == 0 ? q : out + q;
  }
  return out;
}

void orc_resample_filtered_f32(const float *src, int sw, int sh, float *dst, int dw, int dh, int mode, int contract) {
  const float sx = (float)sw / (float)dw, sy = (float)sh / (float)dh;
  for (int y = 0; y < dh; ++y) {
    const float ym = mapped_coord(sy, y, contract);
    for (int x = 0; x < dw; ++x)
      dst[(long)y * dw + x] = interp_filtered(src, sw, sh, mapped_coord(sx, x, contract), ym, mode);
  }
}

void orc_resample_nn_f32(const float *src, int sw, int sh, float *dst, int dw, int dh, int contract) {
  resample_nn<float>(src, sw, sh, dst, dw, dh, contract);
}

void orc_resample_lf_f32(const float *src, int sw, int sh, float *dst, int dw, int dh, int contract) {
  resample_lf<float>(src, sw, sh, dst, dw, dh, contract);
}

void orc_pyramid_decompose_f32(float **gauss, float **lap, int w, int h, int levels, const float *mask,
                               int msize, int bmode, int contract, int nthreads) {
  pyramid_decompose<float>(gauss, lap, w, h, levels, mask, msize, bmode, contract, nthreads);
}

void orc_pyramid_decompose_f64(double **gauss, double **lap, int w, int h, int levels, const double *mask,
                               int msize, int bmode, int nthreads) {
  pyramid_decompose<double>(gauss, lap, w, h, levels, mask, msize, bmode, 0, nthreads);
}

// Restore (Gaussian_Laplacian_Pyramid/src/main.cpp:238-245): G_l = LF(G_{l+1}) + L_l.
void orc_pyramid_collapse_f32(float **out, float **lap, int w, int h, int levels, int contract) {
  std::vector<int> lw(levels), lh(levels);
  lw[0] = w;
  lh[0] = h;
  for (int l = 1; l < levels; ++l) {
    lw[l] = lw[l - 1] / 2;
    lh[l] = lh[l - 1] / 2;
  }
  for (int l = levels - 2; l >= 0; --l) {
    std::vector<float> up((size_t)lw[l] * lh[l]);
    resample_lf<float>(out[l + 1], lw[l + 1], lh[l + 1], up.data(), lw[l], lh[l], contract);
    for (long p = 0; p < (long)lw[l] * lh[l]; ++p) out[l][p] = up[p] + lap[l][p];
  }
}

// ---------------------------------------------------------------------------
// Differentiation oracle (FP64).  Forward: y1 = conv(x, mask) with boundary
// `bmode`; y = bilateral(y1) with the spatial mask `smask` and range sigma
// sigma_r over the same boundary; loss = mean((y - t)^2).
// Adjoint (hand-derived, FP64):
//   w_po = s_o * exp(-c (y1_{q} - y1_p)^2), q = r(p+o), c = 1/(2 sigma_r^2)
//   y_p = N_p / W_p, N_p = sum_o w_po y1_q, W_p = sum_o w_po
//   g_p = dL/dy_p = 2 (y_p - t_p) / n
//   dL/dy1_q += g_p / W_p * w_po * (1 - 2c (y1_q - y_p)(y1_q - y1_p))
//   dL/dy1_p += g_p / W_p * sum_o w_po (y1_q - y_p) * 2c (y1_q - y1_p)
//   dL/dc     = sum_p g_p / W_p * sum_o w_po (y1_q - y_p) * (-(y1_q - y1_p)^2)
//   dL/dsigma = dL/dc * (-1 / sigma^3)
//   dL/dx_{r(p+o)} += m_o * dL/dy1_p ;  dL/dm_o = sum_p dL/dy1_p * x_{r(p+o)}
// CONSTANT taps carry no gradient; CLAMP/MIRROR/REPEAT scatter to the remapped
// pixel, which is the transpose of the boundary remap.
// ---------------------------------------------------------------------------
namespace {

struct C5Fwd {
  std::vector<double> y1, y, W;
};

void c5_forward(const double *x, int w, int h, const double *mask, int mk, const double *smask, int sk,
                double sigma_r, int bmode, int nthreads, C5Fwd &f) {
  const long n = (long)w * h;
  f.y1.assign(n, 0.0);
  f.y.assign(n, 0.0);
  f.W.assign(n, 0.0);
  local_op<double>(x, w, 0, 0, w, h, f.y1.data(), w, 0, 0, w, h, mask, nullptr, mk, mk, ORC_SUM, bmode, 0.0,
                   0, nthreads);
  const int r = sk / 2;
  const double c = 0.5 / (sigma_r * sigma_r);
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int py = 0; py < h; ++py)
    for (int px = 0; px < w; ++px) {
      const double ctr = f.y1[(long)py * w + px];
      double N = 0, Wt = 0;
      for (int oy = 0; oy < sk; ++oy)
        for (int ox = 0; ox < sk; ++ox) {
          const int qx = remap_idx(bmode, px + ox - r, 0, w), qy = remap_idx(bmode, py + oy - r, 0, h);
          const double v = (qx == kConstIdx || qy == kConstIdx) ? 0.0 : f.y1[(long)qy * w + qx];
          const double d = v - ctr;
          const double wt = smask[oy * sk + ox] * std::exp(-c * d * d);
          N += wt * v;
          Wt += wt;
        }
      f.W[(long)py * w + px] = Wt;
      f.y[(long)py * w + px] = N / Wt;
    }
}

}  // namespace

double orc_c5_loss_f64(const double *x, const double *t, int w, int h, const double *mask, int mk,
                       const double *smask, int sk, double sigma_r, int bmode, int nthreads) {
  C5Fwd f;
  c5_forward(x, w, h, mask, mk, smask, sk, sigma_r, bmode, nthreads, f);
  const long n = (long)w * h;
  double L = 0;
  for (long p = 0; p < n; ++p) L += (f.y[p] - t[p]) * (f.y[p] - t[p]);
  return L / (double)n;
}

double orc_c5_grad_f64(const double *x, const double *t, int w, int h, const double *mask, int mk,
                       const double *smask, int sk, double sigma_r, int bmode, double *dx, double *dmask,
                       double *dsigma, int nthreads) {
  C5Fwd f;
  c5_forward(x, w, h, mask, mk, smask, sk, sigma_r, bmode, nthreads, f);
  const long n = (long)w * h;
  double L = 0;
  for (long p = 0; p < n; ++p) L += (f.y[p] - t[p]) * (f.y[p] - t[p]);
  L /= (double)n;
  const int r = sk / 2;
  const double c = 0.5 / (sigma_r * sigma_r);
  std::vector<double> dy1(n, 0.0);
  double dc = 0;
  for (int py = 0; py < h; ++py)
    for (int px = 0; px < w; ++px) {
      const long p = (long)py * w + px;
      const double g = 2.0 * (f.y[p] - t[p]) / (double)n;
      const double a = g / f.W[p];
      const double ctr = f.y1[p], yp = f.y[p];
      double center_acc = 0;
      for (int oy = 0; oy < sk; ++oy)
        for (int ox = 0; ox < sk; ++ox) {
          const int qx = remap_idx(bmode, px + ox - r, 0, w), qy = remap_idx(bmode, py + oy - r, 0, h);
          const bool cst = (qx == kConstIdx || qy == kConstIdx);
          const double v = cst ? 0.0 : f.y1[(long)qy * w + qx];
          const double d = v - ctr;
          const double wt = smask[oy * sk + ox] * std::exp(-c * d * d);
          if (!cst) dy1[(long)qy * w + qx] += a * wt * (1.0 - 2.0 * c * (v - yp) * d);
          center_acc += wt * (v - yp) * 2.0 * c * d;
          dc += a * wt * (v - yp) * (-d * d);
        }
      dy1[p] += a * center_acc;
    }
  if (dsigma) *dsigma = dc * (-1.0 / (sigma_r * sigma_r * sigma_r));
  const int rm = mk / 2;
  if (dx) std::fill(dx, dx + n, 0.0);
  if (dmask) std::fill(dmask, dmask + mk * mk, 0.0);
  for (int py = 0; py < h; ++py)
    for (int px = 0; px < w; ++px) {
      const double gp = dy1[(long)py * w + px];
      for (int oy = 0; oy < mk; ++oy)
        for (int ox = 0; ox < mk; ++ox) {
          const int qx = remap_idx(bmode, px + ox - rm, 0, w), qy = remap_idx(bmode, py + oy - rm, 0, h);
          if (qx == kConstIdx || qy == kConstIdx) continue;
          if (dx) dx[(long)qy * w + qx] += mask[oy * mk + ox] * gp;
          if (dmask) dmask[oy * mk + ox] += gp * x[(long)qy * w + qx];
        }
    }
  return L;
}

// Harris corner program (samples-public/3_Preprocessing/Harris_Corner/src/main.cpp:56-166,
// 258-307, SIZE 3): every local operator reads through the boundary remap
// (CONSTANT taps read 0).
//   dx = (short)(sum_dom(in * cx) / 6), dy likewise with cy (Domain: zero cells
//        skipped; short sum, C division truncating toward zero)
//   sx = dx * dx, sy = dy * dy, sxy = dx * dy (short)
//   Gx = (short)(sum_mask(sx * m) / 16) over the 3x3 [1 2 1; 2 4 2; 1 2 1] mask
//        (int sum), Gy, Gxy likewise
//   R  = (float)(Gx * Gy - Gxy * Gxy) - (k * (float)(Gx + Gy)) * (float)(Gx + Gy),
//        each float operation rounded separately; out = R > threshold
void orc_harris_u8(const uint8_t *in, int w, int h, int bmode, float k, float threshold, uint8_t *out,
                   int nthreads) {
  static const int cx[9] = {-1, 0, 1, -1, 0, 1, -1, 0, 1};
  static const int cy[9] = {-1, -1, -1, 0, 0, 0, 1, 1, 1};
  static const int g[9] = {1, 2, 1, 2, 4, 2, 1, 2, 1};
  const long n = (long)w * h;
  std::vector<int16_t> sx(n), sy(n), sxy(n);
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      int16_t ax = 0, ay = 0;
      for (int oy = -1; oy <= 1; ++oy)
        for (int ox = -1; ox <= 1; ++ox) {
          const int rx = remap_idx(bmode, x + ox, 0, w), ry = remap_idx(bmode, y + oy, 0, h);
          const int v = (rx == kConstIdx || ry == kConstIdx) ? 0 : in[(long)ry * w + rx];
          const int kx = cx[(oy + 1) * 3 + ox + 1], ky = cy[(oy + 1) * 3 + ox + 1];
          if (kx) ax = (int16_t)(ax + (int16_t)(v * kx));
          if (ky) ay = (int16_t)(ay + (int16_t)(v * ky));
        }
      const int16_t dx = (int16_t)(ax / 6), dy = (int16_t)(ay / 6);
      const long p = (long)y * w + x;
      sx[p] = (int16_t)(dx * dx);
      sy[p] = (int16_t)(dy * dy);
      sxy[p] = (int16_t)(dx * dy);
    }
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      int a = 0, b = 0, c = 0;
      for (int oy = -1; oy <= 1; ++oy)
        for (int ox = -1; ox <= 1; ++ox) {
          const int rx = remap_idx(bmode, x + ox, 0, w), ry = remap_idx(bmode, y + oy, 0, h);
          const bool cst = rx == kConstIdx || ry == kConstIdx;
          const long q = cst ? 0 : (long)ry * w + rx;
          const int m = g[(oy + 1) * 3 + ox + 1];
          a += (cst ? 0 : sx[q]) * m;
          b += (cst ? 0 : sy[q]) * m;
          c += (cst ? 0 : sxy[q]) * m;
        }
      const int gx = (int16_t)(a / 16), gy = (int16_t)(b / 16), gxy = (int16_t)(c / 16);
      const float det = (float)(gx * gy - gxy * gxy);
      const float tr = (float)(gx + gy);
      const float kt = k * tr;
      const float kt2 = kt * tr;
      const float R = det - kt2;
      out[(long)y * w + x] = R > threshold ? 1 : 0;
    }
}

// Unsharp program (samples-public/1_Local_Operators/Unsharp/src/main.cpp:53-149,203-247,
// SIZE 3), the blur reading the luminance through the boundary remap:
//   gray  = (float)((double)(0.2126f * powf(R, c)) + 0.7152 * powf(G, c) + 0.0722 * powf(B, c)),
//           c = 1.0f / 2.2f (the sample's float and double literals)
//   blur  = sum_mask gray * m, row-major, products and sums rounded separately
//   sharp = 2 * gray - blur;  ratio = sharp / max(gray, 0.01f)
//   out   = (R * ratio, G * ratio, B * ratio, A), each channel the float
//           product converted to uchar as the CPU back end does: truncated to an
//           int, low byte kept
// gray_out (may be NULL) receives the luminance.
void orc_unsharp_u8x4(const uint8_t *rgba, int w, int h, int bmode, uint8_t *out, float *gray_out, int nthreads) {
  static const float m[9] = {0.057118f, 0.124758f, 0.057118f, 0.124758f, 0.272496f,
                             0.124758f, 0.057118f, 0.124758f, 0.057118f};
  const long n = (long)w * h;
  std::vector<float> gray(n);
  const float c = 1.0f / 2.2f;
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (long p = 0; p < n; ++p) {
    const float xg = powf((float)rgba[4 * p], c), yg = powf((float)rgba[4 * p + 1], c),
                zg = powf((float)rgba[4 * p + 2], c);
    const float t0 = 0.2126f * xg;
    gray[p] = (float)(((double)t0 + 0.7152 * (double)yg) + 0.0722 * (double)zg);
  }
#pragma omp parallel for schedule(static) num_threads(nthreads > 0 ? nthreads : 1)
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      float blur = 0.0f;
      for (int oy = -1; oy <= 1; ++oy)
        for (int ox = -1; ox <= 1; ++ox) {
          const int rx = remap_idx(bmode, x + ox, 0, w), ry = remap_idx(bmode, y + oy, 0, h);
          const float v = (rx == kConstIdx || ry == kConstIdx) ? 0.0f : gray[(long)ry * w + rx];
          const float t = m[(oy + 1) * 3 + ox + 1] * v;
          blur = blur + t;
        }
      const long p = (long)y * w + x;
      const float g2 = 2.0f * gray[p];
      const float sharp = g2 - blur;
      const float ratio = sharp / std::max(gray[p], 0.01f);
      for (int ch = 0; ch < 3; ++ch) {
        const float v = (float)rgba[4 * p + ch] * ratio;
        out[4 * p + ch] = (uint8_t)((int32_t)v & 0xff);
      }
      out[4 * p + 3] = rgba[4 * p + 3];
    }
  if (gray_out) std::copy(gray.begin(), gray.end(), gray_out);
}

// Adjoint of the bilateral filter in FP64, the forward of
// samples-public/3_Preprocessing/Bilateral_Filter/src/main.cpp:63-77 (the
// `bilateral` template above, taps through the boundary remap, CONSTANT taps
// reading cval):  y_p = N_p / W_p,  N_p = sum_o w_po v_q,  W_p = sum_o w_po,
// w_po = smask_o exp(-c (v_q - in_p)^2),  c = 1 / (2 sigma_r^2),  q = r(p + o).
// Given g = dL/dy:
//   a_p = g_p / W_p
//   dL/din_q += a_p w_po (1 - 2c (v_q - y_p)(v_q - in_p))    (q a pixel, not the constant)
//   dL/din_p += a_p sum_o w_po (v_q - y_p) 2c (v_q - in_p)
//   dL/dc     = sum_p a_p sum_o w_po (v_q - y_p) (-(v_q - in_p)^2),  dL/dsigma_r = -dL/dc / sigma_r^3
// grad_in (w x h, dense) is overwritten; returns dL/dsigma_r.
double orc_bilateral_adjoint_f64(const double *in, const double *g, int w, int h, const double *smask, int size,
                                 double sigma_r, int bmode, double cval, double *grad_in) {
  const int r = size / 2;
  const double c = 0.5 / (sigma_r * sigma_r);
  const long n = (long)w * h;
  std::fill(grad_in, grad_in + n, 0.0);
  double dc = 0.0;
  std::vector<double> vq((size_t)size * size);
  std::vector<long> iq((size_t)size * size);
  for (int py = 0; py < h; ++py)
    for (int px = 0; px < w; ++px) {
      const long p = (long)py * w + px;
      const double ctr = in[p];
      double N = 0.0, W = 0.0;
      for (int oy = 0; oy < size; ++oy)
        for (int ox = 0; ox < size; ++ox) {
          const int k = oy * size + ox;
          const int qx = remap_idx(bmode, px + ox - r, 0, w), qy = remap_idx(bmode, py + oy - r, 0, h);
          iq[k] = (qx == kConstIdx || qy == kConstIdx) ? -1 : (long)qy * w + qx;
          vq[k] = iq[k] < 0 ? cval : in[iq[k]];
          const double d = vq[k] - ctr;
          const double wt = smask[k] * std::exp(-c * d * d);
          N += wt * vq[k];
          W += wt;
        }
      const double y = N / W, a = g[p] / W;
      double ctr_acc = 0.0;
      for (int k = 0; k < size * size; ++k) {
        const double d = vq[k] - ctr;
        const double wt = smask[k] * std::exp(-c * d * d);
        if (iq[k] >= 0) grad_in[iq[k]] += a * wt * (1.0 - 2.0 * c * (vq[k] - y) * d);
        ctr_acc += wt * (vq[k] - y) * 2.0 * c * d;
        dc += a * wt * (vq[k] - y) * (-d * d);
      }
      grad_in[p] += a * ctr_acc;
    }
  return dc * (-1.0 / (sigma_r * sigma_r * sigma_r));
}

}  // extern "C"

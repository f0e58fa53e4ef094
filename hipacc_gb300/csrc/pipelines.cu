// pipelines.cu -- two multi-kernel sample programs of the reference as hand-fused
// kernel chains, with their plain per-kernel launch structure for comparison.
//
// Harris corner (samples-public/3_Preprocessing/Harris_Corner/src/main.cpp:56-166,
// 258-307, the 3x3 configuration): nine kernels in the reference --
//   dx = (short)(sum over Domain(mx) in * mx / 6), dy likewise with my
//        (mx = [-1 0 1] in every row, my = its transpose; short sums, C
//        division truncating toward zero)
//   sx = dx^2, sy = dy^2, sxy = dx * dy                     (short)
//   Gx = (short)(sum over the 3x3 mask [1 2 1; 2 4 2; 1 2 1] of sx * m / 16),
//        Gy, Gxy likewise (int sums)
//   R  = (float)(Gx Gy - Gxy^2) - (k (float)(Gx + Gy)) (float)(Gx + Gy),
//        every float operation rounded separately;  out = R > threshold ? 1 : 0
// Every local operator reads through the boundary remap (CONSTANT taps read
// 0).  Fused form: one kernel per 64 x 16 tile stages the u8 input with a
// 2-pixel halo, forms the products on the tile plus a 1-pixel halo in shared
// memory (a halo cell outside the image holds the products at its remapped
// position, as the Gaussian reads them), and writes the 0/1 image: 1 byte in
// and 1 byte out per pixel instead of the nine launches' short intermediates.
//
// Unsharp (samples-public/1_Local_Operators/Unsharp/src/main.cpp:53-149,203-247,
// 3x3): five kernels in the reference --
//   gray  = 0.2126f * powf(R, c) + 0.7152 * powf(G, c) + 0.0722 * powf(B, c),
//           c = 1.0f / 2.2f; the two last literals are double, so the sum is
//           evaluated in double and rounded to float
//   blur  = 3x3 convolution of gray (products and sums rounded separately)
//   sharp = 2 gray - blur;  ratio = sharp / max(gray, 0.01f)
//   out   = (R ratio, G ratio, B ratio, A), each channel the float product
//           converted to uchar as the CPU back end does (truncated to an int,
//           low byte kept)
// The luminance depends on the bytes only: the powf terms come from 256-entry
// tables computed on the host with the host's powf (the CPU back end's own
// function) and the double products split into float pairs.  The double sum
// is reproduced by an exact float-float sum; a pixel whose sum lies within a
// tiny margin of a float rounding midpoint (about 1 in 10^5) is recomputed in
// FP64, so the result equals the double evaluation bit for bit.  Fused form:
// one kernel per 32 x 16 tile stages the luminance with a 1-pixel halo and
// writes the uchar4 result: 8 bytes per pixel instead of the five launches'
// float intermediates.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "hgb_internal.cuh"

namespace hgb {
namespace {

// ------------------------------------------------------------------ Harris
constexpr int HC_TW = 64, HC_TH = 16, HC_T = 256;
constexpr int HC_IW = HC_TW + 4, HC_IH = HC_TH + 4;  // staged input, 2-pixel halo
constexpr int HC_DW = HC_TW + 2, HC_DH = HC_TH + 2;  // products, 1-pixel halo

struct HarrisParams {
  const uint8_t *in;
  int64_t in_p, in_b;
  uint8_t *out;
  int64_t out_p, out_b;
  int w, h, bmode;
  float k, threshold;
  // plain launch structure: short intermediates [image][h][w]
  int16_t *dx, *dy, *sx, *sy, *sxy, *dxy;
};

__device__ __forceinline__ int hc_in(const HarrisParams &p, const uint8_t *img, int vx, int vy) {
  const int rx = remap(p.bmode, vx, 0, p.w), ry = remap(p.bmode, vy, 0, p.h);
  if (rx == (int)0x80000000 || ry == (int)0x80000000) return 0;
  return img[(int64_t)ry * p.in_p + rx];
}

// the two derivative sums at a pixel from a 3x3 neighbourhood v[row][col]
__device__ __forceinline__ void hc_deriv(const int v[3][3], int16_t &dx, int16_t &dy) {
  // Domain order, row-major; the short accumulator of the sample
  int16_t ax = 0, ay = 0;
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    ax = (int16_t)(ax + (int16_t)(-v[r][0]));
    ax = (int16_t)(ax + (int16_t)v[r][2]);
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) ay = (int16_t)(ay + (int16_t)(-v[0][c]));
#pragma unroll
  for (int c = 0; c < 3; ++c) ay = (int16_t)(ay + (int16_t)v[2][c]);
  dx = (int16_t)(ax / 6);
  dy = (int16_t)(ay / 6);
}

__device__ __forceinline__ uint8_t hc_response(const HarrisParams &p, int gx, int gy, int gxy) {
  const float det = __int2float_rn(gx * gy - gxy * gxy);
  const float tr = __int2float_rn(gx + gy);
  const float R = __fsub_rn(det, __fmul_rn(__fmul_rn(p.k, tr), tr));
  return R > p.threshold ? 1 : 0;
}

__global__ void __launch_bounds__(HC_T) harris_fused_kernel(const __grid_constant__ HarrisParams p) {
  __shared__ uint8_t s_in[HC_IH * HC_IW];
  __shared__ int s_sx[HC_DH * HC_DW], s_sy[HC_DH * HC_DW], s_sxy[HC_DH * HC_DW];
  const int b = blockIdx.z, X0 = blockIdx.x * HC_TW, Y0 = blockIdx.y * HC_TH;
  const uint8_t *img = p.in + (int64_t)b * p.in_b;
  const bool inside = X0 - 2 >= 0 && X0 + HC_TW + 2 <= p.w && Y0 - 2 >= 0 && Y0 + HC_TH + 2 <= p.h;
  for (int c = threadIdx.x; c < HC_IH * HC_IW; c += HC_T) {
    const int r = c / HC_IW, q = c - r * HC_IW;
    s_in[c] = inside ? __ldg(img + (int64_t)(Y0 - 2 + r) * p.in_p + X0 - 2 + q)
                     : (uint8_t)hc_in(p, img, X0 - 2 + q, Y0 - 2 + r);
  }
  __syncthreads();
  for (int c = threadIdx.x; c < HC_DH * HC_DW; c += HC_T) {
    const int r = c / HC_DW, q = c - r * HC_DW;
    const int vx = X0 - 1 + q, vy = Y0 - 1 + r;
    int v[3][3];
    int16_t dx = 0, dy = 0;
    if (vx >= 0 && vx < p.w && vy >= 0 && vy < p.h) {
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) v[i][j] = s_in[(r + i) * HC_IW + q + j];
      hc_deriv(v, dx, dy);
    } else if (p.bmode != HGB_BOUNDARY_CONSTANT) {
      // the Gaussian reads the products at the remapped position
      const int ux = remap(p.bmode, vx, 0, p.w), uy = remap(p.bmode, vy, 0, p.h);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) v[i][j] = hc_in(p, img, ux - 1 + j, uy - 1 + i);
      hc_deriv(v, dx, dy);
    }
    s_sx[c] = (int16_t)(dx * dx);
    s_sy[c] = (int16_t)(dy * dy);
    s_sxy[c] = (int16_t)(dx * dy);
  }
  __syncthreads();
  const int tx = threadIdx.x % HC_TW;
  uint8_t *out = p.out + (int64_t)b * p.out_b;
  for (int py = threadIdx.x / HC_TW; py < HC_TH; py += HC_T / HC_TW) {
    const int x = X0 + tx, y = Y0 + py;
    if (x >= p.w || y >= p.h) continue;
    int a = 0, bb = 0, cc = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const int m = (i == 1 ? 2 : 1) * (j == 1 ? 2 : 1);
        const int o = (py + i) * HC_DW + tx + j;
        a += s_sx[o] * m;
        bb += s_sy[o] * m;
        cc += s_sxy[o] * m;
      }
    out[(int64_t)y * p.out_p + x] = hc_response(p, (int16_t)(a / 16), (int16_t)(bb / 16), (int16_t)(cc / 16));
  }
}

// ---- the reference's nine launches (one pixel per thread, short intermediates)
__device__ __forceinline__ bool hc_pixel(const HarrisParams &p, int &x, int &y, int &b) {
  x = blockIdx.x * 32 + (threadIdx.x & 31);
  y = blockIdx.y * 8 + (threadIdx.x >> 5);
  b = blockIdx.z;
  return x < p.w && y < p.h;
}
__device__ __forceinline__ int64_t hc_at(const HarrisParams &p, int b, int x, int y) {
  return ((int64_t)b * p.h + y) * p.w + x;
}

__global__ void __launch_bounds__(256) harris_deriv_kernel(const __grid_constant__ HarrisParams p, int which) {
  int x, y, b;
  if (!hc_pixel(p, x, y, b)) return;
  const uint8_t *img = p.in + (int64_t)b * p.in_b;
  int v[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) v[i][j] = hc_in(p, img, x - 1 + j, y - 1 + i);
  int16_t dx, dy;
  hc_deriv(v, dx, dy);
  (which ? p.dy : p.dx)[hc_at(p, b, x, y)] = which ? dy : dx;
}

__global__ void __launch_bounds__(256) harris_square_kernel(const __grid_constant__ HarrisParams p, int which) {
  int x, y, b;
  if (!hc_pixel(p, x, y, b)) return;
  const int64_t o = hc_at(p, b, x, y);
  const int16_t a = which == 1 ? p.dy[o] : p.dx[o], c = which == 0 ? p.dx[o] : p.dy[o];
  (which == 0 ? p.sx : which == 1 ? p.sy : p.sxy)[o] = (int16_t)(a * c);
}

__global__ void __launch_bounds__(256) harris_gauss_kernel(const __grid_constant__ HarrisParams p, const int16_t *src,
                                                           int16_t *dst) {
  int x, y, b;
  if (!hc_pixel(p, x, y, b)) return;
  int s = 0;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int rx = remap(p.bmode, x - 1 + j, 0, p.w), ry = remap(p.bmode, y - 1 + i, 0, p.h);
      const int v = (rx == (int)0x80000000 || ry == (int)0x80000000) ? 0 : src[hc_at(p, b, rx, ry)];
      s += v * ((i == 1 ? 2 : 1) * (j == 1 ? 2 : 1));
    }
  dst[hc_at(p, b, x, y)] = (int16_t)(s / 16);
}

__global__ void __launch_bounds__(256) harris_response_kernel(const __grid_constant__ HarrisParams p) {
  int x, y, b;
  if (!hc_pixel(p, x, y, b)) return;
  const int64_t o = hc_at(p, b, x, y);
  // the sample's Gaussians of sx and sy land in the dx and dy images
  p.out[(int64_t)b * p.out_b + (int64_t)y * p.out_p + x] = hc_response(p, p.dx[o], p.dy[o], p.dxy[o]);
}

// ------------------------------------------------------------------ Unsharp
constexpr int US_TW = 32, US_TH = 16, US_T = 256;
constexpr int US_GW = US_TW + 2, US_GH = US_TH + 2;

// luminance terms per byte value (host-computed, see the header comment)
struct UnsTables {
  float t0[256];          // 0.2126f * powf(v, c)
  float b1h[256], b1l[256];  // 0.7152 * powf(v, c) as a float pair
  float b2h[256], b2l[256];  // 0.0722 * powf(v, c) as a float pair
  double b1[256], b2[256];   // the double products, for the FP64 recomputation
};

struct UnsharpParams {
  const uchar4 *in;
  int64_t in_p, in_b;  // uchar4 elements
  uchar4 *out;
  int64_t out_p, out_b;
  int w, h, bmode;
  int tiles_x, tiles_y, ntiles;
  const UnsTables *tab;  // device copy
  // plain launch structure: float intermediates [image][h][w]
  float *gray, *blur, *sharp, *ratio;
};

__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (float)(((double)t0 + b1) + b2) for the bytes (r, g, bl)
__device__ __forceinline__ float uns_gray(const UnsTables &T, const float *t0, const float *b1h, const float *b1l,
                                          const float *b2h, const float *b2l, int r, int g, int bl) {
  const float a = t0[r];
  float s, e1, e2;
  two_sum(a, b1h[g], s, e1);
  two_sum(s, b2h[bl], s, e2);
  const float e = __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(b1l[g], b2l[bl]));
  const float y = __fadd_rn(s, e);
  if (y == 0.0f) return y;
  // distance of the exact sum from the rounding midpoints around y
  const float rho = __fadd_rn(__fsub_rn(s, y), e);
  const float ulp = __int_as_float(__float_as_int(y) & 0x7f800000) * 1.1920928955078125e-7f;  // 2^-23
  const bool pow2 = (__float_as_int(y) & 0x007fffff) == 0;
  const float below = pow2 ? 0.25f * ulp : 0.5f * ulp;
  const float margin = y * 9.094947017729282e-13f;  // 2^-40: far above every error of the float-float sum
  if (fabsf(rho - 0.5f * ulp) > margin && fabsf(rho + below) > margin) return y;
  return (float)__dadd_rn(__dadd_rn((double)a, T.b1[g]), T.b2[bl]);
}

__device__ __forceinline__ uchar4 uns_scale(uchar4 v, float r) {
  // (uchar)(v * r): truncated to an int, low byte kept
  v.x = (unsigned char)(__float2int_rz(__fmul_rn((float)v.x, r)) & 0xff);
  v.y = (unsigned char)(__float2int_rz(__fmul_rn((float)v.y, r)) & 0xff);
  v.z = (unsigned char)(__float2int_rz(__fmul_rn((float)v.z, r)) & 0xff);
  return v;
}

__device__ __forceinline__ float uns_blur(const float *g, int stride) {
  const float m0 = 0.057118f, m1 = 0.124758f, m2 = 0.272496f;
  const float m[9] = {m0, m1, m0, m1, m2, m1, m0, m1, m0};
  float s = 0.0f;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) s = __fadd_rn(s, __fmul_rn(m[i * 3 + j], g[i * stride + j]));
  return s;
}

__device__ __forceinline__ float uns_ratio(float g, float blur) {
  const float sharp = __fsub_rn(__fmul_rn(2.0f, g), blur);
  return __fdiv_rn(sharp, fmaxf(g, 0.01f));
}

__device__ __forceinline__ uchar4 uns_load(const UnsharpParams &p, const uchar4 *img, int vx, int vy, bool &cst) {
  const int rx = remap(p.bmode, vx, 0, p.w), ry = remap(p.bmode, vy, 0, p.h);
  cst = rx == (int)0x80000000 || ry == (int)0x80000000;
  return cst ? make_uchar4(0, 0, 0, 0) : img[(int64_t)ry * p.in_p + rx];
}

__global__ void __launch_bounds__(US_T) unsharp_fused_kernel(const __grid_constant__ UnsharpParams p) {
  __shared__ float t0[256], b1h[256], b1l[256], b2h[256], b2l[256];
  __shared__ float s_g[US_GH * US_GW];
  __shared__ uchar4 s_px[US_TH * US_TW];
  const UnsTables &T = *p.tab;
  for (int i = threadIdx.x; i < 256; i += US_T) {
    t0[i] = T.t0[i];
    b1h[i] = T.b1h[i];
    b1l[i] = T.b1l[i];
    b2h[i] = T.b2h[i];
    b2l[i] = T.b2l[i];
  }
  // persistent: the CTA walks tiles blockIdx.x, blockIdx.x + gridDim.x, ...
  for (int t = blockIdx.x; t < p.ntiles; t += gridDim.x) {
    const int per = p.tiles_x * p.tiles_y;
    const int b = t / per, r0 = t - b * per;
    const int Y0 = (r0 / p.tiles_x) * US_TH, X0 = (r0 % p.tiles_x) * US_TW;
    const uchar4 *img = p.in + (int64_t)b * p.in_b;
    __syncthreads();  // tables staged / the previous tile's reads done
    for (int c = threadIdx.x; c < US_GH * US_GW; c += US_T) {
      const int r = c / US_GW, q = c - r * US_GW;
      bool cst;
      const uchar4 v = uns_load(p, img, X0 - 1 + q, Y0 - 1 + r, cst);
      s_g[c] = cst ? 0.0f : uns_gray(T, t0, b1h, b1l, b2h, b2l, v.x, v.y, v.z);
      if (r >= 1 && r <= US_TH && q >= 1 && q <= US_TW) s_px[(r - 1) * US_TW + q - 1] = v;
    }
    __syncthreads();
    const int tx = threadIdx.x % US_TW;
    uchar4 *out = p.out + (int64_t)b * p.out_b;
    for (int py = threadIdx.x / US_TW; py < US_TH; py += US_T / US_TW) {
      const int x = X0 + tx, y = Y0 + py;
      if (x >= p.w || y >= p.h) continue;
      const float g = s_g[(py + 1) * US_GW + tx + 1];
      const float ratio = uns_ratio(g, uns_blur(&s_g[py * US_GW + tx], US_GW));
      out[(int64_t)y * p.out_p + x] = uns_scale(s_px[py * US_TW + tx], ratio);
    }
  }
}

// ---- the reference's five launches (one pixel per thread, float intermediates)
__device__ __forceinline__ bool us_pixel(const UnsharpParams &p, int &x, int &y, int &b) {
  x = blockIdx.x * 32 + (threadIdx.x & 31);
  y = blockIdx.y * 8 + (threadIdx.x >> 5);
  b = blockIdx.z;
  return x < p.w && y < p.h;
}
__device__ __forceinline__ int64_t us_at(const UnsharpParams &p, int b, int x, int y) {
  return ((int64_t)b * p.h + y) * p.w + x;
}

__global__ void __launch_bounds__(256) unsharp_gray_kernel(const __grid_constant__ UnsharpParams p) {
  int x, y, b;
  if (!us_pixel(p, x, y, b)) return;
  const UnsTables &T = *p.tab;
  const uchar4 v = p.in[(int64_t)b * p.in_b + (int64_t)y * p.in_p + x];
  p.gray[us_at(p, b, x, y)] = uns_gray(T, T.t0, T.b1h, T.b1l, T.b2h, T.b2l, v.x, v.y, v.z);
}

__global__ void __launch_bounds__(256) unsharp_blur_kernel(const __grid_constant__ UnsharpParams p) {
  int x, y, b;
  if (!us_pixel(p, x, y, b)) return;
  float g[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const int rx = remap(p.bmode, x - 1 + j, 0, p.w), ry = remap(p.bmode, y - 1 + i, 0, p.h);
      g[i * 3 + j] = (rx == (int)0x80000000 || ry == (int)0x80000000) ? 0.0f : p.gray[us_at(p, b, rx, ry)];
    }
  p.blur[us_at(p, b, x, y)] = uns_blur(g, 3);
}

__global__ void __launch_bounds__(256) unsharp_sharp_kernel(const __grid_constant__ UnsharpParams p) {
  int x, y, b;
  if (!us_pixel(p, x, y, b)) return;
  const int64_t o = us_at(p, b, x, y);
  p.sharp[o] = __fsub_rn(__fmul_rn(2.0f, p.gray[o]), p.blur[o]);
}

__global__ void __launch_bounds__(256) unsharp_ratio_kernel(const __grid_constant__ UnsharpParams p) {
  int x, y, b;
  if (!us_pixel(p, x, y, b)) return;
  const int64_t o = us_at(p, b, x, y);
  p.ratio[o] = __fdiv_rn(p.sharp[o], fmaxf(p.gray[o], 0.01f));
}

__global__ void __launch_bounds__(256) unsharp_scale_kernel(const __grid_constant__ UnsharpParams p) {
  int x, y, b;
  if (!us_pixel(p, x, y, b)) return;
  p.out[(int64_t)b * p.out_b + (int64_t)y * p.out_p + x] =
      uns_scale(p.in[(int64_t)b * p.in_b + (int64_t)y * p.in_p + x], p.ratio[us_at(p, b, x, y)]);
}

// host tables, built once per process with the host's powf; device copies per device
std::mutex g_uns_mu;
bool g_uns_host_ready = false;
UnsTables g_uns_host;
constexpr int kMaxDev = 64;
UnsTables *g_uns_dev[kMaxDev] = {};

int unsharp_tables(const UnsTables **out) {
  int dev = 0;
  HGB_CHECK_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDev) return set_error(HGB_ERR_LIMIT, "hgb_unsharp: device index too large");
  std::lock_guard<std::mutex> lk(g_uns_mu);
  if (!g_uns_host_ready) {
    const float c = 1.0f / 2.2f;
    for (int v = 0; v < 256; ++v) {
      const float pv = powf((float)v, c);
      g_uns_host.t0[v] = 0.2126f * pv;
      const double d1 = 0.7152 * (double)pv, d2 = 0.0722 * (double)pv;
      g_uns_host.b1[v] = d1;
      g_uns_host.b2[v] = d2;
      g_uns_host.b1h[v] = (float)d1;
      g_uns_host.b1l[v] = (float)(d1 - (double)g_uns_host.b1h[v]);
      g_uns_host.b2h[v] = (float)d2;
      g_uns_host.b2l[v] = (float)(d2 - (double)g_uns_host.b2h[v]);
    }
    g_uns_host_ready = true;
  }
  if (!g_uns_dev[dev]) {
    UnsTables *d = nullptr;
    HGB_CHECK_CUDA(cudaMalloc((void **)&d, sizeof(UnsTables)));
    const cudaError_t e = cudaMemcpy(d, &g_uns_host, sizeof(UnsTables), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(d);
      return cuda_error(e, "hgb_unsharp: table upload");
    }
    g_uns_dev[dev] = d;
  }
  *out = g_uns_dev[dev];
  return HGB_OK;
}

}  // namespace
}  // namespace hgb

using namespace hgb;

extern "C" int hgb_harris_corner(const hgb_view *in, const hgb_view *out, float k, float threshold, int boundary,
                                 int mode, void *stream) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  rc = check_view(out, "out");
  if (rc) return rc;
  HGB_REQUIRE(in->dtype == HGB_U8 && out->dtype == HGB_U8, "hgb_harris_corner: u8 images expected");
  HGB_REQUIRE(in->width == out->width && in->height == out->height && in->batch == out->batch,
              "hgb_harris_corner: size mismatch");
  HGB_REQUIRE(boundary >= 0 && boundary <= 4, "hgb_harris_corner: bad boundary");
  HGB_REQUIRE(mode == 0 || mode == 1, "hgb_harris_corner: mode must be 0 (fused) or 1 (nine launches)");
  HarrisParams p;
  memset(&p, 0, sizeof(p));
  p.in = (const uint8_t *)in->data;
  p.in_p = in->pitch;
  p.in_b = in->batch_stride;
  p.out = (uint8_t *)out->data;
  p.out_p = out->pitch;
  p.out_b = out->batch_stride;
  p.w = in->width;
  p.h = in->height;
  p.bmode = boundary;
  p.k = k;
  p.threshold = threshold;
  cudaStream_t st = (cudaStream_t)stream;
  if (mode == 0) {
    cudaEvent_t ev = before_launch(st);
    harris_fused_kernel<<<dim3(cdiv(p.w, HC_TW), cdiv(p.h, HC_TH), in->batch), HC_T, 0, st>>>(p);
    return after_launch("harris_fused_kernel", st, ev);
  }
  const size_t px = (size_t)p.w * p.h * in->batch;
  Workspace ws;
  rc = workspace_get(px * 2 * 6, &ws);
  if (rc) return rc;
  int16_t *base = (int16_t *)ws.base;
  p.dx = base;
  p.dy = base + px;
  p.sx = base + 2 * px;
  p.sy = base + 3 * px;
  p.sxy = base + 4 * px;
  p.dxy = base + 5 * px;
  const dim3 g(cdiv(p.w, 32), cdiv(p.h, 8), in->batch);
  cudaEvent_t ev = before_launch(st);
  harris_deriv_kernel<<<g, 256, 0, st>>>(p, 0);
  harris_deriv_kernel<<<g, 256, 0, st>>>(p, 1);
  harris_square_kernel<<<g, 256, 0, st>>>(p, 0);
  harris_square_kernel<<<g, 256, 0, st>>>(p, 1);
  harris_square_kernel<<<g, 256, 0, st>>>(p, 2);
  // as the sample: the Gaussians of sx and sy overwrite dx and dy
  harris_gauss_kernel<<<g, 256, 0, st>>>(p, p.sx, p.dx);
  harris_gauss_kernel<<<g, 256, 0, st>>>(p, p.sy, p.dy);
  harris_gauss_kernel<<<g, 256, 0, st>>>(p, p.sxy, p.dxy);
  harris_response_kernel<<<g, 256, 0, st>>>(p);
  return after_launch("harris nine launches", st, ev);
}

extern "C" int hgb_unsharp(const hgb_view *in, const hgb_view *out, int boundary, int mode, void *stream) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  rc = check_view(out, "out");
  if (rc) return rc;
  HGB_REQUIRE(in->dtype == HGB_U8X4 && out->dtype == HGB_U8X4, "hgb_unsharp: uchar4 images expected");
  HGB_REQUIRE(in->width == out->width && in->height == out->height && in->batch == out->batch,
              "hgb_unsharp: size mismatch");
  HGB_REQUIRE(in->data != out->data, "hgb_unsharp: in and out must differ");
  HGB_REQUIRE(in->pitch % 4 == 0 && out->pitch % 4 == 0 && in->batch_stride % 4 == 0 && out->batch_stride % 4 == 0 &&
                  (uintptr_t)in->data % 4 == 0 && (uintptr_t)out->data % 4 == 0,
              "hgb_unsharp: uchar4 rows must be 4-byte aligned");
  HGB_REQUIRE(boundary >= 0 && boundary <= 4, "hgb_unsharp: bad boundary");
  HGB_REQUIRE(mode == 0 || mode == 1, "hgb_unsharp: mode must be 0 (fused) or 1 (five launches)");
  UnsharpParams p;
  memset(&p, 0, sizeof(p));
  p.in = (const uchar4 *)in->data;
  p.in_p = in->pitch / 4;
  p.in_b = in->batch_stride / 4;
  p.out = (uchar4 *)out->data;
  p.out_p = out->pitch / 4;
  p.out_b = out->batch_stride / 4;
  p.w = in->width;
  p.h = in->height;
  p.bmode = boundary;
  rc = unsharp_tables(&p.tab);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (mode == 0) {
    p.tiles_x = cdiv(p.w, US_TW);
    p.tiles_y = cdiv(p.h, US_TH);
    p.ntiles = p.tiles_x * p.tiles_y * in->batch;
    const int grid = std::min(p.ntiles, num_sms() * std::max(1, resident_ctas((const void *)unsharp_fused_kernel, US_T, 0)));
    cudaEvent_t ev = before_launch(st);
    unsharp_fused_kernel<<<grid, US_T, 0, st>>>(p);
    return after_launch("unsharp_fused_kernel", st, ev);
  }
  const size_t px = (size_t)p.w * p.h * in->batch;
  Workspace ws;
  rc = workspace_get(px * 4 * 4, &ws);
  if (rc) return rc;
  float *base = (float *)ws.base;
  p.gray = base;
  p.blur = base + px;
  p.sharp = base + 2 * px;
  p.ratio = base + 3 * px;
  const dim3 g(cdiv(p.w, 32), cdiv(p.h, 8), in->batch);
  cudaEvent_t ev = before_launch(st);
  unsharp_gray_kernel<<<g, 256, 0, st>>>(p);
  unsharp_blur_kernel<<<g, 256, 0, st>>>(p);
  unsharp_sharp_kernel<<<g, 256, 0, st>>>(p);
  unsharp_ratio_kernel<<<g, 256, 0, st>>>(p);
  unsharp_scale_kernel<<<g, 256, 0, st>>>(p);
  return after_launch("unsharp five launches", st, ev);
}

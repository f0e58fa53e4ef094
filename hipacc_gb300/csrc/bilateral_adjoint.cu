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
#include <cmath>
#include <cstring>

#include "hgb_internal.cuh"

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
  const size_t nparts = (size_t)cdiv(p.w, BA_TW) * cdiv(p.h, BA_TH) * p.batch;
  Workspace ws;
  rc = workspace_get(px * 8 + nparts * 8 + 256, &ws);
  if (rc) return rc;
  p.dc_part = (double *)ws.base;
  p.a = (float *)((char *)ws.base + (nparts * 8 + 255) / 256 * 256);
  p.y = p.a + px;
  cudaStream_t st = (cudaStream_t)stream;
  switch (size) {
    case 3: return launch_bil_adjoint<3>(p, st);
    case 5: return launch_bil_adjoint<5>(p, st);
    case 7: return launch_bil_adjoint<7>(p, st);
    case 9: return launch_bil_adjoint<9>(p, st);
    case 11: return launch_bil_adjoint<11>(p, st);
    default: return launch_bil_adjoint<13>(p, st);
  }
}

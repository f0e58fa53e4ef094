// band.cuh -- edge bands and boundary pre-images for the adjoint kernels.
//
// A tile path that takes groups of four horizontally adjacent pixels whose
// taps stay inside the image leaves out a band of radius R along the edges:
// rows [0, R) and [H-R, H) whole, then, for the rows in between, columns
// [0, L) and [W-wr, W) with L = R rounded up to 4 and wr = W - 4 floor((W -
// R) / 4) (the image must be wide enough that the two do not meet).  Those pixels go
// through the boundary's pre-images one pixel per thread, from a flat list of
// the batch's band pixels that every CTA takes an equal contiguous share of.
#pragma once

#include "hgb_internal.cuh"

namespace hgb {

__host__ __device__ __forceinline__ int band_left(int R) { return (R + 3) / 4 * 4; }
__host__ __device__ __forceinline__ int band_right(int W, int R) { return W - 4 * ((W - R) / 4); }
__host__ __device__ __forceinline__ int band_size(int W, int H, int R) {
  return 2 * R * W + (H - 2 * R) * (band_left(R) + band_right(W, R));
}
__device__ __forceinline__ void band_pos(int k, int W, int H, int R, int &y, int &x) {
  if (k < 2 * R * W) {
    const int yy = k / W;
    x = k - yy * W;
    y = yy < R ? yy : H - 2 * R + yy;
    return;
  }
  k -= 2 * R * W;
  const int L = band_left(R), mid = (H - 2 * R) * L;
  if (k < mid) {
    y = R + k / L;
    x = k - (y - R) * L;
    return;
  }
  k -= mid;
  const int wr = band_right(W, R);
  const int yy = k / wr;
  y = R + yy;
  x = W - wr + (k - yy * wr);
}

// the contiguous share of n band entries that this CTA takes
__device__ __forceinline__ void cta_share(int64_t n, int64_t &k0, int64_t &k1) {
  k0 = n * blockIdx.x / gridDim.x;
  k1 = n * (blockIdx.x + 1) / gridDim.x;
}

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

}  // namespace hgb

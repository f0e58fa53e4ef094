// binning.cu -- hgb_histogram: binned data of the histogram binning kernel.
//
// Reference: Kernel::binned_data (dsl/kernel.hpp:163-200) with the binning
// function of samples-public/2_Global_Operators/Histogram/src/main.cpp:41-47,
//   bin((unsigned)(pixel / 255.0f * num_bins)) = 1,  reduce = left + right,
// run on the GPU by hipaccApplyBinningSegmented (runtime/hipacc_cu.tpp:410-464,
// device code runtime/hipacc_cu_red.hpp:527-641) and on the CPU by
// BINNING_CPU_2D (runtime/hipacc_cpu_red.hpp:70-126), whose Put drops bin
// indices past the last bin.  The float-to-unsigned conversion here saturates
// (negative and NaN products land in bin 0), where C leaves it undefined.
//
// GB300 form: one resident wave of CTAs, each with private histograms in
// shared memory updated by shared-memory atomics -- for u8 pixels and up to
// 256 bins one column per lane (a warp's 32 updates land in 32 banks),
// otherwise one copy per warp up to 1024 bins and one copy beyond -- the
// image read as 16-pixel chunks with 16-byte loads where the layout allows
// (several chunks' loads in flight per thread), and one global atomic add per
// non-empty private bin at the end.  Integer sums, so the result does not
// depend on the order.  u8 pixels map through a 256-entry table computed
// with the same float arithmetic, replicated once per shared-memory bank --
// unless the table is the identity up to a limit and past the last bin above
// it (256 bins: values 0..254 to bins 0..254, 255 dropped), in which case the
// pixel is its own bin index, no table is read and half the shared memory
// holds twice the CTAs.
#include <algorithm>

#include "hgb_internal.cuh"

namespace hgb {
namespace {

constexpr int HB_T = 256;
constexpr unsigned kMaxBins = 16384;

struct HistParams {
  const char *in;
  int64_t pitch, bstride;
  int ox, oy, w, h, batch;
  int es;      // element size (1: u8, 4: f32)
  int dense;   // window rows back to back over the batch: one flat run
  int vec;     // 16-byte loads legal for every chunk
  unsigned nb;
  int layout;  // private histograms per CTA: 0 one, 1 one per warp, 2 one column per lane
  int direct;  // u8, lane columns: value v < lim is bin v, values >= lim pass the last bin
  unsigned lim;
  uint32_t *bins;
};

__device__ __forceinline__ uint32_t bin_of(float px, unsigned nb) {
  // pixel / 255 * num_bins with the sample's two roundings, truncated
  return __float2uint_rz(__fmul_rn(__fdiv_rn(px, 255.0f), (float)nb));
}

template <typename T>
__global__ void __launch_bounds__(HB_T) hist_kernel(const __grid_constant__ HistParams p) {
  extern __shared__ uint32_t hist_smem[];
  const unsigned copies = p.layout == 2 ? 32u : (p.layout == 1 ? (unsigned)(HB_T / 32) : 1u);
  const unsigned nall = p.nb * copies;
  // u8 only: the value -> bin table, one copy per bank (entry v of lane l at
  // v * 32 + l), so a warp's 32 lookups never conflict
  uint32_t *lut = hist_smem + nall;
  for (unsigned i = threadIdx.x; i < nall; i += HB_T) hist_smem[i] = 0u;
  // lane columns: bin i of lane l at i * 32 + l, so a warp's 32 updates hit 32
  // banks; per-warp copies: warps do not contend on a bin
  const unsigned lane = threadIdx.x & 31;
  uint32_t *sb = hist_smem + (p.layout == 1 ? (threadIdx.x >> 5) * p.nb : 0u);
  if constexpr (sizeof(T) == 1)
    if (!p.direct)
      for (int i = threadIdx.x; i < 256 * 32; i += HB_T) lut[i] = bin_of((float)(i >> 5), p.nb);
  __syncthreads();
  auto put = [&](T px) {
    if constexpr (sizeof(T) == 1) {
      if (p.direct) {
        if ((uint32_t)px < p.lim) atomicAdd(&sb[((uint32_t)px << 5) | lane], 1u);
        return;
      }
    }
    uint32_t idx;
    if constexpr (sizeof(T) == 1)
      idx = lut[((uint32_t)px << 5) | (threadIdx.x & 31)];
    else
      idx = bin_of((float)px, p.nb);
    if (idx < p.nb) atomicAdd(&sb[p.layout == 2 ? (idx << 5) | lane : idx], 1u);
  };
  // items: 16-pixel chunks of rows; a dense window is one row per batch
  const int64_t row_len = p.dense ? (int64_t)p.w * p.h * p.batch : p.w;
  const int64_t rows = p.dense ? 1 : (int64_t)p.h * p.batch;
  const int64_t cpr = (row_len + 15) / 16;
  const int64_t items = rows * cpr;
  // U chunks per thread and pass, all loads issued before the updates (more
  // bytes in flight per SM: a resident wave holds few CTAs)
  constexpr int NV = 16 * sizeof(T) / 16;
  constexpr int U = sizeof(T) == 1 ? 4 : 2;
  const int64_t stride = (int64_t)gridDim.x * HB_T;
  for (int64_t it0 = (int64_t)blockIdx.x * HB_T + threadIdx.x; it0 < items; it0 += U * stride) {
    uint4 v[U][NV];
    const T *src[U];
    int n[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t it = it0 + u * stride;
      n[u] = 0;
      src[u] = nullptr;
      if (it < items) {
        const int64_t row = it / cpr, chunk = it - row * cpr;
        const char *base;
        if (p.dense) {
          base = p.in + ((int64_t)p.oy * p.pitch + (int64_t)p.ox * p.es);
        } else {
          const int b = (int)(row / p.h), y = (int)(row - (int64_t)b * p.h);
          base = p.in + (int64_t)b * p.bstride + (int64_t)(p.oy + y) * p.pitch + (int64_t)p.ox * p.es;
        }
        src[u] = reinterpret_cast<const T *>(base) + chunk * 16;
        const int64_t left = row_len - chunk * 16;
        n[u] = left < 16 ? (int)left : 16;
        if (p.vec && n[u] == 16) {
#pragma unroll
          for (int k = 0; k < NV; ++k) v[u][k] = ldg16(reinterpret_cast<const char *>(src[u]) + 16 * k);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (p.vec && n[u] == 16) {
        const T *e = reinterpret_cast<const T *>(v[u]);
#pragma unroll
        for (int k = 0; k < 16; ++k) put(e[k]);
      } else {
        for (int k = 0; k < n[u]; ++k) put(src[u][k]);
      }
    }
  }
  __syncthreads();
  for (unsigned i = threadIdx.x; i < p.nb; i += HB_T) {
    uint32_t c = 0;
    if (p.layout == 2)
      for (int k = 0; k < 32; ++k) c += hist_smem[(i << 5) | ((k + i) & 31)];  // rotate to spread banks
    else
      for (unsigned k = 0; k < copies; ++k) c += hist_smem[k * p.nb + i];
    if (c) atomicAdd(&p.bins[i], c);
  }
}

// u8 pixels, identity table, dense rows, 16-byte loads: one flat run of n
// bytes.  Every byte goes to lane column slot v (256 slots; the slots from
// lim on, which the table sends past the last bin, are never published), so
// a pixel costs a byte extract, an address and one shared-memory atomic.
// (Per-thread 16-bit counter columns updated by plain load / add / store
// measured slower, 22.8 against 15.7 us on 4096^2: each update waits for the
// previous one of the same thread, and 64 KB per CTA leaves 12 warps per SM.)
__global__ void __launch_bounds__(HB_T) hist_u8_direct_kernel(const __grid_constant__ HistParams p, int64_t n) {
  __shared__ uint32_t h[256 * 32];
  for (int i = threadIdx.x; i < 256 * 32; i += HB_T) h[i] = 0u;
  __syncthreads();
  const unsigned lane = threadIdx.x & 31;
  uint32_t *hl = h + lane;
  const uint8_t *src = reinterpret_cast<const uint8_t *>(p.in) + ((int64_t)p.oy * p.pitch + p.ox);
  const int64_t nchunks = n >> 4;
  const int64_t stride = (int64_t)gridDim.x * HB_T;
  constexpr int U = 4;  // chunks in flight per thread
  auto count = [&](uint32_t w) {
#pragma unroll
    for (int k = 0; k < 4; ++k) atomicAdd(hl + (__byte_perm(w, 0u, 0x4440 + k) << 5), 1u);
  };
  for (int64_t c0 = (int64_t)blockIdx.x * HB_T + threadIdx.x; c0 < nchunks; c0 += U * stride) {
    uint4 v[U];
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (c0 + u * stride < nchunks) v[u] = ldg16(src + 16 * (c0 + u * stride));
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (c0 + u * stride < nchunks) {
        count(v[u].x);
        count(v[u].y);
        count(v[u].z);
        count(v[u].w);
      }
  }
  // the last n mod 16 bytes: block 0
  if (blockIdx.x == 0)
    for (int64_t i = (nchunks << 4) + threadIdx.x; i < n; i += HB_T) atomicAdd(hl + ((uint32_t)src[i] << 5), 1u);
  __syncthreads();
  for (unsigned i = threadIdx.x; i < p.lim && i < p.nb; i += HB_T) {
    uint32_t c = 0;
    for (int k = 0; k < 32; ++k) c += h[(i << 5) | ((k + i) & 31)];  // rotate to spread banks
    if (c) atomicAdd(&p.bins[i], c);
  }
}

}  // namespace
}  // namespace hgb

using namespace hgb;

extern "C" int hgb_histogram(const hgb_view *in, const hgb_window *win, unsigned num_bins, uint32_t *bins_dev,
                             uint32_t *bins_host, void *stream) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  HGB_REQUIRE(in->dtype == HGB_U8 || in->dtype == HGB_F32, "hgb_histogram: u8 or f32 pixels expected");
  HGB_REQUIRE(num_bins >= 1 && num_bins <= kMaxBins, "hgb_histogram: num_bins must be 1..16384");
  HGB_REQUIRE(bins_dev || bins_host, "hgb_histogram: no result buffer");
  const hgb_window w = window_or_full(win, *in);
  rc = check_window(w, *in, "window");
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  uint32_t *bins = bins_dev;
  if (!bins) {
    Workspace ws;
    rc = workspace_get((size_t)num_bins * 4, &ws);
    if (rc) return rc;
    bins = (uint32_t *)ws.base;
  }
  HistParams p;
  memset(&p, 0, sizeof(p));
  p.in = (const char *)in->data;
  p.pitch = in->pitch;
  p.bstride = in->batch_stride;
  p.ox = w.offset_x;
  p.oy = w.offset_y;
  p.w = w.width;
  p.h = w.height;
  p.batch = in->batch;
  p.es = dtype_size(in->dtype);
  // full-width rows back to back (and whole images back to back in a batch): one flat run
  p.dense = (w.width == in->width && (int64_t)in->width * p.es == in->pitch &&
             (in->batch == 1 || (w.height == in->height && in->batch_stride == in->pitch * in->height)))
                ? 1
                : 0;
  const uintptr_t first = (uintptr_t)p.in + (uintptr_t)((int64_t)w.offset_y * p.pitch + (int64_t)w.offset_x * p.es);
  p.vec = (first % 16 == 0) && (p.dense || (p.pitch % 16 == 0 && (in->batch == 1 || p.bstride % 16 == 0))) ? 1 : 0;
  p.nb = num_bins;
  // measured on 4096^2 images: lane columns help u8 (23.0 vs 24.8 us), per-warp copies f32 (24.8 vs 37 us)
  p.layout = (in->dtype == HGB_U8 && num_bins <= 256) ? 2 : (num_bins <= 1024 ? 1 : 0);
  p.bins = bins;
  if (in->dtype == HGB_U8 && p.layout == 2) {
    // the value -> bin table with the kernel's float arithmetic: identity up to
    // some value and past the last bin from there on?
    unsigned lim = 256;
    bool ident = true;
    for (unsigned v = 0; v < 256 && ident; ++v) {
      const unsigned b = (unsigned)(((float)v / 255.0f) * (float)num_bins);
      if (v < lim && b != v) {
        if (b >= num_bins) lim = v;
        else ident = false;
      } else if (v >= lim && b < num_bins) {
        ident = false;
      }
    }
    p.direct = ident ? 1 : 0;
    p.lim = lim;
  }
  const size_t copies = p.layout == 2 ? 32 : (p.layout == 1 ? HB_T / 32 : 1);
  const size_t smem = ((size_t)num_bins * copies + (in->dtype == HGB_U8 && !p.direct ? 256 * 32 : 0)) * 4;
  HGB_CHECK_CUDA(cudaMemsetAsync(bins, 0, (size_t)num_bins * 4, st));
  if (in->dtype == HGB_U8 && p.direct && p.dense && p.vec) {
    const int64_t n = (int64_t)w.width * w.height * in->batch;
    const int per_sm = resident_ctas((const void *)hist_u8_direct_kernel, HB_T, 0);
    const int grid =
        (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)num_sms() * per_sm, (n / 16 + HB_T - 1) / HB_T));
    cudaEvent_t ev = before_launch(st);
    hist_u8_direct_kernel<<<grid, HB_T, 0, st>>>(p, n);
    rc = after_launch("hist_u8_direct_kernel", st, ev);
    if (rc) return rc;
    if (bins_host) {
      HGB_CHECK_CUDA(cudaMemcpyAsync(bins_host, bins, (size_t)num_bins * 4, cudaMemcpyDeviceToHost, st));
      HGB_CHECK_CUDA(cudaStreamSynchronize(st));
    }
    return HGB_OK;
  }
  const void *kern = in->dtype == HGB_U8 ? (const void *)hist_kernel<uint8_t> : (const void *)hist_kernel<float>;
  rc = ensure_dynamic_smem(kern, smem);
  if (rc) return rc;
  const int64_t items = ((int64_t)w.width * w.height * in->batch + 15) / 16;
  const int per_sm = resident_ctas(kern, HB_T, smem);
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)num_sms() * per_sm, (items + HB_T - 1) / HB_T));
  cudaEvent_t ev = before_launch(st);
  if (in->dtype == HGB_U8)
    hist_kernel<uint8_t><<<grid, HB_T, smem, st>>>(p);
  else
    hist_kernel<float><<<grid, HB_T, smem, st>>>(p);
  rc = after_launch("hist_kernel", st, ev);
  if (rc) return rc;
  if (bins_host) {
    HGB_CHECK_CUDA(cudaMemcpyAsync(bins_host, bins, (size_t)num_bins * 4, cudaMemcpyDeviceToHost, st));
    HGB_CHECK_CUDA(cudaStreamSynchronize(st));
  }
  return HGB_OK;
}

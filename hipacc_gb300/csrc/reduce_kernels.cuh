// reduce_kernels.cuh -- single-pass global reduction kernels (hgb_reduce and
// its allocation-free variant).
//
// Replaces hipaccApplyReductionShared (runtime/hipacc_cu.tpp:312-408) and its
// device code (runtime/hipacc_cu_red.hpp:140-346): no per-call allocation, a
// fixed grid of (SMs x 4) CTAs, 16-byte loads, warp shuffles, a block combine,
// and one last-block combine of the per-block partials behind a fenced ticket
// (reduce_common.cuh).  The fold order depends only on the grid, so results
// are reproducible run to run.  Float sums keep per-thread Kahan partials,
// merge them pairwise in FP32 and combine the block partials in FP64.
#pragma once

#include <cfloat>
#include <climits>
#include <cstring>
#include <type_traits>

#include "reduce_common.cuh"

namespace hgb {
namespace {

// accumulator and fold rules per (storage type, op)
template <typename T, int OP>
struct Red;

template <typename T, int OP>
struct IntRed {
  static constexpr bool kSigned = T(-1) < T(0);
  using A = typename std::conditional<kSigned, long long, unsigned long long>::type;
  static __device__ __forceinline__ A identity() {
    if (OP == HGB_REDUCE_SUM) return A(0);
    if (OP == HGB_REDUCE_PROD) return A(1);
    if (OP == HGB_REDUCE_MIN) return kSigned ? A(LLONG_MAX) : A(ULLONG_MAX);
    return kSigned ? A(LLONG_MIN) : A(0);
  }
  static __device__ __forceinline__ A fold(A a, A b) {
    if (OP == HGB_REDUCE_SUM) return a + b;
    if (OP == HGB_REDUCE_PROD) return a * b;
    if (OP == HGB_REDUCE_MIN) return a < b ? a : b;
    return a > b ? a : b;
  }
  static __device__ __forceinline__ A lift(T v) { return A(v); }
  // 8-byte result: sums widened; min/max/prod in the input's width
  static __device__ __forceinline__ unsigned long long finish(A a) {
    if (OP == HGB_REDUCE_SUM) return (unsigned long long)a;
    if (OP == HGB_REDUCE_PROD) {
      const T t = (T)a;
      return kSigned ? (unsigned long long)(long long)t : (unsigned long long)t;
    }
    return (unsigned long long)a;
  }
};

template <int OP> struct Red<uint8_t, OP> : IntRed<uint8_t, OP> {};
template <int OP> struct Red<uint16_t, OP> : IntRed<uint16_t, OP> {};
template <int OP> struct Red<int16_t, OP> : IntRed<int16_t, OP> {};
template <int OP> struct Red<uint32_t, OP> : IntRed<uint32_t, OP> {};
template <int OP> struct Red<int32_t, OP> : IntRed<int32_t, OP> {};
template <int OP> struct Red<unsigned long long, OP> : IntRed<unsigned long long, OP> {};

// floating point: SUM uses Kahan pairs (value = s - c); MIN/MAX/PROD a float
template <typename T, int OP>
struct FltRed {
  using A = typename std::conditional<OP == HGB_REDUCE_SUM, Kahan, float>::type;
  static __device__ __forceinline__ A identity() {
    if constexpr (OP == HGB_REDUCE_SUM) return Kahan{0.0f, 0.0f};
    else if constexpr (OP == HGB_REDUCE_PROD) return 1.0f;
    else if constexpr (OP == HGB_REDUCE_MIN) return __int_as_float(0x7f800000);  // +inf
    else return __int_as_float(0xff800000);
  }
  static __device__ __forceinline__ A fold_elem(A a, float v) {
    if constexpr (OP == HGB_REDUCE_SUM) return kahan_add(a, v);
    else if constexpr (OP == HGB_REDUCE_PROD) return __fmul_rn(a, v);
    else if constexpr (OP == HGB_REDUCE_MIN) return a < v ? a : v;
    else return a > v ? a : v;
  }
  static __device__ __forceinline__ A fold(A a, A b) {
    if constexpr (OP == HGB_REDUCE_SUM) return kahan_merge(a, b);
    else return fold_elem(a, b);
  }
};
template <int OP> struct Red<float, OP> : FltRed<float, OP> {};
template <int OP> struct Red<__nv_bfloat16, OP> : FltRed<__nv_bfloat16, OP> {};
template <int OP> struct Red<__half, OP> : FltRed<__half, OP> {};

template <int OP>
struct Red<double, OP> {
  using A = double;
  static __device__ __forceinline__ A identity() {
    if (OP == HGB_REDUCE_SUM) return 0.0;
    if (OP == HGB_REDUCE_PROD) return 1.0;
    if (OP == HGB_REDUCE_MIN) return __longlong_as_double(0x7ff0000000000000ll);
    return __longlong_as_double((long long)0xfff0000000000000ull);
  }
  static __device__ __forceinline__ A fold(A a, A b) {
    if (OP == HGB_REDUCE_SUM) return __dadd_rn(a, b);
    if (OP == HGB_REDUCE_PROD) return __dmul_rn(a, b);
    if (OP == HGB_REDUCE_MIN) return a < b ? a : b;
    return a > b ? a : b;
  }
};

template <typename A>
__device__ __forceinline__ A shfl_down_any(A v, int d) {
  if constexpr (std::is_same<A, Kahan>::value) {
    Kahan r;
    r.s = __shfl_down_sync(0xffffffffu, v.s, d);
    r.c = __shfl_down_sync(0xffffffffu, v.c, d);
    return r;
  } else {
    return __shfl_down_sync(0xffffffffu, v, d);
  }
}

struct RedParams {
  const char *in;
  int64_t pitch, bstride;
  int ox, oy, w, h, batch;
  int chunks_per_row;  // 16-byte chunks per window row
  int vec;
  void *partials;
  unsigned int *ticket;
  unsigned long long *acc;  // integer accumulator (zero at rest)
  unsigned long long *result_dev;
};

template <typename T, int OP>
__device__ __forceinline__ typename Red<T, OP>::A fold_value(typename Red<T, OP>::A a, T v) {
  if constexpr (std::is_same<T, float>::value || std::is_same<T, __nv_bfloat16>::value ||
                std::is_same<T, __half>::value)
    return Red<T, OP>::fold_elem(a, Storage<T>::to_f(v));
  else if constexpr (std::is_same<T, double>::value)
    return Red<T, OP>::fold(a, v);
  else
    return Red<T, OP>::fold(a, Red<T, OP>::lift(v));
}

template <typename T, int OP>
__device__ __forceinline__ typename Red<T, OP>::A block_fold(typename Red<T, OP>::A a) {
  using R = Red<T, OP>;
  using A = typename R::A;
  __shared__ A s_part[32];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) a = R::fold(a, shfl_down_any(a, d));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) s_part[warp] = a;
  __syncthreads();
  if (warp == 0) {
    a = lane < (int)(blockDim.x >> 5) ? s_part[lane] : R::identity();
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) a = R::fold(a, shfl_down_any(a, d));
  }
  __syncthreads();
  return a;  // valid in thread 0
}

// fold one 16-byte chunk (V elements, the last chunk of a row may be partial)
template <typename T, int OP>
__device__ __forceinline__ typename Red<T, OP>::A fold_chunk(typename Red<T, OP>::A acc, const uint4 &v, int valid) {
  constexpr int V = 16 / sizeof(T);
  const T *e = reinterpret_cast<const T *>(&v);
#pragma unroll
  for (int q = 0; q < V; ++q)
    if (q < valid) acc = fold_value<T, OP>(acc, e[q]);
  return acc;
}

// u8 sums: four bytes per dp4a into a 32-bit partial (at most 2^24 chunks of
// 16 bytes per partial before it is folded into the 64-bit accumulator)
__device__ __forceinline__ uint32_t byte_sum16(const uint4 &v, uint32_t s) {
  s = __dp4a(v.x, 0x01010101u, s);
  s = __dp4a(v.y, 0x01010101u, s);
  s = __dp4a(v.z, 0x01010101u, s);
  return __dp4a(v.w, 0x01010101u, s);
}

template <typename T, int OP>
__global__ void __launch_bounds__(256) reduce_kernel(const __grid_constant__ RedParams p) {
  using R = Red<T, OP>;
  using A = typename R::A;
  constexpr int V = 16 / sizeof(T);
  constexpr bool kByteSum = std::is_same<T, uint8_t>::value && OP == HGB_REDUCE_SUM;
  constexpr int U = 4;  // chunks in flight per thread
  A acc = R::identity();
  uint32_t bsum = 0;
  int bsum_n = 0;
  const int cpr = p.chunks_per_row;
  const int64_t items = (int64_t)p.batch * p.h * cpr;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // chunk position as (row of the batch, chunk of the row), advanced by the
  // grid stride without a division per chunk
  const int s_c = (int)(stride % cpr);
  const int64_t s_r = stride / cpr;
  const int s_ry = (int)(s_r % p.h), s_rb = (int)(s_r / p.h);  // the row stride as (images, rows)
  int64_t it = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int c = (int)(it % cpr);
  int64_t rg = it / cpr;
  int b = (int)(rg / p.h), y = (int)(rg - (int64_t)b * p.h);
  auto advance = [&]() {
    it += stride;
    c += s_c;
    y += s_ry;
    b += s_rb;
    if (c >= cpr) {
      c -= cpr;
      ++y;
    }
    if (y >= p.h) {  // y < 2h here: one wrap at most
      y -= p.h;
      ++b;
    }
  };
  while (it < items) {
    uint4 v[U];
    int valid[U];
    int n = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (it < items) {
        const T *row = reinterpret_cast<const T *>(p.in + b * p.bstride + (int64_t)(p.oy + y) * p.pitch) + p.ox;
        const int x0 = c * V;
        valid[u] = min(V, p.w - x0);
        if (p.vec && valid[u] == V) {
          v[u] = ldg16(row + x0);
        } else {
          T tmp[V];
#pragma unroll
          for (int q = 0; q < V; ++q) tmp[q] = q < valid[u] ? row[x0 + q] : T(0);
          memcpy(&v[u], tmp, 16);
        }
        ++n;
        advance();
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (u < n) {
        if constexpr (kByteSum) {
          bsum = byte_sum16(v[u], bsum);  // padding bytes of a partial chunk are zero
          if (++bsum_n == (1 << 24)) {
            acc = R::fold(acc, (A)bsum);
            bsum = 0;
            bsum_n = 0;
          }
        } else {
          acc = fold_chunk<T, OP>(acc, v[u], valid[u]);
        }
      }
    }
  }
  if constexpr (kByteSum) acc = R::fold(acc, (A)bsum);
  acc = block_fold<T, OP>(acc);
  if constexpr (std::is_integral<T>::value && OP != HGB_REDUCE_PROD) {
    // integers: order-preserving 64-bit keys folded with relaxed atomics,
    // published by the CTA that takes the last ticket (no combine loop)
    using R2 = Red<T, OP>;
    constexpr unsigned long long kSign = R2::kSigned ? 0x8000000000000000ull : 0ull;
    if (threadIdx.x == 0) {
      const unsigned long long u = (unsigned long long)acc ^ kSign;
      if (OP == HGB_REDUCE_SUM)
        atomicAdd(p.acc, (unsigned long long)acc);
      else if (OP == HGB_REDUCE_MAX)
        atomicMax(p.acc, u);
      else
        atomicMax(p.acc, ~u);
      if (ticket_acq_rel(p.ticket) == gridDim.x - 1) {
        const unsigned long long v = ld_relaxed_u64(p.acc);
        A a;
        if (OP == HGB_REDUCE_SUM)
          a = (A)v;
        else if (OP == HGB_REDUCE_MAX)
          a = (A)(v ^ kSign);
        else
          a = (A)(~v ^ kSign);
        *p.result_dev = R2::finish(a);
        *p.acc = 0ull;
        *p.ticket = 0u;
      }
    }
    return;
  }
  A *parts = reinterpret_cast<A *>(p.partials);
  if (threadIdx.x == 0) parts[blockIdx.x] = acc;
  if (!take_last_ticket(p.ticket)) return;
  // last block: combine partials in block order
  const int n = gridDim.x;
  unsigned long long bits;
  if constexpr (std::is_same<A, Kahan>::value) {
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const float2 v = __ldcg(reinterpret_cast<const float2 *>(parts) + i);
      s += (double)v.x - (double)v.y;
    }
    __shared__ double s_d[32];
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) s += __shfl_down_sync(0xffffffffu, s, d);
    if ((threadIdx.x & 31) == 0) s_d[threadIdx.x >> 5] = s;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += s_d[i];
    bits = __double_as_longlong(t);
  } else {
    A a = R::identity();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      A v;
      if constexpr (sizeof(A) == 8) {
        const unsigned long long u = __ldcg(reinterpret_cast<const unsigned long long *>(parts) + i);
        memcpy(&v, &u, 8);
      } else {
        const unsigned int u = __ldcg(reinterpret_cast<const unsigned int *>(parts) + i);
        memcpy(&v, &u, 4);
      }
      a = R::fold(a, v);
    }
    a = block_fold<T, OP>(a);
    if constexpr (std::is_same<A, float>::value)
      bits = __double_as_longlong((double)a);
    else if constexpr (std::is_same<A, double>::value)
      bits = __double_as_longlong(a);
    else
      bits = R::finish(a);
  }
  if (threadIdx.x == 0) *p.result_dev = bits;
  release_ticket(p.ticket);
}

template <typename T>
int launch_reduce(int op, const RedParams &p, int grid, cudaStream_t st) {
  cudaEvent_t ev = before_launch(st);
  switch (op) {
    case HGB_REDUCE_SUM: reduce_kernel<T, HGB_REDUCE_SUM><<<grid, 256, 0, st>>>(p); break;
    case HGB_REDUCE_MIN: reduce_kernel<T, HGB_REDUCE_MIN><<<grid, 256, 0, st>>>(p); break;
    case HGB_REDUCE_MAX: reduce_kernel<T, HGB_REDUCE_MAX><<<grid, 256, 0, st>>>(p); break;
    default: reduce_kernel<T, HGB_REDUCE_PROD><<<grid, 256, 0, st>>>(p); break;
  }
  return after_launch("reduce_kernel", st, ev);
}

// Fill RedParams for `in` / `win` (everything but the scratch pointers) and
// choose the grid: SMs x 4 CTAs, fewer for small windows.
inline int reduce_setup(const hgb_view *in, const hgb_window *winp, int op, RedParams *p, int *grid) {
  int rc = check_view(in, "in");
  if (rc) return rc;
  HGB_REQUIRE(op >= HGB_REDUCE_SUM && op <= HGB_REDUCE_PROD, "hgb_reduce: bad op");
  HGB_REQUIRE(in->dtype != HGB_U8X4, "hgb_reduce: vector pixels are not reducible");
  hgb_window win = window_or_full(winp, *in);
  rc = check_window(win, *in, "window");
  if (rc) return rc;
  const int es = dtype_size(in->dtype);
  p->in = (const char *)in->data;
  p->pitch = in->pitch;
  p->bstride = in->batch_stride;
  p->ox = win.offset_x;
  p->oy = win.offset_y;
  p->w = win.width;
  p->h = win.height;
  p->batch = in->batch;
  const int V = 16 / es;
  p->chunks_per_row = cdiv(win.width, V);
  const uintptr_t base = (uintptr_t)in->data + (uintptr_t)win.offset_x * es;
  p->vec = base % 16 == 0 && in->pitch % 16 == 0 && (in->batch == 1 || in->batch_stride % 16 == 0);
  const int64_t items = (int64_t)p->batch * p->h * p->chunks_per_row;
  int g = num_sms() * 4;
  if ((int64_t)g * 256 > items) g = (int)((items + 255) / 256);
  *grid = g < 1 ? 1 : g;
  return HGB_OK;
}

inline int reduce_launch(int dtype, int op, const RedParams &p, int grid, cudaStream_t st) {
  switch (dtype) {
    case HGB_U8: return launch_reduce<uint8_t>(op, p, grid, st);
    case HGB_U16: return launch_reduce<uint16_t>(op, p, grid, st);
    case HGB_I16: return launch_reduce<int16_t>(op, p, grid, st);
    case HGB_U32: return launch_reduce<uint32_t>(op, p, grid, st);
    case HGB_I32: return launch_reduce<int32_t>(op, p, grid, st);
    case HGB_U64: return launch_reduce<unsigned long long>(op, p, grid, st);
    case HGB_F32: return launch_reduce<float>(op, p, grid, st);
    case HGB_BF16: return launch_reduce<__nv_bfloat16>(op, p, grid, st);
    case HGB_F16: return launch_reduce<__half>(op, p, grid, st);
    case HGB_F64: return launch_reduce<double>(op, p, grid, st);
  }
  return set_error(HGB_ERR_UNSUPPORTED, "hgb_reduce: dtype");
}

}  // namespace
}  // namespace hgb


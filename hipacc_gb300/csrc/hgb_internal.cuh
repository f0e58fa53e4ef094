// hgb_internal.cuh -- shared device/host helpers of libhipacc_gb300.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/hipacc_gb300.h"

namespace hgb {

// ---------------------------------------------------------------- errors
int set_error(int status, const std::string &msg);   // records msg, returns status
int cuda_error(cudaError_t e, const char *what);      // HGB_ERR_CUDA with the CUDA message
inline int ok() { return HGB_OK; }

#define HGB_CHECK_CUDA(call)                                     \
  do {                                                           \
    cudaError_t hgb_e_ = (call);                                 \
    if (hgb_e_ != cudaSuccess) return ::hgb::cuda_error(hgb_e_, #call); \
  } while (0)

#define HGB_REQUIRE(cond, msg)                                            \
  do {                                                                    \
    if (!(cond)) return ::hgb::set_error(HGB_ERR_INVALID, (msg));         \
  } while (0)

// check the launch just issued, then time it when timing is on
int after_launch(const char *kernel, cudaStream_t stream, cudaEvent_t start);
// returns a started event when timing is on (else nullptr)
cudaEvent_t before_launch(cudaStream_t stream);

// ---------------------------------------------------------------- workspace
// Per-device scratch owned by the library: reduction partials, tickets,
// work-lists.  The ticket region is zeroed once at allocation and every
// kernel that uses a ticket resets it before it exits.
struct Workspace {
  void *base = nullptr;     // general scratch
  size_t bytes = 0;
  unsigned int *tickets = nullptr;  // kTickets counters, zero between uses
  unsigned long long *acc = nullptr;  // kAcc accumulators, zero between uses
};
constexpr int kTickets = 64;
constexpr int kAcc = 64;
// accumulator / ticket slots of the fused and standalone reductions
constexpr int kSlotSobel = 0;   // acc[0] sum, acc[1] max; ticket[0]
constexpr int kSlotReduce = 2;  // acc[2]; ticket[1]
constexpr int kTicketSobelClaim = 3;  // tile counter of the streaming Sobel
int workspace_get(size_t bytes, Workspace *ws);  // grows on demand

int num_sms();
// Per-device, thread-safe kernel set-up: raise a kernel's dynamic shared
// memory limit (once per device and size), and its resident CTAs per SM for a
// launch shape (cached per device).
int ensure_dynamic_smem(const void *kernel, size_t bytes);
int resident_ctas(const void *kernel, int threads, size_t smem);

// ---------------------------------------------------------------- dtypes
inline int dtype_size(int dt) {
  switch (dt) {
    case HGB_U8: return 1;
    case HGB_U8X4: return 4;
    case HGB_I16: case HGB_U16: case HGB_F16: case HGB_BF16: return 2;
    case HGB_I32: case HGB_U32: case HGB_F32: return 4;
    case HGB_U64: case HGB_F64: return 8;
  }
  return 0;
}
inline bool is_float_storage(int dt) { return dt == HGB_F32 || dt == HGB_BF16 || dt == HGB_F16; }

int check_view(const hgb_view *v, const char *name);
inline char *image_ptr(const hgb_view &v, int b) { return (char *)v.data + (int64_t)b * v.batch_stride; }

// window defaulting to the whole view
inline hgb_window window_or_full(const hgb_window *w, const hgb_view &v) {
  if (w) return *w;
  hgb_window r{0, 0, v.width, v.height};
  return r;
}
int check_window(const hgb_window &w, const hgb_view &v, const char *name);

// ---------------------------------------------------------------- device
// Boundary remap (lib/AST/BorderHandling.cpp:41-120); identical to the
// oracle's remap_idx.  UNDEFINED is clamped so that no access leaves the
// image; MIRROR repeats the reflection until the index is in range.
// Returns INT_MIN for CONSTANT out of range.
__host__ __device__ __forceinline__ int remap(int mode, int idx, int lo, int hi) {
  if (idx >= lo && idx < hi) return idx;
  switch (mode) {
    case HGB_BOUNDARY_REPEAT: {
      const int w = hi - lo;
      int r = (idx - lo) % w;
      if (r < 0) r += w;
      return lo + r;
    }
    case HGB_BOUNDARY_MIRROR:
      // bounded: each pass moves idx strictly closer to the window
      for (int it = 0; it < 64 && (idx < lo || idx >= hi); ++it) {
        if (idx >= hi) idx = hi - (idx + 1 - hi);
        if (idx < lo) idx = lo + (lo - idx - 1);
      }
      return idx < lo ? lo : (idx >= hi ? hi - 1 : idx);
    case HGB_BOUNDARY_CONSTANT:
      return (int)0x80000000;
    default:
      return idx < lo ? lo : hi - 1;
  }
}

template <typename T> struct Storage;
// u8 pixels: widened exactly; written as the samples' (uchar)(x + 0.5f), with
// values outside [0, 255] saturated (the C cast leaves them undefined; NaN
// gives 255, as fminf returns the number)
template <> struct Storage<uint8_t> {
  static __device__ __forceinline__ float load(const uint8_t *p) { return (float)__ldg(p); }
  static __device__ __forceinline__ float to_f(uint8_t v) { return (float)v; }
  static __device__ __forceinline__ uint8_t from_f(float v) {
    return (uint8_t)__float2uint_rz(fminf(__fadd_rn(v, 0.5f), 255.0f));
  }
};
template <> struct Storage<float> {
  static __device__ __forceinline__ float load(const float *p) { return __ldg(p); }
  static __device__ __forceinline__ float to_f(float v) { return v; }
  static __device__ __forceinline__ float from_f(float v) { return v; }
};
template <> struct Storage<__nv_bfloat16> {
  static __device__ __forceinline__ float load(const __nv_bfloat16 *p) { return __bfloat162float(__ldg(p)); }
  static __device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }
  static __device__ __forceinline__ __nv_bfloat16 from_f(float v) { return __float2bfloat16_rn(v); }
};
template <> struct Storage<__half> {
  static __device__ __forceinline__ float load(const __half *p) { return __half2float(__ldg(p)); }
  static __device__ __forceinline__ float to_f(__half v) { return __half2float(v); }
  static __device__ __forceinline__ __half from_f(float v) { return __float2half_rn(v); }
};

// 16-byte read-only streaming load / store
__device__ __forceinline__ uint4 ldg16(const void *p) {
  uint4 r;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
               : "l"(p));
  return r;
}
__device__ __forceinline__ void stg16(void *p, uint4 v) {
  asm volatile("st.global.v4.u32 [%0], {%1,%2,%3,%4};" ::"l"(p), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w)
               : "memory");
}

// Packed FP32 pairs (sm_100+ f32x2 arithmetic): two lanes per instruction,
// each lane rounded exactly like the scalar instruction (fma.rn / add.rn /
// mul.rn), so results are bit-identical to the scalar forms.
using f2 = unsigned long long;
__device__ __forceinline__ f2 f2_pack(float lo, float hi) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ float f2_lo(f2 v) { return __uint_as_float((unsigned)(v & 0xffffffffull)); }
__device__ __forceinline__ float f2_hi(f2 v) { return __uint_as_float((unsigned)(v >> 32)); }
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
  f2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
  f2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
  f2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// unpack 16 bytes of storage into floats
template <typename T> struct Vec16;
template <> struct Vec16<float> {
  static constexpr int N = 4;
  static __device__ __forceinline__ void unpack(uint4 v, float *f) {
    f[0] = __uint_as_float(v.x); f[1] = __uint_as_float(v.y);
    f[2] = __uint_as_float(v.z); f[3] = __uint_as_float(v.w);
  }
};
template <> struct Vec16<__nv_bfloat16> {
  static constexpr int N = 8;
  static __device__ __forceinline__ void unpack(uint4 v, float *f) {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      f[2 * i] = __uint_as_float(w[i] << 16);
      f[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
    }
  }
};
template <> struct Vec16<uint8_t> {
  static constexpr int N = 16;
  static __device__ __forceinline__ void unpack(uint4 v, float *f) {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int b = 0; b < 4; ++b) f[4 * i + b] = (float)((w[i] >> (8 * b)) & 0xffu);
  }
};
template <> struct Vec16<__half> {
  static constexpr int N = 8;
  static __device__ __forceinline__ void unpack(uint4 v, float *f) {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      __half2 h = *reinterpret_cast<const __half2 *>(&w[i]);
      float2 t = __half22float2(h);
      f[2 * i] = t.x;
      f[2 * i + 1] = t.y;
    }
  }
};

__host__ __device__ constexpr int round_up(int a, int b) { return (a + b - 1) / b * b; }
__host__ __device__ constexpr int cdiv(int a, int b) { return (a + b - 1) / b; }

}  // namespace hgb

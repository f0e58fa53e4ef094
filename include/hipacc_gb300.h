/*
 * hipacc_gb300.h -- C ABI of libhipacc_gb300.so, the GB300 (sm_103a) kernels
 * for the image-processing hot path of Hipacc's generated code: local
 * operators, point operators, global reductions and pyramid construction,
 * plus reduced-precision storage, batched/persistent pyramid launches and
 * adjoint kernels.
 *
 * Every entry point returns an int status (HGB_OK = 0) and records a
 * thread-local message readable with hgb_last_error().  Nothing aborts the
 * process and no kernel traps: device-side failures (bounded-wait timeouts)
 * come back as HGB_ERR_TIMEOUT.  Pointers named *_dev are device addresses;
 * `stream` is a cudaStream_t (NULL = legacy default stream).  All launches are
 * asynchronous unless a host result is requested.
 *
 * The comment above each entry point names the reference interface it
 * replaces (paths inside the Hipacc source tree).
 */
#ifndef HIPACC_GB300_H
#define HIPACC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HGB_ABI_VERSION 1

#if defined(__GNUC__)
#define HGB_API __attribute__((visibility("default")))
#else
#define HGB_API
#endif

typedef enum hgb_status {
  HGB_OK = 0,
  HGB_ERR_INVALID = 1,     /* bad argument: null pointer, size, dtype, window */
  HGB_ERR_UNSUPPORTED = 2, /* valid request this build has no kernel for */
  HGB_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  HGB_ERR_ALLOC = 4,       /* device or host allocation failed */
  HGB_ERR_TIMEOUT = 5,     /* a bounded device-side wait expired */
  HGB_ERR_LIMIT = 6,       /* request exceeds a fixed capacity */
  HGB_ERR_INTERNAL = 7     /* a device-side consistency check failed (a library defect) */
} hgb_status;

/* pixel storage types */
typedef enum hgb_dtype {
  HGB_U8 = 0,
  HGB_U8X4 = 1, /* uchar4, RGBA */
  HGB_I16 = 2,
  HGB_U16 = 3,
  HGB_I32 = 4,
  HGB_U32 = 5,
  HGB_U64 = 6,
  HGB_F16 = 7,
  HGB_BF16 = 8,
  HGB_F32 = 9,
  HGB_F64 = 10
} hgb_dtype;

/* hipacc::Boundary numbering (dsl/image.hpp:46-52) */
typedef enum hgb_boundary {
  HGB_BOUNDARY_UNDEFINED = 0,
  HGB_BOUNDARY_CLAMP = 1,
  HGB_BOUNDARY_REPEAT = 2,
  HGB_BOUNDARY_MIRROR = 3,
  HGB_BOUNDARY_CONSTANT = 4
} hgb_boundary;

/* hipacc::Reduce numbering (dsl/kernel.hpp:48-54); MEDIAN is not implemented
 * by the reference either */
typedef enum hgb_reduce_op { HGB_REDUCE_SUM = 0, HGB_REDUCE_MIN = 1, HGB_REDUCE_MAX = 2, HGB_REDUCE_PROD = 3 } hgb_reduce_op;

/* A device image or a batch of equally sized device images.
 * Replaces HipaccImageCudaRaw<T> (runtime/hipacc_cu.hpp:113-160): stride is in
 * bytes here and a batch dimension is added. */
typedef struct hgb_view {
  void *data;           /* device address of pixel (0,0) of image 0 */
  int32_t dtype;        /* hgb_dtype */
  int32_t width;        /* pixels */
  int32_t height;       /* rows */
  int32_t batch;        /* images, >= 1 */
  int64_t pitch;        /* bytes between rows */
  int64_t batch_stride; /* bytes between images (ignored when batch == 1) */
} hgb_view;

/* Accessor window / IterationSpace ROI (HipaccAccessorBase,
 * runtime/hipacc_base.hpp:76-85; IterationSpace, dsl/iterationspace.hpp:118-133).
 * A NULL window means the whole image. */
typedef struct hgb_window {
  int32_t offset_x, offset_y, width, height;
} hgb_window;

/* ------------------------------------------------------------------ */
/* runtime                                                             */
/* ------------------------------------------------------------------ */

/* Library ABI version (HGB_ABI_VERSION of the build). */
HGB_API int hgb_abi_version(void);

/* hipaccInitCUDA (runtime/hipacc_cu_standalone.hpp:113-163): select the
 * device, create its context and report its name into `name` (may be NULL). */
HGB_API int hgb_init(int device, char *name, size_t name_len);

/* Message of the last failing call on this thread ("" if none). */
HGB_API const char *hgb_last_error(void);

/* -time-kernels / hipacc_last_kernel_timing (runtime/hipacc_base.hpp:54-66,
 * runtime/hipacc_cu_standalone.hpp:297-326): when on, every launch is
 * bracketed by CUDA events on its stream and synchronised; the duration in ms
 * is kept per thread. */
HGB_API int hgb_set_timing(int on);
HGB_API float hgb_last_kernel_timing(void);

/* Tile-configuration autotuning (replaces the compile-time -use-config /
 * -pixels-per-thread choices, include/hipacc/Device/TargetDescription.h:53-191):
 * when enabled, the first call of an operator for a new shape class times
 * each tile configuration and keeps the fastest; choices persist as JSON. */
HGB_API int hgb_autotune_enable(int on);
HGB_API int hgb_autotune_clear(void);
HGB_API int hgb_autotune_count(void);
HGB_API int hgb_autotune_save(const char *path);
HGB_API int hgb_autotune_load(const char *path);

/* Device status word: HGB_OK, or the error a kernel recorded since the last
 * call (HGB_ERR_TIMEOUT when a bounded wait on a TMA copy or an inter-tile
 * dependency expired, HGB_ERR_INTERNAL when a kernel's consistency check
 * failed).  Synchronises the device and clears the word. */
HGB_API int hgb_device_status(int *status);

/* Reserve the per-device workspace (reduction partials, tickets, work-lists)
 * up front, e.g. before stream capture.  Calls grow it on demand otherwise. */
HGB_API int hgb_workspace_reserve(size_t bytes);

/* Image memory: hipaccCreateMemory<T> (runtime/hipacc_cu.tpp:50-81, row pitch
 * rounded up to `alignment` bytes, 0 = 256), hipaccWriteMemory (84-116),
 * hipaccReadMemory (165-193), hipaccCopyMemory / hipaccCopyMemoryRegion
 * (runtime/hipacc_cu_standalone.hpp:165-216).  `host` buffers are dense rows
 * of width * element size bytes. */
typedef struct hgb_image hgb_image;
HGB_API int hgb_image_create(int dtype, int width, int height, int alignment, const void *host_init, hgb_image **out);
HGB_API int hgb_image_destroy(hgb_image *img);
HGB_API int hgb_image_get_view(const hgb_image *img, hgb_view *out);
HGB_API int hgb_image_write(hgb_image *img, const void *host, void *stream);
HGB_API int hgb_image_read(const hgb_image *img, void *host, void *stream);
/* hgb_image_read without the final stream synchronisation: the copy is
 * queued on `stream` and `host` is valid once the stream reaches it (for
 * pipelines that overlap one frame's read-back with the next frame's upload;
 * no counterpart in the reference, whose hipaccReadMemory blocks). */
HGB_API int hgb_image_read_async(const hgb_image *img, void *host, void *stream);
HGB_API int hgb_image_copy(const hgb_image *src, hgb_image *dst, void *stream);
HGB_API int hgb_image_copy_region(const hgb_image *src, const hgb_window *src_win, hgb_image *dst,
                          const hgb_window *dst_win, void *stream);

/* Streams and whole-program graphs: the CUDA-graph mode of Hipacc's generated
 * host code (hipaccLaunchKernelCudaGraph, runtime/hipacc_cu_standalone.hpp:331-356;
 * graph assembly in lib/Rewrite/Rewrite.cpp:423-477).  Calls issued on a stream
 * between hgb_graph_begin and hgb_graph_end are recorded, not run; the graph
 * replays them with one launch.  Independent branches are expressed with
 * hgb_stream_wait: `waiter` waits for the work queued so far on `signaller`
 * (a fork or a join edge).  Calls that synchronise (host results, image
 * read-back) or allocate (hgb_image_create, the first growth of the workspace:
 * call hgb_workspace_reserve first) cannot be recorded. */
HGB_API int hgb_stream_create(void **stream);
HGB_API int hgb_stream_destroy(void *stream);
HGB_API int hgb_stream_synchronize(void *stream);
HGB_API int hgb_stream_wait(void *waiter, void *signaller);
typedef struct hgb_graph hgb_graph;
HGB_API int hgb_graph_begin(void *stream);
HGB_API int hgb_graph_end(void *stream, hgb_graph **out);
HGB_API int hgb_graph_launch(const hgb_graph *graph, void *stream);
HGB_API int hgb_graph_destroy(hgb_graph *graph);

/* ------------------------------------------------------------------ */
/* local operators                                                     */
/* ------------------------------------------------------------------ */

/* One generated local-operator kernel (lib/AST/ASTTranslate.cpp:510-1197,
 * launched by hipaccLaunchKernel, runtime/hipacc_cu_standalone.hpp:277-329):
 *   out(is) = fold_{mask cells c} reduce(init, mask[c] * in(acc + c))
 * Kernel::convolve (dsl/kernel.hpp:241-267) when `mask` is set, and
 * Kernel::reduce(Domain) (dsl/kernel.hpp:270-296) over `domain` (non-zero
 * cells) otherwise; both may be given (mask(dom) * input(dom)).  The fold is
 * row-major from get_init(reduce) (lib/AST/Convolution.cpp:90-100), SUM as
 * fused multiply-add.  Boundary remap per lib/AST/BorderHandling.cpp:41-407.
 * in/out: f32, bf16 or f16 storage (same or different), or u8 in with u8 or
 * f32 out; FP32 arithmetic.  u8 results are written as the image samples'
 * (uchar)(v + 0.5f) (samples-public/1_Local_Operators/Gaussian_Blur/src/main.cpp),
 * saturated to [0, 255].
 * mask_w, mask_h <= 15; `mask` / `domain` are host arrays (mask_h rows of
 * mask_w); `mask_dev` (may replace `mask`) is a device array read at launch.
 * in->batch == out->batch images are processed in one launch. */
HGB_API int hgb_local_op(const hgb_view *in, const hgb_window *acc, const hgb_view *out, const hgb_window *iter,
                 const float *mask, const float *mask_dev, const uint8_t *domain, int mask_w, int mask_h,
                 int reduce, int boundary, float const_val, void *stream);

/* Separable local operator: the reference writes it as two local operators
 * with a 1xK and a Kx1 mask and an intermediate image; here one kernel keeps
 * the row pass in shared memory (FP32), which gives the FP32 two-pass result
 * bit for bit.  K <= 15, odd. */
HGB_API int hgb_separable(const hgb_view *in, const hgb_view *out, const float *row_taps, const float *col_taps, int k,
                  int boundary, float const_val, void *stream);

/* Bilateral filter (samples-public/3_Preprocessing/Bilateral_Filter/src/main.cpp:63-77):
 * out = sum s*in / sum s, s = exp(-c_r (in - centre)^2) * smask, c_r = 0.5/sigma_r^2.
 * size odd <= 13.  flags bit 0: compute the range weights with packed half
 * precision exponentials (f16/bf16 storage only; error stated by the tests). */
HGB_API int hgb_bilateral(const hgb_view *in, const hgb_view *out, const float *smask, int size, float sigma_r,
                  int boundary, float const_val, int flags, void *stream);

/* Sobel magnitude min(|gx|+|gy|, 255) over u8 with the two integer masks'
 * Domains (samples-public/3_Preprocessing/Sobel/src/main.cpp:56-67), with the
 * global reductions of the result fused into the same kernel: the u64 sum and
 * u8 max land in sum_dev / max_dev (either may be NULL).  size 3, 5 or 7. */
HGB_API int hgb_sobel_mag(const hgb_view *in, const hgb_view *out, const int *mask_x, const int *mask_y, int size,
                  int boundary, int const_val, uint64_t *sum_dev, uint32_t *max_dev, void *stream);

/* ------------------------------------------------------------------ */
/* point operators                                                     */
/* ------------------------------------------------------------------ */

/* uchar4 -> uchar gray (samples-public/0_Point_Operators/Color_Conversion,
 * integer form): out = (wr*R + wg*G + wb*B) >> shift, 16-byte vector I/O. */
HGB_API int hgb_point_gray(const hgb_view *in, const hgb_view *out, int wr, int wg, int wb, int shift, void *stream);

/* Element-wise combination of two images of the same size (the
 * DifferenceOfGaussian / Restore point kernels,
 * samples-public/5_Other/Gaussian_Laplacian_Pyramid/src/main.cpp:74-107):
 * op 0: out = a - b, 1: out = a + b, 2: out = alpha*a + beta*b.  Float storage. */
HGB_API int hgb_point_binary(int op, const hgb_view *a, const hgb_view *b, const hgb_view *out, float alpha, float beta,
                     void *stream);

/* Storage conversion between f32, bf16, f16 (round to nearest even) and u8. */
HGB_API int hgb_convert(const hgb_view *in, const hgb_view *out, void *stream);

/* Resampling accessor read as a point operator (Interpolate::NN / LF / B5 /
 * CF / L3, lib/AST/Interpolate.cpp:85-113, runtime/hipacc_cu_interpolate.hpp:173-616,
 * runtime/hipacc_cpu_interpolate.hpp:157-520): out(x,y) = in at the mapped
 * position scale/2 + scale*x, CLAMP taps.  imode 1 = NN, 2 = LF (bilinear),
 * 3 = B5 (binomial, 4x4 taps), 4 = CF (cubic a = -0.5, 4x4), 5 = L3 (Lanczos-3,
 * 6x6, the reference's tap weights).  f32 images. */
HGB_API int hgb_resample(const hgb_view *in, const hgb_view *out, int imode, void *stream);

/* ------------------------------------------------------------------ */
/* multi-kernel programs as fused chains                               */
/* ------------------------------------------------------------------ */

/* The Harris corner program (samples-public/3_Preprocessing/Harris_Corner/
 * src/main.cpp:56-166,258-307, 3x3 masks; nine kernels there: two
 * derivatives over Domains with a /6, three squares, three integer Gaussians
 * with a /16, the response R = det - k trace^2 against `threshold`).  u8 in,
 * u8 out (0 or 1 per pixel), every local operator reading through `boundary`
 * (CONSTANT taps read 0).  mode 0: one fused kernel (the intermediates stay
 * in shared memory); mode 1: the nine launches with short intermediates in
 * the library workspace (for comparison).  Bit-exact either way. */
HGB_API int hgb_harris_corner(const hgb_view *in, const hgb_view *out, float k, float threshold, int boundary,
                              int mode, void *stream);

/* The Unsharp program (samples-public/1_Local_Operators/Unsharp/src/main.cpp:
 * 53-149,203-247, 3x3; five kernels there: gamma-corrected luminance, Gaussian
 * blur through `boundary`, sharpen, ratio, scale of the RGB channels).
 * uchar4 in and out (alpha copied).  The luminance's powf terms are the host
 * C library's (the CPU back end's function) and its double sum is reproduced
 * exactly, so the result equals the CPU back end's bit for bit; a channel
 * product outside [0, 256) keeps the low byte of its truncation to an int, as
 * the CPU back end's conversion does.  mode 0: one fused kernel; mode 1: the
 * five launches with float intermediates in the library workspace. */
HGB_API int hgb_unsharp(const hgb_view *in, const hgb_view *out, int boundary, int mode, void *stream);

/* ------------------------------------------------------------------ */
/* global reductions                                                   */
/* ------------------------------------------------------------------ */

/* Kernel::reduced_data (dsl/kernel.hpp:121-161) /
 * hipaccApplyReductionShared (runtime/hipacc_cu.tpp:312-408): one pass over
 * `in` (window may be NULL) with warp shuffles, a block combine and a
 * last-block combine behind a release/acquire ticket.  Result types:
 *   u8/u16/u32 SUM -> uint64, MIN/MAX -> same width as input (stored in a u32/u64 slot)
 *   i16/i32 SUM -> int64;  u64 SUM -> uint64
 *   f32/f16/bf16 SUM -> per-thread Kahan partials, FP64 cross-block combine;
 *   the 8-byte result is a double (the float result is its rounding)
 *   f32/f16/bf16 MIN/MAX/PROD -> folded in float, delivered widened to a double
 *   f64 -> double
 * `result_dev` (device, 8 bytes) and/or `result_host` (8 bytes; the call then
 * synchronises the stream). */
HGB_API int hgb_reduce(const hgb_view *in, const hgb_window *win, int op, void *result_dev, void *result_host,
               void *stream);

/* hgb_reduce for callers that cannot allocate device memory (no counterpart
 * in the reference).  hgb_reduce grows a library workspace with cudaMalloc on
 * first use.  Some callers cannot allow that: real-time frame loops that must
 * never block in the CUDA allocator, and plug-ins inside a host program whose
 * device memory belongs to the host's own allocator with a fixed budget.
 * This entry point allocates nothing: its
 * scratch is a fixed 16.25 KiB array in the library's device memory (block
 * partials for at most 1024 blocks; larger launches return HGB_ERR_LIMIT),
 * held by every GPU that loads the library until exit.  The first call on a
 * device resolves the array's address.  Every call shares the array: calls
 * that overlap on the GPU race.  Same
 * arguments, results and determinism as hgb_reduce. */
HGB_API int hgb_reduce_noalloc(const hgb_view *in, const hgb_window *win, int op, void *result_dev,
                               void *result_host, void *stream);

/* Binned data (Kernel::binned_data, dsl/kernel.hpp:163-200;
 * hipaccApplyBinningSegmented, runtime/hipacc_cu.tpp:410-464) of the
 * histogram binning function (samples-public/2_Global_Operators/Histogram/
 * src/main.cpp:41-47): for every pixel of the window (of every image of the
 * batch), bin (unsigned)(pixel / 255.0f * num_bins) += 1.  Indices past the
 * last bin are dropped (BINNING_CPU_2D, runtime/hipacc_cpu_red.hpp:70-126);
 * negative or NaN products count in bin 0.  u8 or f32 pixels, num_bins
 * 1..16384.  `bins_dev` (num_bins uint32, overwritten) and/or `bins_host`
 * (the call then synchronises the stream). */
HGB_API int hgb_histogram(const hgb_view *in, const hgb_window *win, unsigned num_bins, uint32_t *bins_dev,
                          uint32_t *bins_host, void *stream);

/* ------------------------------------------------------------------ */
/* pyramids (Pyramid / traverse, dsl/pyramid.hpp:97-318;                */
/* hipaccCreatePyramid, runtime/hipacc_cu.tpp:466-497)                  */
/* ------------------------------------------------------------------ */

/* A plan for the Laplacian pyramids of `n_images` FP32 images of uneven
 * sizes: level l is floor(w / 2^l) x floor(h / 2^l) (dsl/pyramid.hpp:103-114),
 * reduce = 5x5 mask + nearest-neighbour 2x downsample, expand = linear
 * filtering upsample, as the Gaussian_Laplacian_Pyramid sample.  The plan
 * owns the device arena of all levels and the tile work-list. */
typedef struct hgb_pyramid_plan hgb_pyramid_plan;
HGB_API int hgb_pyramid_plan_create(int n_images, const int *widths, const int *heights, int levels, const float *mask5,
                            int boundary, hgb_pyramid_plan **out);
HGB_API int hgb_pyramid_plan_destroy(hgb_pyramid_plan *plan);
/* Device views of level `level` of image `image`: Gaussian G_l and
 * Laplacian L_l (L of the last level is not defined; G of level 0 is the input
 * slot the caller fills). */
HGB_API int hgb_pyramid_level_view(const hgb_pyramid_plan *plan, int image, int level, hgb_view *gauss, hgb_view *lap);
/* Build all levels of all images.  mode 0: one persistent launch over the tile
 * work-list with bounded inter-level waits; mode 1: one launch per level over
 * all images; mode 2: per image, per level plain launches (blur, subsample,
 * difference), the reference's launch structure. */
HGB_API int hgb_pyramid_decompose(hgb_pyramid_plan *plan, int mode, void *stream);
/* Collapse (Restore): G_l = LF(G_{l+1}) + L_l from the bottom level up,
 * into the plan's Gaussian levels. */
HGB_API int hgb_pyramid_collapse(hgb_pyramid_plan *plan, void *stream);
/* Test support for the plan's bounded device-side waits (no counterpart in
 * the reference, whose kernels do not wait on one another).  `max_polls`
 * limits every wait of the plan's later launches (0 = the default, 2^22
 * polls).  kind 0: normal operation.  kind 1 (persistent form): the tiles of
 * `level` are claimed but never published, so the waits of level + 1 on them
 * run out.  kind 2: the tiles of `level` expect their staged box but no copy
 * is issued, so their barrier waits run out with nothing in flight.  Either
 * way the launch ends by itself, the device status word reads
 * HGB_ERR_TIMEOUT (hgb_device_status) and the context stays usable; nothing
 * faults or traps. */
HGB_API int hgb_pyramid_plan_wait_test(hgb_pyramid_plan *plan, long long max_polls, int kind, int level);
/* Measurement support for the single-launch form (no counterpart in the
 * reference): when `trace_dev` is set, each CTA of a later mode-0 launch whose
 * grid has at most `capacity` CTAs writes one record of 8 int64 at
 * trace_dev[8 * cta]: start and end on the global timer (ns) and on the SM
 * clock, SM clock cycles spent claiming tiles, waiting for previous levels and
 * running tiles, then (tiles taken) | (waits that polled) << 32.  NULL turns
 * it off. */
HGB_API int hgb_pyramid_plan_trace(hgb_pyramid_plan *plan, long long *trace_dev, long long capacity);

/* ------------------------------------------------------------------ */
/* adjoints                                                            */
/* ------------------------------------------------------------------ */

/* Adjoint of the SUM local operator out = conv(in, mask) with the boundary
 * transposed: CLAMP/MIRROR/REPEAT gather every output that read a pixel
 * through the remap, CONSTANT taps carry no gradient.
 *   grad_in  (may be NULL) = conv^T(grad_out)
 *   grad_mask_dev (may be NULL, mask_w*mask_h floats) = sum_p grad_out(p) * in(remap(p+c)),
 *   deterministic: block partials combined in FP64 in a fixed order.  With
 *   CONSTANT, taps outside the image count as reading 0 in grad_mask (the
 *   constant is not an argument here): exact for a forward with constant 0. 
 * mask is a device array (mask_dev) or host array (mask). */
HGB_API int hgb_local_op_adjoint(const hgb_view *in, const hgb_view *grad_out, const hgb_view *grad_in, const float *mask,
                         const float *mask_dev, int mask_w, int mask_h, int boundary, float *grad_mask_dev,
                         void *stream);

/* Adjoint of the bilateral filter hgb_bilateral (the body of
 * samples-public/3_Preprocessing/Bilateral_Filter/src/main.cpp:63-77, FP32
 * storage): for grad_out = dL/dy it returns
 *   grad_in (may be NULL)        = dL/din, with the boundary transposed: every
 *                                  tap that read a pixel through CLAMP / MIRROR /
 *                                  REPEAT sends its gradient there, CONSTANT taps
 *                                  carry none;
 *   grad_sigma_dev (may be NULL) = dL/dsigma_r (one float, summed over the batch,
 *                                  combined in FP64 in a fixed order).
 * The range weights are recomputed, never stored.  Same smask / size / sigma_r /
 * boundary / const_val as the forward; size odd, 3..13.  Uses the library
 * workspace (8 bytes per pixel): calls sharing it must be ordered on one
 * stream. */
HGB_API int hgb_bilateral_adjoint(const hgb_view *in, const hgb_view *grad_out, const float *smask, int size,
                                  float sigma_r, int boundary, float const_val, const hgb_view *grad_in,
                                  float *grad_sigma_dev, void *stream);

/* Adjoint of the separable filter hgb_separable (FP32 storage).  The forward
 * is the reference's two local operators, t = conv(in, row taps as 1 x K)
 * and out = conv(t, column taps as K x 1), each with the boundary (the
 * separable form has no reference primitive: lib/AST/Convolution.cpp:397-435
 * is the 2-D convolve it splits).  For grad_out = dL/dout:
 *   grad_in (may be NULL)               = dL/din, boundary transposed as in
 *                                         hgb_local_op_adjoint;
 *   grad_row_dev, grad_col_dev (may be
 *   NULL, k floats each, device)        = dL/drow_taps, dL/dcol_taps, combined in
 *                                         FP64 in a fixed order.
 * Same taps / k / boundary / const_val as the forward (const_val recomputes t;
 * the tap gradients count CONSTANT taps outside as reading 0).  Composed from
 * hgb_local_op and hgb_local_op_adjoint; uses the library workspace (8 bytes
 * per pixel): calls sharing it must be ordered on one stream. */
HGB_API int hgb_separable_adjoint(const hgb_view *in, const hgb_view *grad_out, const float *row_taps,
                                  const float *col_taps, int k, int boundary, float const_val,
                                  const hgb_view *grad_in, float *grad_row_dev, float *grad_col_dev, void *stream);

/* Adjoint of the MIN / MAX local operator: Kernel::reduce(Domain,
 * Reduce::MIN/MAX) (domain given, mask NULL) and Kernel::convolve(mask,
 * Reduce::MIN/MAX) (mask given, domain NULL or all ones); dsl/kernel.hpp:241-315,
 * lib/AST/Convolution.cpp:43-100.  The forward starts at FLT_MAX (MIN) or
 * FLT_MIN (MAX) and takes acc = acc < v ? acc : v (MIN) or acc > v ? acc : v
 * (MAX) per tap in row-major order.  Each output's gradient goes to the pixel
 * read by the tap that last replaced the running value (times its mask weight
 * for convolve); nothing flows when no tap replaced the initial value or when
 * the winner was a CONSTANT tap outside the image.  grad_in is gathered per
 * pixel in a fixed order (deterministic).  FP32 storage, masks up to 15 x 15.
 * Uses the library workspace (1 byte per pixel). */
HGB_API int hgb_local_op_minmax_adjoint(const hgb_view *in, const hgb_view *grad_out, const hgb_view *grad_in,
                                        const float *mask, const uint8_t *domain, int mask_w, int mask_h,
                                        int reduce, int boundary, float const_val, void *stream);

/* Forward + adjoint of the differentiation workload
 *   y1 = conv(x, mask), y = bilateral(y1; smask, sigma_r), loss = mean((y - t)^2)
 * in two fused kernels (forward with the loss gradient in its epilogue;
 * adjoint of the bilateral and of the convolution with the bilateral weights
 * recomputed).  x, t, grad_x: f32 batch views of the same size.  mask_dev and
 * sigma_dev are device parameters; outputs: loss_dev (double), grad_x,
 * grad_mask_dev (mask_k^2 floats), grad_sigma_dev (float).  mode 0 = fused,
 * mode 1 = the unfused chain of plain kernels (for comparison). */
HGB_API int hgb_conv_bilateral_mse(const hgb_view *x, const hgb_view *t, const float *mask_dev, int mask_k,
                           const float *smask, int smask_k, const float *sigma_dev, int boundary, int mode,
                           double *loss_dev, const hgb_view *grad_x, float *grad_mask_dev, float *grad_sigma_dev,
                           void *stream);

#ifdef __cplusplus
}
#endif

#endif /* HIPACC_GB300_H */

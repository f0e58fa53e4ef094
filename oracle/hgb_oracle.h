/*
 * hgb_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the semantics of the code Hipacc's CPU back end emits for
 * the image-processing hot path (local operators, point operators, global
 * reductions, pyramid construction) plus FP64 twins and the hand adjoint used
 * as the differentiation oracle.  Only tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline / reference arm may load this library; the product
 * library (libhipacc_gb300.so) never links or calls it.
 *
 * Every function cites the reference file:line whose behaviour it restates.
 * Numbering of the enums equals the reference enums so that values can be
 * passed through unchanged:
 *   boundary: hipacc::Boundary  (dsl/image.hpp:46-52)
 *   reduce:   hipacc::Reduce    (dsl/kernel.hpp:48-54)
 *
 * Floating-point contraction: the reference's generated C code is
 * `_tmp += mask * in` (lib/AST/Convolution.cpp:43-87).  Whether the C compiler
 * contracts that into an FMA depends on the target (GCC on aarch64 does by
 * default, x86-64 without -mfma does not).  Every float routine therefore has a
 * `contract` flag: 1 = the FMA-contracted form (acc = fma(m, x, acc)), 0 = the
 * separately rounded form.  The library is compiled with -ffp-contract=off so
 * that the flag alone decides.
 */
#ifndef HGB_ORACLE_H
#define HGB_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_UNDEFINED = 0, ORC_CLAMP = 1, ORC_REPEAT = 2, ORC_MIRROR = 3, ORC_CONSTANT = 4 };
enum { ORC_SUM = 0, ORC_MIN = 1, ORC_MAX = 2, ORC_PROD = 3 };

/* Boundary remap of one index (lib/AST/BorderHandling.cpp:41-120).
 * Returns the in-range index, or -2147483648 when CONSTANT reads the constant. */
int orc_remap(int mode, int idx, int lower, int upper);

/* Generic local operator (convolve / reduce(Domain)) over float images.
 * Strides are in elements.  acc_* is the Accessor window on `in`, is_* the
 * IterationSpace window on `out` (dsl/image.hpp:574-612, dsl/kernel.hpp:241-296). */
void orc_local_op_f32(const float *in, long in_stride, int acc_ox, int acc_oy, int acc_w, int acc_h,
                      float *out, long out_stride, int is_ox, int is_oy, int is_w, int is_h,
                      const float *mask, const uint8_t *domain, int mw, int mh,
                      int reduce, int bmode, float cval, int contract, int nthreads);
void orc_local_op_f64(const double *in, long in_stride, int acc_ox, int acc_oy, int acc_w, int acc_h,
                      double *out, long out_stride, int is_ox, int is_oy, int is_w, int is_h,
                      const double *mask, const uint8_t *domain, int mw, int mh,
                      int reduce, int bmode, double cval, int contract, int nthreads);

/* Separable filter as the reference expresses it: two local operators with a
 * 1xK and a Kx1 mask, FP32 intermediate image. */
void orc_separable_f32(const float *in, int w, int h, float *out, const float *row_taps,
                       const float *col_taps, int k, int bmode, float cval, int contract,
                       int nthreads);
void orc_separable_f64(const double *in, int w, int h, double *out, const double *row_taps,
                       const double *col_taps, int k, int bmode, double cval, int nthreads);

/* Sobel magnitude min(|gx|+|gy|, 255) with integer masks over their Domains
 * (samples-public/3_Preprocessing/Sobel/src/main.cpp:56-67, dsl/mask.hpp:238-250). */
void orc_sobel_mag_u8(const uint8_t *in, int w, int h, long in_stride, uint8_t *out, long out_stride,
                      const int *mask_x, const int *mask_y, int size, int bmode, int cval,
                      int nthreads);

/* RGBA -> gray point operator (wr*R + wg*G + wb*B) >> shift. */
void orc_rgba_to_gray_u8(const uint8_t *in, int w, int h, long in_stride_px, uint8_t *out,
                         long out_stride, int wr, int wg, int wb, int shift, int nthreads);

/* REDUCTION_CPU_2D (runtime/hipacc_cpu_red.hpp:19-68) restated: per-thread
 * partials over contiguous row blocks, each seeded by the first pixel of its
 * first row, then a serial combine in thread order. */
uint64_t orc_reduce_sum_u8_u64(const uint8_t *in, int w, int h, long stride, int nthreads);
uint32_t orc_reduce_max_u8(const uint8_t *in, int w, int h, long stride, int nthreads);
float    orc_reduce_f32(const float *in, int w, int h, long stride, int op, int nthreads);
double   orc_reduce_f32_exact(const float *in, int w, int h, long stride, int op);

/* Binning (Kernel::binned_data, dsl/kernel.hpp:163-200; CPU back end
 * BINNING_CPU_2D, runtime/hipacc_cpu_red.hpp:70-126) with the binning
 * function of samples-public/2_Global_Operators/Histogram/src/main.cpp:41-47:
 * bin (unsigned)(pixel / 255.0f * num_bins) += 1; indices >= num_bins are
 * dropped (the macro's Put).  Negative or NaN products go to bin 0 and
 * products >= 2^32 to 2^32 - 1 (the saturating conversion; C leaves them
 * undefined).  u8 pixels are widened to float first.  bins are overwritten. */
void orc_histogram_f32(const float *in, int w, int h, long stride, unsigned num_bins, uint32_t *bins);
void orc_histogram_u8(const uint8_t *in, int w, int h, long stride, unsigned num_bins, uint32_t *bins);

/* Bilateral filter (samples-public/3_Preprocessing/Bilateral_Filter/src/main.cpp:63-77)
 * with a float range sigma and float output p/d. */
void orc_bilateral_f32(const float *in, int w, int h, long stride, float *out, long out_stride,
                       const float *smask, int size, float sigma_r, int bmode, float cval,
                       int contract, int nthreads);
void orc_bilateral_f64(const double *in, int w, int h, long stride, double *out, long out_stride,
                       const double *smask, int size, double sigma_r, int bmode, double cval,
                       int nthreads);

/* Nearest-neighbour and linear-filtering resampling of a whole image
 * (lib/AST/Interpolate.cpp:85-113, runtime/hipacc_cpu_interpolate.hpp:157-197). */
void orc_resample_nn_f32(const float *src, int sw, int sh, float *dst, int dw, int dh, int contract);
void orc_resample_lf_f32(const float *src, int sw, int sh, float *dst, int dw, int dh, int contract);
/* B5 / CF / L3 resampling accessors (mode 3 / 4 / 5, hipacc::Interpolate
 * numbering) of the CPU back end with clamped taps; `contract` applies to the
 * mapped coordinate only (the GPU maps with one fused multiply-add). */
void orc_resample_filtered_f32(const float *src, int sw, int sh, float *dst, int dw, int dh, int mode, int contract);

/* Laplacian pyramid (samples-public/5_Other/Gaussian_Laplacian_Pyramid/src/main.cpp:199-248).
 * gauss[l] (l = 0..levels-1) and lap[l] (l = 0..levels-2) are caller buffers of
 * the level sizes w_l = w_{l-1}/2 (dsl/pyramid.hpp:103-114); gauss[0] is the input. */
void orc_pyramid_decompose_f32(float **gauss, float **lap, int w, int h, int levels,
                               const float *mask, int msize, int bmode, int contract,
                               int nthreads);
void orc_pyramid_decompose_f64(double **gauss, double **lap, int w, int h, int levels,
                               const double *mask, int msize, int bmode, int nthreads);
/* Collapse: out[l] = LF(out[l+1]) + lap[l], out[levels-1] = gauss bottom (Restore). */
void orc_pyramid_collapse_f32(float **out, float **lap, int w, int h, int levels, int contract);

/* Differentiation workload in FP64: y1 = conv(x, mask), y = bilateral(y1, smask,
 * sigma_r), loss = mean((y - t)^2).  `orc_c5_loss_f64` is the forward only (for
 * finite differences); `orc_c5_grad_f64` adds the hand adjoint. */
double orc_c5_loss_f64(const double *x, const double *t, int w, int h, const double *mask, int mk,
                       const double *smask, int sk, double sigma_r, int bmode, int nthreads);
/* Harris corner program of the Harris_Corner sample (3x3), out 0 / 1. */
void orc_harris_u8(const uint8_t *in, int w, int h, int bmode, float k, float threshold, uint8_t *out,
                   int nthreads);
/* Unsharp program of the Unsharp sample (3x3): uchar4 in and out; gray_out
 * (may be NULL) receives the luminance image. */
void orc_unsharp_u8x4(const uint8_t *rgba, int w, int h, int bmode, uint8_t *out, float *gray_out, int nthreads);
/* Adjoint of the bilateral filter (FP64): dL/din into grad_in (dense w x h) for
 * dL/dy = g; returns dL/dsigma_r. */
double orc_bilateral_adjoint_f64(const double *in, const double *g, int w, int h, const double *smask, int size,
                                 double sigma_r, int bmode, double cval, double *grad_in);
double orc_c5_grad_f64(const double *x, const double *t, int w, int h, const double *mask, int mk,
                       const double *smask, int sk, double sigma_r, int bmode, double *dx,
                       double *dmask, double *dsigma, int nthreads);

#ifdef __cplusplus
}
#endif

#endif

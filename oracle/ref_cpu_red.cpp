// ref_cpu_red.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Instantiates the reference's own CPU reduction macro REDUCTION_CPU_2D
// (runtime/hipacc_cpu_red.hpp:19-68), included where it lies in the reference
// tree by oracle/Makefile, to pin the restated reduce_2d in hgb_oracle.cpp.
// Built twice: without OpenMP (one partial) and with -DUSE_OPENMP (one
// partial per core, libgomp static schedule).  Also instantiates the binning
// macro BINNING_CPU_2D (runtime/hipacc_cpu_red.hpp:70-126) with the binning
// function of samples-public/2_Global_Operators/Histogram/src/main.cpp:41-47
// (bin(pixel / 255 * num_bins) = 1, reduce = sum).
#include <cstdint>
#include <vector>

#include "hipacc_cpu_red.hpp"

#ifdef USE_OPENMP
#define HGB_SUFFIX(n) n##_omp
namespace hgb_ref_omp {
#else
#define HGB_SUFFIX(n) n##_serial
namespace hgb_ref_serial {
#endif
// the macros define inline functions; a namespace per build keeps the serial
// and OpenMP instances apart in the shared library

static inline float hgb_red_sum(float a, float b) { return a + b; }
static inline float hgb_red_max(float a, float b) { return a > b ? a : b; }

REDUCTION_CPU_2D(hgb_sum, float, hgb_red_sum, 1)
REDUCTION_CPU_2D(hgb_max, float, hgb_red_max, 1)

// the histogram sample's binning function, in the form the CPU back end emits
// (the bin write goes through the macro's <name>Put, which drops indices
// beyond the last bin)
static inline unsigned hgb_bin_sum(unsigned a, unsigned b) { return a + b; }
inline void hgb_histPut(unsigned *_lmem, unsigned _offset, unsigned idx, unsigned val);
inline void hgb_hist(unsigned *_lmem, unsigned _offset, unsigned num_bins, int x, int y, float pixel) {
  (void)x;
  (void)y;
  hgb_histPut(_lmem, _offset, (unsigned)(pixel / 255.0f * num_bins), 1u);
}
typedef unsigned uint;
BINNING_CPU_2D(hgb_histogram, float, uint, hgb_bin_sum, hgb_hist, 1)

}  // namespace

#ifdef USE_OPENMP
using namespace hgb_ref_omp;
#else
using namespace hgb_ref_serial;
#endif

extern "C" float HGB_SUFFIX(ref_cpu_red_sum_f32)(float *in, int w, int h) {
  return hgb_sumKernel(in, w, h, w);
}
extern "C" float HGB_SUFFIX(ref_cpu_red_max_f32)(float *in, int w, int h) {
  return hgb_maxKernel(in, w, h, w);
}
extern "C" int HGB_SUFFIX(ref_cpu_red_cores)(void) { return GET_NUM_CORES; }
extern "C" void HGB_SUFFIX(ref_cpu_histogram_f32)(float *in, int w, int h, unsigned num_bins, unsigned *bins) {
  const std::vector<unsigned> r = hgb_histogramKernel(in, num_bins, w, h, w);
  for (unsigned i = 0; i < num_bins; ++i) bins[i] = r[i];
}

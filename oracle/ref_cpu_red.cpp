// ref_cpu_red.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Instantiates the reference's own CPU reduction macro REDUCTION_CPU_2D
// (runtime/hipacc_cpu_red.hpp:19-68), included where it lies in the reference
// tree by oracle/Makefile, to pin the restated reduce_2d in hgb_oracle.cpp.
// Built twice: without OpenMP (one partial) and with -DUSE_OPENMP (one
// partial per core, libgomp static schedule).
#include <cstdint>
#include <vector>

#include "hipacc_cpu_red.hpp"

static inline float hgb_red_sum(float a, float b) { return a + b; }
static inline float hgb_red_max(float a, float b) { return a > b ? a : b; }

REDUCTION_CPU_2D(hgb_sum, float, hgb_red_sum, 1)
REDUCTION_CPU_2D(hgb_max, float, hgb_red_max, 1)

#ifdef USE_OPENMP
#define HGB_SUFFIX(n) n##_omp
#else
#define HGB_SUFFIX(n) n##_serial
#endif

extern "C" float HGB_SUFFIX(ref_cpu_red_sum_f32)(float *in, int w, int h) {
  return hgb_sumKernel(in, w, h, w);
}
extern "C" float HGB_SUFFIX(ref_cpu_red_max_f32)(float *in, int w, int h) {
  return hgb_maxKernel(in, w, h, w);
}
extern "C" int HGB_SUFFIX(ref_cpu_red_cores)(void) { return GET_NUM_CORES; }

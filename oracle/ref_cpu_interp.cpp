// ref_cpu_interp.cpp -- TEST INFRASTRUCTURE ONLY.
//
// Instantiates the reference's own CPU back-end interpolation macros
// (runtime/hipacc_cpu_interpolate.hpp: INTERPOLATE_LINEAR_FILTERING_CPU,
// INTERPOLATE_BINOMIAL5_FILTERING_CPU, INTERPOLATE_CUBIC_FILTERING_CPU,
// INTERPOLATE_LANCZOS_FILTERING_CPU), included where it lies in the reference
// tree by oracle/Makefile, with clamped taps over the whole image, to pin the
// restated resampling accessors in hgb_oracle.cpp.  The output pixel (x, y)
// reads the accessor at the cell-centred mapped position scale/2 + scale*x
// (lib/AST/Interpolate.cpp:85-113), computed without contraction.
#include <cmath>

#include "hipacc_cpu_interpolate.hpp"

namespace hgb_ref_interp {
INTERPOLATE_LINEAR_FILTERING_CPU(lf_clamp, float, IMG_PARM(float), NO_PARM(float), IMG, BH_CLAMP_LOWER, BH_CLAMP_UPPER,
                                 BH_CLAMP_LOWER, BH_CLAMP_UPPER)
INTERPOLATE_BINOMIAL5_FILTERING_CPU(b5_clamp, float, IMG_PARM(float), NO_PARM(float), IMG, BH_CLAMP_LOWER,
                                    BH_CLAMP_UPPER, BH_CLAMP_LOWER, BH_CLAMP_UPPER)
INTERPOLATE_CUBIC_FILTERING_CPU(cf_clamp, float, IMG_PARM(float), NO_PARM(float), IMG, BH_CLAMP_LOWER, BH_CLAMP_UPPER,
                                BH_CLAMP_LOWER, BH_CLAMP_UPPER)
INTERPOLATE_LANCZOS_FILTERING_CPU(l3_clamp, float, IMG_PARM(float), NO_PARM(float), IMG, BH_CLAMP_LOWER,
                                  BH_CLAMP_UPPER, BH_CLAMP_LOWER, BH_CLAMP_UPPER)
}  // namespace hgb_ref_interp

// mode: 2 = LF, 3 = B5, 4 = CF, 5 = L3 (hipacc::Interpolate numbering)
extern "C" int ref_cpu_interp_f32(int mode, const float *src, int sw, int sh, float *dst, int dw, int dh) {
  using namespace hgb_ref_interp;
  const float sx = (float)sw / (float)dw, sy = (float)sh / (float)dh;
  for (int y = 0; y < dh; ++y) {
    const float ym = sy / 2 + sy * (float)y;
    for (int x = 0; x < dw; ++x) {
      const float xm = sx / 2 + sx * (float)x;
      float v;
      switch (mode) {
        case 2: v = lf_clamp(src, sw, xm, ym, sw, sh, 0, 0); break;
        case 3: v = b5_clamp(src, sw, xm, ym, sw, sh, 0, 0); break;
        case 4: v = cf_clamp(src, sw, xm, ym, sw, sh, 0, 0); break;
        case 5: v = l3_clamp(src, sw, xm, ym, sw, sh, 0, 0); break;
        default: return 1;
      }
      dst[(long)y * dw + x] = v;
    }
  }
  return 0;
}

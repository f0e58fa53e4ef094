// RGBA -> gray point operator (samples-public/0_Point_Operators/Color_Conversion,
// integer weights) and global reductions of a float image
// (samples-public/2_Global_Operators/Reduction_Sum / Reduction_Max).
#include <hipacc_gb300/hipacc.hpp>

#include "common.hpp"

using namespace hipacc;

int main() {
  hipaccInitCUDA(0);
  const int width = 640, height = 480;
  std::vector<unsigned char> raw = random_bytes(width * height * 4, 11);
  Image<uchar4> in(width, height, reinterpret_cast<const uchar4 *>(raw.data()));
  Image<uchar> out(width, height);
  Accessor<uchar4> acc(in);
  IterationSpace<uchar> iter(out);
  ColorConversion conv(iter, acc);
  conv.execute();
  const uchar *g = out.data();
  for (int p = 0; p < width * height; ++p)
    REQUIRE(g[p] == ((77 * raw[4 * p] + 150 * raw[4 * p + 1] + 29 * raw[4 * p + 2]) >> 8));
  std::vector<float> f = random_floats(width * height, 12);
  Image<float> fi(width, height, f.data());
  Image<float> fo(width, height);
  Accessor<float> facc(fi);
  IterationSpace<float> fit(fo);
  Reduction<float> rsum(fit, facc, Reduce::SUM), rmax(fit, facc, Reduce::MAX);
  double s = 0.0;
  float m = 0.0f;
  for (float v : f) {
    s += v;
    m = std::max(m, v);
  }
  REQUIRE(std::fabs(rsum.reduced_data() - s) <= 1e-6 * s);
  REQUIRE(rmax.reduced_data() == m);
  std::printf("Test PASSED\n");
  return 0;
}

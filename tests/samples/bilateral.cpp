// Bilateral filter in the shape of samples-public/3_Preprocessing/Bilateral_Filter
// (13x13 spatial Gaussian sigma_d = 3, float range sigma 0.1) with REPEAT.
#include <hipacc_gb300/hipacc.hpp>

#include "common.hpp"

using namespace hipacc;

int main() {
  hipaccInitCUDA(0);
  const int width = 300, height = 200, S = 13, R = 6;
  const float sigma_r = 0.1f;
  std::vector<float> coef(S * S);
  for (int j = 0; j < S; ++j)
    for (int i = 0; i < S; ++i) coef[j * S + i] = (float)std::exp(-((i - R) * (i - R) + (j - R) * (j - R)) / 18.0);
  std::vector<float> input = random_floats(width * height, 31);
  Image<float> in(width, height, input.data());
  Image<float> out(width, height);
  Mask<float> mask(S, S, coef.data());
  BoundaryCondition<float> bound(in, mask, Boundary::REPEAT);
  Accessor<float> acc(bound);
  IterationSpace<float> iter(out);
  BilateralFilter<float> filter(iter, acc, mask, sigma_r);
  filter.execute();
  const float *o = out.data();
  const float c_r = 0.5f / (sigma_r * sigma_r);
  double worst = 0.0;
  for (int y = 0; y < height; ++y)
    for (int x = 0; x < width; ++x) {
      const float ctr = input[(size_t)y * width + x];
      float d = 0.0f, p = 0.0f;
      for (int j = -R; j <= R; ++j)
        for (int i = -R; i <= R; ++i) {
          const float v = input[(size_t)(((y + j) % height + height) % height) * width + ((x + i) % width + width) % width];
          const float diff = v - ctr;
          const float s = std::exp(-c_r * diff * diff) * coef[(j + R) * S + i + R];
          d += s;
          p += s * v;
        }
      worst = std::max(worst, (double)std::fabs(o[(size_t)y * width + x] - p / d));
    }
  std::printf("max abs error vs the float reference: %.3g\n", worst);
  REQUIRE(worst <= 2e-5);
  std::printf("Test PASSED\n");
  return 0;
}

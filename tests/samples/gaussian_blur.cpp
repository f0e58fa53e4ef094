// Gaussian blur in the shape of samples-public/1_Local_Operators/Gaussian_Blur:
// Image, Mask, BoundaryCondition(CLAMP), Accessor, IterationSpace and a
// convolution kernel executed on the GPU; a naive reference loop checks every
// pixel including the borders.
#include <hipacc_gb300/hipacc.hpp>

#include "common.hpp"

using namespace hipacc;

int main() {
  hipaccInitCUDA(0);
  hipaccEnableTiming(true);
  const int width = 1024, height = 768;
  const float coef[5][5] = {{0.005008f, 0.017300f, 0.026151f, 0.017300f, 0.005008f},
                            {0.017300f, 0.059761f, 0.090339f, 0.059761f, 0.017300f},
                            {0.026151f, 0.090339f, 0.136565f, 0.090339f, 0.026151f},
                            {0.017300f, 0.059761f, 0.090339f, 0.059761f, 0.017300f},
                            {0.005008f, 0.017300f, 0.026151f, 0.017300f, 0.005008f}};
  std::vector<float> input = random_floats(width * height, 7);
  Image<float> in(width, height, input.data());
  Image<float> out(width, height);
  Mask<float> mask(coef);
  BoundaryCondition<float> bound(in, mask, Boundary::CLAMP);
  Accessor<float> acc(bound);
  IterationSpace<float> iter(out);
  Convolution<float> filter(iter, acc, mask);
  filter.execute();
  std::printf("GPU: %.3f ms, %.1f Mpixel/s\n", hipacc_last_kernel_timing(),
              width * height / hipacc_last_kernel_timing() / 1000.0);
  const float *output = out.data();
  for (int y = 0; y < height; ++y)
    for (int x = 0; x < width; ++x) {
      float sum = 0.0f;
      for (int yf = -2; yf <= 2; ++yf)
        for (int xf = -2; xf <= 2; ++xf)
          sum = std::fma(coef[yf + 2][xf + 2],
                         input[(size_t)clampi(y + yf, 0, height - 1) * width + clampi(x + xf, 0, width - 1)], sum);
      REQUIRE(output[(size_t)y * width + x] == sum);
    }
  std::printf("Test PASSED\n");
  return 0;
}

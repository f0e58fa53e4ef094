// Sobel magnitude with MIRROR and the global sum / max of the result, in the
// shape of samples-public/3_Preprocessing/Sobel + 2_Global_Operators.
#include <hipacc_gb300/hipacc.hpp>

#include "common.hpp"

using namespace hipacc;

int main() {
  hipaccInitCUDA(0);
  const int width = 1000, height = 777;
  const int cx[3][3] = {{-1, 0, 1}, {-2, 0, 2}, {-1, 0, 1}};
  const int cy[3][3] = {{-1, -2, -1}, {0, 0, 0}, {1, 2, 1}};
  std::vector<unsigned char> input = random_bytes(width * height, 3);
  Image<uchar> in(width, height, input.data());
  Image<uchar> out(width, height);
  Mask<int> mask_x(cx), mask_y(cy);
  BoundaryCondition<uchar> bound(in, mask_x, Boundary::MIRROR);
  Accessor<uchar> acc(bound);
  IterationSpace<uchar> iter(out);
  SobelMagnitude sobel(iter, acc, mask_x, mask_y);
  sobel.execute();
  const unsigned long long sum = sobel.reduced_sum();
  const unsigned max = sobel.reduced_max();
  const uchar *output = out.data();
  unsigned long long rsum = 0;
  unsigned rmax = 0;
  for (int y = 0; y < height; ++y)
    for (int x = 0; x < width; ++x) {
      int gx = 0, gy = 0;
      for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i) {
          const int v = input[(size_t)mirror(y + j, height) * width + mirror(x + i, width)];
          gx += cx[j + 1][i + 1] * v;
          gy += cy[j + 1][i + 1] * v;
        }
      const int m = std::min(std::abs(gx) + std::abs(gy), 255);
      REQUIRE(output[(size_t)y * width + x] == m);
      rsum += m;
      rmax = std::max<unsigned>(rmax, m);
    }
  REQUIRE(sum == rsum);
  REQUIRE(max == rmax);
  std::printf("sum %llu max %u\nTest PASSED\n", sum, max);
  return 0;
}

// Whole-program graph in the shape of Hipacc's CUDA-graph mode
// (samples-public/common/config/cuda-graph.conf): a Gaussian blur, a Sobel
// magnitude with its fused sum / max, and an RGBA->gray conversion recorded
// once into a CudaGraph -- the gray conversion on a second stream as an
// independent branch (fork / join) -- and replayed.  The replayed results are
// checked against plain CPU loops of the three kernels (the blur's taps
// row-major as fused multiply-adds, the Sobel samples' integer arithmetic, the
// integer gray weights) and against the eager execution; then new inputs are
// written and the same graph replayed again, so that a replay that re-used
// stale results would fail.
#include <hipacc_gb300/hipacc.hpp>

#include "common.hpp"

using namespace hipacc;

int main() {
  hipaccInitCUDA(0);
  const int width = 1000, height = 600;
  const float coef[3][3] = {{0.0625f, 0.125f, 0.0625f}, {0.125f, 0.25f, 0.125f}, {0.0625f, 0.125f, 0.0625f}};
  const int sx[3][3] = {{-1, 0, 1}, {-2, 0, 2}, {-1, 0, 1}};
  const int sy[3][3] = {{-1, -2, -1}, {0, 0, 0}, {1, 2, 1}};
  std::vector<float> f = random_floats(width * height, 21);
  std::vector<unsigned char> u = random_bytes(width * height, 22);
  std::vector<unsigned char> rgba = random_bytes(width * height * 4, 23);

  // eager reference results
  Image<float> fin(width, height, f.data()), fout_e(width, height), fout_g(width, height);
  Image<uchar> uin(width, height, u.data()), mag_e(width, height), mag_g(width, height);
  Image<uchar4> cin(width, height, reinterpret_cast<const uchar4 *>(rgba.data()));
  Image<uchar> gray_e(width, height), gray_g(width, height);
  Mask<float> blur(coef);
  Mask<int> mx(sx), my(sy);
  BoundaryCondition<float> fb(fin, blur, Boundary::MIRROR);
  Accessor<float> fa(fb);
  BoundaryCondition<uchar> ub(uin, mx, Boundary::CLAMP);
  Accessor<uchar> ua(ub);
  Accessor<uchar4> ca(cin);
  IterationSpace<float> fi_e(fout_e), fi_g(fout_g);
  IterationSpace<uchar> mi_e(mag_e), mi_g(mag_g), gi_e(gray_e), gi_g(gray_g);
  Convolution<float> conv_e(fi_e, fa, blur), conv_g(fi_g, fa, blur);
  SobelMagnitude sob_e(mi_e, ua, mx, my), sob_g(mi_g, ua, mx, my);
  ColorConversion col_e(gi_e, ca), col_g(gi_g, ca);
  conv_e.execute();
  sob_e.execute();
  col_e.execute();

  // the same program recorded once, the conversion as a parallel branch
  hgb_workspace_reserve(1 << 20);
  CudaGraph graph;
  Stream side;
  graph.begin();
  side.wait(graph.stream());  // fork
  hipaccSetStream(side.get());
  col_g.execute();
  hipaccSetStream(graph.stream().get());
  conv_g.execute();
  sob_g.execute();
  graph.stream().wait(side);  // join
  graph.end();
  for (int i = 0; i < 10; ++i) graph.launch();
  graph.synchronize();

  // CPU loops of the three kernels on the current host inputs
  auto check_all = [&](const std::vector<float> &fi, const std::vector<unsigned char> &ui,
                       const std::vector<unsigned char> &ci, bool with_eager) {
    const float *b = fout_g.data();
    const float *a = with_eager ? fout_e.data() : nullptr;
    for (int y = 0; y < height; ++y)
      for (int x = 0; x < width; ++x) {
        float acc = 0.0f;
        for (int j = -1; j <= 1; ++j)
          for (int i = -1; i <= 1; ++i)
            acc = std::fmaf(coef[j + 1][i + 1], fi[(size_t)mirror(y + j, height) * width + mirror(x + i, width)], acc);
        REQUIRE(b[(size_t)y * width + x] == acc);
        if (a) REQUIRE(a[(size_t)y * width + x] == acc);
      }
    const uchar *m2 = mag_g.data();
    const uchar *m1 = with_eager ? mag_e.data() : nullptr;
    unsigned long long s = 0;
    unsigned mx_ = 0;
    for (int y = 0; y < height; ++y)
      for (int x = 0; x < width; ++x) {
        int gx = 0, gy = 0;
        for (int j = -1; j <= 1; ++j)
          for (int i = -1; i <= 1; ++i) {
            const int v = ui[(size_t)clampi(y + j, 0, height - 1) * width + clampi(x + i, 0, width - 1)];
            gx += sx[j + 1][i + 1] * v;
            gy += sy[j + 1][i + 1] * v;
          }
        const int m = std::min(std::abs(gx) + std::abs(gy), 255);
        REQUIRE(m2[(size_t)y * width + x] == m);
        if (m1) REQUIRE(m1[(size_t)y * width + x] == m);
        s += (unsigned)m;
        mx_ = std::max<unsigned>(mx_, (unsigned)m);
      }
    REQUIRE(sob_g.reduced_sum() == s && sob_g.reduced_max() == mx_);
    if (with_eager) REQUIRE(sob_e.reduced_sum() == s && sob_e.reduced_max() == mx_);
    const uchar *g2 = gray_g.data();
    const uchar *g1 = with_eager ? gray_e.data() : nullptr;
    for (int p = 0; p < width * height; ++p) {
      const int g = (77 * ci[4 * p] + 150 * ci[4 * p + 1] + 29 * ci[4 * p + 2]) >> 8;
      REQUIRE(g2[p] == g);
      if (g1) REQUIRE(g1[p] == g);
    }
  };
  check_all(f, u, rgba, true);

  // new inputs into the same device images, the same graph replayed
  f = random_floats(width * height, 31);
  u = random_bytes(width * height, 32);
  rgba = random_bytes(width * height * 4, 33);
  fin = f.data();
  uin = u.data();
  cin = reinterpret_cast<const uchar4 *>(rgba.data());
  graph.launch();
  graph.synchronize();
  check_all(f, u, rgba, false);
  std::printf("Test PASSED\n");
  return 0;
}

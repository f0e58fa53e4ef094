// Whole-program graph in the shape of Hipacc's CUDA-graph mode
// (samples-public/common/config/cuda-graph.conf): a Gaussian blur, a Sobel
// magnitude with its fused sum / max, and an RGBA->gray conversion recorded
// once into a CudaGraph -- the gray conversion on a second stream as an
// independent branch (fork / join) -- and replayed; the replayed results must
// equal the eagerly executed ones bit for bit.
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

  const float *a = fout_e.data(), *b = fout_g.data();
  for (int p = 0; p < width * height; ++p) REQUIRE(a[p] == b[p]);
  const uchar *m1 = mag_e.data(), *m2 = mag_g.data();
  unsigned long long s = 0;
  for (int p = 0; p < width * height; ++p) {
    REQUIRE(m1[p] == m2[p]);
    s += m2[p];
  }
  REQUIRE(sob_g.reduced_sum() == s && sob_g.reduced_sum() == sob_e.reduced_sum());
  REQUIRE(sob_g.reduced_max() == sob_e.reduced_max());
  const uchar *g1 = gray_e.data(), *g2 = gray_g.data();
  for (int p = 0; p < width * height; ++p) REQUIRE(g1[p] == g2[p]);
  std::printf("Test PASSED\n");
  return 0;
}

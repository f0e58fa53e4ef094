// Laplacian pyramid with Pyramid / traverse in the shape of
// samples-public/5_Other/Gaussian_Laplacian_Pyramid: per level a blur, a
// nearest-neighbour subsample and a difference with a linear-filtering
// accessor, each its own kernel launch.  The batched persistent form
// (LaplacianPyramidBatch) must produce the same pyramid bit for bit.
#include <hipacc_gb300/hipacc.hpp>

#include "common.hpp"

using namespace hipacc;

int main() {
  hipaccInitCUDA(0);
  const int width = 601, height = 403, depth = 5;
  const float b1[5] = {1.f / 16, 4.f / 16, 6.f / 16, 4.f / 16, 1.f / 16};
  float coef[5][5];
  for (int j = 0; j < 5; ++j)
    for (int i = 0; i < 5; ++i) coef[j][i] = (float)((double)b1[j] * (double)b1[i]);
  std::vector<float> input = random_floats(width * height, 21);
  Image<float> gaus(width, height, input.data());
  Image<float> tmp(width, height);
  Image<float> lap(width, height);
  Mask<float> mask(coef);
  Pyramid<float> pgaus(gaus, depth), ptmp(tmp, depth), plap(lap, depth);
  traverse(pgaus, ptmp, plap, [&]() {
    if (!pgaus.is_top_level()) {
      BoundaryCondition<float> bound(pgaus(-1), mask, Boundary::MIRROR);
      Accessor<float> acc1(bound);
      IterationSpace<float> iter1(ptmp(-1));
      Convolution<float> blur(iter1, acc1, mask);
      blur.execute();
      Accessor<float> acc2(ptmp(-1), Interpolate::NN);
      IterationSpace<float> iter2(pgaus(0));
      Copy<float> sub(iter2, acc2);
      sub.execute();
      Accessor<float> acc3(pgaus(-1));
      Accessor<float> acc4(pgaus(0), Interpolate::LF);
      IterationSpace<float> iter3(plap(-1));
      Difference<float> dog(iter3, acc3, acc4);
      dog.execute();
    }
    traverse();
  });
  // the batched persistent launch of the same decomposition
  std::vector<int> ws{width}, hs{height};
  LaplacianPyramidBatch batch(ws, hs, depth, &coef[0][0], Boundary::MIRROR);
  Image<float> staging(width, height, input.data());
  hgb_view sv = staging.view(), g0 = batch.gauss(0, 0);
  check(hgb_convert(&sv, &g0, nullptr), "level upload");  // f32 -> f32 copy between pitched views
  batch.decompose(0);
  for (int l = 0; l < depth; ++l) {
    hgb_view bv = batch.gauss(0, l);
    Image<float> readback(bv.width, bv.height);
    hgb_view rv = readback.view();
    check(hgb_convert(&bv, &rv, nullptr), "level readback");
    const float *a = pgaus(l).data(), *c = readback.data();
    for (int i = 0; i < bv.width * bv.height; ++i) REQUIRE(a[i] == c[i]);
    if (l + 1 < depth) {
      hgb_view lb = batch.laplace(0, l);
      Image<float> lr(lb.width, lb.height);
      hgb_view lrv = lr.view();
      check(hgb_convert(&lb, &lrv, nullptr), "laplace readback");
      const float *la = plap(l).data(), *lc = lr.data();
      for (int i = 0; i < lb.width * lb.height; ++i) REQUIRE(la[i] == lc[i]);
    }
  }
  std::printf("Test PASSED\n");
  return 0;
}

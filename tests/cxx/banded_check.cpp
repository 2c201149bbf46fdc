// Banded LU with partial pivoting (helfem_gb300/csrc/banded.hpp) against
// the residual of dense matrices with the same band: random, shifted into
// indefiniteness, and with tiny diagonals that force row interchanges.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "banded.hpp"

int main() {
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  int bad = 0;
  const int sizes[] = {1, 5, 50, 300};
  const int bands[] = {1, 3, 14};
  for (int n : sizes)
    for (int w : bands)
      for (int kind = 0; kind < 3; ++kind) {
        std::vector<double> A((size_t)n * n, 0.0);
        for (int j = 0; j < n; ++j)
          for (int i = std::max(0, j - w); i <= std::min(n - 1, j + w); ++i) A[i + (size_t)j * n] = U(rng);
        for (int i = 0; i < n; ++i) {
          if (kind == 1) A[i + (size_t)i * n] -= 0.5;           // indefinite shift
          if (kind == 2) A[i + (size_t)i * n] *= 1e-6;          // pivoting needed
        }
        hfg::BandedLU lu;
        lu.reset(n, w, w);
        for (int j = 0; j < n; ++j)
          for (int i = std::max(0, j - w); i <= std::min(n - 1, j + w); ++i) lu.at(i, j) = A[i + (size_t)j * n];
        if (!lu.factor()) { std::printf("singular n %d w %d kind %d\n", n, w, kind); ++bad; continue; }
        std::vector<double> b(n), x(n);
        for (int i = 0; i < n; ++i) b[i] = x[i] = U(rng);
        lu.solve(x.data());
        double rmax = 0.0, amax = 0.0, xmax = 0.0;
        for (int i = 0; i < n; ++i) {
          double r = -b[i];
          for (int j = 0; j < n; ++j) r += A[i + (size_t)j * n] * x[j];
          rmax = std::max(rmax, std::fabs(r));
          xmax = std::max(xmax, std::fabs(x[i]));
        }
        for (double v : A) amax = std::max(amax, std::fabs(v));
        const double rel = rmax / (amax * xmax * n);
        if (!(rel < 1e-14)) { std::printf("residual n %d w %d kind %d rel %.3e\n", n, w, kind, rel); ++bad; }
      }
  // the shift-invert form: dense F and S, band w kept, theta inside the spectrum
  for (int n : {40, 200}) {
    const int w = 6;
    std::vector<double> F((size_t)n * n), S((size_t)n * n);
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const double d = std::fabs((double)(i - j));
        F[i + (size_t)j * n] = (i == j ? 2.0 + i : 0.0) + 0.3 / (1.0 + d) + (d > w ? 0.01 : 0.0);
        S[i + (size_t)j * n] = (i == j ? 1.0 : 0.0) + (d <= 1 ? 0.1 : 0.0);
      }
    const double theta = 7.3;
    hfg::BandedLU lu;
    if (!hfg::factor_shifted_band(F.data(), n, S.data(), n, n, w, theta, lu)) { ++bad; continue; }
    std::vector<double> b(n), x(n);
    for (int i = 0; i < n; ++i) b[i] = x[i] = U(rng);
    lu.solve(x.data());
    double rmax = 0.0;
    for (int i = 0; i < n; ++i) {
      double r = -b[i];
      for (int j = std::max(0, i - w); j <= std::min(n - 1, i + w); ++j)
        r += (F[i + (size_t)j * n] - theta * S[i + (size_t)j * n]) * x[j];
      rmax = std::max(rmax, std::fabs(r));
    }
    if (!(rmax < 1e-11)) { std::printf("shifted band n %d residual %.3e\n", n, rmax); ++bad; }
  }
  std::printf(bad ? "FAIL\n" : "ok\n");
  return bad ? 1 : 0;
}

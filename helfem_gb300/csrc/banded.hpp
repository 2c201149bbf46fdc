// LU factorisation with partial pivoting of a banded matrix and the solve,
// for the shift-invert preconditioner of the SCF refinement: the Fock
// blocks of the finite-element basis are banded (bandwidth nn-1) apart from
// exchange, so (F_band - theta S) z = r costs n (nn-1)^2 instead of n^3.
//
// Storage (the usual band layout for pivoted banded LU): column-major
// ld x n with ld = 2 kl + ku + 1; A(i, j) sits at ab[(kl + ku + i - j) +
// j * ld] for max(0, j - ku) <= i <= min(n - 1, j + kl); the first kl rows
// hold the fill-in of U that row interchanges create.
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

namespace hfg {

struct BandedLU {
  int n = 0, kl = 0, ku = 0, ld = 0;
  std::vector<double> ab;
  std::vector<int> piv;

  void reset(int n_, int kl_, int ku_) {
    n = n_;
    kl = kl_;
    ku = ku_;
    ld = 2 * kl + ku + 1;
    ab.assign((size_t)ld * n, 0.0);
    piv.assign(n, 0);
  }
  double& at(int i, int j) { return ab[(size_t)(kl + ku + i - j) + (size_t)j * ld]; }
  double at(int i, int j) const { return ab[(size_t)(kl + ku + i - j) + (size_t)j * ld]; }

  // in place; false when a pivot column is exactly zero (singular)
  bool factor() {
    int ju = 0;  // last column touched by the interchanges so far
    for (int j = 0; j < n; ++j) {
      const int km = std::min(kl, n - 1 - j);
      int jp = 0;
      double best = std::fabs(at(j, j));
      for (int i = 1; i <= km; ++i) {
        const double v = std::fabs(at(j + i, j));
        if (v > best) { best = v; jp = i; }
      }
      piv[j] = j + jp;
      if (best == 0.0) return false;
      ju = std::max(ju, std::min(j + ku + jp, n - 1));
      if (jp != 0)
        for (int c = j; c <= ju; ++c) std::swap(at(j, c), at(j + jp, c));
      const double inv = 1.0 / at(j, j);
      for (int i = 1; i <= km; ++i) at(j + i, j) *= inv;
      for (int c = j + 1; c <= ju; ++c) {
        const double u = at(j, c);
        if (u == 0.0) continue;
        for (int i = 1; i <= km; ++i) at(j + i, c) -= at(j + i, j) * u;
      }
    }
    return true;
  }

  // b <- A^-1 b
  void solve(double* b) const {
    const int kv = kl + ku;
    for (int j = 0; j < n; ++j) {
      const int km = std::min(kl, n - 1 - j);
      if (piv[j] != j) std::swap(b[j], b[piv[j]]);
      const double bj = b[j];
      if (bj != 0.0)
        for (int i = 1; i <= km; ++i) b[j + i] -= at(j + i, j) * bj;
    }
    for (int j = n - 1; j >= 0; --j) {
      b[j] /= at(j, j);
      const double bj = b[j];
      if (bj != 0.0)
        for (int i = std::max(0, j - kv); i < j; ++i) b[i] -= at(i, j) * bj;
    }
  }
};

// Factor M = band_w(F) - theta band_w(S) for dense column-major n x n F and
// S (leading dimensions ldf, lds; entries with |i - j| > w are dropped) into
// lu. Returns false when M is singular.
inline bool factor_shifted_band(const double* F, int ldf, const double* S, int lds, int n, int w, double theta,
                                BandedLU& lu) {
  lu.reset(n, w, w);
  for (int j = 0; j < n; ++j)
    for (int i = std::max(0, j - w); i <= std::min(n - 1, j + w); ++i)
      lu.at(i, j) = F[i + (size_t)j * ldf] - theta * S[i + (size_t)j * lds];
  return lu.factor();
}

}  // namespace hfg

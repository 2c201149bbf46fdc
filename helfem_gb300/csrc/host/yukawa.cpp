// Host tables of the Yukawa-screened exchange kernel e^{-lambda r12}/r12
// (TwoDBasisT::compute_yukawa, src/atomic/TwoDBasis.cpp:736-758; the radial
// factors of libhelfemqc/include/CoulombExchangeFE.h:175-217 in Yukawa mode,
// RadialBasis.cpp:321-330 and 719-737, quadrature.cpp:163-197).
//
// The kernel separates as 4 pi lambda sum_L i_L(lambda r<) k_L(lambda r>)
// sum_M Y_L^M Y_L^M*, with the modified spherical Bessel functions
//   i_L(x) = sqrt(pi / 2x) I_{L+1/2}(x),   k_L(x) = sqrt(2 / (pi x)) K_{L+1/2}(x)
// (libhelfem/include/math.h:48-110). For x -> 0, 4 pi lambda i_L k_L tends to
// the bare 4 pi/(2L+1) r<^L / r>^{L+1}. i_L is summed from its Taylor series
// below x = 0.5 (the closed form is 0/0 there) and taken from the C++17
// special functions above; k_L from std::cyl_bessel_k.
#include <algorithm>
#include <cmath>
#include <stdexcept>

#include "atom.hpp"

namespace hfg {

double bessel_il(double x, int L) {
  const double ax = std::fabs(x);
  double v;
  if (ax < 0.5) {
    double dfac = 1.0;  // (2L+1)!!
    for (int j = 3; j <= 2 * L + 1; j += 2) dfac *= j;
    double term = std::pow(ax, L) / dfac;
    v = term;
    const double h = 0.5 * ax * ax;
    for (int k = 1; k < 200; ++k) {
      term *= h / ((double)k * (2.0 * L + 2.0 * k + 1.0));
      v += term;
      if (std::fabs(term) <= 1e-18 * std::fabs(v)) break;
    }
  } else {
    v = std::cyl_bessel_i(L + 0.5, ax) * std::sqrt(M_PI / (2.0 * ax));
  }
  return (x < 0.0 && (L & 1)) ? -v : v;
}

double bessel_kl(double x, int L) { return std::cyl_bessel_k(L + 0.5, x) * std::sqrt(2.0 / (M_PI * x)); }

void AtomHost::build_yukawa(double lambda) {
  if (!(lambda > 0.0)) throw std::invalid_argument("Yukawa screening parameter must be positive");
  const int nn = rad.nn, nel = rad.nel, n2 = nn * nn;
  y_lambda = lambda;
  y_rs.assign((size_t)NL * nel * n2, 0.0);
  y_rb.assign((size_t)NL * nel * n2, 0.0);
  y_tk.assign((size_t)NL * nel * n2 * n2, 0.0);
  rad.prepare_twoe();
#pragma omp parallel for collapse(2) schedule(dynamic)
  for (int L = 0; L < NL; ++L)
    for (int e = 0; e < nel; ++e) {
      const size_t le = (size_t)L * nel + e;
      const double scale = (2.0 * L + 1.0) * lambda;
      auto a = rad.weighted_integral([L, lambda](double r) { return bessel_il(lambda * r, L); }, e);
      for (int i = 0; i < n2; ++i) y_rs[le * n2 + i] = scale * a[i];
      if (e > 0) {  // the outer factor is never used on the innermost element
        auto b = rad.weighted_integral([L, lambda](double r) { return bessel_kl(lambda * r, L); }, e);
        std::copy(b.begin(), b.end(), y_rb.begin() + le * n2);
      }
      const std::vector<double> T = rad.twoe_separable([L, lambda](double r) { return bessel_il(lambda * r, L); },
                                                       [L, lambda](double r) { return bessel_kl(lambda * r, L); }, e);
      int r = 0;
      const std::vector<double> Lc = pivoted_cholesky(T, n2, chol_tol, r);
      // exchange ordering: K_ac = sum_bd (ab|cd) P_bd, rows (a + c nn), cols (b + d nn)
      double* out = &y_tk[le * n2 * n2];
      std::vector<double> Lt((size_t)n2 * r);
      for (int p = 0; p < r; ++p)
        for (int ab = 0; ab < n2; ++ab) Lt[(size_t)ab * r + p] = Lc[ab + (size_t)p * n2];
      for (int d = 0; d < nn; ++d)
        for (int b = 0; b < nn; ++b)
          for (int c = 0; c < nn; ++c)
            for (int a2 = 0; a2 < nn; ++a2) {
              double s = 0.0;
              const double* x = &Lt[(a2 + (size_t)b * nn) * r];
              const double* y = &Lt[(c + (size_t)d * nn) * r];
              for (int p = 0; p < r; ++p) s += x[p] * y[p];
              out[(a2 + (size_t)c * nn) + (size_t)(b + d * nn) * n2] = scale * s;
            }
    }
}

}  // namespace hfg

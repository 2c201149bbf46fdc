// Range-separated exchange with the erfc kernel: the pair tables.
//
//   erfc expansion      libhelfem/src/erfc_expn.cpp (Angyan, Gerber and
//                       Marsman, J. Phys. A 39, 8613 (2006), eqs. 21-30)
//   pair integrals      libhelfem/src/RadialBasis.cpp:742-811,
//                       libhelfem/src/quadrature.cpp:203-249
//   exchange ordering   libhelfemqc/include/CoulombExchangeFE.h:275-295,
//                       libhelfem/src/utils.cpp:54-80
//
// Phi_L(X, x) (X >= x) is the Legendre coefficient of erfc(mu r12)/(mu r12)
// at X = mu r>, x = mu r<: the general closed form where both arguments
// are large enough, the Taylor series in x otherwise (x < 0.4 or X < 0.5,
// the reference's choice). The pair integrals use the radial basis's
// modified Gauss-Chebyshev rule on both elements; when both electrons are in
// the same element the inner rule is repeated on as many sub-intervals as it
// has points (the electronic cusp), and the table is symmetrised.
#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <vector>

#include "atom.hpp"

namespace hfg {
namespace {

double dfact(int n) {
  double v = 1.0;
  for (int k = n; k >= 2; k -= 2) v *= k;
  return v;
}
double fact(int n) {
  double v = 1.0;
  for (int k = 2; k <= n; ++k) v *= k;
  return v;
}
// the reference's binomial for the series coefficients: for n < -1 it
// recurses as C(n, m) = (-1)^m C(n + m - 1, m), which is not the
// generalised binomial
double binom_reference(int n, int m) {
  if (n == -1) return (m % 2) ? -1.0 : 1.0;
  if (n == 0) return m == 0 ? 1.0 : 0.0;
  if (m == 0) return 1.0;
  if (m == 1) return n;
  if (n > 0 && m > n) return 0.0;
  if (n < 0) return binom_reference(n + m - 1, m) * ((m % 2) ? -1.0 : 1.0);
  double v = 1.0;
  const int k = std::min(m, n - m);
  for (int i = 0; i < k; ++i) v *= double(n - i) / double(i + 1);
  return v;
}
double binom_exact(int n, int m) {
  double v = 1.0;
  for (int i = 0; i < m; ++i) v *= double(n - i) / double(i + 1);
  return v;
}

double Fn(int n, double X, double x) {  // eq. 22
  const double ep = std::exp(-std::pow(X + x, 2)), em = std::exp(-std::pow(X - x, 2));
  const double pre = -1.0 / (4.0 * X * x);
  double F = 0.0;
  for (int p = 0; p <= n; ++p)
    F += std::pow(pre, p + 1) * (fact(n + p) / (fact(p) * fact(n - p))) *
         (std::pow(-1.0, n - p) * ep - em);
  return 2.0 / std::sqrt(M_PI) * F;
}
double Hn(int n, double X, double x) {  // eq. 24, X >= x
  const double a = std::pow(X, 2 * n + 1), b = std::pow(x, 2 * n + 1);
  return ((a + b) * std::erfc(X + x) - (a - b) * std::erfc(X - x)) / (2.0 * std::pow(x * X, n + 1));
}
double phi_general(int n, double X, double x) {  // eq. 21
  double s = 0.0;
  for (int m = 1; m <= n; ++m) {
    const double Xm = std::pow(X, m), xm = std::pow(x, m);
    s += Fn(n - m, X, x) * ((Xm * Xm + xm * xm) / (Xm * xm));
  }
  return Fn(n, X, x) + s + Hn(n, X, x);
}
double Dnk(int n, int k, double X, bool exact) {  // eqs. 28, 29
  const double pre = std::exp(-X * X) / std::sqrt(M_PI) * std::pow(2.0, n + 1) * std::pow(X, 2 * n + 1);
  if (k == 0) {
    double s = 0.0;
    for (int m = 1; m <= n; ++m) s += 1.0 / (dfact(2 * (n - m) + 1) * std::pow(2.0 * X * X, m));
    return std::erfc(X) + pre * s;
  }
  double s = 0.0;
  for (int m = 1; m <= k; ++m)
    s += (exact ? binom_exact(m - k - 1, m - 1) : binom_reference(m - k - 1, m - 1)) *
         std::pow(2.0 * X * X, k - m) / dfact(2 * (n + k - m) + 1);
  return pre * (2.0 * n + 1.0) / (fact(k) * (2.0 * (n + k) + 1.0)) * s;
}
// the series coefficients D_nk(X) of one outer argument, made on demand
// (the same values the series would compute term by term)
struct SeriesCoef {
  double X = 0.0;
  std::vector<double> D;
  double at(int n, int k, bool exact) {
    while ((int)D.size() <= k) D.push_back(Dnk(n, (int)D.size(), X, exact));
    return D[k];
  }
};

double phi_short(int n, double X, double x, bool exact, SeriesCoef& c) {  // eq. 30
  if (x == 0.0 && n > 0) return 0.0;
  if (n == 0 && x == 0.0 && X == 0.0) return 1.0;
  double P = 0.0;
  for (int k = 0; k <= 200; k += 2) {
    const double d = c.at(n, k, exact) * std::pow(x, n + 2 * k) + c.at(n, k + 1, exact) * std::pow(x, n + 2 * (k + 1));
    P += d;
    if (std::fabs(d) < 2.220446049250313e-16 * std::max(std::fabs(P), 1.0)) return P / std::pow(X, n + 1);
  }
  throw std::runtime_error("erfc kernel: short-range series did not converge");
}

}  // namespace

double erfc_phi(int n, double A, double B, bool exact) {
  const double X = std::max(A, B), x = std::min(A, B);
  SeriesCoef c;
  c.X = X;
  if (x < 0.4 || X < 0.5) return phi_short(n, X, x, exact, c);
  return phi_general(n, X, x);
}

void AtomHost::build_erfc(double mu, bool exact_binomial) {
  if (!(mu > 0.0)) throw std::invalid_argument("erfc range-separation parameter must be positive");
  const int nn = rad.nn, nel = rad.nel, n2 = nn * nn;
  e_mu = mu;
  e_exact = exact_binomial;
  e_tk.assign((size_t)NL * nel * nel * n2 * n2, 0.0);
  std::vector<double> xq, wq;
  cheb_rule(nquad, xq, wq);
  const int nq = (int)xq.size();
  // the inner rule on nq sub-intervals (pairs within one element)
  std::vector<double> xs((size_t)nq * nq), ws((size_t)nq * nq);
  for (int ii = 0; ii < nq; ++ii) {
    const double a = ii * 2.0 / nq - 1.0, b = (ii + 1) * 2.0 / nq - 1.0, mid = 0.5 * (a + b), len = 0.5 * (b - a);
    for (int q = 0; q < nq; ++q) {
      xs[(size_t)ii * nq + q] = mid + xq[q] * len;
      ws[(size_t)ii * nq + q] = wq[q] * len;
    }
  }
  // weighted pair products of the padded primitives at a rule:
  // out[q + (a + b nn) * npts] = w_q sf B_a B_b(r_q)
  auto pairs = [&](int e, const std::vector<double>& x, const std::vector<double>& w, std::vector<double>& out) {
    std::vector<double> Bv;
    rad.B(e, x, 0, Bv);
    const size_t np = x.size();
    out.assign(np * n2, 0.0);
    for (int b = 0; b < nn; ++b)
      for (int a = 0; a < nn; ++a)
        for (size_t q = 0; q < np; ++q)
          out[q + (size_t)(a + b * nn) * np] = w[q] * rad.sf(e) * Bv[q + (size_t)a * np] * Bv[q + (size_t)b * np];
  };
#pragma omp parallel for collapse(3) schedule(dynamic)
  for (int L = 0; L < NL; ++L)
    for (int ea = 0; ea < nel; ++ea)
      for (int eb = 0; eb < nel; ++eb) {
        const bool same = (ea == eb);
        const std::vector<double>& xk = same ? xs : xq;
        const std::vector<double>& wk = same ? ws : wq;
        const size_t nk = xk.size();
        std::vector<double> Pi, Pk, F((size_t)nq * nk), FP((size_t)nq * n2), T((size_t)n2 * n2);
        pairs(ea, xq, wq, Pi);
        pairs(eb, xk, wk, Pk);
        // series coefficients per point (the outer argument of a pair is
        // one of its two points)
        std::vector<SeriesCoef> ci(nq), ck(nk);
        for (int a = 0; a < nq; ++a) ci[a].X = mu * (rad.mid(ea) + rad.sf(ea) * xq[a]);
        for (size_t b = 0; b < nk; ++b) ck[b].X = mu * (rad.mid(eb) + rad.sf(eb) * xk[b]);
        for (size_t b = 0; b < nk; ++b)
          for (int a = 0; a < nq; ++a) {
            const double A1 = ci[a].X, B1 = ck[b].X;
            SeriesCoef& c = (A1 >= B1) ? ci[a] : ck[b];
            const double X = std::max(A1, B1), x = std::min(A1, B1);
            F[a + (size_t)b * nq] = (x < 0.4 || X < 0.5) ? phi_short(L, X, x, exact_binomial, c)
                                                         : phi_general(L, X, x);
          }
        // FP = F Pk (nq x n2), T = Pi^T FP (n2 x n2): (ij|kl), rows i + j nn, cols k + l nn
        std::fill(FP.begin(), FP.end(), 0.0);
        for (int c = 0; c < n2; ++c)
          for (size_t b = 0; b < nk; ++b) {
            const double pk = Pk[b + (size_t)c * nk];
            if (pk == 0.0) continue;
            for (int a = 0; a < nq; ++a) FP[a + (size_t)c * nq] += F[a + (size_t)b * nq] * pk;
          }
        for (int c = 0; c < n2; ++c)
          for (int r = 0; r < n2; ++r) {
            double s = 0.0;
            for (int a = 0; a < nq; ++a) s += Pi[a + (size_t)r * nq] * FP[a + (size_t)c * nq];
            T[r + (size_t)c * n2] = s;
          }
        if (same)
          for (int c = 0; c < n2; ++c)
            for (int r = 0; r < c; ++r) {
              const double v = 0.5 * (T[r + (size_t)c * n2] + T[c + (size_t)r * n2]);
              T[r + (size_t)c * n2] = T[c + (size_t)r * n2] = v;
            }
        // exchange ordering, times mu: out[t = j + k nn, v = i + l nn] = mu (ij|kl)
        double* out = &e_tk[(((size_t)L * nel + ea) * nel + eb) * n2 * n2];
        for (int l = 0; l < nn; ++l)
          for (int k = 0; k < nn; ++k)
            for (int j = 0; j < nn; ++j)
              for (int i = 0; i < nn; ++i)
                out[(j + (size_t)k * nn) + (size_t)(i + l * nn) * n2] =
                    mu * T[(i + (size_t)j * nn) + (size_t)(k + l * nn) * n2];
      }
}

}  // namespace hfg

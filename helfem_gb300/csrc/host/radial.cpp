// FP64 host tabulation of the finite-element radial basis.
//
// Follows HelFEM's radial machinery in what it computes:
//   Gauss-Lobatto LIP nodes           libhelfem/include/lobatto.h:35-108
//   modified Gauss-Chebyshev rule     libhelfem/include/chebyshev.h:31-55
//   LIP values/derivatives            libhelfem/include/LIPBasis_eval.h:29-100
//   B/r deflation on element 0        libhelfem/include/LIPBasis.h:74-101
//   radial integrals (R = B/r form)   libhelfem/src/RadialBasis.cpp:245-257
//   R and dR/dr on a grid             libhelfem/src/RadialBasis.cpp:868-901
//   in-element 2e tensor              libhelfem/src/quadrature.cpp:36-161
// The reference converges each integral by doubling a Gauss-Lobatto rule
// until it is stable to 8 eps. Here every integral is evaluated once with a
// Gauss-Legendre rule that is exact for the polynomial integrands (element 0,
// the inner r'^L moments) and far past convergence for the analytic ones
// (their r = 0 pole lies outside the element), which gives the same values to
// a few ulps at a fraction of the cost.
#include <cmath>
#include <map>
#include <mutex>
#include <stdexcept>
#include <utility>

#include "atom.hpp"

namespace hfg {

namespace {
// rules are computed once per order (the tabulation asks for the same few
// orders thousands of times, from several threads)
std::mutex gl_mutex;
std::map<int, std::pair<std::vector<double>, std::vector<double>>> gl_cache;
}  // namespace

void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  {
    std::lock_guard<std::mutex> g(gl_mutex);
    auto it = gl_cache.find(n);
    if (it != gl_cache.end()) {
      x = it->second.first;
      w = it->second.second;
      return;
    }
  }
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    double pp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        const double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      const double z1 = z;
      z = z1 - p1 / pp;
      if (std::fabs(z - z1) < 1e-16) {
        // one more evaluation for the weight at the converged node
        p1 = 1.0; p2 = 0.0;
        for (int j = 1; j <= n; ++j) {
          const double p3 = p2;
          p2 = p1;
          p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
        }
        pp = n * (z * p1 - p2) / (z * z - 1.0);
        break;
      }
    }
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
  }
  std::lock_guard<std::mutex> g(gl_mutex);
  gl_cache.emplace(n, std::make_pair(x, w));
}

void gauss_lobatto(int n, std::vector<double>& x, std::vector<double>& w) {
  if (n < 2) throw std::invalid_argument("Gauss-Lobatto rule needs at least 2 nodes");
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  // interior nodes are the roots of P'_{n-1}; Newton from Chebyshev-Gauss-
  // Lobatto guesses, using (1-x^2) P'_{n-1} = (n-1)(P_{n-2} - x P_{n-1})
  const int N = n - 1;
  for (int i = 0; i < n; ++i) {
    double z = -std::cos(M_PI * i / N);
    if (i == 0) { x[i] = -1.0; continue; }
    if (i == N) { x[i] = 1.0; continue; }
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int j = 2; j <= N; ++j) {
        const double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
        p0 = p1;
        p1 = p2;
      }
      // f = (p0 - z p1) ~ (1-z^2) P'_N / N ; f' = -(N+1) p1 ... use
      // g(z) = P'_N(z), g'(z) = (2 z P'_N - N(N+1) P_N)/(1-z^2)
      const double dP = N * (p0 - z * p1) / (1.0 - z * z);
      const double d2P = (2.0 * z * dP - N * (N + 1.0) * p1) / (1.0 - z * z);
      const double dz = dP / d2P;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[i] = z;
  }
  for (int i = 0; i < n; ++i) {
    double p0 = 1.0, p1 = x[i];
    for (int j = 2; j <= N; ++j) {
      const double p2 = ((2.0 * j - 1.0) * x[i] * p1 - (j - 1.0) * p0) / j;
      p0 = p1;
      p1 = p2;
    }
    w[i] = 2.0 / (N * (N + 1.0) * p1 * p1);
  }
}

void cheb_rule(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 1; i <= n; ++i) {
    const double ang = i * M_PI / (n + 1);
    const double s = std::sin(ang), c = std::cos(ang), s2 = s * s;
    // stored reversed: ascending in x
    w[n - i] = 16.0 / 3.0 / (n + 1) * s2 * s2;
    x[n - i] = 1.0 - 2.0 * i / (n + 1.0) + 2.0 / M_PI * (1.0 + 2.0 / 3.0 * s2) * c * s;
  }
}

void lip_eval(const std::vector<double>& x, const std::vector<double>& nodes, int nder,
              std::vector<double>& out) {
  const int np = (int)x.size(), n = (int)nodes.size();
  out.assign((size_t)np * n, 0.0);
  std::vector<double> inv(n);
  for (int fi = 0; fi < n; ++fi) {
    for (int p = 0; p < n; ++p) inv[p] = (p == fi) ? 0.0 : 1.0 / (nodes[fi] - nodes[p]);
    for (int ix = 0; ix < np; ++ix) {
      double acc = 0.0;
      if (nder == 0) {
        acc = 1.0;
        for (int p = 0; p < n; ++p)
          if (p != fi) acc *= (x[ix] - nodes[p]) * inv[p];
      } else if (nder == 1) {
        for (int d1 = 0; d1 < n; ++d1) {
          if (d1 == fi) continue;
          double v = inv[d1];
          for (int p = 0; p < n; ++p)
            if (p != fi && p != d1) v *= (x[ix] - nodes[p]) * inv[p];
          acc += v;
        }
      } else if (nder == 2) {
        for (int d1 = 0; d1 < n; ++d1) {
          if (d1 == fi) continue;
          for (int d2 = 0; d2 < d1; ++d2) {
            if (d2 == fi) continue;
            double v = inv[d1] * inv[d2];
            for (int p = 0; p < n; ++p)
              if (p != fi && p != d1 && p != d2) v *= (x[ix] - nodes[p]) * inv[p];
            acc += v;
          }
        }
        acc *= 2.0;
      } else {
        throw std::invalid_argument("lip_eval: nder <= 2");
      }
      out[ix + (size_t)fi * np] = acc;
    }
  }
}

int RadialBasis::nfun(int e) const {
  int n = nn;
  if (e == 0) --n;
  if (e == nel - 1) --n;
  return n;
}

void RadialBasis::B(int e, const std::vector<double>& x, int nder, std::vector<double>& out) const {
  lip_eval(x, nodes, nder, out);
  const int np = (int)x.size();
  const double scale = std::pow(sf(e), -nder);
  for (int p = 0; p < nn; ++p)
    for (int ix = 0; ix < np; ++ix)
      out[ix + (size_t)p * np] = valid(e, p) ? out[ix + (size_t)p * np] * scale : 0.0;
}

void RadialBasis::R(int e, const std::vector<double>& x, std::vector<double>& out) const {
  const int np = (int)x.size();
  if (e == 0) {
    // B_u = (x+1)/(x_u+1) * Lred_u(x), r = sf*(x+1)  =>  B_u/r = Lred_u/(sf (x_u+1))
    std::vector<double> red, rn(nodes.begin() + 1, nodes.end());
    lip_eval(x, rn, 0, red);
    out.assign((size_t)np * nn, 0.0);
    for (int p = 1; p < nn; ++p) {
      if (!valid(e, p)) continue;
      const double f = 1.0 / (sf(0) * (nodes[p] + 1.0));
      for (int ix = 0; ix < np; ++ix) out[ix + (size_t)p * np] = red[ix + (size_t)(p - 1) * np] * f;
    }
    return;
  }
  B(e, x, 0, out);
  for (int p = 0; p < nn; ++p)
    for (int ix = 0; ix < np; ++ix) out[ix + (size_t)p * np] /= (mid(e) + sf(e) * x[ix]);
}

void RadialBasis::dR(int e, const std::vector<double>& x, std::vector<double>& out) const {
  const int np = (int)x.size();
  if (e == 0) {
    std::vector<double> red, rn(nodes.begin() + 1, nodes.end());
    lip_eval(x, rn, 1, red);
    out.assign((size_t)np * nn, 0.0);
    for (int p = 1; p < nn; ++p) {
      if (!valid(e, p)) continue;
      const double f = 1.0 / (sf(0) * sf(0) * (nodes[p] + 1.0));
      for (int ix = 0; ix < np; ++ix) out[ix + (size_t)p * np] = red[ix + (size_t)(p - 1) * np] * f;
    }
    return;
  }
  std::vector<double> b0, b1;
  B(e, x, 0, b0);
  B(e, x, 1, b1);
  out.assign((size_t)np * nn, 0.0);
  for (int p = 0; p < nn; ++p)
    for (int ix = 0; ix < np; ++ix) {
      const double r = mid(e) + sf(e) * x[ix];
      out[ix + (size_t)p * np] = (-b0[ix + (size_t)p * np] / r + b1[ix + (size_t)p * np]) / r;
    }
}

std::vector<double> RadialBasis::radial_integral(int k, int e) const {
  std::vector<double> x, w, Rv;
  gauss_legendre(128, x, w);
  R(e, x, Rv);
  const int np = (int)x.size();
  std::vector<double> wt(np);
  for (int i = 0; i < np; ++i) {
    const double r = mid(e) + sf(e) * x[i];
    wt[i] = w[i] * sf(e) * std::pow(r, k + 2);
  }
  std::vector<double> M((size_t)nn * nn, 0.0);
  for (int b = 0; b < nn; ++b)
    for (int a = 0; a <= b; ++a) {
      double s = 0.0;
      for (int i = 0; i < np; ++i) s += Rv[i + (size_t)a * np] * Rv[i + (size_t)b * np] * wt[i];
      M[a + (size_t)b * nn] = M[b + (size_t)a * nn] = s;
    }
  return M;
}

std::vector<double> RadialBasis::kinetic(int e) const {
  std::vector<double> x, w, dB;
  gauss_legendre(64, x, w);
  B(e, x, 1, dB);
  const int np = (int)x.size();
  std::vector<double> M((size_t)nn * nn, 0.0);
  for (int b = 0; b < nn; ++b)
    for (int a = 0; a <= b; ++a) {
      double s = 0.0;
      for (int i = 0; i < np; ++i) s += dB[i + (size_t)a * np] * dB[i + (size_t)b * np] * w[i];
      M[a + (size_t)b * nn] = M[b + (size_t)a * nn] = 0.5 * s * sf(e);
    }
  return M;
}

std::vector<double> RadialBasis::weighted_integral(const std::function<double(double)>& f, int e) const {
  std::vector<double> x, w, Bv;
  gauss_legendre(128, x, w);
  B(e, x, 0, Bv);
  const int np = (int)x.size();
  std::vector<double> wt(np);
  for (int i = 0; i < np; ++i) wt[i] = w[i] * sf(e) * f(mid(e) + sf(e) * x[i]);
  std::vector<double> M((size_t)nn * nn, 0.0);
  for (int b = 0; b < nn; ++b)
    for (int a = 0; a <= b; ++a) {
      double s = 0.0;
      for (int i = 0; i < np; ++i) s += Bv[i + (size_t)a * np] * Bv[i + (size_t)b * np] * wt[i];
      M[a + (size_t)b * nn] = M[b + (size_t)a * nn] = s;
    }
  return M;
}

std::vector<double> RadialBasis::twoe(int L, int e) const {
  return twoe_separable([L](double r) { return std::pow(r, L); }, [L](double r) { return std::pow(r, -L - 1.0); },
                        e);
}

void twoe_points(std::vector<double>& xo, std::vector<double>& wo, std::vector<double>& xi, std::vector<double>& wi,
                 std::vector<double>& xin) {
  gauss_legendre(TWOE_NO, xo, wo);
  gauss_legendre(TWOE_NI, xi, wi);
  xin.resize((size_t)TWOE_NO * TWOE_NI);
  for (int p = 0; p < TWOE_NO; ++p)
    for (int q = 0; q < TWOE_NI; ++q) xin[q + (size_t)p * TWOE_NI] = -1.0 + 0.5 * (xo[p] + 1.0) * (xi[q] + 1.0);
}

void RadialBasis::prepare_twoe() {
  std::vector<double> xo, wo, xi, wi, xin;
  twoe_points(xo, wo, xi, wi, xin);
  lip_eval(xo, nodes, 0, tw_Bo);
  lip_eval(xin, nodes, 0, tw_Bin);
}

std::vector<double> RadialBasis::twoe_separable(const std::function<double(double)>& fin,
                                                const std::function<double(double)>& fout, int e) const {
  // (ij|kl) = int dr B_iB_j(r) fout(r) G_kl(r) + (ij <-> kl),
  // G_kl(r) = int_{rmin}^{r} B_k B_l fin(r') dr'  (bare kernel: polynomial,
  // exact Gauss rule)
  const int no = TWOE_NO, ni = TWOE_NI;
  std::vector<double> xo, wo, xi, wi, xin;
  twoe_points(xo, wo, xi, wi, xin);
  const double rmin = bval[e];
  std::vector<double> Bo_raw, Bin_raw;
  const std::vector<double>* Bo = &tw_Bo;
  const std::vector<double>* Bin = &tw_Bin;
  if (tw_Bo.empty() || tw_Bin.empty()) {
    lip_eval(xo, nodes, 0, Bo_raw);
    lip_eval(xin, nodes, 0, Bin_raw);
    Bo = &Bo_raw;
    Bin = &Bin_raw;
  }
  const size_t npin = xin.size();
  std::vector<double> win(npin);
  for (int p = 0; p < no; ++p) {
    const double ro = mid(e) + sf(e) * xo[p];
    const double half = 0.5 * (ro - rmin);
    for (int q = 0; q < ni; ++q) {
      const double r = rmin + half * (xi[q] + 1.0);
      win[q + (size_t)p * ni] = half * wi[q] * fin(r);
    }
  }
  // invalid primitives (the dropped r = 0 and r = Rmax functions) are zero
  std::vector<char> ok(nn);
  for (int k = 0; k < nn; ++k) ok[k] = valid(e, k);
  const int n2 = nn * nn;
  std::vector<double> G((size_t)no * n2, 0.0);  // G[p*n2 + k + l*nn]
  for (int p = 0; p < no; ++p)
    for (int l = 0; l < nn; ++l)
      for (int k = 0; k <= l; ++k) {
        if (!ok[k] || !ok[l]) continue;
        double s = 0.0;
        for (int q = 0; q < ni; ++q) {
          const size_t iq = q + (size_t)p * ni;
          s += win[iq] * (*Bin)[iq + (size_t)k * npin] * (*Bin)[iq + (size_t)l * npin];
        }
        G[(size_t)p * n2 + k + l * nn] = G[(size_t)p * n2 + l + k * nn] = s;
      }
  // T1[ij, kl] = sum_p wb[p, ij] G[p, kl] (p ascending) is symmetric under
  // i <-> j and k <-> l: it is accumulated over the valid pairs i <= j,
  // k <= l only, as rank-1 updates with a contiguous inner loop
  std::vector<int> pi, pj;
  for (int j = 0; j < nn; ++j)
    for (int i = 0; i <= j; ++i)
      if (ok[i] && ok[j]) { pi.push_back(i); pj.push_back(j); }
  const int np = (int)pi.size();
  std::vector<double> wb((size_t)no * np), Gp((size_t)no * np);
  for (int p = 0; p < no; ++p) {
    const double ro = mid(e) + sf(e) * xo[p];
    const double wp = wo[p] * sf(e) * fout(ro);
    for (int a = 0; a < np; ++a) {
      wb[(size_t)p * np + a] = wp * (*Bo)[p + (size_t)pi[a] * no] * (*Bo)[p + (size_t)pj[a] * no];
      Gp[(size_t)p * np + a] = G[(size_t)p * n2 + pi[a] + pj[a] * nn];
    }
  }
  std::vector<double> T1((size_t)np * np, 0.0);  // T1[a + b*np], a = ij pair, b = kl pair
  // four consecutive p per sweep over T1 (each entry still sums p in order)
  static_assert(TWOE_NO % 4 == 0, "outer rule length must be a multiple of 4");
  for (int p = 0; p < no; p += 4) {
    const double* w0 = &wb[(size_t)p * np];
    const double* w1 = w0 + np;
    const double* w2 = w1 + np;
    const double* w3 = w2 + np;
    for (int b = 0; b < np; ++b) {
      const double g0 = Gp[(size_t)p * np + b], g1 = Gp[(size_t)(p + 1) * np + b];
      const double g2 = Gp[(size_t)(p + 2) * np + b], g3 = Gp[(size_t)(p + 3) * np + b];
      double* Tc = &T1[(size_t)b * np];
      for (int a = 0; a < np; ++a) {
        double t = Tc[a];
        t += w0[a] * g0;
        t += w1[a] * g1;
        t += w2[a] * g2;
        t += w3[a] * g3;
        Tc[a] = t;
      }
    }
  }
  // T = T1 + T1^T, expanded to all (i, j), (k, l)
  std::vector<double> T((size_t)n2 * n2, 0.0);
  for (int b = 0; b < np; ++b)
    for (int a = 0; a < np; ++a) {
      const double v = (a == b) ? 2.0 * T1[a + (size_t)a * np] : T1[a + (size_t)b * np] + T1[b + (size_t)a * np];
      const int i = pi[a], j = pj[a], k = pi[b], l = pj[b];
      const size_t ij = i + (size_t)j * nn, ji = j + (size_t)i * nn, kl = k + (size_t)l * nn, lk = l + (size_t)k * nn;
      T[ij + kl * n2] = T[ji + kl * n2] = T[ij + lk * n2] = T[ji + lk * n2] = v;
    }
  return T;
}

}  // namespace hfg

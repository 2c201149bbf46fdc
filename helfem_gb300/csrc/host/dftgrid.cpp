// Host tables of the atomic DFT grid (src/atomic/dftgrid.cpp:470-576,
// src/general/angular.cpp:21-70): the element radial rule (modified
// Gauss-Chebyshev, nquad points), the angular product rule (ldft Chebyshev
// points in cos(theta) x mdft uniform phi points), the radial functions and
// their derivatives at the radial points, and the real angular coupling
// tables that let the device evaluate the density and the Fock matrix in
// separable form.
#include <cmath>
#include <stdexcept>

#include "atom.hpp"

namespace hfg {
namespace {

// normalised associated Legendre Theta_l^m(x), m >= 0, Condon-Shortley phase
double theta_lm(int l, int m, double x) {
  if (m > l) return 0.0;
  const double s = std::sqrt(std::max((1.0 - x) * (1.0 + x), 0.0));
  double c = std::sqrt((2.0 * m + 1.0) / (4.0 * M_PI));
  for (int k = 1; k <= m; ++k) c *= std::sqrt((2.0 * k - 1.0) / (2.0 * k));
  double pmm = ((m & 1) ? -1.0 : 1.0) * c * std::pow(s, m);
  if (l == m) return pmm;
  double pm1 = x * std::sqrt(2.0 * m + 3.0) * pmm;
  if (l == m + 1) return pm1;
  double p2 = pmm, p1 = pm1;
  for (int ll = m + 2; ll <= l; ++ll) {
    const double a = std::sqrt((4.0 * ll * ll - 1.0) / ((double)ll * ll - (double)m * m));
    const double b = std::sqrt(((ll - 1.0) * (ll - 1.0) - (double)m * m) / (4.0 * (ll - 1.0) * (ll - 1.0) - 1.0));
    const double p = a * (x * p1 - b * p2);
    p2 = p1;
    p1 = p;
  }
  return p1;
}

}  // namespace

void ylm(int l, int m, double cth, double phi, double& re, double& im) {
  if (std::abs(m) > l) { re = im = 0.0; return; }
  const int am = std::abs(m);
  double t = theta_lm(l, am, cth);
  if (m < 0 && (am & 1)) t = -t;  // Y_l^{-m} = (-1)^m conj(Y_l^m)
  re = t * std::cos(m * phi);
  im = t * std::sin(m * phi);
}

void AtomHost::build_dft_grid(int ld, int md) {
  int mmx = 0;
  for (int m : mval) mmx = std::max(mmx, std::abs(m));
  ldft = ld > 0 ? ld : 4 * lmax + 12;
  mdft = md > 0 ? md : 4 * mmx + 12;
  std::vector<double> xc, wc;
  cheb_rule(ldft, xc, wc);
  nap = ldft * mdft;
  const double dphi = 2.0 * M_PI / mdft;
  std::vector<double> cth(nap), ph(nap);
  xc_wang.assign(nap, 0.0);
  xc_isin.assign(nap, 0.0);
  for (int i = 0; i < ldft; ++i)
    for (int j = 0; j < mdft; ++j) {
      const int a = i * mdft + j;
      cth[a] = xc[i];
      ph[a] = j * dphi;
      xc_wang[a] = wc[i] * dphi;
      xc_isin[a] = 1.0 / std::sqrt((1.0 - xc[i]) * (1.0 + xc[i]));
    }
  // Y, dY/dtheta at every angular point
  std::vector<double> Yr((size_t)nang * nap), Yi((size_t)nang * nap), Tr((size_t)nang * nap), Ti((size_t)nang * nap);
  for (int al = 0; al < nang; ++al) {
    const int l = lval[al], m = mval[al];
    for (int a = 0; a < nap; ++a) {
      double yr, yi;
      ylm(l, m, cth[a], ph[a], yr, yi);
      const double s = std::sqrt((1.0 - cth[a]) * (1.0 + cth[a]));
      const double cot = cth[a] / s;
      // dY/dtheta = m cot(theta) Y_l^m + sqrt((l-m)(l+m+1)) e^{-i phi} Y_l^{m+1}
      double tr = m * cot * yr, ti = m * cot * yi;
      if (m < l) {
        double ur, ui;
        ylm(l, m + 1, cth[a], ph[a], ur, ui);
        const double f = std::sqrt((double)(l - m) * (l + m + 1));
        const double cr = std::cos(ph[a]), ci = -std::sin(ph[a]);
        tr += f * (cr * ur - ci * ui);
        ti += f * (cr * ui + ci * ur);
      }
      Yr[al * (size_t)nap + a] = yr;
      Yi[al * (size_t)nap + a] = yi;
      Tr[al * (size_t)nap + a] = tr;
      Ti[al * (size_t)nap + a] = ti;
    }
  }
  const size_t n2 = (size_t)nang * nang;
  xc_W.assign(n2 * nap, 0.0);
  xc_Wt.assign(n2 * nap, 0.0);
  xc_Wp.assign(n2 * nap, 0.0);
  for (int be = 0; be < nang; ++be)
    for (int al = 0; al < nang; ++al) {
      const size_t o = (al + (size_t)be * nang) * nap;
      for (int a = 0; a < nap; ++a) {
        const double ar = Yr[al * (size_t)nap + a], ai = Yi[al * (size_t)nap + a];
        const double br = Yr[be * (size_t)nap + a], bi = Yi[be * (size_t)nap + a];
        const double tr = Tr[al * (size_t)nap + a], ti = Ti[al * (size_t)nap + a];
        xc_W[o + a] = ar * br + ai * bi;   // Re[Ya conj(Yb)]
        xc_Wt[o + a] = tr * br + ti * bi;  // Re[dYa conj(Yb)]
        // Re[(i m) Ya conj(Yb)] = -m Im[Ya conj(Yb)] = -m (ai br - ar bi)
        xc_Wp[o + a] = -mval[al] * (ai * br - ar * bi);
      }
    }
  // radial side
  const int nn = rad.nn, nel = rad.nel;
  std::vector<double> xq, wq;
  cheb_rule(nquad, xq, wq);
  xc_r.assign((size_t)nel * nquad, 0.0);
  xc_wr.assign((size_t)nel * nquad, 0.0);
  xc_R.assign((size_t)nel * nquad * nn, 0.0);
  xc_dR.assign((size_t)nel * nquad * nn, 0.0);
  for (int e = 0; e < nel; ++e) {
    std::vector<double> Rv, dRv;
    rad.R(e, xq, Rv);
    rad.dR(e, xq, dRv);
    for (int q = 0; q < nquad; ++q) {
      const double r = rad.mid(e) + rad.sf(e) * xq[q];
      xc_r[(size_t)e * nquad + q] = r;
      xc_wr[(size_t)e * nquad + q] = rad.sf(e) * wq[q] * r * r;
      for (int p = 0; p < nn; ++p) {
        xc_R[((size_t)e * nquad + q) * nn + p] = Rv[q + (size_t)p * nquad];
        xc_dR[((size_t)e * nquad + q) * nn + p] = dRv[q + (size_t)p * nquad];
      }
    }
  }
}

}  // namespace hfg

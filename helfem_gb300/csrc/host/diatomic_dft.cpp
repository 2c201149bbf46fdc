// Host tables of the pure-m diatomic DFT grid (src/diatomic/dftgrid_purem.cpp).
//
// When the orbitals do not mix m the density is phi-independent and the phi
// integral of every matrix element is 2 pi delta(m_s, m_t)
// (dftgrid_purem.cpp:34-80, main.cpp:316-330). On mu element e the grid is the
// product of the element's modified Gauss-Chebyshev rule of 5 Nnodes points in
// mu (main.cpp:191, basis.cpp:496-503) and lang Chebyshev points in cos(nu);
// the point weight is w = 2 pi wang wr Rhalf^3 sinh mu (sinh^2 mu + sin^2 nu)
// and the gradient scale factor h = Rhalf sqrt(sinh^2 mu + sin^2 nu)
// (dftgrid_purem.cpp:92-117). The basis value of dummy function (s, p) is
// Y_s(nu, phi = 0) B_p(mu); its nu derivative uses
// dY/dnu = m cot(nu) Y_l^m + sqrt((l-m)(l+m+1)) Y_l^{m+1} (dftgrid_purem.cpp:63-73).
//
// Everything the device needs factorises into per-(element, mu point) radial
// rows, per-(element, point) weights and per-(pair, nu point) angular
// products, as in the atomic grid. The pairs are unordered (s <= t): the
// density, the potential and the Fock tiles are symmetric under s <-> t.
#include <algorithm>
#include <cmath>
#include <stdexcept>

#include "atom.hpp"
#include "diatomic.hpp"

namespace hfg {

void DiatomicHost::build_xc_grid(int lang) {
  int lmx = 0;
  for (int l : lval) lmx = std::max(lmx, l);
  xc_lang = lang > 0 ? lang : 4 * lmx + 12;
  xc_nq = 5 * nn;
  const int na = xc_lang, nq = xc_nq;
  std::vector<double> cth, wang;
  cheb_rule(na, cth, wang);
  std::vector<double> sth(na), cot(na);
  for (int a = 0; a < na; ++a) {
    sth[a] = std::sqrt(std::max((1.0 - cth[a]) * (1.0 + cth[a]), 0.0));
    cot[a] = sth[a] > 0.0 ? cth[a] / sth[a] : 0.0;
  }
  // angular values per function
  std::vector<double> Y((size_t)nang * na), dY((size_t)nang * na);
  for (int s = 0; s < nang; ++s) {
    const int l = lval[s], m = mval[s];
    for (int a = 0; a < na; ++a) {
      double y, im;
      ylm(l, m, cth[a], 0.0, y, im);
      double d = m * cot[a] * y;
      if (m < l) {
        double u;
        ylm(l, m + 1, cth[a], 0.0, u, im);
        d += std::sqrt((double)(l - m) * (double)(l + m + 1)) * u;
      }
      Y[(size_t)s * na + a] = y;
      dY[(size_t)s * na + a] = d;
    }
  }
  // same-m unordered pairs s <= t
  xc_ps.clear();
  xc_pt.clear();
  xc_mult.clear();
  for (int t = 0; t < nang; ++t)
    for (int s = 0; s <= t; ++s)
      if (mval[s] == mval[t]) {
        xc_ps.push_back(s);
        xc_pt.push_back(t);
        xc_mult.push_back(s == t ? 1.0 : 2.0);
      }
  xc_npair = (int)xc_ps.size();
  xc_W.assign((size_t)xc_npair * na, 0.0);
  xc_Wt.assign((size_t)xc_npair * na, 0.0);
  for (int k = 0; k < xc_npair; ++k) {
    const int s = xc_ps[k], t = xc_pt[k];
    for (int a = 0; a < na; ++a) {
      const size_t ia = (size_t)s * na + a, ib = (size_t)t * na + a;
      xc_W[(size_t)k * na + a] = Y[ia] * Y[ib];
      xc_Wt[(size_t)k * na + a] = dY[ia] * Y[ib] + Y[ia] * dY[ib];
    }
  }
  // mirror shells (same l, opposite m) and the Fock-side pair list
  std::vector<int> mir(nang, -1);
  for (int s = 0; s < nang; ++s)
    for (int s2 = 0; s2 < nang; ++s2)
      if (mval[s] != 0 && lval[s2] == lval[s] && mval[s2] == -mval[s]) mir[s] = s2;
  xc_fk.clear();
  xc_fms.clear();
  xc_fmt.clear();
  for (int k = 0; k < xc_npair; ++k) {
    const int s = xc_ps[k], t = xc_pt[k], m = mval[s];
    const bool mirrored = mir[s] >= 0 && mir[t] >= 0;
    if (m < 0 && mirrored) continue;  // written by its +m mirror
    xc_fk.push_back(k);
    xc_fms.push_back(m > 0 && mirrored ? mir[s] : -1);
    xc_fmt.push_back(m > 0 && mirrored ? mir[t] : -1);
  }
  // radial rows and point weights
  std::vector<double> xq, wq;
  cheb_rule(nq, xq, wq);
  std::vector<double> Bv, dBv;
  lip_eval(xq, nodes, 0, Bv);   // [q + p*nq]
  lip_eval(xq, nodes, 1, dBv);
  xc_R.assign((size_t)nel * nq * nn, 0.0);
  xc_dR.assign((size_t)nel * nq * nn, 0.0);
  xc_w.assign((size_t)nel * nq * na, 0.0);
  xc_hinv.assign((size_t)nel * nq * na, 0.0);
  const double R3 = Rhalf * Rhalf * Rhalf;
  for (int e = 0; e < nel; ++e) {
    const double sf = 0.5 * (bval[e + 1] - bval[e]), mid = 0.5 * (bval[e + 1] + bval[e]);
    for (int q = 0; q < nq; ++q) {
      const size_t eq = (size_t)e * nq + q;
      for (int p = 0; p < nn; ++p) {
        xc_R[eq * nn + p] = Bv[q + (size_t)p * nq];
        xc_dR[eq * nn + p] = dBv[q + (size_t)p * nq] / sf;
      }
      const double mu = mid + sf * xq[q], wr = sf * wq[q];
      const double sh = std::sinh(mu);
      for (int a = 0; a < na; ++a) {
        const double s2 = sh * sh + sth[a] * sth[a];
        const double h = Rhalf * std::sqrt(s2);
        xc_w[eq * na + a] = 2.0 * M_PI * wang[a] * wr * R3 * sh * s2;
        xc_hinv[eq * na + a] = h > 0.0 ? 1.0 / h : 0.0;
      }
    }
  }
}

}  // namespace hfg

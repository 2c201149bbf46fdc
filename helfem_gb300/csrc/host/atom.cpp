// Atom set-up: the host-side equivalent of HelFEM's TwoDBasisT constructor,
// one-electron matrices and compute_tei (src/atomic/TwoDBasis.cpp:66-94,
// 265-374, 708-735; libhelfemqc/include/CoulombExchangeFE.h:180-217), plus
// the Gaunt coupling lists that TwoDBasisT::coulomb / exchange rebuild on
// every call (TwoDBasis.cpp:787-788, 889-890) and that are built once here.
#include <algorithm>
#include <cmath>
#include <limits>
#include <stdexcept>

#include "atom.hpp"

namespace hfg {

// Greedy pivoted Cholesky with an absolute tolerance on the residual
// diagonal, the factorisation HelFEM uses for the in-element tensor
// (libhelfem/src/RadialBasis.cpp:670-709). A is n x n column-major;
// returns n x r column-major.
std::vector<double> pivoted_cholesky(const std::vector<double>& A, int n, double tol, int& rank) {
  std::vector<double> D(n);
  for (int i = 0; i < n; ++i) D[i] = A[i + (size_t)i * n];
  std::vector<char> done(n, 0);
  std::vector<double> L;
  rank = 0;
  for (int k = 0; k < n; ++k) {
    int piv = -1;
    double pv = tol;
    for (int i = 0; i < n; ++i)
      if (!done[i] && D[i] > pv) { piv = i; pv = D[i]; }
    if (piv < 0) break;
    done[piv] = 1;
    const double s = std::sqrt(pv);
    L.resize((size_t)(rank + 1) * n);
    double* col = &L[(size_t)rank * n];
    for (int i = 0; i < n; ++i) {
      if (done[i] && i != piv) { col[i] = 0.0; continue; }
      double v = A[i + (size_t)piv * n];
      for (int j = 0; j < rank; ++j) v -= L[i + (size_t)j * n] * L[piv + (size_t)j * n];
      col[i] = v / s;
    }
    col[piv] = s;
    ++rank;
    for (int i = 0; i < n; ++i)
      if (!done[i]) D[i] -= col[i] * col[i];
  }
  return L;
}

void AtomHost::build(int Z_, int nnodes, const std::vector<double>& bval, const std::vector<int>& lv,
                     const std::vector<int>& mv, int nquad_, double tol, bool twoe_host) {
  if (nnodes < 3) throw std::invalid_argument("need at least 3 nodes per element");
  if (bval.size() < 2) throw std::invalid_argument("need at least one element");
  for (size_t i = 1; i < bval.size(); ++i)
    if (!(bval[i] > bval[i - 1])) throw std::invalid_argument("element boundaries must increase");
  if (bval[0] != 0.0) throw std::invalid_argument("first element boundary must be r = 0");
  if (lv.empty() || lv.size() != mv.size()) throw std::invalid_argument("bad angular basis");
  for (size_t i = 0; i < lv.size(); ++i)
    if (lv[i] < 0 || std::abs(mv[i]) > lv[i]) throw std::invalid_argument("bad (l,m) pair");
  Z = Z_;
  chol_tol = tol > 0 ? tol : 1e-12;
  rad.nn = nnodes;
  rad.bval = bval;
  rad.nel = (int)bval.size() - 1;
  rad.nrad = rad.nel * (nnodes - 1) - 1;
  std::vector<double> w;
  gauss_lobatto(nnodes, rad.nodes, w);
  nquad = nquad_ > 0 ? nquad_ : 5 * nnodes;
  lval = lv;
  mval = mv;
  nang = (int)lval.size();
  nbf = nang * rad.nrad;
  lmax = *std::max_element(lval.begin(), lval.end());
  NL = 2 * lmax + 1;

  const int nn = rad.nn, nel = rad.nel, n2 = nn * nn;
  rs.assign((size_t)NL * nel * n2, 0.0);
  rb.assign((size_t)NL * nel * n2, 0.0);
  chol.assign((size_t)NL * nel, {});
  chol_rank.assign((size_t)NL * nel, 0);
  std::vector<std::vector<double>> cholpad((size_t)NL * nel);

  twoe_on_host = twoe_host;
  rad.prepare_twoe();
#pragma omp parallel for collapse(2) schedule(dynamic)
  for (int L = 0; L < NL; ++L)
    for (int e = 0; e < nel; ++e) {
      const size_t le = (size_t)L * nel + e;
      auto a = rad.radial_integral(L, e);
      std::copy(a.begin(), a.end(), rs.begin() + le * n2);
      if (e > 0) {  // r_big is never used on the innermost element
        auto b = rad.radial_integral(-L - 1, e);
        std::copy(b.begin(), b.end(), rb.begin() + le * n2);
      }
      if (!twoe_host) continue;
      const std::vector<double> T = rad.twoe(L, e);
      int r = 0;
      cholpad[le] = pivoted_cholesky(T, n2, chol_tol, r);
      chol_rank[le] = r;
      // compact reference layout: rows (a + b*Ni) over valid primitives
      const int p0 = rad.pfirst(e), ni = rad.nfun(e);
      std::vector<double>& c = chol[le];
      c.assign((size_t)ni * ni * r, 0.0);
      for (int p = 0; p < r; ++p)
        for (int b = 0; b < ni; ++b)
          for (int a2 = 0; a2 < ni; ++a2)
            c[(a2 + (size_t)b * ni) + (size_t)p * ni * ni] =
                cholpad[le][(a2 + p0) + (size_t)(b + p0) * nn + (size_t)p * n2];
    }
  rmax = 0;
  for (int r : chol_rank) rmax = std::max(rmax, r);
  if (twoe_host) {
    cholp.assign((size_t)NL * nel * n2 * rmax, 0.0);
    tk.assign((size_t)NL * nel * n2 * n2, 0.0);
  } else {
    chol.clear();
    cholp.clear();
    tk.clear();
  }
#pragma omp parallel for collapse(2) schedule(dynamic) if (twoe_host)
  for (int L = 0; L < NL; ++L)
    for (int e = 0; e < nel; ++e) {
      if (!twoe_host) continue;
      const size_t le = (size_t)L * nel + e;
      const int r = chol_rank[le];
      std::copy(cholpad[le].begin(), cholpad[le].begin() + (size_t)n2 * r, cholp.begin() + le * n2 * rmax);
      // exchange ordering: K_ac = sum_bd (ab|cd) P_bd, rows (a + c nn), cols (b + d nn);
      // the factor rows are transposed first so that each dot product is contiguous
      double* out = &tk[le * n2 * n2];
      const std::vector<double>& Lc = cholpad[le];
      std::vector<double> Lt((size_t)n2 * r);
      for (int p = 0; p < r; ++p)
        for (int ab = 0; ab < n2; ++ab) Lt[(size_t)ab * r + p] = Lc[ab + (size_t)p * n2];
      for (int d = 0; d < nn; ++d)
        for (int b = 0; b < nn; ++b)
          for (int c = 0; c < nn; ++c)
            for (int a = 0; a < nn; ++a) {
              double s = 0.0;
              const double* x = &Lt[(a + (size_t)b * nn) * r];
              const double* y = &Lt[(c + (size_t)d * nn) * r];
              for (int p = 0; p < r; ++p) s += x[p] * y[p];
              out[(a + (size_t)c * nn) + (size_t)(b + d * nn) * n2] = s;
            }
    }

  // one-electron radial matrices (assembled with shared boundary functions)
  const int nr = rad.nrad;
  Srad.assign((size_t)nr * nr, 0.0);
  Trad = Tlrad = Vrad = Srad;
  for (int e = 0; e < nel; ++e) {
    const auto s = rad.radial_integral(0, e);
    const auto t = rad.kinetic(e);
    const auto tl = rad.radial_integral(-2, e);
    const auto v = rad.radial_integral(-1, e);
    for (int q = 0; q < nn; ++q)
      for (int p = 0; p < nn; ++p) {
        if (!rad.valid(e, p) || !rad.valid(e, q)) continue;
        const size_t o = rad.g(e, p) + (size_t)rad.g(e, q) * nr, i = p + (size_t)q * nn;
        Srad[o] += s[i];
        Trad[o] += t[i];
        Tlrad[o] += 0.5 * tl[i];
        Vrad[o] += v[i];
      }
  }
  build_couplings();
}

// c(l_out, l_in, L) = (2 l_out + 1)^-1 sum_{m_out, m_in} G(l_out, m_out, L, m_out - m_in, l_in)^2
static double channel_average(int lout, int lin, int L) {
  double c = 0.0;
  for (int mo = -lout; mo <= lout; ++mo)
    for (int mi = -lin; mi <= lin; ++mi) {
      const int M = mo - mi;
      if (std::abs(M) > L) continue;
      const double g = gaunt_coeff(lout, mo, L, M, lin);
      c += g * g;
    }
  return c / (2 * lout + 1);
}

void AtomHost::build_couplings_spherical() {
  for (int i = 0; i < nang; ++i)
    if (lval[i] != i || mval[i] != 0)
      throw std::invalid_argument("spherically averaged basis: angular functions must be (l, 0), l = 0..lmax");
  chans.assign(1, {0, 0});
  jket_ptr.assign(1, 0);
  jket_blk.clear();
  jket_coef.clear();
  for (int l = 0; l < nang; ++l) {
    jket_blk.push_back(l + l * nang);
    jket_coef.push_back(1.0);
  }
  jket_ptr.push_back((int)jket_blk.size());
  jbra_ptr.assign(1, 0);
  jbra_chan.clear();
  jbra_coef.clear();
  for (int j = 0; j < nang; ++j)
    for (int i = 0; i < nang; ++i) {
      if (i == j) {
        jbra_chan.push_back(0);
        jbra_coef.push_back(4.0 * M_PI);
      }
      jbra_ptr.push_back((int)jbra_chan.size());
    }
  kjk_ptr.assign(1, 0);
  kent_L.clear();
  kent_ptr.assign(1, 0);
  kterm_blk.clear();
  kterm_coef.clear();
  for (int k = 0; k < nang; ++k)
    for (int j = 0; j < nang; ++j) {
      if (j == k) {
        for (int L = 0; L < NL; ++L) {
          const size_t first = kterm_blk.size();
          for (int lin = 0; lin < nang; ++lin) {
            if (L < std::abs(lin - j) || L > lin + j) continue;
            const double c = channel_average(j, lin, L);
            if (c == 0.0) continue;
            kterm_blk.push_back(lin + lin * nang);
            kterm_coef.push_back(4.0 * M_PI / (2 * L + 1) * c);
          }
          if (kterm_blk.size() == first) continue;
          kent_L.push_back(L);
          kent_ptr.push_back((int)kterm_blk.size());
        }
      }
      kjk_ptr.push_back((int)kent_L.size());
    }
}

void AtomHost::build_couplings() {
  if (spherical) {
    build_couplings_spherical();
    return;
  }
  int mmx = -1 << 30, mmn = 1 << 30;
  for (int m : mval) { mmx = std::max(mmx, m); mmn = std::min(mmn, m); }
  const int Mmax = mmx - mmn;
  // J channels (L, M), |M| <= min(L, Mmax)  (TwoDBasis.cpp:794-800)
  chans.clear();
  std::vector<int> chan_of((size_t)NL * (2 * Mmax + 1), -1);
  for (int L = 0; L < NL; ++L)
    for (int M = -std::min(L, Mmax); M <= std::min(L, Mmax); ++M) {
      chan_of[(size_t)L * (2 * Mmax + 1) + (M + Mmax)] = (int)chans.size();
      chans.push_back({L, M});
    }
  const int nch = (int)chans.size();
  // ket contraction (TwoDBasis.cpp:803-822): every coupled L, zero or not
  std::vector<std::vector<std::pair<int, double>>> ket(nch);
  for (int l = 0; l < nang; ++l)
    for (int k = 0; k < nang; ++k) {
      const int lk = lval[k], mk = mval[k], ll = lval[l], ml = mval[l];
      const int M = mk - ml;
      for (int L = std::max(std::abs(lk - ll), std::abs(M)); L <= lk + ll; ++L) {
        const double c = gaunt_coeff(lk, mk, L, M, ll);
        if (c == 0.0) continue;
        ket[chan_of[(size_t)L * (2 * Mmax + 1) + (M + Mmax)]].push_back({k + l * nang, c});
      }
    }
  jket_ptr.assign(1, 0);
  jket_blk.clear();
  jket_coef.clear();
  for (int c = 0; c < nch; ++c) {
    for (auto& t : ket[c]) { jket_blk.push_back(t.first); jket_coef.push_back(t.second); }
    jket_ptr.push_back((int)jket_blk.size());
  }
  // bra scatter (TwoDBasis.cpp:853-874), with 4 pi/(2L+1)
  jbra_ptr.assign(1, 0);
  jbra_chan.clear();
  jbra_coef.clear();
  for (int j = 0; j < nang; ++j)
    for (int i = 0; i < nang; ++i) {
      const int li = lval[i], mi = mval[i], lj = lval[j], mj = mval[j];
      const int M = mj - mi;
      for (int L = std::max(std::abs(lj - li), std::abs(M)); L <= lj + li; ++L) {
        const double c = gaunt_coeff(lj, mj, L, M, li);
        if (c == 0.0) continue;
        jbra_chan.push_back(chan_of[(size_t)L * (2 * Mmax + 1) + (M + Mmax)]);
        jbra_coef.push_back(c * 4.0 * M_PI / (2 * L + 1));
      }
      jbra_ptr.push_back((int)jbra_chan.size());
    }
  // exchange recoupling (TwoDBasis.cpp:916-970)
  kjk_ptr.assign(1, 0);
  kent_L.clear();
  kent_ptr.assign(1, 0);
  kterm_blk.clear();
  kterm_coef.clear();
  for (int k = 0; k < nang; ++k)
    for (int j = 0; j < nang; ++j) {
      const int lj = lval[j], mj = mval[j], lk = lval[k], mk = mval[k];
      std::vector<std::vector<std::pair<int, double>>> perL(NL);
      for (int i = 0; i < nang; ++i)
        for (int l = 0; l < nang; ++l) {
          const int li = lval[i], mi = mval[i], ll = lval[l], ml = mval[l];
          const int M = mj - mi;
          if (M != mk - ml) continue;
          const int Lmin = std::max({std::abs(li - lj), std::abs(lk - ll), std::abs(M)});
          const int Lmax = std::min(li + lj, lk + ll);
          for (int L = Lmin; L <= Lmax; ++L) {
            const double c = gaunt_coeff(lj, mj, L, M, li) * gaunt_coeff(lk, mk, L, M, ll);
            if (c == 0.0) continue;
            perL[L].push_back({i + l * nang, 4.0 * M_PI / (2 * L + 1) * c});
          }
        }
      for (int L = 0; L < NL; ++L) {
        if (perL[L].empty()) continue;
        kent_L.push_back(L);
        for (auto& t : perL[L]) { kterm_blk.push_back(t.first); kterm_coef.push_back(t.second); }
        kent_ptr.push_back((int)kterm_blk.size());
      }
      kjk_ptr.push_back((int)kent_L.size());
    }
}

}  // namespace hfg

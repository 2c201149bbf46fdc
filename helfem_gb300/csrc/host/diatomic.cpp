// FP64 host tabulation of the diatomic (prolate spheroidal) basis.
//
// Computes what HelFEM's diatomic TwoDBasis caches in compute_tei and uses in
// its one-electron matrices:
//   Legendre P_L^M, Q_L^M of cosh(mu)  src/legendre/Legendre.h:30-330
//   radial FE basis in mu              src/diatomic/basis.cpp:522-540
//   pure-function list                 src/diatomic/basis.cpp:712-736
//   disjoint P/Q integrals             src/diatomic/basis.cpp:1382-1430,
//                                      350-395 (Plm_integral / Qlm_integral)
//   in-element 2-channel kernel        src/diatomic/quadrature.cpp:175-255
//   sign-carrying pivoted factor       src/diatomic/basis.cpp:1432-1545
//   one-electron radial blocks         src/diatomic/basis.cpp:253-290,395-410
//   overlap / kinetic / nuclear        src/diatomic/basis.cpp:1033-1140
//   mod_coeff (cos^2 coupling)         src/general/gaunt.cpp:254-275
// The reference refines Gauss-Chebyshev / Gauss-Lobatto rules until each
// block is stable to eps(double). Here every integral is evaluated once with
// a Gauss-Legendre rule far past convergence for its analytic integrand; on
// the element touching mu = 0, where Q_L^M(cosh mu) is singular, the outer
// variable of the in-element kernel is mapped mu = mu_e t^3, which makes the
// integrand smooth. (The Q integrals of that element are never used: it is
// never the outer element of a disjoint pair.)
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <unordered_map>

#include "atom.hpp"
#include "diatomic.hpp"

namespace hfg {

// ---------------------------------------------------------------------------
// Associated Legendre functions of x = cosh(mu) > 1
// ---------------------------------------------------------------------------
void legendre_pq(int Lmax, int Mmax, double mu, double* P, double* Q) {
  const int NLs = Lmax + 1;
  const double x = std::cosh(mu), w = std::sinh(mu);
  for (int i = 0; i < (Mmax + 1) * NLs; ++i) P[i] = Q[i] = 0.0;
  // P: P_M^M = (2M-1)!! w^M, P_{M+1}^M = (2M+1) x P_M^M, upward in L
  double diag = 1.0;
  for (int M = 0; M <= Mmax && M <= Lmax; ++M) {
    if (M > 0) diag *= (2 * M - 1) * w;
    double* pm = P + M * NLs;
    pm[M] = diag;
    if (M + 1 <= Lmax) pm[M + 1] = (2 * M + 1) * x * diag;
    for (int L = M + 1; L < Lmax; ++L) pm[L + 1] = ((2 * L + 1) * x * pm[L] - (L + M) * pm[L - 1]) / (L + 1 - M);
  }
  // Q_0^0 = 1/2 ln((x+1)/(x-1)) = -ln tanh(mu/2), exactly in mu
  const double q00 = -std::log(std::tanh(0.5 * mu));
  if (mu < 1.0 / std::max(Lmax, 1)) {
    // near x = 1: Q_L = P_L Q_0 - W_L with W obeying the Legendre recurrence
    // (W_0 = 0, W_1 = 1); Q_L^1 from the x-derivative times w
    double pl0 = 1.0, pl1 = x, wl0 = 0.0, wl1 = 1.0, dp0 = 0.0, dp1 = 1.0, dw0 = 0.0, dw1 = 0.0;
    Q[0] = q00;
    if (Mmax >= 1) Q[NLs] = -1.0 / w;
    if (Lmax >= 1) {
      Q[1] = pl1 * q00 - wl1;
      if (Mmax >= 1) Q[NLs + 1] = w * dp1 * q00 - pl1 / w - w * dw1;
    }
    for (int k = 1; k < Lmax; ++k) {
      const double pl2 = ((2 * k + 1) * x * pl1 - k * pl0) / (k + 1);
      const double wl2 = ((2 * k + 1) * x * wl1 - k * wl0) / (k + 1);
      const double dp2 = ((2 * k + 1) * (pl1 + x * dp1) - k * dp0) / (k + 1);
      const double dw2 = ((2 * k + 1) * (wl1 + x * dw1) - k * dw0) / (k + 1);
      Q[k + 1] = pl2 * q00 - wl2;
      if (Mmax >= 1) Q[NLs + k + 1] = w * dp2 * q00 - pl2 / w - w * dw2;
      pl0 = pl1; pl1 = pl2; wl0 = wl1; wl1 = wl2; dp0 = dp1; dp1 = dp2; dw0 = dw1; dw1 = dw2;
    }
  } else {
    // Miller: backward recurrence from well past Lmax, where the minimal
    // solution dominates; normalised on Q_0^0 and Q_0^1 = -1/w
    const int N = Lmax + (int)std::ceil(37.0 / mu) + 20;
    for (int M = 0; M <= std::min(Mmax, 1); ++M) {
      double* qm = Q + M * NLs;
      double nxt = 0.0, cur = 1e-280;
      for (int L = N; L >= 1; --L) {
        const double prev = ((2 * L + 1) * x * cur - (L - M + 1) * nxt) / (L + M);
        nxt = cur;
        cur = prev;
        if (L - 1 <= Lmax) qm[L - 1] = cur;
        if (std::fabs(cur) > 1e250) {
          cur *= 1e-250;
          nxt *= 1e-250;
          for (int l = L - 1; l <= Lmax; ++l) qm[l] *= 1e-250;
        }
      }
      const double s = (M == 0 ? q00 : -1.0 / w) / qm[0];
      for (int l = 0; l <= Lmax; ++l) qm[l] *= s;
    }
  }
  // M >= 2: Q_L^{M+1} = -2 M x / w Q_L^M + (L+M)(L-M+1) Q_L^{M-1}
  for (int M = 1; M < Mmax; ++M)
    for (int L = 0; L <= Lmax; ++L)
      Q[(M + 1) * NLs + L] = -2.0 * M * x / w * Q[M * NLs + L] + (double)(L + M) * (L - M + 1) * Q[(M - 1) * NLs + L];
  for (int i = 0; i < (Mmax + 1) * NLs; ++i) {
    if (!std::isfinite(P[i]) || (P[i] != 0.0 && std::fabs(P[i]) < DBL_MIN)) P[i] = 0.0;
    if (!std::isfinite(Q[i]) || (Q[i] != 0.0 && std::fabs(Q[i]) < DBL_MIN)) Q[i] = 0.0;
  }
}

namespace {

constexpr int NGL_1E = 96;   // one-electron and disjoint integrals
constexpr int NGL_OUT = 64;  // in-element kernel, outer variable
constexpr int NGL_IN = 64;   // in-element kernel, inner variable

// Gaunt values are needed many times over the same small index space
struct GauntCache {
  std::unordered_map<uint64_t, double> m;
  double coeff(int L, int M, int l, int mm, int lp) {
    if (L < 0 || l < 0 || lp < 0) return 0.0;
    const uint64_t key = ((((uint64_t)L * 256 + (M + 128)) * 256 + l) * 256 + (mm + 128)) * 256 + lp;
    auto it = m.find(key);
    if (it != m.end()) return it->second;
    const double v = gaunt_coeff(L, M, l, mm, lp);
    m.emplace(key, v);
    return v;
  }
  // int Y_lj^mj* cos^2 Y_L^M Y_li^mi: cos^2 = (2/3) sqrt(pi) Y_0^0 + (4/15) sqrt(5 pi) Y_2^0
  // applied to Y_L^M and expanded in Y_Lp^M
  double mod(int lj, int mj, int L, int M, int li, int mi) {
    if (mj != M + mi) return 0.0;
    const double c0 = 2.0 / 3.0 * std::sqrt(M_PI), c2 = 4.0 / 15.0 * std::sqrt(5.0 * M_PI);
    double v = c0 * coeff(L, M, 0, 0, L) * coeff(lj, mj, li, mi, L);
    for (int Lp = std::max(std::max(L - 2, 0), std::abs(M)); Lp <= L + 2; ++Lp)
      v += c2 * coeff(Lp, M, 2, 0, L) * coeff(lj, mj, li, mi, Lp);
    return v;
  }
};

double lm_factor(int L, int M, double Rhalf) {
  const int Ma = std::abs(M);
  double fr = 1.0;
  for (int p = L + Ma; p > L - Ma; --p) fr *= p;
  return ((M & 1) ? -1.0 : 1.0) * 4.0 * M_PI * std::pow(Rhalf, 5) / fr;
}

// diagonal-pivoted, sign-carrying Cholesky of the symmetric N x N matrix W
// (column-major): W ~ B diag(s) B', pivot on the largest |residual diagonal|,
// stop at thresh * max|diag W|
void sign_cholesky(const std::vector<double>& W, int N, double thresh, std::vector<double>& B,
                   std::vector<double>& s) {
  std::vector<double> d(N);
  double dmax0 = 0.0;
  for (int i = 0; i < N; ++i) {
    d[i] = W[i + (size_t)i * N];
    dmax0 = std::max(dmax0, std::fabs(d[i]));
  }
  B.clear();
  s.clear();
  for (int it = 0; it < N; ++it) {
    int piv = 0;
    double best = -1.0;
    for (int i = 0; i < N; ++i)
      if (std::fabs(d[i]) > best) { best = std::fabs(d[i]); piv = i; }
    const double dp = d[piv];
    if (dmax0 <= 0.0 || std::fabs(dp) <= thresh * dmax0) break;
    const double sg = dp >= 0.0 ? 1.0 : -1.0;
    const int r = (int)s.size();
    std::vector<double> col(W.begin() + (size_t)piv * N, W.begin() + (size_t)(piv + 1) * N);
    for (int q = 0; q < r; ++q) {
      const double f = s[q] * B[piv + (size_t)q * N];
      if (f == 0.0) continue;
      const double* bq = B.data() + (size_t)q * N;
      for (int i = 0; i < N; ++i) col[i] -= f * bq[i];
    }
    const double inv = 1.0 / std::sqrt(std::fabs(dp));
    for (int i = 0; i < N; ++i) {
      col[i] *= inv;
      d[i] -= sg * col[i] * col[i];
    }
    d[piv] = 0.0;
    B.insert(B.end(), col.begin(), col.end());
    s.push_back(sg);
  }
}

}  // namespace

int DiatomicHost::lm_index(int L, int Mabs) const {
  for (int i = 0; i < nlm; ++i)
    if (lm_L[i] == L && lm_M[i] == Mabs) return i;
  return -1;
}

void DiatomicHost::build(int Z1_, int Z2_, double Rhalf_, int nnodes, const std::vector<double>& bval_,
                         const std::vector<int>& lval_, const std::vector<int>& mval_, double thresh,
                         bool twoe_host) {
  if (nnodes < 3 || nnodes > 17) throw std::invalid_argument("diatomic: nnodes must be in [3, 17]");
  if (bval_.size() < 3) throw std::invalid_argument("diatomic: need at least two elements");
  for (size_t i = 1; i < bval_.size(); ++i)
    if (!(bval_[i] > bval_[i - 1])) throw std::invalid_argument("diatomic: element boundaries must increase");
  if (bval_[0] != 0.0) throw std::invalid_argument("diatomic: the first boundary must be mu = 0");
  if (lval_.empty() || lval_.size() != mval_.size()) throw std::invalid_argument("diatomic: bad angular basis");
  if (!(Rhalf_ > 0.0)) throw std::invalid_argument("diatomic: Rhalf must be positive");
  Z1 = Z1_;
  Z2 = Z2_;
  Rhalf = Rhalf_;
  cd_thresh = thresh > 0 ? thresh : 1e-12;
  twoe_on_host = twoe_host;
  nn = nnodes;
  bval = bval_;
  nel = (int)bval.size() - 1;
  nrad = nel * (nn - 1);
  lval = lval_;
  mval = mval_;
  nang = (int)lval.size();
  mmax = 0;
  for (int i = 0; i < nang; ++i) {
    if (lval[i] < 0 || std::abs(mval[i]) > lval[i]) throw std::invalid_argument("diatomic: need |m| <= l");
    mmax = std::max(mmax, std::abs(mval[i]));
  }
  ndummy = nang * nrad;
  pure.clear();
  for (int a = 0; a < nang; ++a)
    for (int j = (mval[a] == 0 ? 0 : 1); j < nrad; ++j) pure.push_back(a * nrad + j);
  nbf = (int)pure.size();
  std::vector<double> w;
  gauss_lobatto(nn, nodes, w);
  // (L,|M|) map: |M|-major, L ascending
  std::vector<std::pair<int, int>> lm;
  Lmax = 0;
  for (int i = 0; i < nang; ++i)
    for (int j = 0; j < nang; ++j) {
      const int M = mval[j] - mval[i];
      for (int L = std::max(std::abs(lval[j] - lval[i]) - 2, std::abs(M)); L <= lval[j] + lval[i] + 2; ++L) {
        lm.emplace_back(std::abs(M), L);
        Lmax = std::max(Lmax, L);
      }
    }
  std::sort(lm.begin(), lm.end());
  lm.erase(std::unique(lm.begin(), lm.end()), lm.end());
  nlm = (int)lm.size();
  lm_L.resize(nlm);
  lm_M.resize(nlm);
  for (int i = 0; i < nlm; ++i) {
    lm_M[i] = lm[i].first;
    lm_L[i] = lm[i].second;
  }
  tabulate_radial();
  build_couplings();
}

void DiatomicHost::tabulate_radial() {
  const int n2 = nn * nn;
  const int Mtop = nlm ? *std::max_element(lm_M.begin(), lm_M.end()) : 0;
  const size_t tile = (size_t)n2;
  p0.assign(twoe_on_host ? (size_t)nlm * nel * tile : 0, 0.0);
  p2 = p0;
  q0 = p0;
  q2 = p0;
  std::vector<std::vector<double>> fB((size_t)nlm * nel), fS((size_t)nlm * nel);
  std::vector<double> xg, wg, xo, wo, xi, wi;
  gauss_legendre(NGL_1E, xg, wg);
  gauss_legendre(NGL_OUT, xo, wo);
  gauss_legendre(NGL_IN, xi, wi);
  const int NLs = Lmax + 1, NMs = Mtop + 1;
  // one-electron radial blocks, assembled
  I10.assign((size_t)nrad * nrad, 0.0);
  I11 = I10;
  I12 = I10;
  Im1 = I10;
  Trad = I10;
  std::vector<double> Bv, dBv;
  lip_eval(xg, nodes, 0, Bv);
  lip_eval(xg, nodes, 1, dBv);
  auto valid = [&](int e, int p) { return e * (nn - 1) + p < nrad; };
  for (int e = 0; e < nel; ++e) {
    const double sf = 0.5 * (bval[e + 1] - bval[e]), mid = 0.5 * (bval[e + 1] + bval[e]);
    for (int q = 0; q < NGL_1E; ++q) {
      const double mu = mid + sf * xg[q], wq = wg[q] * sf, sh = std::sinh(mu), ch = std::cosh(mu);
      for (int b = 0; b < nn; ++b) {
        if (!valid(e, b)) continue;
        const int gb = e * (nn - 1) + b;
        for (int a = 0; a < nn; ++a) {
          if (!valid(e, a)) continue;
          const int ga = e * (nn - 1) + a;
          const double bb = Bv[q + (size_t)a * NGL_1E] * Bv[q + (size_t)b * NGL_1E] * wq;
          const size_t o = ga + (size_t)gb * nrad;
          I10[o] += bb * sh;
          I11[o] += bb * sh * ch;
          I12[o] += bb * sh * ch * ch;
          Im1[o] += bb / sh;
          Trad[o] += dBv[q + (size_t)a * NGL_1E] * dBv[q + (size_t)b * NGL_1E] * wq * sh / (sf * sf);
        }
      }
    }
  }
  if (!twoe_on_host) {  // the two-electron tables come from the device tabulation
    cd_rank.clear();
    cd_B.clear();
    cd_s.clear();
    rmax = 0;
    return;
  }
#pragma omp parallel
  {
    std::vector<double> PL(NMs * NLs), QL(NMs * NLs);
    std::vector<double> B1, B2, xr(1);
#pragma omp for schedule(dynamic)
    for (int e = 0; e < nel; ++e) {
      const double mus = bval[e], mue = bval[e + 1];
      const double sf = 0.5 * (mue - mus), mid = 0.5 * (mue + mus);
      // ---- disjoint integrals (GL on the element)
      {
        std::vector<double> Pq((size_t)NGL_1E * NMs * NLs), Qq((size_t)NGL_1E * NMs * NLs);
        for (int q = 0; q < NGL_1E; ++q)
          legendre_pq(Lmax, Mtop, mid + sf * xg[q], Pq.data() + (size_t)q * NMs * NLs,
                      Qq.data() + (size_t)q * NMs * NLs);
        for (int ilm = 0; ilm < nlm; ++ilm) {
          const int L = lm_L[ilm], M = lm_M[ilm];
          double* d_p0 = p0.data() + ((size_t)ilm * nel + e) * tile;
          double* d_p2 = p2.data() + ((size_t)ilm * nel + e) * tile;
          double* d_q0 = q0.data() + ((size_t)ilm * nel + e) * tile;
          double* d_q2 = q2.data() + ((size_t)ilm * nel + e) * tile;
          for (int q = 0; q < NGL_1E; ++q) {
            const double mu = mid + sf * xg[q], wq = wg[q] * sf, sh = std::sinh(mu), ch = std::cosh(mu);
            const double pv = Pq[(size_t)q * NMs * NLs + M * NLs + L] * wq * sh;
            const double qv = Qq[(size_t)q * NMs * NLs + M * NLs + L] * wq * sh;
            for (int b = 0; b < nn; ++b) {
              if (!valid(e, b)) continue;
              for (int a = 0; a < nn; ++a) {
                if (!valid(e, a)) continue;
                const double bb = Bv[q + (size_t)a * NGL_1E] * Bv[q + (size_t)b * NGL_1E];
                const size_t o = a + (size_t)b * nn;
                d_p0[o] += bb * pv;
                d_p2[o] += bb * pv * ch * ch;
                d_q0[o] += bb * qv;
                d_q2[o] += bb * qv * ch * ch;
              }
            }
          }
        }
      }
      // ---- in-element kernel
      std::vector<double> mu1(NGL_OUT), w1(NGL_OUT), mu2((size_t)NGL_OUT * NGL_IN), w2((size_t)NGL_OUT * NGL_IN);
      for (int q = 0; q < NGL_OUT; ++q) {
        if (e == 0) {
          const double t = 0.5 * (xo[q] + 1.0);
          mu1[q] = mus + (mue - mus) * t * t * t;
          w1[q] = 0.5 * wo[q] * 3.0 * (mue - mus) * t * t;
        } else {
          mu1[q] = mid + sf * xo[q];
          w1[q] = sf * wo[q];
        }
        const double h = 0.5 * (mu1[q] - mus);
        for (int r = 0; r < NGL_IN; ++r) {
          mu2[(size_t)q * NGL_IN + r] = mus + h * (xi[r] + 1.0);
          w2[(size_t)q * NGL_IN + r] = h * wi[r];
        }
      }
      std::vector<double> ref1(NGL_OUT), ref2((size_t)NGL_OUT * NGL_IN);
      for (int q = 0; q < NGL_OUT; ++q) ref1[q] = (mu1[q] - mid) / sf;
      for (size_t i = 0; i < ref2.size(); ++i) ref2[i] = (mu2[i] - mid) / sf;
      lip_eval(ref1, nodes, 0, B1);  // [q + p*NGL_OUT]
      lip_eval(ref2, nodes, 0, B2);  // [i + p*NGL_OUT*NGL_IN]
      const size_t n2i = ref2.size();
      for (int p = 0; p < nn; ++p)
        if (!valid(e, p)) {
          for (int q = 0; q < NGL_OUT; ++q) B1[q + (size_t)p * NGL_OUT] = 0.0;
          for (size_t i = 0; i < n2i; ++i) B2[i + (size_t)p * n2i] = 0.0;
        }
      std::vector<double> P1((size_t)NGL_OUT * NMs * NLs), Q1((size_t)NGL_OUT * NMs * NLs);
      std::vector<double> P2(n2i * NMs * NLs), Q2s(NMs * NLs);
      for (int q = 0; q < NGL_OUT; ++q)
        legendre_pq(Lmax, Mtop, mu1[q], P1.data() + (size_t)q * NMs * NLs, Q1.data() + (size_t)q * NMs * NLs);
      for (size_t i = 0; i < n2i; ++i) legendre_pq(Lmax, Mtop, mu2[i], P2.data() + i * NMs * NLs, Q2s.data());
      // unique pairs a <= b
      std::vector<int> pa, pb;
      for (int b = 0; b < nn; ++b)
        for (int a = 0; a <= b; ++a) { pa.push_back(a); pb.push_back(b); }
      const int np = (int)pa.size();
      // element-dependent, channel-independent factors: hyperbolic functions
      // of the quadrature points and the basis pair products (pair-contiguous)
      std::vector<double> sh1(NGL_OUT), ch1(NGL_OUT), sh2(n2i), ch2(n2i);
      for (int q = 0; q < NGL_OUT; ++q) { sh1[q] = std::sinh(mu1[q]); ch1[q] = std::cosh(mu1[q]); }
      for (size_t i = 0; i < n2i; ++i) { sh2[i] = std::sinh(mu2[i]); ch2[i] = std::cosh(mu2[i]); }
      std::vector<double> BB1((size_t)NGL_OUT * np), BB2(n2i * np);
      for (int q = 0; q < NGL_OUT; ++q)
        for (int k = 0; k < np; ++k)
          BB1[(size_t)q * np + k] = B1[q + (size_t)pa[k] * NGL_OUT] * B1[q + (size_t)pb[k] * NGL_OUT];
      for (size_t i = 0; i < n2i; ++i)
        for (int k = 0; k < np; ++k) BB2[i * np + k] = B2[i + (size_t)pa[k] * n2i] * B2[i + (size_t)pb[k] * n2i];
      // Channels in chunks of CH: the inner and outer integrals of a chunk
      // are formed with q outermost, so that each q's slice of the pair
      // products (NGL_IN x np) is read once per chunk instead of once per
      // channel. Per channel, q and pair the operations are unchanged.
      constexpr int CH = 8;
      const size_t qs = (size_t)NGL_OUT * np;  // one channel's [q][pair] block
      std::vector<double> inner0(CH * qs), inner2(CH * qs), outer0(CH * qs), outer2(CH * qs);
      std::vector<double> res((size_t)4 * np * np), Tt((size_t)3 * np * np);
      std::vector<double> W((size_t)4 * n2 * n2);
      std::vector<int> pidx(n2);
      for (int b = 0; b < nn; ++b)
        for (int a = 0; a < nn; ++a) {
          const int lo = std::min(a, b), hi = std::max(a, b);
          pidx[a + b * nn] = lo + hi * (hi + 1) / 2;
        }
      for (int ilm0 = 0; ilm0 < nlm; ilm0 += CH) {
        const int nch = std::min(CH, nlm - ilm0);
        for (int q = 0; q < NGL_OUT; ++q) {
          const double sh = sh1[q], ch = ch1[q];
          const double* bq = BB1.data() + (size_t)q * np;
          for (int c = 0; c < nch; ++c) {
            const int ilm = ilm0 + c;
            const size_t lmo = (size_t)lm_M[ilm] * NLs + lm_L[ilm];
            const double wq0 = w1[q] * sh * Q1[(size_t)q * NMs * NLs + lmo];
            double* o0 = outer0.data() + c * qs + (size_t)q * np;
            double* o2 = outer2.data() + c * qs + (size_t)q * np;
            double* i0 = inner0.data() + c * qs + (size_t)q * np;
            double* i2 = inner2.data() + c * qs + (size_t)q * np;
            for (int k = 0; k < np; ++k) {
              const double bb = bq[k];
              o0[k] = wq0 * bb;
              o2[k] = wq0 * ch * ch * bb;
              i0[k] = 0.0;
              i2[k] = 0.0;
            }
            for (int r = 0; r < NGL_IN; ++r) {
              const size_t ii = (size_t)q * NGL_IN + r;
              const double wr0 = w2[ii] * sh2[ii] * P2[ii * NMs * NLs + lmo], wr2 = wr0 * ch2[ii] * ch2[ii];
              const double* bi = BB2.data() + ii * np;
              for (int k = 0; k < np; ++k) {
                const double bb = bi[k];
                i0[k] += wr0 * bb;
                i2[k] += wr2 * bb;
              }
            }
          }
        }
        for (int c = 0; c < nch; ++c) {
          const int ilm = ilm0 + c;
          // res_kl[c + d*np] = sum_q outer_k[q][c] inner_l[q][d], q ascending,
          // in 4 x 8 register blocks
          const double* outs[2] = {outer0.data() + c * qs, outer2.data() + c * qs};
          const double* ins[2] = {inner0.data() + c * qs, inner2.data() + c * qs};
          for (int k = 0; k < 2; ++k)
            for (int l = 0; l < 2; ++l) {
              double* R = res.data() + (size_t)(2 * k + l) * np * np;
              const double* Ok = outs[k];
              const double* Il = ins[l];
              for (int d0 = 0; d0 < np; d0 += 4)
                for (int c0 = 0; c0 < np; c0 += 8) {
                  if (d0 + 4 <= np && c0 + 8 <= np) {
                    double acc[4][8] = {};
                    for (int q = 0; q < NGL_OUT; ++q) {
                      const double* oq = Ok + (size_t)q * np + c0;
                      const double* iq = Il + (size_t)q * np + d0;
                      for (int dd = 0; dd < 4; ++dd) {
                        const double v = iq[dd];
                        for (int cc = 0; cc < 8; ++cc) acc[dd][cc] += oq[cc] * v;
                      }
                    }
                    for (int dd = 0; dd < 4; ++dd)
                      for (int cc = 0; cc < 8; ++cc) R[(c0 + cc) + (size_t)(d0 + dd) * np] = acc[dd][cc];
                  } else {
                    for (int d = d0; d < std::min(np, d0 + 4); ++d)
                      for (int cx = c0; cx < std::min(np, c0 + 8); ++cx) {
                        double acc = 0.0;
                        for (int q = 0; q < NGL_OUT; ++q) acc += Ok[(size_t)q * np + cx] * Il[(size_t)q * np + d];
                        R[cx + (size_t)d * np] = acc;
                      }
                  }
                }
            }
          // T_kl(c, d) = res_kl(c, d) + res_lk(d, c): T00, T02 (= T20 transposed) and T22
          const double* r00 = res.data();
          const double* r02 = res.data() + (size_t)np * np;
          const double* r20 = res.data() + (size_t)2 * np * np;
          const double* r22 = res.data() + (size_t)3 * np * np;
          double* t00 = Tt.data();
          double* t02 = Tt.data() + (size_t)np * np;
          double* t22 = Tt.data() + (size_t)2 * np * np;
          for (int d0 = 0; d0 < np; d0 += 16)
            for (int c0 = 0; c0 < np; c0 += 16)
              for (int d = d0; d < std::min(np, d0 + 16); ++d)
                for (int cx = c0; cx < std::min(np, c0 + 16); ++cx) {
                  const size_t cd = cx + (size_t)d * np, dc = d + (size_t)cx * np;
                  t00[cd] = r00[cd] + r00[dc];
                  t02[cd] = r02[cd] + r20[dc];
                  t22[cd] = r22[cd] + r22[dc];
                }
          // W = [[T00, -T02], [-T02^T, T22]] over the pair index of (a, b).
          // It is symmetric as assembled: T_kl(c, d) and T_lk(d, c) are the
          // same two terms summed in the other order, so the reference's
          // 0.5 (W + W^T) leaves every entry unchanged.
          const int N = 2 * n2;
          for (int col = 0; col < n2; ++col) {
            const size_t dcol = (size_t)pidx[col] * np;
            double* w0 = W.data() + (size_t)col * N;
            double* w1c = W.data() + (size_t)(n2 + col) * N;
            for (int row = 0; row < n2; ++row) {
              const size_t cd = pidx[row] + dcol;
              w0[row] = t00[cd];
              w1c[row] = -t02[cd];
              w0[n2 + row] = -t02[pidx[col] + (size_t)pidx[row] * np];
              w1c[n2 + row] = t22[cd];
            }
          }
          sign_cholesky(W, N, cd_thresh, fB[(size_t)ilm * nel + e], fS[(size_t)ilm * nel + e]);
        }
      }
    }
  }
  rmax = 1;
  for (auto& s : fS) rmax = std::max(rmax, (int)s.size());
  const int N = 2 * n2;
  cd_rank.assign((size_t)nlm * nel, 0);
  cd_B.assign((size_t)nlm * nel * N * rmax, 0.0);
  cd_s.assign((size_t)nlm * nel * rmax, 0.0);
  for (size_t t = 0; t < fS.size(); ++t) {
    const int r = (int)fS[t].size();
    cd_rank[t] = r;
    std::copy(fB[t].begin(), fB[t].end(), cd_B.begin() + t * N * rmax);
    std::copy(fS[t].begin(), fS[t].end(), cd_s.begin() + t * rmax);
  }
}

void DiatomicHost::twoe_rules(TwoeRules& R) const {
  R.n1e = NGL_1E;
  R.no = NGL_OUT;
  R.ni = NGL_IN;
  gauss_legendre(NGL_1E, R.xg, R.wg);
  gauss_legendre(NGL_OUT, R.xo, R.wo);
  gauss_legendre(NGL_IN, R.xi, R.wi);
  lip_eval(R.xg, nodes, 0, R.Bg);
  lip_eval(R.xo, nodes, 0, R.B1g);
  // reference coordinates (mu - mid) / sf of the in-element points: on an
  // element after the first, mu_1 = mid + sf x_q and the inner points run
  // over [mu_s, mu_1]; on the first (mu_s = 0), mu_1 = mu_e t^3
  std::vector<double> r1z(NGL_OUT), r2g((size_t)NGL_OUT * NGL_IN), r2z((size_t)NGL_OUT * NGL_IN);
  for (int q = 0; q < NGL_OUT; ++q) {
    const double t = 0.5 * (R.xo[q] + 1.0), t3 = t * t * t;
    r1z[q] = 2.0 * t3 - 1.0;
    for (int r = 0; r < NGL_IN; ++r) {
      r2g[(size_t)q * NGL_IN + r] = 0.5 * (1.0 + R.xo[q]) * (1.0 + R.xi[r]) - 1.0;
      r2z[(size_t)q * NGL_IN + r] = t3 * (1.0 + R.xi[r]) - 1.0;
    }
  }
  lip_eval(r1z, nodes, 0, R.B1z);
  lip_eval(r2g, nodes, 0, R.B2g);
  lip_eval(r2z, nodes, 0, R.B2z);
}

void DiatomicHost::build_couplings() {
  GauntCache G;
  nM = 4 * mmax + 1;
  // angular coupling table
  al_ptr.assign((size_t)nang * (Lmax + 1) * nM + 1, 0);
  al_b.clear();
  al_c0.clear();
  al_c2.clear();
  for (int a = 0; a < nang; ++a)
    for (int L = 0; L <= Lmax; ++L)
      for (int M = -2 * mmax; M <= 2 * mmax; ++M) {
        const int idx = al_index(a, L, M);
        al_ptr[idx] = (int)al_b.size();
        if (std::abs(M) <= L) {
          for (int b = 0; b < nang; ++b) {
            if (mval[b] != mval[a] - M) continue;
            if (L < std::max(std::abs(lval[a] - lval[b]) - 2, std::abs(M)) || L > lval[a] + lval[b] + 2) continue;
            const double c0 = G.mod(lval[a], mval[a], L, M, lval[b], mval[b]);
            const double c2 = G.coeff(lval[a], mval[a], L, M, lval[b]);
            if (c0 == 0.0 && c2 == 0.0) continue;
            al_b.push_back(b);
            al_c0.push_back(c0);
            al_c2.push_back(c2);
          }
        }
      }
  al_ptr.back() = (int)al_b.size();
  auto al_len = [&](int a, int L, int M) {
    if (std::abs(M) > 2 * mmax || std::abs(M) > L) return 0;
    const int i = al_index(a, L, M);
    return al_ptr[i + 1] - al_ptr[i];
  };
  // Coulomb channels: signed (L, M) that some (i, j) pair couples, ordered
  ch_L.clear(); ch_M.clear(); ch_ilm.clear(); ch_fac.clear();
  std::vector<std::pair<int, int>> LM;
  for (int i = 0; i < nang; ++i)
    for (int j = 0; j < nang; ++j) {
      const int M = mval[j] - mval[i];
      for (int L = std::max(std::abs(lval[j] - lval[i]) - 2, std::abs(M)); L <= lval[j] + lval[i] + 2; ++L)
        LM.emplace_back(L, M);
    }
  std::sort(LM.begin(), LM.end());
  LM.erase(std::unique(LM.begin(), LM.end()), LM.end());
  std::vector<int> chan_of((size_t)(Lmax + 1) * nM, -1);
  for (auto& p : LM) {
    chan_of[(size_t)p.first * nM + p.second + 2 * mmax] = (int)ch_L.size();
    ch_L.push_back(p.first);
    ch_M.push_back(p.second);
    ch_ilm.push_back(lm_index(p.first, std::abs(p.second)));
    ch_fac.push_back(lm_factor(p.first, p.second, Rhalf));
  }
  // bra lists per output block (i, j): channel (L, M = mj - mi), couplings of
  // the (j; L, M; i) entry
  jbra_ptr.assign((size_t)nang * nang + 1, 0);
  jbra_chan.clear(); jbra_c0.clear(); jbra_c2.clear();
  for (int j = 0; j < nang; ++j)
    for (int i = 0; i < nang; ++i) {
      const int ij = i + j * nang;
      jbra_ptr[ij] = (int)jbra_chan.size();
      const int M = mval[j] - mval[i];
      if (std::abs(M) > 2 * mmax) continue;
      for (int L = 0; L <= Lmax; ++L) {
        if (!al_len(j, L, M)) continue;
        const int idx = al_index(j, L, M);
        for (int u = al_ptr[idx]; u < al_ptr[idx + 1]; ++u)
          if (al_b[u] == i) {
            const int ch = chan_of[(size_t)L * nM + M + 2 * mmax];
            if (ch < 0) throw std::logic_error("diatomic: missing Coulomb channel");
            jbra_chan.push_back(ch);
            jbra_c0.push_back(al_c0[u]);
            jbra_c2.push_back(al_c2[u]);
          }
      }
    }
  jbra_ptr.back() = (int)jbra_chan.size();  // filled in output-block order i + j*nang
  // exchange entries: per output block (j, k), every (L, |M|) with a signed
  // M = +-|M| for which both (j; L, M) and (k; L, M) couple something
  kjk_ptr.assign((size_t)nang * nang + 1, 0);
  kent_L.clear(); kent_Ma.clear(); kent_ilm.clear();
  for (int k = 0; k < nang; ++k)
    for (int j = 0; j < nang; ++j) {
      kjk_ptr[j + k * nang] = (int)kent_L.size();
      for (int ilm = 0; ilm < nlm; ++ilm) {
        const int L = lm_L[ilm], Ma = lm_M[ilm];
        bool any = false;
        for (int sgn = 0; sgn < (Ma ? 2 : 1) && !any; ++sgn) {
          const int M = sgn ? -Ma : Ma;
          any = al_len(j, L, M) > 0 && al_len(k, L, M) > 0;
        }
        if (!any) continue;
        kent_L.push_back(L);
        kent_Ma.push_back(Ma);
        kent_ilm.push_back(ilm);
      }
    }
  kjk_ptr.back() = (int)kent_L.size();
  // entries were appended in (k, j) order = output-block order j + k*nang
}

// D = dense one-electron matrix over the dummy basis (0: S, 1: T, 2: V)
void DiatomicHost::dense_one_electron(int which, std::vector<double>& D) const {
  GauntCache G;
  const size_t nd = (size_t)ndummy;
  D.assign(nd * nd, 0.0);
  auto add = [&](int ia, int ja, const std::vector<double>& R, double f) {
    if (f == 0.0) return;
    for (int c = 0; c < nrad; ++c)
      for (int r = 0; r < nrad; ++r)
        D[((size_t)ja * nrad + c) * nd + (size_t)ia * nrad + r] += f * R[r + (size_t)c * nrad];
  };
  for (int ia = 0; ia < nang; ++ia) {
    const int li = lval[ia], mi = mval[ia];
    if (which == 1) {
      add(ia, ia, Trad, 0.5 * Rhalf);
      add(ia, ia, I10, 0.5 * Rhalf * li * (li + 1));
      if (mi != 0) add(ia, ia, Im1, 0.5 * Rhalf * mi * mi);
      continue;
    }
    for (int ja = 0; ja < nang; ++ja) {
      const int lj = lval[ja], mj = mval[ja];
      if (mi != mj) continue;
      if (which == 0) {
        if (li == lj) add(ia, ja, I12, std::pow(Rhalf, 3));
        // cos^2 coupling = (2/3)sqrt(pi) <Y00> + (4/15)sqrt(5pi) <Y20>
        const double c2 = 2.0 / 3.0 * std::sqrt(M_PI) * G.coeff(lj, mj, 0, 0, li) +
                          4.0 / 15.0 * std::sqrt(5.0 * M_PI) * G.coeff(lj, mj, 2, 0, li);
        add(ia, ja, I10, -c2 * std::pow(Rhalf, 3));
      } else {
        if (li == lj) add(ia, ja, I11, -(double)(Z1 + Z2) * Rhalf * Rhalf);
        if (Z1 != Z2) {
          const double c1 = 2.0 * std::sqrt(M_PI / 3.0) * G.coeff(lj, mj, 1, 0, li);
          add(ia, ja, I10, -(double)(Z2 - Z1) * c1 * Rhalf * Rhalf);
        }
      }
    }
  }
}

static void gather_pure(const std::vector<double>& D, const std::vector<int>& idx, int ndummy,
                        std::vector<double>& out) {
  const size_t n = idx.size();
  out.assign(n * n, 0.0);
  for (size_t c = 0; c < n; ++c)
    for (size_t r = 0; r < n; ++r) out[r + c * n] = D[(size_t)idx[r] + (size_t)idx[c] * ndummy];
}

void DiatomicHost::overlap(std::vector<double>& S) const {
  std::vector<double> D;
  dense_one_electron(0, D);
  gather_pure(D, pure, ndummy, S);
}
void DiatomicHost::kinetic(std::vector<double>& T) const {
  std::vector<double> D;
  dense_one_electron(1, D);
  gather_pure(D, pure, ndummy, T);
}
void DiatomicHost::nuclear(std::vector<double>& V) const {
  std::vector<double> D;
  dense_one_electron(2, D);
  gather_pure(D, pure, ndummy, V);
}

void DiatomicHost::one_electron_block(int which, int mblock, std::vector<double>& out, int& n_out) const {
  // the block only couples shells with m == mblock: build it from those
  GauntCache G;
  std::vector<int> shells;
  for (int a = 0; a < nang; ++a)
    if (mval[a] == mblock) shells.push_back(a);
  const int f0 = mblock == 0 ? 0 : 1, nr = nrad - f0;
  const int ns = (int)shells.size();
  n_out = ns * nr;
  out.assign((size_t)n_out * n_out, 0.0);
  auto add = [&](int si, int sj, const std::vector<double>& R, double f) {
    if (f == 0.0) return;
    for (int c = 0; c < nr; ++c)
      for (int r = 0; r < nr; ++r)
        out[((size_t)sj * nr + c) * n_out + (size_t)si * nr + r] += f * R[(r + f0) + (size_t)(c + f0) * nrad];
  };
  for (int si = 0; si < ns; ++si) {
    const int li = lval[shells[si]], mi = mval[shells[si]];
    if (which == 1) {
      add(si, si, Trad, 0.5 * Rhalf);
      add(si, si, I10, 0.5 * Rhalf * li * (li + 1));
      if (mi != 0) add(si, si, Im1, 0.5 * Rhalf * mi * mi);
      continue;
    }
    for (int sj = 0; sj < ns; ++sj) {
      const int lj = lval[shells[sj]], mj = mval[shells[sj]];
      if (which == 0) {
        if (li == lj) add(si, sj, I12, std::pow(Rhalf, 3));
        const double c2 = 2.0 / 3.0 * std::sqrt(M_PI) * G.coeff(lj, mj, 0, 0, li) +
                          4.0 / 15.0 * std::sqrt(5.0 * M_PI) * G.coeff(lj, mj, 2, 0, li);
        add(si, sj, I10, -c2 * std::pow(Rhalf, 3));
      } else {
        if (li == lj) add(si, sj, I11, -(double)(Z1 + Z2) * Rhalf * Rhalf);
        if (Z1 != Z2) {
          const double c1 = 2.0 * std::sqrt(M_PI / 3.0) * G.coeff(lj, mj, 1, 0, li);
          add(si, sj, I10, -(double)(Z2 - Z1) * c1 * Rhalf * Rhalf);
        }
      }
    }
  }
}

}  // namespace hfg

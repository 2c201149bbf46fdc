// Host-side (FP64) description of one atom: the finite-element radial basis,
// the integrals HelFEM's TwoDBasisT::compute_tei caches, and the Gaunt
// coupling lists, laid out for the device.
//
// Element layout (FiniteElementBasis.cpp:51-64, 305-313): every element is an
// nn x nn "primitive" tile. Primitive p of element e is the global radial
// function g(e,p) = e*(nn-1) + p - 1; consecutive elements share one function
// (g(e,nn-1) == g(e+1,0)); g == -1 (element 0, p = 0) and g == Nrad (last
// element, p = nn-1) are the functions removed by the Dirichlet conditions and
// are stored as zero rows/columns. Per-element matrices are stored padded to
// nn x nn, column-major.
#pragma once

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace hfg {

double gaunt_coeff(int L, int M, int l, int m, int lp);

// greedy pivoted Cholesky of the n x n column-major A with an absolute
// tolerance on the residual diagonal: n x rank column-major factor
std::vector<double> pivoted_cholesky(const std::vector<double>& A, int n, double tol, int& rank);
// modified spherical Bessel functions i_L, k_L (normalisation in yukawa.cpp)
double bessel_il(double x, int L);
double bessel_kl(double x, int L);

// 1-D rules and Lagrange interpolating polynomials
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w);
void gauss_lobatto(int n, std::vector<double>& x, std::vector<double>& w);
void cheb_rule(int n, std::vector<double>& x, std::vector<double>& w);
// d^n L_i(x)/dx^n for all nodes, out[ix + i*npts]
void lip_eval(const std::vector<double>& x, const std::vector<double>& nodes, int nder,
              std::vector<double>& out);
// quadrature of the in-element two-electron tensor: outer Gauss-Legendre rule
// (TWOE_NO points) on the element and, for outer point p, the inner rule
// (TWOE_NI points) on [r_min, r_p], whose reference coordinates are
// xin[q + p*TWOE_NI] = -1 + (xo[p] + 1)(xi[q] + 1)/2
constexpr int TWOE_NO = 128, TWOE_NI = 48;
void twoe_points(std::vector<double>& xo, std::vector<double>& wo, std::vector<double>& xi, std::vector<double>& wi,
                 std::vector<double>& xin);

struct RadialBasis {
  int nn = 0;    // nodes (functions) per element
  int nel = 0;
  int nrad = 0;
  std::vector<double> bval;   // nel+1
  std::vector<double> nodes;  // Gauss-Lobatto nodes on [-1,1]
  int g(int e, int p) const { return e * (nn - 1) + p - 1; }
  bool valid(int e, int p) const { const int q = g(e, p); return q >= 0 && q < nrad; }
  double sf(int e) const { return 0.5 * (bval[e + 1] - bval[e]); }
  double mid(int e) const { return 0.5 * (bval[e + 1] + bval[e]); }
  int first(int e) const { return e == 0 ? 0 : g(e, 0); }
  int nfun(int e) const;
  int pfirst(int e) const { return e == 0 ? 1 : 0; }  // first valid primitive
  // B (nder 0/1) at reference points x: out[ix + p*npts] in primitive index
  // space (invalid primitives zero)
  void B(int e, const std::vector<double>& x, int nder, std::vector<double>& out) const;
  // R = B/r and dR/dr (deflated analytically on element 0)
  void R(int e, const std::vector<double>& x, std::vector<double>& out) const;
  void dR(int e, const std::vector<double>& x, std::vector<double>& out) const;
  // int R_a R_b r^(k+2) dr, nn x nn padded
  std::vector<double> radial_integral(int k, int e) const;
  // int B_a B_b f(r) dr = int R_a R_b f(r) r^2 dr, nn x nn padded
  std::vector<double> weighted_integral(const std::function<double(double)>& f, int e) const;
  std::vector<double> kinetic(int e) const;  // 1/2 int B'_a B'_b dr
  // in-element (ab|cd)_L, (nn^2 x nn^2) padded, pair index a + b*nn
  std::vector<double> twoe(int L, int e) const;
  // in-element tensor of a separable kernel g(r<, r>) = fin(r<) fout(r>):
  // (ab|cd) = int int B_aB_b(r) B_cB_d(r') g(r<, r>), same layout as twoe
  std::vector<double> twoe_separable(const std::function<double(double)>& fin,
                                     const std::function<double(double)>& fout, int e) const;
  // LIP values at the in-element tensor's quadrature points, which in
  // reference coordinates do not depend on the element (filled by
  // prepare_twoe before parallel tabulation; computed per call otherwise)
  std::vector<double> tw_Bo, tw_Bin;
  void prepare_twoe();
};

struct AtomHost {
  int Z = 0;
  RadialBasis rad;
  int nquad = 0;
  int nang = 0, nbf = 0, NL = 0, lmax = 0;
  std::vector<int> lval, mval;
  double chol_tol = 1e-12;

  // per (L, e): padded nn x nn
  std::vector<double> rs, rb;  // [(L*nel+e)*nn*nn]
  // per (L, e): pivoted Cholesky factor, compact reference layout (Ni^2 x r)
  std::vector<std::vector<double>> chol;
  std::vector<int> chol_rank;
  // per (L, e): padded J-ordered factor nn^2 x rmax (zero-padded columns)
  int rmax = 0;
  std::vector<double> cholp;  // [(L*nel+e)*nn*nn*rmax]
  // per (L, e): exchange-ordered in-element tensor rebuilt from the factor,
  //   Tk[(a + c*nn) + (b + d*nn)*nn^2] = sum_p Lc(a+b*nn,p) Lc(c+d*nn,p)
  std::vector<double> tk;

  // radial one-electron blocks assembled (nrad x nrad)
  std::vector<double> Srad, Trad, Tlrad, Vrad;

  // ---- Gaunt coupling lists ----------------------------------------------
  // J: channels (L,M); ket terms (k,l,coef); bra terms per output (i,j)
  struct Chan { int L, M; };
  std::vector<Chan> chans;
  std::vector<int> jket_ptr;      // [nchan+1]
  std::vector<int> jket_blk;      // angular block index k + l*nang
  std::vector<double> jket_coef;
  std::vector<int> jbra_ptr;      // [nang*nang+1], output block i + j*nang
  std::vector<int> jbra_chan;
  std::vector<double> jbra_coef;  // includes 4pi/(2L+1)
  // K: per output block (j + k*nang): L entries, each with (i + l*nang, coef)
  std::vector<int> kjk_ptr;       // [nang*nang+1] -> entries
  std::vector<int> kent_L;        // per entry
  std::vector<int> kent_ptr;      // [nent+1] -> terms
  std::vector<int> kterm_blk;
  std::vector<double> kterm_coef; // includes 4pi/(2L+1)

  // ---- DFT grid (src/atomic/dftgrid.cpp:470-576, angular.cpp:21-70) -----
  // per element: nquad Chebyshev radial points; angular product rule of
  // ldft cos(theta) Chebyshev points x mdft uniform phi points (nap total)
  int ldft = 0, mdft = 0, nap = 0;
  std::vector<double> xc_wang;     // [nap] angular weights
  std::vector<double> xc_isin;     // [nap] 1/sin(theta)
  // real angular tables, [(alpha + beta*nang)*nap + a]:
  //   W   = Re[Y_alpha conj(Y_beta)]
  //   Wt  = Re[dY_alpha/dtheta conj(Y_beta)]
  //   Wp  = Re[(i m_alpha) Y_alpha conj(Y_beta)]
  std::vector<double> xc_W, xc_Wt, xc_Wp;
  // per element e and radial point q: r, total radial weight wrad*r^2,
  // R and dR/dr of the nn primitives: [(e*nquad + q)*nn + p]
  std::vector<double> xc_r, xc_wr, xc_R, xc_dR;
  void build_dft_grid(int ldft, int mdft);

  // ---- Yukawa-screened (range-separated) exchange ----------------------
  // (src/atomic/TwoDBasis.cpp:736-758, 1001-1131): e^{-lambda r12}/r12 =
  // 4 pi lambda sum_LM i_L(lambda r<) k_L(lambda r>) Y Y*, with the modified
  // spherical Bessel functions i_L = sqrt(pi/2x) I_{L+1/2}, k_L =
  // sqrt(2/(pi x)) K_{L+1/2}. The tables below carry the factor (2L+1) lambda
  // relative to the bare ones, so that the bare coupling coefficients (which
  // include 4 pi/(2L+1)) give 4 pi lambda: per (L, e) padded nn x nn
  // y_rs = (2L+1) lambda int B B i_L(lambda r), y_rb = int B B k_L(lambda r),
  // and y_tk the exchange-ordered in-element tensor (scaled likewise).
  double y_lambda = 0.0;
  std::vector<double> y_rs, y_rb, y_tk;
  void build_yukawa(double lambda);
  // Range-separated exchange with the erfc kernel (host/erfc.cpp):
  // erfc(mu r12)/r12 = sum_LM (4 pi/(2L+1)) mu Phi_L(mu r>, mu r<) Y Y*
  // does not separate into r< / r> factors, so every element pair (a, b)
  // has its own exchange-ordered table, mu times the pair's (ij|kl)_L:
  // e_tk[((L*nel + a)*nel + b)*n2*n2 + t + v*n2], t = j + k nn (output),
  // v = i + l nn (density), padded. exact_binomial selects the
  // generalised binomial in the short-range series instead of the
  // reference's rule.
  double e_mu = 0.0;
  bool e_exact = false;
  std::vector<double> e_tk;
  void build_erfc(double mu, bool exact_binomial);

  // twoe_host = false leaves the in-element factors (chol, cholp, tk,
  // chol_rank, rmax) to the device tabulation
  void build(int Z, int nnodes, const std::vector<double>& bval, const std::vector<int>& lval,
             const std::vector<int>& mval, int nquad, double chol_tol, bool twoe_host = true);
  bool twoe_on_host = true;
  // Spherically averaged basis (src/sadatom/basis.cpp): angular functions
  // (l, 0) for l = 0..lmax, one per l channel, set before build(). The
  // coupling lists then carry the channel-averaged coefficients instead of
  // the Gaunt products: J has the one multipole L = 0, summed over every
  // diagonal block and scattered to every diagonal block with 4 pi
  // (basis.cpp:186-207); K(l_out, l_out) = -sum_L K_L[sum_l_in (4 pi/(2L+1))
  // c(l_out, l_in, L) P(l_in, l_in)] with c the m-averaged squared Gaunt
  // coefficient (basis.cpp:209-312).
  bool spherical = false;
  void build_couplings();
  void build_couplings_spherical();
};

// normalised Y_l^m(theta, phi) with the Condon-Shortley phase (value of the
// reference's ::spherical_harmonics, src/general/spherical_harmonics.cpp)
void ylm(int l, int m, double cth, double phi, double& re, double& im);

}  // namespace hfg

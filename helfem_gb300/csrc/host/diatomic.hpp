// Host-side (FP64) description of one diatomic molecule in prolate
// spheroidal coordinates (mu, nu, phi): the finite-element basis in mu, the
// integrals HelFEM's diatomic TwoDBasis::compute_tei caches, the angular
// coupling tables and the one-electron radial blocks, laid out for the
// device.
//
// Radial layout (src/diatomic/basis.cpp:522-540): element e owns an nn x nn
// primitive tile; primitive p is the global function g(e,p) = e*(nn-1) + p,
// valid for g < nrad = nel*(nn-1) (the mu = 0 function is kept, the mu_max
// one dropped). The "dummy" basis is nang*nrad functions (AO index
// iang*nrad + irad); the pure basis drops the mu = 0 function of every m != 0
// shell (basis.cpp:712-736).
#pragma once

#include <vector>

namespace hfg {

// P[M*(Lmax+1) + L], Q[...] of x = cosh(mu), Hobson convention (no
// Condon-Shortley phase), for 0 <= M <= Mmax, 0 <= L <= Lmax. Non-finite and
// subnormal values are returned as 0.
void legendre_pq(int Lmax, int Mmax, double mu, double* P, double* Q);

struct DiatomicHost {
  int Z1 = 0, Z2 = 0;
  double Rhalf = 0.0;
  int nn = 0, nel = 0, nrad = 0, nang = 0, ndummy = 0, nbf = 0;
  std::vector<double> bval, nodes;
  std::vector<int> lval, mval;
  std::vector<int> pure;  // [nbf] dummy index of each pure function
  int mmax = 0;           // max |m| of the basis
  int Lmax = 0;           // max multipole L
  // (L,|M|) multipoles, |M|-major then L (basis.cpp:553-620)
  int nlm = 0;
  std::vector<int> lm_L, lm_M;
  int lm_index(int L, int Mabs) const;
  // per (ilm, e), padded nn x nn column-major: int B_a B_b sinh cosh^k P (k = 0, 2)
  // and the same with Q
  std::vector<double> p0, p2, q0, q2;
  // per (ilm, e): sign-carrying factor of the 2-channel in-element kernel,
  // padded (2 nn^2 x rmax), row = channel*nn^2 + a + b*nn
  int rmax = 0;
  std::vector<int> cd_rank;
  std::vector<double> cd_B, cd_s;  // cd_s: [(ilm*nel+e)*rmax]
  double cd_thresh = 1e-12;
  // assembled one-electron radial blocks (nrad x nrad, column-major):
  // int B B sinh, sinh cosh, sinh cosh^2, 1/sinh, and int B' B' sinh
  std::vector<double> I10, I11, I12, Im1, Trad;

  // ---- angular coupling table ---------------------------------------------
  // For angular function a, multipole L and signed M (|M| <= 2 mmax): the
  // functions b with mb = ma - M that couple, with
  //   c0 = int Y_a* cos^2(nu) Y_L^M Y_b   (the reference's mod_coeff)
  //   c2 = int Y_a* Y_L^M Y_b             (its coeff)
  // Serves the Coulomb ket and bra sums and the exchange recoupling.
  int nM = 0;  // 4*mmax + 1
  std::vector<int> al_ptr;  // [(a*(Lmax+1) + L)*nM + M + 2 mmax] (+1)
  std::vector<int> al_b;
  std::vector<double> al_c0, al_c2;
  int al_index(int a, int L, int M) const { return (a * (Lmax + 1) + L) * nM + M + 2 * mmax; }

  // ---- Coulomb channels (signed (L, M)) and bra lists ----------------------
  std::vector<int> ch_L, ch_M, ch_ilm;
  std::vector<double> ch_fac;  // (-1)^M 4 pi Rhalf^5 (L-|M|)!/(L+|M|)!
  std::vector<int> jbra_ptr;   // [nang*nang+1] output block i + j*nang
  std::vector<int> jbra_chan;
  std::vector<double> jbra_c0, jbra_c2;
  // ---- exchange entries per output block j + k*nang: (L, |M|) --------------
  std::vector<int> kjk_ptr;    // [nang*nang+1]
  std::vector<int> kent_L, kent_Ma, kent_ilm;

  // ---- pure-m DFT grid (src/diatomic/dftgrid_purem.cpp:34-199) -----------
  // Per mu element: xc_nq Chebyshev points in mu; xc_lang Chebyshev points in
  // cos(nu); the phi integral is analytic (2 pi). Only same-m angular pairs
  // couple, and every quantity is symmetric under s <-> t, so the tables run
  // over unordered pairs k = (s <= t): xc_ps[k] = s, xc_pt[k] = t,
  // xc_mult[k] = 2 (s != t) or 1.
  int xc_lang = 0, xc_nq = 0, xc_npair = 0;
  std::vector<int> xc_ps, xc_pt;
  std::vector<double> xc_mult;
  std::vector<double> xc_W, xc_Wt;     // [k*lang + a]: Y_s Y_t and Y_s' Y_t + Y_s Y_t' (phi = 0)
  std::vector<double> xc_R, xc_dR;     // [(e*nq + q)*nn + p]: B_p, dB_p/dmu
  std::vector<double> xc_w, xc_hinv;   // [(e*nq + q)*lang + a]: weight, 1/h
  // Fock-side pair list: V_xc is one phi-independent field, so the tile of a
  // -m pair equals that of its +m mirror (same l's). xc_fk lists the pairs
  // whose tiles are built (m >= 0, or without a mirror); xc_fms / xc_fmt are
  // the mirror shells the same tile is also written to (-1: none).
  std::vector<int> xc_fk, xc_fms, xc_fmt;
  void build_xc_grid(int lang);

  // twoe_on_host = false: the two-electron tables (p0..q2, cd_*) are left
  // to the device tabulation, which fills p0..q2, cd_rank and rmax
  void build(int Z1, int Z2, double Rhalf, int nnodes, const std::vector<double>& bval,
             const std::vector<int>& lval, const std::vector<int>& mval, double cd_thresh,
             bool twoe_on_host = true);
  bool twoe_on_host = true;
  // quadrature rules of the two-electron tabulation and the LIP values at
  // its reference points, for the device tabulation: B1*/B2* are the outer
  // and inner points of the elements after the first (*g) and of the first
  // (*z, mu = mu_1 t^3), laid out [q + p*no] and [(q*ni + r) + p*no*ni]
  struct TwoeRules {
    int n1e = 0, no = 0, ni = 0;
    std::vector<double> xg, wg, xo, wo, xi, wi, Bg, B1g, B1z, B2g, B2z;
  };
  void twoe_rules(TwoeRules& R) const;
  // pure-basis one-electron matrices (nbf x nbf, column-major)
  void overlap(std::vector<double>& S) const;
  void kinetic(std::vector<double>& T) const;
  void nuclear(std::vector<double>& V) const;
  // the same restricted to the pure functions with m == mblock (symmetry
  // block, pure order): n_out functions
  void one_electron_block(int which, int mblock, std::vector<double>& out, int& n_out) const;

 private:
  void tabulate_radial();
  void tabulate_twoe();
  void build_couplings();
  void dense_one_electron(int which, std::vector<double>& D) const;
};

}  // namespace hfg

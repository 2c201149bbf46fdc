// helfem_gb300/TwoDBasis.hpp — header-only C++ shim over the C ABI that
// re-exposes the reference's member-function signatures for the Fock-build
// path, so that a C++ driver written against HelFEM switches by changing the
// type it instantiates:
//
//   atomic   TwoDBasisT<double>::coulomb / exchange / compute_tei / overlap /
//            kinetic / nuclear, compute_yukawa / rs_exchange
//                                        (src/atomic/TwoDBasis.h:180-227)
//   diatomic TwoDBasis::coulomb / exchange / compute_tei / overlap /
//            kinetic / nuclear           (src/diatomic/basis.h:300-337)
//   DFTGrid::eval_Fxc(x, c, P, H, Exc, Nel, thr) and the Pa/Pb overload
//                                        (src/atomic/dftgrid.h:156-159)
//   diatomic PureMDFTGrid::eval_Fxc, both overloads
//                                        (src/diatomic/dftgrid_purem.h:154-161)
//   sadatom  TwoDBasis::coulomb / exchange / rs_exchange / compute_tei /
//            compute_yukawa / compute_erfc / overlap / kinetic / kinetic_l /
//            nuclear                     (src/sadatom/basis.h:25-130)
//   sadatom  DFTGrid::eval_Fxc, both overloads
//                                        (src/sadatom/dftgrid.h:124-127)
//
// Matrix is any column-major dense type with Matrix(rows, cols), rows(),
// cols() and data() (Eigen::MatrixXd, helfem::Matrix). Status codes come back
// as the reference's exception types: a missing compute_tei is
// std::logic_error("Primitive teis have not been computed!\n") as in
// TwoDBasis.cpp:775-776, bad shapes are std::runtime_error (as
// dftgrid_common.h:130-134 throws), bad arguments std::invalid_argument,
// allocation failures std::bad_alloc.
#pragma once

#include <algorithm>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../helfem_gb300.h"

namespace helfem_gb300 {

inline void check(hfg_status s) {
  if (s == HFG_OK) return;
  const std::string msg = hfg_last_error();
  switch (s) {
    case HFG_ERR_ARG: throw std::invalid_argument(msg);
    case HFG_ERR_STATE: throw std::logic_error(msg);
    case HFG_ERR_NOMEM: throw std::bad_alloc();
    default: throw std::runtime_error(msg);
  }
}

namespace detail {
template <class Matrix>
void require_square(const Matrix& P, size_t n, const char* who) {
  if ((size_t)P.rows() != n || (size_t)P.cols() != n)
    throw std::runtime_error(std::string(who) + ": density matrix has the wrong size");
}
inline void no_tei() { throw std::logic_error("Primitive teis have not been computed!\n"); }
}  // namespace detail

// ---------------------------------------------------------------- atomic
template <class Matrix>
class AtomicTwoDBasis {
 public:
  AtomicTwoDBasis(int Z, int nnodes, int nquad, std::vector<double> bval, std::vector<int> lval,
                  std::vector<int> mval)
      : Z_(Z), nnodes_(nnodes), nquad_(nquad), bval_(std::move(bval)), lval_(std::move(lval)),
        mval_(std::move(mval)) {
    // one-electron matrices are available before compute_tei, as in the reference
    host_ = make(true);
  }
  ~AtomicTwoDBasis() = default;
  AtomicTwoDBasis(const AtomicTwoDBasis&) = delete;
  AtomicTwoDBasis& operator=(const AtomicTwoDBasis&) = delete;

  // caches the integrals on the device; the flag is accepted for signature
  // compatibility (both J and K tables are always built)
  void compute_tei(bool /*exchange*/) { gpu_ = make(false); }

  size_t Nbf() const { return (size_t)dims().nbf; }
  size_t Nrad() const { return (size_t)dims().nrad; }
  size_t Nang() const { return lval_.size(); }

  Matrix overlap() const { return one(hfg_overlap); }
  Matrix kinetic() const { return one(hfg_kinetic); }
  Matrix nuclear() const { return one(hfg_nuclear); }

  Matrix coulomb(const Matrix& P) const {
    if (!gpu_) detail::no_tei();
    detail::require_square(P, Nbf(), "coulomb");
    Matrix J(P.rows(), P.cols());
    check(hfg_coulomb_host(gpu_.get(), P.data(), J.data()));
    return J;
  }
  Matrix exchange(const Matrix& P) const {
    if (!gpu_) detail::no_tei();
    detail::require_square(P, Nbf(), "exchange");
    Matrix K(P.rows(), P.cols());
    check(hfg_exchange_host(gpu_.get(), P.data(), K.data()));
    return K;
  }

  // range-separated exchange with the Yukawa kernel exp(-lambda r12)/r12
  // (TwoDBasis.h compute_yukawa / rs_exchange); compute_tei first
  void compute_yukawa(double lambda) {
    if (!gpu_) detail::no_tei();
    check(hfg_atom_compute_yukawa(gpu_.get(), lambda));
  }
  Matrix rs_exchange(const Matrix& P) const {
    if (!gpu_) detail::no_tei();
    detail::require_square(P, Nbf(), "rs_exchange");
    Matrix K(P.rows(), P.cols());
    check(hfg_rs_exchange_host(gpu_.get(), P.data(), K.data(), 0));
    return K;
  }

  hfg_atom* handle() const { return gpu_.get(); }

 private:
  struct Del {
    void operator()(hfg_atom* a) const { hfg_atom_destroy(a); }
  };
  std::unique_ptr<hfg_atom, Del> make(bool host_only) const {
    hfg_atom_desc d{Z_, nnodes_, nquad_, (int)bval_.size() - 1, bval_.data(), (int)lval_.size(),
                    lval_.data(), mval_.data(), 0.0, host_only ? 1 : 0};
    hfg_atom* a = nullptr;
    check(hfg_atom_create(&d, &a));
    return std::unique_ptr<hfg_atom, Del>(a);
  }
  hfg_atom_dims_t dims() const {
    hfg_atom_dims_t d{};
    check(hfg_atom_get_dims(host_.get(), &d));
    return d;
  }
  Matrix one(hfg_status (*fn)(const hfg_atom*, double*)) const {
    const size_t n = Nbf();
    Matrix M(n, n);
    check(fn(host_.get(), M.data()));
    return M;
  }

  int Z_, nnodes_, nquad_;
  std::vector<double> bval_;
  std::vector<int> lval_, mval_;
  std::unique_ptr<hfg_atom, Del> host_, gpu_;
};

// DFTGrid::eval_Fxc over an atomic basis (the grid is built on the device on
// first use; Ekin of meta-GGAs is not part of this path and returns 0)
template <class Matrix>
class AtomicDFTGrid {
 public:
  explicit AtomicDFTGrid(const AtomicTwoDBasis<Matrix>* basis) : b_(basis) {}
  void eval_Fxc(int x_func, int c_func, const Matrix& P, Matrix& H, double& Exc, double& Nel, double& Ekin,
                double thr) const {
    if (!b_->handle()) detail::no_tei();
    detail::require_square(P, b_->Nbf(), "eval_Fxc");
    H = Matrix(P.rows(), P.cols());
    check(hfg_xc_host(b_->handle(), x_func, c_func, P.data(), nullptr, H.data(), nullptr, &Exc, &Nel, thr));
    Ekin = 0.0;
  }
  void eval_Fxc(int x_func, int c_func, const Matrix& Pa, const Matrix& Pb, Matrix& Ha, Matrix& Hb, double& Exc,
                double& Nel, double& Ekin, double thr) const {
    if (!b_->handle()) detail::no_tei();
    detail::require_square(Pa, b_->Nbf(), "eval_Fxc");
    detail::require_square(Pb, b_->Nbf(), "eval_Fxc");
    Ha = Matrix(Pa.rows(), Pa.cols());
    Hb = Matrix(Pb.rows(), Pb.cols());
    check(hfg_xc_host(b_->handle(), x_func, c_func, Pa.data(), Pb.data(), Ha.data(), Hb.data(), &Exc, &Nel, thr));
    Ekin = 0.0;
  }

 private:
  const AtomicTwoDBasis<Matrix>* b_;
};

// -------------------------------------------------------------- diatomic
template <class Matrix>
class DiatomicTwoDBasis {
 public:
  DiatomicTwoDBasis(int Z1, int Z2, double Rhalf, int nnodes, std::vector<double> bval, std::vector<int> lval,
                    std::vector<int> mval)
      : Z1_(Z1), Z2_(Z2), Rhalf_(Rhalf), nnodes_(nnodes), bval_(std::move(bval)), lval_(std::move(lval)),
        mval_(std::move(mval)) {
    host_ = make(true);
  }
  DiatomicTwoDBasis(const DiatomicTwoDBasis&) = delete;
  DiatomicTwoDBasis& operator=(const DiatomicTwoDBasis&) = delete;

  void compute_tei(bool /*exchange*/) { gpu_ = make(false); }

  size_t Nbf() const { return (size_t)dims().nbf; }
  size_t Ndummy() const { return (size_t)dims().ndummy; }
  size_t Nrad() const { return (size_t)dims().nrad; }
  size_t Nang() const { return lval_.size(); }

  Matrix overlap() const { return one(hfg_diatomic_overlap); }
  Matrix kinetic() const { return one(hfg_diatomic_kinetic); }
  Matrix nuclear() const { return one(hfg_diatomic_nuclear); }

  Matrix coulomb(const Matrix& P) const {
    if (!gpu_) detail::no_tei();
    detail::require_square(P, Nbf(), "coulomb");
    Matrix J(P.rows(), P.cols());
    check(hfg_diatomic_coulomb_host(gpu_.get(), P.data(), J.data()));
    return J;
  }
  Matrix exchange(const Matrix& P) const {
    if (!gpu_) detail::no_tei();
    detail::require_square(P, Nbf(), "exchange");
    Matrix K(P.rows(), P.cols());
    check(hfg_diatomic_exchange_host(gpu_.get(), P.data(), K.data(), 0));
    return K;
  }

  hfg_diatomic* handle() const { return gpu_.get(); }

 private:
  struct Del {
    void operator()(hfg_diatomic* d) const { hfg_diatomic_destroy(d); }
  };
  std::unique_ptr<hfg_diatomic, Del> make(bool host_only) const {
    hfg_diatomic_desc d{Z1_, Z2_, Rhalf_, nnodes_, (int)bval_.size() - 1, bval_.data(), (int)lval_.size(),
                        lval_.data(), mval_.data(), 0.0, host_only ? 1 : 0};
    hfg_diatomic* h = nullptr;
    check(hfg_diatomic_create(&d, &h));
    return std::unique_ptr<hfg_diatomic, Del>(h);
  }
  hfg_diatomic_dims_t dims() const {
    hfg_diatomic_dims_t d{};
    check(hfg_diatomic_get_dims(host_.get(), &d));
    return d;
  }
  Matrix one(hfg_status (*fn)(const hfg_diatomic*, double*)) const {
    const size_t n = Nbf();
    Matrix M(n, n);
    check(fn(host_.get(), M.data()));
    return M;
  }

  int Z1_, Z2_;
  double Rhalf_;
  int nnodes_;
  std::vector<double> bval_;
  std::vector<int> lval_, mval_;
  std::unique_ptr<hfg_diatomic, Del> host_, gpu_;
};

// PureMDFTGrid over a diatomic basis: the XC potential when the orbitals do
// not mix m. lang = 0 takes the reference default 4 lmax + 12. External
// functional parameters are not supported (the x_pars/c_pars arguments of the
// reference are absent); Ekin of meta-GGAs is not part of this path and
// returns 0. `beta` is accepted for signature compatibility: Hb is always
// assigned, zero when the beta density is zero (dftgrid_purem.cpp:731-742).
template <class Matrix>
class DiatomicPureMDFTGrid {
 public:
  DiatomicPureMDFTGrid(const DiatomicTwoDBasis<Matrix>* basis, int lang) : b_(basis), lang_(lang) {}
  void eval_Fxc(int x_func, int c_func, const Matrix& P, Matrix& H, double& Exc, double& Nel, double& Ekin,
                double thr) const {
    prepare();
    detail::require_square(P, b_->Nbf(), "eval_Fxc");
    H = Matrix(P.rows(), P.cols());
    check(hfg_diatomic_xc_host(b_->handle(), x_func, c_func, P.data(), nullptr, H.data(), nullptr, &Exc, &Nel, thr));
    Ekin = 0.0;
  }
  void eval_Fxc(int x_func, int c_func, const Matrix& Pa, const Matrix& Pb, Matrix& Ha, Matrix& Hb, double& Exc,
                double& Nel, double& Ekin, bool /*beta*/, double thr) const {
    prepare();
    detail::require_square(Pa, b_->Nbf(), "eval_Fxc");
    detail::require_square(Pb, b_->Nbf(), "eval_Fxc");
    Ha = Matrix(Pa.rows(), Pa.cols());
    Hb = Matrix(Pb.rows(), Pb.cols());
    check(hfg_diatomic_xc_host(b_->handle(), x_func, c_func, Pa.data(), Pb.data(), Ha.data(), Hb.data(), &Exc, &Nel,
                               thr));
    Ekin = 0.0;
  }

 private:
  void prepare() const {
    if (!b_->handle()) detail::no_tei();
    if (!built_) {
      check(hfg_diatomic_dft_grid(b_->handle(), lang_));
      built_ = true;
    }
  }
  const DiatomicTwoDBasis<Matrix>* b_;
  int lang_;
  mutable bool built_ = false;
};

// ----------------------------------------------- spherically averaged atom
// sadatom::basis::TwoDBasis (src/sadatom/basis.h:25-130): one radial channel
// per l = 0..lmax; matrices are Nrad x Nrad, densities and exchange
// matrices a Cube of lmax+1 of them. The one-electron matrices are the
// reference's radial ones: kinetic() without and kinetic_l() the
// coefficient of the l(l+1) centrifugal term.
template <class Matrix, class Cube = std::vector<Matrix>>
class SadatomTwoDBasis {
 public:
  SadatomTwoDBasis(int Z, int nnodes, int nquad, std::vector<double> bval, int lmax)
      : Z_(Z), nnodes_(nnodes), nquad_(nquad), lmax_(lmax), bval_(std::move(bval)) {
    // host tables with at least the p channel, whose kinetic block carries
    // the centrifugal term that kinetic_l() returns
    host_ = make(std::max(lmax_, 1), true);
  }
  SadatomTwoDBasis(const SadatomTwoDBasis&) = delete;
  SadatomTwoDBasis& operator=(const SadatomTwoDBasis&) = delete;

  void compute_tei() { gpu_ = make(lmax_, false); }
  void compute_yukawa(double lambda) {
    if (!gpu_) detail::no_tei();
    check(hfg_atom_compute_yukawa(gpu_.get(), lambda));
  }
  void compute_erfc(double mu) {
    if (!gpu_) detail::no_tei();
    check(hfg_atom_compute_erfc(gpu_.get(), mu, 0));
  }

  size_t Nbf() const { return (size_t)dims().nrad; }

  Matrix overlap() const { return block(hfg_overlap, 0); }
  Matrix kinetic() const { return block(hfg_kinetic, 0); }
  Matrix kinetic_l() const {
    Matrix T0 = block(hfg_kinetic, 0), T1 = block(hfg_kinetic, 1), Tl(T0.rows(), T0.cols());
    const size_t n = (size_t)T0.rows() * T0.cols();
    for (size_t i = 0; i < n; ++i) Tl.data()[i] = 0.5 * (T1.data()[i] - T0.data()[i]);
    return Tl;
  }
  Matrix nuclear() const { return block(hfg_nuclear, 0); }

  Matrix coulomb(const Matrix& P) const {
    if (!gpu_) detail::no_tei();
    if ((size_t)P.rows() != Nbf() || (size_t)P.cols() != Nbf())
      throw std::logic_error("Density matrix does not match basis set!\n");
    Matrix J(P.rows(), P.cols());
    check(hfg_sadatom_coulomb_host(gpu_.get(), P.data(), J.data()));
    return J;
  }
  Cube exchange(const Cube& P) const { return channels(hfg_sadatom_exchange_host, P); }
  Cube rs_exchange(const Cube& P) const { return channels(hfg_sadatom_rs_exchange_host, P); }

  hfg_atom* handle() const { return gpu_.get(); }
  int lmax() const { return lmax_; }

 private:
  struct Del {
    void operator()(hfg_atom* a) const { hfg_atom_destroy(a); }
  };
  std::unique_ptr<hfg_atom, Del> make(int lmax, bool host_only) const {
    hfg_sadatom_desc d{Z_, nnodes_, nquad_, (int)bval_.size() - 1, bval_.data(), lmax, 0.0, host_only ? 1 : 0};
    hfg_atom* a = nullptr;
    check(hfg_sadatom_create(&d, &a));
    return std::unique_ptr<hfg_atom, Del>(a);
  }
  hfg_atom_dims_t dims() const {
    hfg_atom_dims_t d{};
    check(hfg_atom_get_dims(host_.get(), &d));
    return d;
  }
  // channel l's diagonal block of the host handle's block-diagonal matrix
  Matrix block(hfg_status (*fn)(const hfg_atom*, double*), int l) const {
    const hfg_atom_dims_t d = dims();
    const size_t nr = (size_t)d.nrad, nbf = (size_t)d.nbf;
    std::vector<double> full(nbf * nbf);
    check(fn(host_.get(), full.data()));
    Matrix M(nr, nr);
    for (size_t j = 0; j < nr; ++j)
      for (size_t i = 0; i < nr; ++i) M.data()[i + j * nr] = full[(l * nr + i) + (l * nr + j) * nbf];
    return M;
  }
  Cube channels(hfg_status (*fn)(hfg_atom*, const double*, double*, int), const Cube& P) const {
    if (!gpu_) detail::no_tei();
    if ((int)P.size() != lmax_ + 1) throw std::logic_error("Density matrix am does not match basis set!\n");
    const size_t nr = Nbf();
    std::vector<double> in((size_t)(lmax_ + 1) * nr * nr), out(in.size());
    for (int l = 0; l <= lmax_; ++l) {
      if ((size_t)P[l].rows() != nr || (size_t)P[l].cols() != nr)
        throw std::logic_error("Density matrix does not match basis set!\n");
      std::copy(P[l].data(), P[l].data() + nr * nr, in.begin() + (size_t)l * nr * nr);
    }
    check(fn(gpu_.get(), in.data(), out.data(), 0));
    Cube K;
    for (int l = 0; l <= lmax_; ++l) {
      Matrix M(nr, nr);
      std::copy(out.begin() + (size_t)l * nr * nr, out.begin() + (size_t)(l + 1) * nr * nr, M.data());
      K.push_back(std::move(M));
    }
    return K;
  }

  int Z_, nnodes_, nquad_, lmax_;
  std::vector<double> bval_;
  std::unique_ptr<hfg_atom, Del> host_, gpu_;
};

// sadatom::dftgrid::DFTGrid::eval_Fxc (src/sadatom/dftgrid.h:124-127) with
// the reference's convention: P[l] is the channel density over 4 pi and
// H[l] = 4 pi times the XC block of channel l (the SCF divides it by 4 pi,
// src/sadatom/scf.cpp:163-192). External functional parameters are absent
// as for the other grids; `beta` is accepted for signature compatibility.
template <class Matrix, class Cube = std::vector<Matrix>>
class SadatomDFTGrid {
 public:
  explicit SadatomDFTGrid(const SadatomTwoDBasis<Matrix, Cube>* basis) : b_(basis) {}
  void eval_Fxc(int x_func, int c_func, const Cube& P, Cube& H, double& Exc, double& Nel, double thr) const {
    const std::vector<double> Pr = radial(P);
    std::vector<double> Hr(Pr.size());
    check(hfg_sadatom_xc_host(handle(), x_func, c_func, Pr.data(), nullptr, Hr.data(), nullptr, &Exc, &Nel, thr));
    H = spread(Hr);
  }
  void eval_Fxc(int x_func, int c_func, const Cube& Pa, const Cube& Pb, Cube& Ha, Cube& Hb, double& Exc,
                double& Nel, bool /*beta*/, double thr) const {
    const std::vector<double> Pra = radial(Pa), Prb = radial(Pb);
    std::vector<double> Hra(Pra.size()), Hrb(Prb.size());
    check(hfg_sadatom_xc_host(handle(), x_func, c_func, Pra.data(), Prb.data(), Hra.data(), Hrb.data(), &Exc,
                              &Nel, thr));
    Ha = spread(Hra);
    Hb = spread(Hrb);
  }

 private:
  static constexpr double kFourPi = 12.566370614359172953850573533118;
  hfg_atom* handle() const {
    if (!b_->handle()) detail::no_tei();
    return b_->handle();
  }
  // radial density 4 pi sum_l P[l]
  std::vector<double> radial(const Cube& P) const {
    if ((int)P.size() != b_->lmax() + 1) throw std::runtime_error("eval_Fxc: density has the wrong channel count");
    const size_t nr = b_->Nbf();
    std::vector<double> R(nr * nr, 0.0);
    for (const Matrix& M : P) {
      if ((size_t)M.rows() != nr || (size_t)M.cols() != nr)
        throw std::runtime_error("eval_Fxc: density matrix has the wrong size");
      for (size_t i = 0; i < nr * nr; ++i) R[i] += kFourPi * M.data()[i];
    }
    return R;
  }
  Cube spread(const std::vector<double>& Hr) const {
    const size_t nr = b_->Nbf();
    Cube H;
    for (int l = 0; l <= b_->lmax(); ++l) {
      Matrix M(nr, nr);
      for (size_t i = 0; i < nr * nr; ++i) M.data()[i] = kFourPi * Hr[i];
      H.push_back(std::move(M));
    }
    return H;
  }
  const SadatomTwoDBasis<Matrix, Cube>* b_;
};

}  // namespace helfem_gb300

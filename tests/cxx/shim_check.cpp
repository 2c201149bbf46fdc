// Exercises the C++ shim (include/helfem_gb300/TwoDBasis.hpp) the way a
// HelFEM driver would: reference signatures, reference exception types.
//   shim_check host   -> prints the atomic and diatomic overlap traces and
//                        checks that coulomb() before compute_tei() throws
//                        std::logic_error
//   shim_check gpu    -> prints tr(P J), tr(P K) for a fixed density
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "helfem_gb300/TwoDBasis.hpp"

struct Mat {  // minimal column-major matrix with the interface the shim needs
  std::vector<double> v;
  long r = 0, c = 0;
  Mat() = default;
  Mat(long r_, long c_) : v((size_t)r_ * c_, 0.0), r(r_), c(c_) {}
  long rows() const { return r; }
  long cols() const { return c; }
  double* data() { return v.data(); }
  const double* data() const { return v.data(); }
  double& operator()(long i, long j) { return v[(size_t)i + (size_t)j * r]; }
};

static double trace_prod(const Mat& A, const Mat& B) {
  double s = 0.0;
  for (size_t i = 0; i < A.v.size(); ++i) s += A.v[i] * B.v[i];
  return s;
}

int main(int argc, char** argv) {
  const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
  std::vector<double> b = {0.0, 0.5, 2.0, 8.0, 40.0};
  helfem_gb300::AtomicTwoDBasis<Mat> atom(4, 9, 0, b, {0, 1}, {0, 0});
  Mat S = atom.overlap();
  double tr = 0.0;
  for (long i = 0; i < S.rows(); ++i) tr += S(i, i);
  std::printf("atomic nbf %zu trS %.15e\n", atom.Nbf(), tr);
  std::vector<double> bd = {0.0, 0.8, 2.0, 4.7};
  helfem_gb300::DiatomicTwoDBasis<Mat> mol(1, 1, 0.7, 9, bd, {0, 1, 1, 1}, {0, 0, 1, -1});
  Mat Sd = mol.overlap();
  double trd = 0.0;
  for (long i = 0; i < Sd.rows(); ++i) trd += Sd(i, i);
  std::printf("diatomic nbf %zu trS %.15e\n", mol.Nbf(), trd);
  helfem_gb300::SadatomTwoDBasis<Mat> sad(10, 9, 0, b, 1);
  Mat Ss = sad.overlap(), Tl = sad.kinetic_l();
  double trs = 0.0, trl = 0.0;
  for (long i = 0; i < Ss.rows(); ++i) {
    trs += Ss(i, i);
    trl += Tl(i, i);
  }
  std::printf("sadatom nrad %zu trS %.15e trTl %.15e\n", sad.Nbf(), trs, trl);
  Mat P(atom.Nbf(), atom.Nbf());
  for (long i = 0; i < P.rows(); ++i)
    for (long j = 0; j < P.cols(); ++j) P(i, j) = 1e-2 / (1.0 + i + j);
  if (!gpu) {
    try {
      atom.coulomb(P);
      std::printf("no exception\n");
      return 1;
    } catch (const std::logic_error& e) {
      std::printf("logic_error: %s", e.what());
    }
    try {
      sad.exchange(std::vector<Mat>(2, Mat(sad.Nbf(), sad.Nbf())));
      std::printf("no exception\n");
      return 1;
    } catch (const std::logic_error& e) {
      std::printf("sadatom logic_error: %s", e.what());
    }
    return 0;
  }
  atom.compute_tei(true);
  Mat J = atom.coulomb(P), K = atom.exchange(P);
  std::printf("atomic trPJ %.15e trPK %.15e\n", trace_prod(P, J), trace_prod(P, K));
  mol.compute_tei(true);
  Mat Pd(mol.Nbf(), mol.Nbf());
  for (long i = 0; i < Pd.rows(); ++i)
    for (long j = 0; j < Pd.cols(); ++j) Pd(i, j) = 1e-3 / (1.0 + i + j);
  Mat Jd = mol.coulomb(Pd), Kd = mol.exchange(Pd);
  std::printf("diatomic trPJ %.15e trPK %.15e\n", trace_prod(Pd, Jd), trace_prod(Pd, Kd));
  // pure-m XC: LDA restricted and PBE unrestricted
  helfem_gb300::DiatomicPureMDFTGrid<Mat> grid(&mol, 0);
  Mat Hx, Ha, Hb;
  double exc = 0.0, nel = 0.0, ekin = 0.0, exc2 = 0.0, nel2 = 0.0;
  grid.eval_Fxc(1, 7, Pd, Hx, exc, nel, ekin, 1e-12);
  Mat Pb(mol.Nbf(), mol.Nbf());
  for (long i = 0; i < Pb.rows(); ++i)
    for (long j = 0; j < Pb.cols(); ++j) Pb(i, j) = 0.5 * Pd(i, j);
  grid.eval_Fxc(101, 130, Pd, Pb, Ha, Hb, exc2, nel2, ekin, true, 1e-12);
  std::printf("diatomic-xc trPH %.15e Exc %.15e Nel %.15e trPHa %.15e trPbHb %.15e Exc2 %.15e\n",
              trace_prod(Pd, Hx), exc, nel, trace_prod(Pd, Ha), trace_prod(Pb, Hb), exc2);
  // spherically averaged atom: J of the radial density, K of two channels,
  // LDA on the reference's grid convention (densities over 4 pi)
  sad.compute_tei();
  std::vector<Mat> Pc(2, Mat(sad.Nbf(), sad.Nbf()));
  Mat Pr(sad.Nbf(), sad.Nbf());
  for (int l = 0; l < 2; ++l)
    for (long i = 0; i < Pr.rows(); ++i)
      for (long j = 0; j < Pr.cols(); ++j) {
        Pc[l](i, j) = 1e-2 / (1.0 + l + i + j);
        Pr(i, j) += Pc[l](i, j);
      }
  Mat Js = sad.coulomb(Pr);
  std::vector<Mat> Ks = sad.exchange(Pc);
  helfem_gb300::SadatomDFTGrid<Mat> sgrid(&sad);
  std::vector<Mat> Pq(2, Mat(sad.Nbf(), sad.Nbf())), Hq;
  for (int l = 0; l < 2; ++l)
    for (size_t i = 0; i < Pq[l].v.size(); ++i) Pq[l].v[i] = Pc[l].v[i] / 12.566370614359172953850573533118;
  double sexc = 0.0, snel = 0.0;
  sgrid.eval_Fxc(1, 7, Pq, Hq, sexc, snel, 1e-12);
  std::printf("sadatom trPJ %.15e trPK0 %.15e trPK1 %.15e trPH %.15e Exc %.15e\n", trace_prod(Pr, Js),
              trace_prod(Pc[0], Ks[0]), trace_prod(Pc[1], Ks[1]), trace_prod(Pr, Hq[1]), sexc);
  try {
    mol.coulomb(Mat(3, 3));
  } catch (const std::runtime_error& e) {
    std::printf("runtime_error: %s\n", e.what());
  }
  return 0;
}

// Oracle (test infrastructure only): C++17/OpenMP restatement of HelFEM's
// atomic Coulomb and exchange builds. The GPU product is compared
// against it, and it is the timed CPU baseline; nothing in the product links it.
//
// Restated from (paths inside the HelFEM project):
//   src/atomic/TwoDBasis.cpp:773-877   TwoDBasisT::coulomb  (ket contraction
//                                       into Paux[L][M], per-(L,M) FE
//                                       assembly, bra scatter)
//   src/atomic/TwoDBasis.cpp:879-999   TwoDBasisT::exchange (OpenMP
//                                       collapse(2) over (jang,kang),
//                                       Rmat[L] recoupling, density-block
//                                       screening at 10*eps, K -= K_block)
//   libhelfemqc/include/CoulombExchangeFE.h:432-482
//                                       assemble_J_FE_one_multipole_cached_chol
//   libhelfemqc/include/CoulombExchangeFE.h:484-530
//                                       assemble_K_FE_one_multipole_cached_chol
// The loop structure, the memory traffic pattern (full Nrad x Nrad
// temporaries per (L,M) and per (jang,kang,L)) and the parallel decomposition
// follow the reference so that the CPU timing is representative of it. Small
// dense products are written as plain loops (the reference uses Eigen).
//
// Matrices are column-major doubles; the AO index is iang*Nrad + irad.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// Plain-data description of an atom's tabulated integrals.
struct ora_atom {
  int nrad, nang, nel, NL;
  int gmax;                 // Gaunt table bound (all l <= gmax)
  const int* lval;          // [nang]
  const int* mval;          // [nang]
  const int* first;         // [nel] first radial function of element
  const int* ni;            // [nel] functions in element
  const double* rs;         // r_small blocks, column-major ni x ni
  const int64_t* rs_off;    // [NL*nel]
  const double* rb;         // r_big blocks (element 0 unused)
  const int64_t* rb_off;    // [NL*nel]
  const double* chol;       // Cholesky factors (ni^2 x rank), column-major
  const int64_t* chol_off;  // [NL*nel]
  const int* chol_rank;     // [NL*nel]
  const double* gaunt;      // dense table, see gidx()
};

int ora_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// thread count of the following oracle calls (the reference's tests run
// with OMP_NUM_THREADS=1); n <= 0 restores every host core
void ora_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : omp_get_num_procs());
#else
  (void)n;
#endif
}

}  // extern "C"

namespace {

// coeff(a, ma, b, mb, c) = int Y_a^ma* Y_b^mb Y_c^(ma-mb)
inline double gcoeff(const ora_atom& A, int a, int ma, int b, int mb, int c) {
  const int g = A.gmax, w = 2 * g + 1;
  if (a < 0 || b < 0 || c < 0 || a > g || b > g || c > g) return 0.0;
  if (std::abs(ma) > a || std::abs(mb) > b || std::abs(ma - mb) > c) return 0.0;
  const size_t idx = ((((size_t)a * w + (ma + g)) * (g + 1) + b) * w + (mb + g)) * (g + 1) + c;
  return A.gaunt[idx];
}

// Nrad x Nrad column-major block helpers
inline const double* blk(const double* M, int nbf, int nrad, int ia, int ja) {
  return M + (size_t)ja * nrad * nbf + (size_t)ia * nrad;
}

// assemble_J_FE_one_multipole_cached_chol (CoulombExchangeFE.h:432-482)
void assemble_J(const ora_atom& A, int L, const std::vector<double>& P,
                std::vector<double>& J) {
  const int nrad = A.nrad, nel = A.nel;
  std::fill(J.begin(), J.end(), 0.0);
  std::vector<double> Psub, scal;
  for (int je = 0; je < nel; ++je) {
    const int jf = A.first[je], nj = A.ni[je];
    Psub.assign((size_t)nj * nj, 0.0);
    for (int b = 0; b < nj; ++b)
      for (int a = 0; a < nj; ++a) Psub[a + b * nj] = P[(size_t)(jf + a) + (size_t)(jf + b) * nrad];
    const double* rsj = A.rs + A.rs_off[L * nel + je];
    double jsmall = 0.0, jbig = 0.0;
    for (int b = 0; b < nj; ++b)
      for (int a = 0; a < nj; ++a) jsmall += rsj[a + b * nj] * Psub[b + a * nj];
    if (je > 0) {
      const double* rbj = A.rb + A.rb_off[L * nel + je];
      for (int b = 0; b < nj; ++b)
        for (int a = 0; a < nj; ++a) jbig += rbj[a + b * nj] * Psub[b + a * nj];
    }
    for (int ie = 0; ie < je; ++ie) {
      const int f = A.first[ie], n = A.ni[ie];
      const double* rsi = A.rs + A.rs_off[L * nel + ie];
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) J[(size_t)(f + a) + (size_t)(f + b) * nrad] += jbig * rsi[a + b * n];
    }
    for (int ie = je + 1; ie < nel; ++ie) {
      const int f = A.first[ie], n = A.ni[ie];
      const double* rbi = A.rb + A.rb_off[L * nel + ie];
      for (int b = 0; b < n; ++b)
        for (int a = 0; a < n; ++a) J[(size_t)(f + a) + (size_t)(f + b) * nrad] += jsmall * rbi[a + b * n];
    }
    // factored in-element term: J = Lc (Lc^T vec P)
    const int r = A.chol_rank[L * nel + je];
    const double* Lc = A.chol + A.chol_off[L * nel + je];
    const int n2 = nj * nj;
    scal.assign(r, 0.0);
    for (int p = 0; p < r; ++p) {
      double s = 0.0;
      for (int q = 0; q < n2; ++q) s += Lc[q + (size_t)p * n2] * Psub[q];
      scal[p] = s;
    }
    for (int q = 0; q < n2; ++q) {
      double s = 0.0;
      for (int p = 0; p < r; ++p) s += Lc[q + (size_t)p * n2] * scal[p];
      const int a = q % nj, b = q / nj;
      J[(size_t)(jf + a) + (size_t)(jf + b) * nrad] += s;
    }
  }
}

// assemble_K_FE_one_multipole_cached_chol (CoulombExchangeFE.h:484-530);
// accumulates into Kb.
void assemble_K(const ora_atom& A, int L, const double* X, double* Kb) {
  const int nrad = A.nrad, nel = A.nel;
  std::vector<double> Psub, tmp, Ksub;
  for (int ie = 0; ie < nel; ++ie) {
    const int fi = A.first[ie], ni = A.ni[ie];
    for (int je = 0; je < nel; ++je) {
      const int fj = A.first[je], nj = A.ni[je];
      Psub.assign((size_t)ni * nj, 0.0);
      for (int b = 0; b < nj; ++b)
        for (int a = 0; a < ni; ++a) Psub[a + b * ni] = X[(size_t)(fi + a) + (size_t)(fj + b) * nrad];
      Ksub.assign((size_t)ni * nj, 0.0);
      if (ie == je) {
        const int r = A.chol_rank[L * nel + ie];
        const double* Lc = A.chol + A.chol_off[L * nel + ie];
        const int n2 = ni * ni;
        tmp.assign((size_t)ni * ni, 0.0);
        for (int p = 0; p < r; ++p) {
          const double* M = Lc + (size_t)p * n2;  // M(a,b) = M[a + b*ni]
          // tmp = Psub * M^T
          for (int c = 0; c < ni; ++c)
            for (int a = 0; a < ni; ++a) {
              double s = 0.0;
              for (int d = 0; d < ni; ++d) s += Psub[a + d * ni] * M[c + d * ni];
              tmp[a + c * ni] = s;
            }
          // Ksub += M * tmp
          for (int c = 0; c < ni; ++c)
            for (int a = 0; a < ni; ++a) {
              double s = 0.0;
              for (int b = 0; b < ni; ++b) s += M[a + b * ni] * tmp[b + c * ni];
              Ksub[a + c * ni] += s;
            }
        }
      } else {
        const double* iint = (ie > je) ? A.rb + A.rb_off[L * nel + ie] : A.rs + A.rs_off[L * nel + ie];
        const double* jint = (ie > je) ? A.rs + A.rs_off[L * nel + je] : A.rb + A.rb_off[L * nel + je];
        tmp.assign((size_t)ni * nj, 0.0);
        // tmp = Psub * jint^T   (ni x nj)
        for (int c = 0; c < nj; ++c)
          for (int a = 0; a < ni; ++a) {
            double s = 0.0;
            for (int d = 0; d < nj; ++d) s += Psub[a + d * ni] * jint[c + d * nj];
            tmp[a + c * ni] = s;
          }
        // Ksub = iint * tmp
        for (int c = 0; c < nj; ++c)
          for (int a = 0; a < ni; ++a) {
            double s = 0.0;
            for (int b = 0; b < ni; ++b) s += iint[a + b * ni] * tmp[b + c * ni];
            Ksub[a + c * ni] = s;
          }
      }
      for (int b = 0; b < nj; ++b)
        for (int a = 0; a < ni; ++a) Kb[(size_t)(fi + a) + (size_t)(fj + b) * nrad] += Ksub[a + b * ni];
    }
  }
}

}  // namespace

extern "C" {

// TwoDBasisT::coulomb (TwoDBasis.cpp:773-877). P, J: nbf x nbf column-major.
void ora_coulomb(const ora_atom* Ap, const double* P, double* J) {
  const ora_atom& A = *Ap;
  const int nrad = A.nrad, nang = A.nang, nbf = nrad * nang;
  int lmx = 0, mmx = -1 << 30, mmn = 1 << 30;
  for (int i = 0; i < nang; ++i) {
    lmx = std::max(lmx, A.lval[i]);
    mmx = std::max(mmx, A.mval[i]);
    mmn = std::min(mmn, A.mval[i]);
  }
  const int Mmax = mmx - mmn;
  const int NL = 2 * lmx + 1;
  const size_t n2 = (size_t)nrad * nrad;
  auto slot = [&](int L, int M) { return (size_t)L * (2 * Mmax + 1) + (M + Mmax); };
  std::vector<std::vector<double>> Paux(NL * (2 * Mmax + 1)), Jaux(NL * (2 * Mmax + 1));
  for (int L = 0; L < NL; ++L)
    for (int M = -std::min(L, Mmax); M <= std::min(L, Mmax); ++M) {
      Paux[slot(L, M)].assign(n2, 0.0);
      Jaux[slot(L, M)].assign(n2, 0.0);
    }
  // ket contraction
  for (int k = 0; k < nang; ++k)
    for (int l = 0; l < nang; ++l) {
      const int lk = A.lval[k], mk = A.mval[k], ll = A.lval[l], ml = A.mval[l];
      const int M = mk - ml;
      const int Lmin = std::max(std::abs(lk - ll), std::abs(M)), Lmax = lk + ll;
      const double* Pb = blk(P, nbf, nrad, k, l);
      for (int L = Lmin; L <= Lmax; ++L) {
        const double cpl = gcoeff(A, lk, mk, L, M, ll);
        std::vector<double>& Pa = Paux[slot(L, M)];
        for (int c = 0; c < nrad; ++c)
          for (int r = 0; r < nrad; ++r) Pa[r + (size_t)c * nrad] += cpl * Pb[r + (size_t)c * nbf];
      }
    }
  // per-(L,M) FE assembly
  std::vector<double> tmp(n2);
  for (int L = 0; L < NL; ++L) {
    const double Lfac = 4.0 * M_PI / (2 * L + 1);
    for (int M = -std::min(L, Mmax); M <= std::min(L, Mmax); ++M) {
      assemble_J(A, L, Paux[slot(L, M)], tmp);
      std::vector<double>& Ja = Jaux[slot(L, M)];
      for (size_t q = 0; q < n2; ++q) Ja[q] += Lfac * tmp[q];
    }
  }
  // bra scatter
  std::memset(J, 0, sizeof(double) * (size_t)nbf * nbf);
  for (int i = 0; i < nang; ++i)
    for (int j = 0; j < nang; ++j) {
      const int li = A.lval[i], mi = A.mval[i], lj = A.lval[j], mj = A.mval[j];
      const int M = mj - mi;
      const int Lmin = std::max(std::abs(lj - li), std::abs(M)), Lmax = lj + li;
      double* Jb = J + (size_t)j * nrad * nbf + (size_t)i * nrad;
      for (int L = Lmin; L <= Lmax; ++L) {
        const double cpl = gcoeff(A, lj, mj, L, M, li);
        if (cpl == 0.0) continue;
        const std::vector<double>& Ja = Jaux[slot(L, M)];
        for (int c = 0; c < nrad; ++c)
          for (int r = 0; r < nrad; ++r) Jb[r + (size_t)c * nbf] += cpl * Ja[r + (size_t)c * nrad];
      }
    }
}

// TwoDBasisT::exchange (TwoDBasis.cpp:879-999). Returns the signed K that is
// added to the Fock matrix.
void ora_exchange(const ora_atom* Ap, const double* P, double* K) {
  const ora_atom& A = *Ap;
  const int nrad = A.nrad, nang = A.nang, nbf = nrad * nang;
  int lmx = 0;
  for (int i = 0; i < nang; ++i) lmx = std::max(lmx, A.lval[i]);
  const int NL = 2 * lmx + 1;
  const size_t n2 = (size_t)nrad * nrad;
  const double bdens_thr = 10.0 * std::numeric_limits<double>::epsilon();
  std::memset(K, 0, sizeof(double) * (size_t)nbf * nbf);

#pragma omp parallel
  {
    std::vector<std::vector<double>> Rmat(NL);
    std::vector<double> Kb(n2);
#pragma omp for collapse(2) schedule(dynamic)
    for (int j = 0; j < nang; ++j)
      for (int k = 0; k < nang; ++k) {
        const int lj = A.lval[j], mj = A.mval[j], lk = A.lval[k], mk = A.mval[k];
        for (int L = 0; L < NL; ++L) Rmat[L].assign(n2, 0.0);
        std::vector<char> couple(NL, 0);
        for (int i = 0; i < nang; ++i) {
          const int li = A.lval[i], mi = A.mval[i];
          for (int l = 0; l < nang; ++l) {
            const int ll = A.lval[l], ml = A.mval[l];
            const int M = mj - mi, Mp = mk - ml;
            if (M != Mp) continue;
            const double* Pb = blk(P, nbf, nrad, i, l);
            double nrm = 0.0;
            for (int c = 0; c < nrad; ++c)
              for (int r = 0; r < nrad; ++r) nrm += Pb[r + (size_t)c * nbf] * Pb[r + (size_t)c * nbf];
            if (std::sqrt(nrm) < bdens_thr) continue;
            const int Lmin = std::max(std::max(std::abs(li - lj), std::abs(lk - ll)), std::abs(M));
            const int Lmax = std::min(li + lj, lk + ll);
            for (int L = Lmin; L <= Lmax; ++L) {
              const double cpl = gcoeff(A, lj, mj, L, M, li) * gcoeff(A, lk, mk, L, M, ll);
              if (cpl == 0.0) continue;
              const double f = 4.0 * M_PI / (2 * L + 1) * cpl;
              std::vector<double>& R = Rmat[L];
              for (int c = 0; c < nrad; ++c)
                for (int r = 0; r < nrad; ++r) R[r + (size_t)c * nrad] += f * Pb[r + (size_t)c * nbf];
              couple[L] = 1;
            }
          }
        }
        std::fill(Kb.begin(), Kb.end(), 0.0);
        for (int L = 0; L < NL; ++L)
          if (couple[L]) assemble_K(A, L, Rmat[L].data(), Kb.data());
        double* Ko = K + (size_t)k * nrad * nbf + (size_t)j * nrad;
        for (int c = 0; c < nrad; ++c)
          for (int r = 0; r < nrad; ++r) Ko[r + (size_t)c * nbf] -= Kb[r + (size_t)c * nrad];
      }
  }
}

}  // extern "C"

// Oracle (test infrastructure only): C++17/OpenMP restatement of HelFEM's
// diatomic exchange build. The GPU product is compared against it, and it is
// the timed CPU baseline of the diatomic path; nothing in the product links it.
//
// Restated from (paths inside the HelFEM project):
//   src/diatomic/basis.cpp:1817-2061   TwoDBasis::exchange: density blocks
//       bucketed by m_i - m_l and screened at 10*eps; OpenMP collapse(2)
//       over the output blocks (jang,kang); four recoupled radial matrices
//       R00, R02, R20, R22 per (L,|M|) with couplings
//         mod*mod, -mod*coeff, -coeff*mod, coeff*coeff  (times LMfac);
//       off-diagonal element pairs: K -= X0 (R00 Y0' + R02 Y2') + X2 (R20 Y0'
//       + R22 Y2'), X = P-type integrals of the inner element and Y = Q-type
//       of the outer one (swapped when the row element is outer);
//       in-element blocks: RI-K with the sign-carrying factor,
//         K -= sum_p sigma_p (M0' R00 M0' - M0' R02 M2' - M2' R20 M0' + M2' R22 M2').
// The reference keeps one Rmat set per coupled (L,|M|) alive per output
// block; this restatement builds them one (L,|M|) at a time (same arithmetic,
// bounded memory). Matrices are column-major; the index is iang*Nrad + irad
// over the dummy (boundary-expanded) basis.

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

struct ora_diatomic {
  int nrad, nang, nel, nn, nlm;
  int Lmax, mmax;             // coupling table bounds
  double Rhalf;
  const int* lval;            // [nang]
  const int* mval;            // [nang]
  const int* first;           // [nel]
  const int* ni;              // [nel]
  const int* lm_L;            // [nlm] (L, |M|) list
  const int* lm_M;
  const double* P0;           // [(ilm*nel+e)*nn*nn], ni x ni column-major, ld nn
  const double* P2;
  const double* Q0;
  const double* Q2;
  const double* cdB;          // factor blocks (2 ni^2 x r), column-major
  const int64_t* cdB_off;     // [nlm*nel]
  const double* cds;          // signs
  const int64_t* cds_off;     // [nlm*nel]
  const int* cd_rank;         // [nlm*nel]
  const double* coef;         // [((j*(Lmax+1) + L)*(4mmax+1) + M+2mmax)*nang + i]
  const double* modc;         // same layout
};

}  // extern "C"

namespace {

inline int lmindex(const ora_diatomic& D, int L, int Ma) {
  for (int i = 0; i < D.nlm; ++i)
    if (D.lm_L[i] == L && D.lm_M[i] == Ma) return i;
  return -1;
}

inline double tab(const ora_diatomic& D, const double* t, int j, int L, int M, int i) {
  if (L < 0 || L > D.Lmax || std::abs(M) > 2 * D.mmax) return 0.0;
  const size_t idx = (((size_t)j * (D.Lmax + 1) + L) * (4 * D.mmax + 1) + (M + 2 * D.mmax)) * D.nang + i;
  return t[idx];
}

double lmfac(const ora_diatomic& D, int L, int M) {
  const int Ma = std::abs(M);
  double fr = 1.0;
  for (int p = L + Ma; p > L - Ma; --p) fr *= p;
  return ((M & 1) ? -1.0 : 1.0) * 4.0 * M_PI * std::pow(D.Rhalf, 5) / fr;
}

// C(n x m) = A(n x k) * B(k x m)^T, ld given
inline void gemm_nt(int n, int m, int k, const double* A, int lda, const double* B, int ldb, double* C, int ldc,
                    double alpha, bool acc) {
  for (int c = 0; c < m; ++c)
    for (int r = 0; r < n; ++r) {
      double s = 0.0;
      for (int t = 0; t < k; ++t) s += A[r + (size_t)t * lda] * B[c + (size_t)t * ldb];
      C[r + (size_t)c * ldc] = (acc ? C[r + (size_t)c * ldc] : 0.0) + alpha * s;
    }
}
// C(n x m) += alpha A(n x k) * B(k x m)
inline void gemm_nn(int n, int m, int k, const double* A, int lda, const double* B, int ldb, double* C, int ldc,
                    double alpha) {
  for (int c = 0; c < m; ++c)
    for (int r = 0; r < n; ++r) {
      double s = 0.0;
      for (int t = 0; t < k; ++t) s += A[r + (size_t)t * lda] * B[t + (size_t)c * ldb];
      C[r + (size_t)c * ldc] += alpha * s;
    }
}

}  // namespace

extern "C" {

int ora_num_threads_d() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// density-block screen: act[i + l*nang] = ||P_il|| >= 10 eps
static void block_activity(const ora_diatomic& D, const double* P, std::vector<char>& act) {
  const int nrad = D.nrad, nang = D.nang;
  const size_t nd = (size_t)nang * nrad;
  act.assign((size_t)nang * nang, 0);
#pragma omp parallel for collapse(2) schedule(static)
  for (int l = 0; l < nang; ++l)
    for (int i = 0; i < nang; ++i) {
      double s = 0.0;
      for (int c = 0; c < nrad; ++c)
        for (int r = 0; r < nrad; ++r) {
          const double v = P[((size_t)l * nrad + c) * nd + (size_t)i * nrad + r];
          s += v * v;
        }
      act[(size_t)i + (size_t)l * nang] = !(std::sqrt(s) < 10 * DBL_EPSILON);
    }
}

// the output block (j,k) of K; R, T, T2, Ks are per-thread work arrays
static void exchange_block(const ora_diatomic& D, const double* P, const std::vector<char>& act, int j, int k,
                           std::vector<double>& R, std::vector<double>& T, std::vector<double>& T2,
                           std::vector<double>& Ks, double* K) {
  const int nrad = D.nrad, nang = D.nang, nel = D.nel, nn = D.nn;
  const size_t nd = (size_t)nang * nrad;
  const int lj = D.lval[j], mj = D.mval[j], lk = D.lval[k], mk = D.mval[k];
  for (int ilm = 0; ilm < D.nlm; ++ilm) {
    const int L = D.lm_L[ilm], Ma = D.lm_M[ilm];
    bool any = false;
    // recouple: every active (i,l) with mi - ml = mj - mk and |mj - mi| = Ma
    for (int i = 0; i < nang; ++i) {
      const int li = D.lval[i], mi = D.mval[i];
      const int M = mj - mi;
      if (std::abs(M) != Ma) continue;
      for (int l = 0; l < nang; ++l) {
        const int ll = D.lval[l], ml = D.mval[l];
        if (mi - ml != mj - mk) continue;
        if (!act[(size_t)i + (size_t)l * nang]) continue;
        const int Lmin = std::max(std::max(std::abs(li - lj), std::abs(lk - ll)) - 2, std::abs(M));
        const int Lmx = std::min(li + lj, lk + ll) + 2;
        if (L < Lmin || L > Lmx) continue;
        const double m1 = tab(D, D.modc, j, L, M, i), c1 = tab(D, D.coef, j, L, M, i);
        const double m2 = tab(D, D.modc, k, L, M, l), c2 = tab(D, D.coef, k, L, M, l);
        const double c00 = m1 * m2, c02 = -m1 * c2, c20 = -c1 * m2, c22 = c1 * c2;
        if (c00 == 0.0 && c02 == 0.0 && c20 == 0.0 && c22 == 0.0) continue;
        if (!any) {
          std::fill(R.begin(), R.end(), 0.0);
          any = true;
        }
        const double f = lmfac(D, L, M);
        const double cc[4] = {f * c00, f * c02, f * c20, f * c22};
        for (int c = 0; c < nrad; ++c)
          for (int r = 0; r < nrad; ++r) {
            const double v = P[((size_t)l * nrad + c) * nd + (size_t)i * nrad + r];
            for (int ch = 0; ch < 4; ++ch) R[(size_t)ch * nrad * nrad + r + (size_t)c * nrad] += cc[ch] * v;
          }
      }
    }
    if (!any) continue;
    const double* R00 = R.data();
    const double* R02 = R00 + (size_t)nrad * nrad;
    const double* R20 = R02 + (size_t)nrad * nrad;
    const double* R22 = R20 + (size_t)nrad * nrad;
    for (int ie = 0; ie < nel; ++ie)
      for (int je = 0; je < nel; ++je) {
        const int fi = D.first[ie], Ni = D.ni[ie], fj = D.first[je], Nj = D.ni[je];
        std::fill(Ks.begin(), Ks.end(), 0.0);
        const size_t ro = (size_t)fi + (size_t)fj * nrad;
        if (ie != je) {
          const size_t oi = ((size_t)ilm * nel + ie) * nn * nn, oj = ((size_t)ilm * nel + je) * nn * nn;
          const double* i0 = (ie > je) ? D.Q0 + oi : D.P0 + oi;
          const double* i2 = (ie > je) ? D.Q2 + oi : D.P2 + oi;
          const double* j0 = (ie > je) ? D.P0 + oj : D.Q0 + oj;
          const double* j2 = (ie > je) ? D.P2 + oj : D.Q2 + oj;
          // T = R00 j0' + R02 j2';  Ks -= i0 T
          gemm_nt(Ni, Nj, Nj, R00 + ro, nrad, j0, nn, T.data(), nn, 1.0, false);
          gemm_nt(Ni, Nj, Nj, R02 + ro, nrad, j2, nn, T.data(), nn, 1.0, true);
          gemm_nn(Ni, Nj, Ni, i0, nn, T.data(), nn, Ks.data(), nn, -1.0);
          gemm_nt(Ni, Nj, Nj, R20 + ro, nrad, j0, nn, T.data(), nn, 1.0, false);
          gemm_nt(Ni, Nj, Nj, R22 + ro, nrad, j2, nn, T.data(), nn, 1.0, true);
          gemm_nn(Ni, Nj, Ni, i2, nn, T.data(), nn, Ks.data(), nn, -1.0);
          for (int c = 0; c < Nj; ++c)
            for (int r = 0; r < Ni; ++r)
              K[((size_t)k * nrad + fj + c) * nd + (size_t)j * nrad + fi + r] += Ks[r + (size_t)c * nn];
        } else {
          const int64_t bo = D.cdB_off[(size_t)ilm * nel + ie];
          const int rk = D.cd_rank[(size_t)ilm * nel + ie];
          const double* B = D.cdB + bo;
          const double* sg = D.cds + D.cds_off[(size_t)ilm * nel + ie];
          const size_t n2 = (size_t)Ni * Ni;
          for (int p = 0; p < rk; ++p) {
            const double* M0 = B + (size_t)p * 2 * n2;  // (Ni x Ni), symmetric
            const double* M2 = M0 + n2;
            // contrib = M0'R00 M0' - M0'R02 M2' - M2'R20 M0' + M2'R22 M2'
            const double* Ms[2] = {M0, M2};
            const double* Rs[4] = {R00 + ro, R02 + ro, R20 + ro, R22 + ro};
            const double sgn[4] = {1.0, -1.0, -1.0, 1.0};
            for (int a = 0; a < 2; ++a)
              for (int b = 0; b < 2; ++b) {
                // T2 = R_ab Mb'   (Ni x Ni)
                for (int c = 0; c < Ni; ++c)
                  for (int r = 0; r < Ni; ++r) {
                    double s = 0.0;
                    for (int t = 0; t < Ni; ++t) s += Rs[2 * a + b][r + (size_t)t * nrad] * Ms[b][c + (size_t)t * Ni];
                    T2[r + (size_t)c * nn] = s;
                  }
                // Ks += sigma sgn Ma' T2
                const double w = sg[p] * sgn[2 * a + b];
                for (int c = 0; c < Ni; ++c)
                  for (int r = 0; r < Ni; ++r) {
                    double s = 0.0;
                    for (int t = 0; t < Ni; ++t) s += Ms[a][t + (size_t)r * Ni] * T2[t + (size_t)c * nn];
                    Ks[r + (size_t)c * nn] += w * s;
                  }
              }
          }
          for (int c = 0; c < Nj; ++c)
            for (int r = 0; r < Ni; ++r)
              K[((size_t)k * nrad + fj + c) * nd + (size_t)j * nrad + fi + r] -= Ks[r + (size_t)c * nn];
        }
      }
  }
}

// K over the dummy basis (ndummy = nang*nrad); P is the expanded density.
// jk == nullptr: every output block; else the n blocks jk[0..n) (j + k*nang),
// the rest of K left zero (a bounded sample for CPU timing).
void ora_dexchange_blocks(const ora_diatomic* Dp, const double* P, double* K, const int* jk, int n) {
  const ora_diatomic& D = *Dp;
  const int nrad = D.nrad, nang = D.nang, nn = D.nn;
  const size_t nd = (size_t)nang * nrad;
  std::memset(K, 0, sizeof(double) * nd * nd);
  std::vector<char> act;
  block_activity(D, P, act);
  const int nblk = jk ? n : nang * nang;
#pragma omp parallel
  {
    std::vector<double> R((size_t)4 * nrad * nrad);
    std::vector<double> T((size_t)nn * nn), T2((size_t)nn * nn), Ks((size_t)nn * nn);
#pragma omp for schedule(dynamic)
    for (int b = 0; b < nblk; ++b) {
      const int jkb = jk ? jk[b] : b;
      exchange_block(D, P, act, jkb % nang, jkb / nang, R, T, T2, Ks, K);
    }
  }
}

void ora_dexchange(const ora_diatomic* Dp, const double* P, double* K) {
  ora_dexchange_blocks(Dp, P, K, nullptr, 0);
}

}  // extern "C"

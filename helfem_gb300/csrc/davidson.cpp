// Reference-preconditioned Davidson for the lowest eigenpairs of an SCF block
// (declarations and the method in davidson.hpp).
#include "davidson.hpp"

#include <algorithm>
#include <cmath>
#include <numeric>

#include "cuda/scf_kernels.cuh"

namespace hfg {
namespace {

void cbl(cublasStatus_t s, const char* what) {
  if (s != CUBLAS_STATUS_SUCCESS)
    throw hfg_abi::CudaError(std::string(what) + ": cuBLAS status " + std::to_string((int)s));
}

void ensure(DBuf& b, size_t doubles) {
  if (b.n < sizeof(double) * doubles) b.alloc(sizeof(double) * doubles);
}

}  // namespace

void jacobi_eigh(int m, std::vector<double> A, std::vector<double>& w, std::vector<double>& V) {
  V.assign((size_t)m * m, 0.0);
  for (int i = 0; i < m; ++i) V[i + (size_t)i * m] = 1.0;
  auto at = [&](int r, int c) -> double& { return A[r + (size_t)c * m]; };
  double norm = 0.0;
  for (double x : A) norm += x * x;
  norm = std::sqrt(norm);
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0;
    for (int c = 0; c < m; ++c)
      for (int r = 0; r < c; ++r) off += at(r, c) * at(r, c);
    if (std::sqrt(off) <= 1e-15 * norm || off == 0.0) break;
    for (int p = 0; p < m - 1; ++p)
      for (int q = p + 1; q < m; ++q) {
        const double apq = at(p, q);
        if (apq == 0.0) continue;
        // rotation that annihilates A(p,q) (Golub & Van Loan, symmetric Schur)
        const double tau = (at(q, q) - at(p, p)) / (2.0 * apq);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
        const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
        for (int k = 0; k < m; ++k) {  // A <- A J (columns p, q)
          const double akp = at(k, p), akq = at(k, q);
          at(k, p) = c * akp - s * akq;
          at(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < m; ++k) {  // A <- J^T A (rows p, q)
          const double apk = at(p, k), aqk = at(q, k);
          at(p, k) = c * apk - s * aqk;
          at(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < m; ++k) {  // V <- V J
          const double vkp = V[k + (size_t)p * m], vkq = V[k + (size_t)q * m];
          V[k + (size_t)p * m] = c * vkp - s * vkq;
          V[k + (size_t)q * m] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> idx(m);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return at(a, a) < at(b, b); });
  std::vector<double> Vs((size_t)m * m);
  w.resize(m);
  for (int j = 0; j < m; ++j) {
    w[j] = at(idx[j], idx[j]);
    std::copy(V.begin() + (size_t)idx[j] * m, V.begin() + (size_t)(idx[j] + 1) * m, Vs.begin() + (size_t)j * m);
  }
  V.swap(Vs);
}

namespace {

// Orthogonalise the u columns of T (device, n x u) against Q[:, :m] (two
// classical Gram-Schmidt passes) and append an orthonormal basis of what is
// left to Q (canonical orthonormalisation: directions with a Gram eigenvalue
// below 1e-14 of the largest are dropped). Returns the new column count.
int append_orthonormal(cublasHandle_t bl, cudaStream_t st, int n, double* Q, int m, double* T, int u,
                       DavidsonWork& w) {
  const double one = 1.0, zero = 0.0, mone = -1.0;
  double* C = w.sm2.as<double>();
  for (int pass = 0; pass < 2 && m > 0; ++pass) {
    cbl(cublasDgemm(bl, CUBLAS_OP_T, CUBLAS_OP_N, m, u, n, &one, Q, n, T, n, &zero, C, m), "Q^T T");
    cbl(cublasDgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, n, u, m, &mone, Q, n, C, m, &one, T, n), "T -= Q C");
  }
  cbl(cublasDgemm(bl, CUBLAS_OP_T, CUBLAS_OP_N, u, u, n, &one, T, n, T, n, &zero, C, u), "T^T T");
  w.h1.resize((size_t)u * u);
  ck(cudaMemcpyAsync(w.h1.data(), C, sizeof(double) * u * u, cudaMemcpyDeviceToHost, st), "D2H gram");
  ck(cudaStreamSynchronize(st), "sync");
  for (int c = 0; c < u; ++c)
    for (int r = 0; r < c; ++r) {
      const double a = 0.5 * (w.h1[r + (size_t)c * u] + w.h1[c + (size_t)r * u]);
      w.h1[r + (size_t)c * u] = w.h1[c + (size_t)r * u] = a;
    }
  std::vector<double> om, W;
  jacobi_eigh(u, w.h1, om, W);
  const double wmax = om.empty() ? 0.0 : om.back();
  std::vector<double> M;
  int kept = 0;
  for (int j = u - 1; j >= 0; --j) {  // largest first
    if (!(om[j] > 1e-14 * wmax) || !(om[j] > 1e-280)) continue;
    const double f = 1.0 / std::sqrt(om[j]);
    for (int i = 0; i < u; ++i) M.push_back(W[i + (size_t)j * u] * f);
    ++kept;
  }
  if (kept == 0) return m;
  ck(cudaMemcpyAsync(C, M.data(), sizeof(double) * M.size(), cudaMemcpyHostToDevice, st), "H2D transform");
  double* Qn = Q + (size_t)m * n;
  cbl(cublasDgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, n, kept, u, &one, T, n, C, u, &zero, Qn, n), "T M");
  if (m > 0) {  // one more pass against the old columns
    double* C2 = w.sm.as<double>();
    cbl(cublasDgemm(bl, CUBLAS_OP_T, CUBLAS_OP_N, m, kept, n, &one, Q, n, Qn, n, &zero, C2, m), "Q^T Qn");
    cbl(cublasDgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, n, kept, m, &mone, Q, n, C2, m, &one, Qn, n), "Qn -= Q C");
  }
  return m + kept;
}

}  // namespace

int davidson_lowest(cublasHandle_t bl, cudaStream_t st, const BlockOperator& apply, int n, int k, int kconv,
                    double* V, const double* Vr, const double* lam, std::vector<double>& theta, DavidsonWork& w,
                    int maxit, double tol, const Preconditioner* pc) {
  const double one = 1.0, zero = 0.0;
  k = std::min(k, n);
  kconv = std::min(kconv, k);
  const int mmax = std::min(n, 4 * k);
  ensure(w.Q, (size_t)n * mmax);
  ensure(w.AQ, (size_t)n * mmax);
  for (DBuf* b : {&w.X, &w.AX, &w.R, &w.T, &w.Zr, &w.Zx, &w.Zt}) ensure(*b, (size_t)n * k);
  ensure(w.sm, (size_t)mmax * mmax);
  ensure(w.sm2, (size_t)mmax * std::max(mmax, k));
  ensure(w.th, (size_t)2 * k);
  ensure(w.nrm, (size_t)k);
  double *Q = w.Q.as<double>(), *AQ = w.AQ.as<double>(), *X = w.X.as<double>(), *AX = w.AX.as<double>();
  double *R = w.R.as<double>(), *T = w.T.as<double>();
  ck(cudaMemcpyAsync(T, V, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, st), "copy guess");
  int m = append_orthonormal(bl, st, n, Q, 0, T, k, w);
  if (m < k) return -1;
  int mo = 0;
  std::vector<double> Hh, wv, Y, nrm(k), th(k);
  for (int it = 0; it < maxit; ++it) {
    apply(Q + (size_t)mo * n, m - mo, AQ + (size_t)mo * n);
    double* Hd = w.sm.as<double>();
    cbl(cublasDgemm(bl, CUBLAS_OP_T, CUBLAS_OP_N, m, m, n, &one, Q, n, AQ, n, &zero, Hd, m), "Q^T F Q");
    Hh.resize((size_t)m * m);
    ck(cudaMemcpyAsync(Hh.data(), Hd, sizeof(double) * m * m, cudaMemcpyDeviceToHost, st), "D2H H");
    ck(cudaStreamSynchronize(st), "sync");
    for (int c = 0; c < m; ++c)
      for (int r = 0; r < c; ++r) {
        const double a = 0.5 * (Hh[r + (size_t)c * m] + Hh[c + (size_t)r * m]);
        Hh[r + (size_t)c * m] = Hh[c + (size_t)r * m] = a;
      }
    jacobi_eigh(m, Hh, wv, Y);
    std::copy(wv.begin(), wv.begin() + k, th.begin());
    double* Yd = w.sm2.as<double>();
    ck(cudaMemcpyAsync(Yd, Y.data(), sizeof(double) * m * k, cudaMemcpyHostToDevice, st), "H2D Y");
    ck(cudaMemcpyAsync(w.th.p, th.data(), sizeof(double) * k, cudaMemcpyHostToDevice, st), "H2D theta");
    cbl(cublasDgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, n, k, m, &one, Q, n, Yd, m, &zero, X, n), "Q Y");
    cbl(cublasDgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, n, k, m, &one, AQ, n, Yd, m, &zero, AX, n), "AQ Y");
    k_dav_residual(AX, X, w.th.as<double>(), n, k, R, w.nrm.as<double>(), st);
    ck(cudaMemcpyAsync(nrm.data(), w.nrm.p, sizeof(double) * k, cudaMemcpyDeviceToHost, st), "D2H norms");
    ck(cudaStreamSynchronize(st), "sync");
    std::vector<int> U;
    bool ok = true;
    for (int j = 0; j < k; ++j) {
      const bool cj = nrm[j] <= tol;
      if (!cj) U.push_back(j);
      if (j < kconv && !cj) ok = false;
    }
    if (ok) {
      ck(cudaMemcpyAsync(V, X, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, st), "copy vectors");
      theta = th;
      return it + 1;
    }
    if (it + 1 == maxit) break;
    const int u = (int)U.size();
    if (m + u > mmax) {  // restart from the Ritz vectors
      ck(cudaMemcpyAsync(Q, X, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, st), "restart Q");
      ck(cudaMemcpyAsync(AQ, AX, sizeof(double) * n * k, cudaMemcpyDeviceToDevice, st), "restart AQ");
      m = k;
    }
    // gather the unconverged residuals and Ritz vectors
    double *Rg = w.Zt.as<double>(), *Xg = w.T.as<double>();
    std::vector<double> thU(u);
    for (int i = 0; i < u; ++i) {
      ck(cudaMemcpyAsync(Rg + (size_t)i * n, R + (size_t)U[i] * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, st),
         "gather R");
      ck(cudaMemcpyAsync(Xg + (size_t)i * n, X + (size_t)U[i] * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, st),
         "gather X");
      thU[i] = th[U[i]];
    }
    double* thd = w.th.as<double>() + k;
    ck(cudaMemcpyAsync(thd, thU.data(), sizeof(double) * u, cudaMemcpyHostToDevice, st), "H2D theta U");
    if (pc) {
      (*pc)(Rg, Xg, thd, u, T);
    } else {
      // corrections in the reference eigenbasis, then back: T = Vr Zt
      cbl(cublasDgemm(bl, CUBLAS_OP_T, CUBLAS_OP_N, n, u, n, &one, Vr, n, Rg, n, &zero, w.Zr.as<double>(), n),
          "Vr^T R");
      cbl(cublasDgemm(bl, CUBLAS_OP_T, CUBLAS_OP_N, n, u, n, &one, Vr, n, Xg, n, &zero, w.Zx.as<double>(), n),
          "Vr^T X");
      const double floor_ = 1e-8 * std::max(1.0, std::fabs(thU.empty() ? 0.0 : thU[0]));
      k_dav_olsen(w.Zr.as<double>(), w.Zx.as<double>(), lam, thd, n, u, floor_, Rg, st);
      cbl(cublasDgemm(bl, CUBLAS_OP_N, CUBLAS_OP_N, n, u, n, &one, Vr, n, Rg, n, &zero, T, n), "Vr Zt");
    }
    mo = m;
    m = append_orthonormal(bl, st, n, Q, m, T, u, w);
    if (m == mo) break;  // no new directions
  }
  return -1;
}

}  // namespace hfg

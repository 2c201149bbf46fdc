// Fock diagonalisation step as a standalone entry point: per symmetry block,
// the orthonormal Fock block F'_k = X_k^T F(idx,idx) X_k, its eigenpairs and
// the AO coefficients C_k = X_k V (src/general/scf_driver_common.h:176-187,
// 432-445; src/general/scf_helpers.cpp:41-50 eig_gsym). In the atomic basis S
// is block diagonal with one radial block per angular function, so
// X_k = I (x) X_rad with X_rad = invh(S_rad) (utils.cpp:120-159, diagonal
// pre-normalisation); blocks of one size are diagonalised together in a
// batched cuSOLVER call.
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <cmath>
#include <map>

#include "cuda/scf_kernels.cuh"
#include "handle.hpp"

namespace {

void cbf(cublasStatus_t s, const char* what) {
  if (s != CUBLAS_STATUS_SUCCESS) throw hfg_abi::CudaError(std::string(what) + ": cuBLAS status " + std::to_string((int)s));
}
void csf(cusolverStatus_t s, const char* what) {
  if (s != CUSOLVER_STATUS_SUCCESS)
    throw hfg_abi::CudaError(std::string(what) + ": cuSOLVER status " + std::to_string((int)s));
}

// the radial overlap with unit diagonal, diag(dn) S diag(dn), dn = S_ii^-1/2
std::vector<double> normalised_overlap(const std::vector<double>& Srad, int nrad) {
  std::vector<double> S(Srad), dn(nrad);
  for (int i = 0; i < nrad; ++i) dn[i] = 1.0 / std::sqrt(S[i + (size_t)i * nrad]);
  for (int c = 0; c < nrad; ++c)
    for (int r = 0; r < nrad; ++r) S[r + (size_t)c * nrad] *= dn[r] * dn[c];
  return S;
}

}  // namespace

extern "C" hfg_status hfg_fock_diag(hfg_atom* a, const double* F, int symmetry, double* C, double* eps, void* stream) {
  return guard([&] {
    need(a && F && C && eps, "hfg_fock_diag: null argument");
    need(symmetry == 1 || symmetry == 2, "hfg_fock_diag: symmetry must be 1 (per m) or 2 (per l,m)");
    a->check_device();
    const hfg::AtomHost& H = a->host;
    const int nbf = H.nbf, nrad = H.rad.nrad, nang = H.nang;
    cudaStream_t st = stream ? (cudaStream_t)stream : a->own_stream;
    hfg_abi::AllocStream alloc_on(st);
    struct Hs {
      cublasHandle_t bl = nullptr;
      cusolverDnHandle_t so = nullptr;
      cusolverDnParams_t pr = nullptr;
      ~Hs() {
        if (pr) cusolverDnDestroyParams(pr);
        if (so) cusolverDnDestroy(so);
        if (bl) cublasDestroy(bl);
      }
    } h;
    cbf(cublasCreate(&h.bl), "cublasCreate");
    cbf(cublasSetStream(h.bl, st), "cublasSetStream");
    csf(cusolverDnCreate(&h.so), "cusolverDnCreate");
    csf(cusolverDnSetStream(h.so, st), "cusolverDnSetStream");
    csf(cusolverDnCreateParams(&h.pr), "cusolverDnCreateParams");
    const double one = 1.0, zero = 0.0;
    const size_t nr2 = (size_t)nrad * nrad;

    // ---- X_rad = diag(dn) U diag(lam^-1/2) U^T diag(dn) from the eigenpairs
    // of the normalised radial overlap, built once per handle ----
    if (!a->d_xrad.p) {
      std::vector<double> S = normalised_overlap(H.Srad, nrad), dn(nrad);
      for (int i = 0; i < nrad; ++i) dn[i] = 1.0 / std::sqrt(H.Srad[i + (size_t)i * nrad]);
      DBuf dS, dw, work, info;
      double* Sd = dS.upload(S);
      dw.alloc(sizeof(double) * nrad);
      int lw = 0;
      csf(cusolverDnDsyevd_bufferSize(h.so, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, nrad, Sd, nrad,
                                      dw.as<double>(), &lw),
          "syevd buffer size");
      work.alloc(sizeof(double) * (size_t)std::max(lw, 1));
      info.alloc(sizeof(int));
      csf(cusolverDnDsyevd(h.so, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, nrad, Sd, nrad, dw.as<double>(),
                           work.as<double>(), lw, info.as<int>()),
          "syevd");
      std::vector<double> U(nr2), lam(nrad);
      ck(cudaMemcpyAsync(U.data(), Sd, sizeof(double) * nr2, cudaMemcpyDeviceToHost, st), "D2H");
      ck(cudaMemcpyAsync(lam.data(), dw.p, sizeof(double) * nrad, cudaMemcpyDeviceToHost, st), "D2H");
      ck(cudaStreamSynchronize(st), "sync");
      need(lam[0] > 0, "hfg_fock_diag: overlap matrix is not positive definite");
      std::vector<double> X(nr2, 0.0), Ul(nr2);
      for (int k = 0; k < nrad; ++k) {
        const double f = 1.0 / std::sqrt(lam[k]);
        for (int r = 0; r < nrad; ++r) Ul[r + (size_t)k * nrad] = U[r + (size_t)k * nrad] * f;
      }
      for (int c = 0; c < nrad; ++c)
        for (int k = 0; k < nrad; ++k) {
          const double u = U[c + (size_t)k * nrad];
          for (int r = 0; r < nrad; ++r) X[r + (size_t)c * nrad] += Ul[r + (size_t)k * nrad] * u;
        }
      for (int c = 0; c < nrad; ++c)
        for (int r = 0; r < nrad; ++r) X[r + (size_t)c * nrad] *= dn[r];
      hfg_abi::AllocStream own(a->own_stream);
      a->d_xrad.upload(X);
      ck(cudaStreamSynchronize(a->own_stream), "sync");
    }
    const double* X = a->d_xrad.as<double>();

    // ---- blocks: unique m ascending (symmetry 1) or one per angular function ----
    std::vector<std::vector<int>> blocks;
    if (symmetry == 1) {
      std::map<int, std::vector<int>> bym;
      for (int i = 0; i < nang; ++i) bym[H.mval[i]].push_back(i);
      for (auto& kv : bym) blocks.push_back(kv.second);
    } else {
      for (int i = 0; i < nang; ++i) blocks.push_back({i});
    }
    const int nblk = (int)blocks.size();
    std::vector<int> nk(nblk), coff(nblk);
    std::map<int, std::vector<int>> by_size;
    int c0 = 0;
    for (int k = 0; k < nblk; ++k) {
      nk[k] = (int)blocks[k].size() * nrad;
      coff[k] = c0;
      c0 += nk[k];
      by_size[nk[k]].push_back(k);
    }
    ck(cudaMemsetAsync(C, 0, sizeof(double) * (size_t)nbf * nbf, st), "memset");
    DBuf dang, dFk, dT1, dBatch, dW, dWork, dInfo, dCk;
    std::vector<char> hwork;
    for (auto& grp : by_size) {
      const int n = grp.first, nb = (int)grp.second.size();
      const size_t n2 = (size_t)n * n;
      dBatch.alloc(sizeof(double) * n2 * nb);
      dW.alloc(sizeof(double) * (size_t)n * nb);
      dInfo.alloc(sizeof(int) * nb);
      dFk.alloc(sizeof(double) * n2);
      dT1.alloc(sizeof(double) * n2);
      for (int q = 0; q < nb; ++q) {
        const int k = grp.second[q], p = (int)blocks[k].size();
        dang.upload(blocks[k]);
        hfg::k_gather_block(F, nbf, nrad, dang.as<int>(), n, dFk.as<double>(), st);
        // F' = (I x X)^T F_k (I x X): two strided-batched radial GEMMs
        cbf(cublasDgemmStridedBatched(h.bl, CUBLAS_OP_N, CUBLAS_OP_N, n, nrad, nrad, &one, dFk.as<double>(), n,
                                      (long long)nrad * n, X, nrad, 0, &zero, dT1.as<double>(), n,
                                      (long long)nrad * n, p),
            "F X");
        cbf(cublasDgemmStridedBatched(h.bl, CUBLAS_OP_T, CUBLAS_OP_N, nrad, n, nrad, &one, X, nrad, 0,
                                      dT1.as<double>(), n, nrad, &zero, dBatch.as<double>() + n2 * q, n, nrad, p),
            "X^T F X");
        ck(cudaStreamSynchronize(st), "sync");  // dang is reused for the next block
      }
      size_t wd = 0, wh = 0;
      csf(cusolverDnXsyevBatched_bufferSize(h.so, h.pr, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                                            CUDA_R_64F, dBatch.p, n, CUDA_R_64F, dW.p, CUDA_R_64F, &wd, &wh, nb),
          "syevBatched buffer size");
      dWork.alloc(std::max<size_t>(wd, 8));
      hwork.resize(std::max<size_t>(wh, 8));
      csf(cusolverDnXsyevBatched(h.so, h.pr, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_R_64F,
                                 dBatch.p, n, CUDA_R_64F, dW.p, CUDA_R_64F, dWork.p, wd, hwork.data(), wh,
                                 dInfo.as<int>(), nb),
          "syevBatched");
      std::vector<int> hinfo(nb);
      ck(cudaMemcpyAsync(hinfo.data(), dInfo.p, sizeof(int) * nb, cudaMemcpyDeviceToHost, st), "D2H");
      ck(cudaStreamSynchronize(st), "sync");
      for (int q = 0; q < nb; ++q)
        if (hinfo[q] != 0) throw std::runtime_error("hfg_fock_diag: eigensolver did not converge");
      dCk.alloc(sizeof(double) * n2);
      for (int q = 0; q < nb; ++q) {
        const int k = grp.second[q], p = (int)blocks[k].size();
        ck(cudaMemcpyAsync(eps + coff[k], dW.as<double>() + (size_t)n * q, sizeof(double) * n,
                           cudaMemcpyDeviceToDevice, st),
           "eps");
        // C_k = (I x X) V: rows of angular function a, columns of the block
        cbf(cublasDgemmStridedBatched(h.bl, CUBLAS_OP_N, CUBLAS_OP_N, nrad, n, nrad, &one, X, nrad, 0,
                                      dBatch.as<double>() + n2 * q, n, nrad, &zero, dCk.as<double>(), n, nrad, p),
            "X V");
        for (int ai = 0; ai < p; ++ai) {
          const int ang = blocks[k][ai];
          ck(cudaMemcpy2DAsync(C + (size_t)coff[k] * nbf + (size_t)ang * nrad, sizeof(double) * nbf,
                               dCk.as<double>() + (size_t)ai * nrad, sizeof(double) * n, sizeof(double) * nrad, n,
                               cudaMemcpyDeviceToDevice, st),
             "scatter C");
        }
        ck(cudaStreamSynchronize(st), "sync");
      }
    }
    a->mark_use(st);
  });
}

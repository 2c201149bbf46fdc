// Atomic SCF on the device: the Fock-builder loop of the reference's atomic
// driver (src/atomic/main.cpp:369-470) with its per-symmetry-block
// orthonormalisation and diagonalisation (src/general/scf_driver_common.h:
// 176-187, 406-445, 459-520; src/general/scf_helpers.cpp:41-50).
//
// The reference hands convergence to OpenOrbitalOptimizer (DIIS, ODA, CG);
// converged energies do not depend on the accelerator, so this driver uses
// Pulay DIIS on the orthonormal-basis Fock blocks with Aufbau occupations
// across blocks (or fixed per-block counts, the reference's --readocc).
//
// Everything large stays on the device: P, J, K, Vxc, F (nbf x nbf), the
// orthonormal blocks and the DIIS history. Two structural facts cut the FP64
// work of the diagonalisation step on GB300 (FP64 ~1/64 of FP32):
//  * S is block diagonal with one radial block per angular function, so the
//    block orthonormaliser is I (x) X_rad with X_rad = invh(S_rad); the
//    transform X^T F X is two strided-batched nrad-sized GEMMs per block
//    instead of two dense block GEMMs;
//  * only occupied orbitals are back-transformed and used for P.
#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <numeric>

#include "cuda/scf_kernels.cuh"
#include "davidson.hpp"
#include "handle.hpp"

namespace {

void cb(cublasStatus_t s, const char* what) {
  if (s != CUBLAS_STATUS_SUCCESS) throw hfg_abi::CudaError(std::string(what) + ": cuBLAS status " + std::to_string((int)s));
}
void cs(cusolverStatus_t s, const char* what) {
  if (s != CUSOLVER_STATUS_SUCCESS)
    throw hfg_abi::CudaError(std::string(what) + ": cuSOLVER status " + std::to_string((int)s));
}

struct Handles {
  cublasHandle_t bl = nullptr;
  cusolverDnHandle_t so = nullptr;
  ~Handles() {
    if (bl) cublasDestroy(bl);
    if (so) cusolverDnDestroy(so);
  }
};

struct Block {
  int key = 0;                // m (symmetry 1) or angular index (symmetry 2)
  std::vector<int> ang;       // angular functions in the block
  int nk = 0;                 // ang.size() * nrad
  DBuf d_ang;
  size_t off = 0;             // offset of the block in a flattened block vector
};

// symmetric eigensolve of an n x n device matrix in place (eigenvectors)
struct Eigh {
  DBuf work, info;
  int lwork = 0;
  void run(cusolverDnHandle_t h, double* A, int n, double* w) {
    int lw = 0;
    cs(cusolverDnDsyevd_bufferSize(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, A, n, w, &lw),
       "syevd buffer size");
    if (lw > lwork) {
      work.alloc(sizeof(double) * (size_t)lw);
      lwork = lw;
    }
    if (!info.p) info.alloc(sizeof(int));
    cs(cusolverDnDsyevd(h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, A, n, w, work.as<double>(), lwork,
                        info.as<int>()),
       "syevd");
  }
};

// Host wall-clock per SCF phase; every phase ends at a point where the host
// waits for the device anyway (a blocking dot product, the eigenvalue copy),
// so the split costs no extra synchronisation.
struct PhaseTimer {
  double ms[7] = {0, 0, 0, 0, 0, 0, 0};
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  void lap(int k) {
    const auto n = std::chrono::steady_clock::now();
    ms[k] += std::chrono::duration<double, std::milli>(n - t).count();
    t = n;
  }
};

}  // namespace

// The SCF proper; throws on failure. bl/so: handles already bound to the
// stream (the engine's workers keep one pair each).
void hfg_scf_impl(hfg_atom* a, const hfg_scf_desc* d, hfg_scf_result* res, double* orbital_energies,
                  cudaStream_t stream, cublasHandle_t bl_in, cusolverDnHandle_t so_in) {
  {
    need(a && d && res, "hfg_scf_run: null argument");
    a->check_device();
    const hfg::AtomHost& H = a->host;
    const int nbf = H.nbf, nrad = H.rad.nrad, nang = H.nang;
    const bool restricted = d->restricted != 0;
    const int nspin = restricted ? 1 : 2;
    need(d->nela >= 0 && d->nelb >= 0 && d->nela + d->nelb > 0, "hfg_scf_run: no electrons");
    need(d->symmetry == 1 || d->symmetry == 2, "hfg_scf_run: symmetry must be 1 (per m) or 2 (per l,m)");
    const bool have_xc = d->x_func != 0 || d->c_func != 0;
    need(hfg::xc_func_supported(d->x_func) && hfg::xc_func_supported(d->c_func), "hfg_scf_run: unsupported functional");
    const double kfrac = d->kfrac >= 0 ? d->kfrac : (have_xc ? 0.0 : 1.0);
    const int maxiter = d->maxiter > 0 ? d->maxiter : 200;
    const double etol = d->e_tol > 0 ? d->e_tol : 1e-10;
    const double dtol = d->diis_tol > 0 ? d->diis_tol : 1e-7;
    const char* venv = std::getenv("HFG_SCF_VERBOSE");
    const bool verbose = venv && venv[0] && venv[0] != '0';
    const double thr = d->dftthr > 0 ? d->dftthr : 1e-12;
    cudaStream_t st = stream ? (cudaStream_t)stream : a->own_stream;
    if (have_xc && !a->xc_ready) a->setup_xc(0, 0);
    hfg_abi::AllocStream alloc_on(st);  // every buffer below is stream-ordered on st

    struct {
      cublasHandle_t bl;
      cusolverDnHandle_t so;
    } hd{bl_in, so_in};

    // ---- symmetry blocks (TwoDBasis.cpp:218-232: unique m ascending) ----
    std::vector<Block> blocks;
    if (d->symmetry == 1) {
      std::map<int, std::vector<int>> bym;
      for (int i = 0; i < nang; ++i) bym[H.mval[i]].push_back(i);
      for (auto& kv : bym) {
        Block b;
        b.key = kv.first;
        b.ang = kv.second;
        blocks.push_back(std::move(b));
      }
    } else {
      for (int i = 0; i < nang; ++i) {
        Block b;
        b.key = i;
        b.ang = {i};
        blocks.push_back(std::move(b));
      }
    }
    const int nblk = (int)blocks.size();
    size_t Lblk = 0;
    int nkmax = 0;
    for (auto& b : blocks) {
      b.nk = (int)b.ang.size() * nrad;
      b.off = Lblk;
      Lblk += (size_t)b.nk * b.nk;
      nkmax = std::max(nkmax, b.nk);
      b.d_ang.upload(b.ang);
    }
    if (d->fixed_occ) need(d->n_fixed_blocks == nblk, "hfg_scf_run: fixed_occ needs one (alpha, beta) pair per block");
    if (d->l_occ) need(d->symmetry == 2 && d->n_l_occ >= 1, "hfg_scf_run: l_occ needs symmetry 2");

    // ---- radial orthonormaliser X = invh(S_rad) (utils.cpp:120-159) ----
    const size_t nr2 = (size_t)nrad * nrad, nb2 = (size_t)nbf * nbf;
    DBuf dX, dtmp, dw;
    {
      std::vector<double> S(H.Srad), dn(nrad);
      for (int i = 0; i < nrad; ++i) dn[i] = 1.0 / std::sqrt(S[i + (size_t)i * nrad]);
      for (int c = 0; c < nrad; ++c)
        for (int r = 0; r < nrad; ++r) S[r + (size_t)c * nrad] *= dn[r] * dn[c];
      DBuf dS;
      double* Sd = dS.upload(S);
      dw.alloc(sizeof(double) * nrad);
      Eigh eg;
      eg.run(hd.so, Sd, nrad, dw.as<double>());
      std::vector<double> lam(nrad);
      ck(cudaMemcpyAsync(lam.data(), dw.p, sizeof(double) * nrad, cudaMemcpyDeviceToHost, st), "D2H");
      ck(cudaStreamSynchronize(st), "sync");
      need(lam[0] > 0, "hfg_scf_run: overlap matrix is not positive definite");
      // X = diag(dn) U diag(lam^-1/2) U^T on the device (one DGEMM)
      const double one_ = 1.0, zero_ = 0.0;
      std::vector<double> f(nrad);
      for (int k = 0; k < nrad; ++k) f[k] = 1.0 / std::sqrt(lam[k]);
      DBuf df, ddn, dUl;
      df.upload(f);
      ddn.upload(dn);
      dUl.alloc(sizeof(double) * nr2);
      hfg::k_scale_cols(Sd, nrad, nrad, df.as<double>(), dUl.as<double>(), st);
      dX.alloc(sizeof(double) * nr2);
      cb(cublasDgemm(hd.bl, CUBLAS_OP_N, CUBLAS_OP_T, nrad, nrad, nrad, &one_, dUl.as<double>(), nrad, Sd, nrad,
                     &zero_, dX.as<double>(), nrad),
         "U L U^T");
      hfg::k_scale_rows(dX.as<double>(), nrad, nrad, ddn.as<double>(), st);
      ck(cudaStreamSynchronize(st), "sync");
    }

    // ---- one-electron matrices, expanded on the device from the radial
    // blocks (the dense nbf^2 matrices never exist on the host) ----
    DBuf dT, dV, dH, dP, dPs[2], dJ, dK[2], dXC[2], dF[2], dE;
    {
      DBuf dTr, dTl, dVr, dl;
      dTr.upload(H.Trad);
      dTl.upload(H.Tlrad);
      dVr.upload(H.Vrad);
      dl.upload(std::vector<int>(H.lval.begin(), H.lval.begin() + nang));
      dT.alloc(sizeof(double) * nb2);
      dV.alloc(sizeof(double) * nb2);
      ck(cudaMemsetAsync(dT.p, 0, sizeof(double) * nb2, st), "memset");
      ck(cudaMemsetAsync(dV.p, 0, sizeof(double) * nb2, st), "memset");
      hfg::k_expand_one_electron(dTr.as<double>(), dTl.as<double>(), dVr.as<double>(), dl.as<int>(), nang, nrad,
                                 (double)H.Z, dT.as<double>(), dV.as<double>(), st);
      ck(cudaStreamSynchronize(st), "sync");  // the radial blocks are freed at the end of this scope
    }
    double* T = dT.as<double>();
    double* V = dV.as<double>();
    dH.alloc(sizeof(double) * nb2);
    hfg::k_add4(dH.as<double>(), T, V, nullptr, nullptr, nb2, st);
    dP.alloc(sizeof(double) * nb2);
    dJ.alloc(sizeof(double) * nb2);
    dE.alloc(sizeof(double) * 2);
    for (int s = 0; s < 2; ++s) {
      dPs[s].alloc(sizeof(double) * nb2);
      dF[s].alloc(sizeof(double) * nb2);
      if (kfrac != 0.0) dK[s].alloc(sizeof(double) * nb2);
      if (have_xc) dXC[s].alloc(sizeof(double) * nb2);
    }

    // ---- per-iteration block buffers ----
    const size_t Ltot = Lblk * nspin;
    DBuf dFo, dEo, dFk, dT1, dVec, dW, dG, dCo, deps;
    dFo.alloc(sizeof(double) * Ltot);  // orthonormal Fock blocks (current)
    dEo.alloc(sizeof(double) * Ltot);  // DIIS errors (current)
    dFk.alloc(sizeof(double) * (size_t)nkmax * nkmax);
    dT1.alloc(sizeof(double) * (size_t)nkmax * nkmax);
    dVec.alloc(sizeof(double) * Ltot);  // eigenvectors, per spin and block
    dW.alloc(sizeof(double) * (size_t)nkmax * nkmax);
    dG.alloc(sizeof(double) * (size_t)nkmax * nkmax);
    dCo.alloc(sizeof(double) * (size_t)nkmax * nkmax);
    deps.alloc(sizeof(double) * (size_t)nbf * nspin);
    const int nhist = 8;
    DBuf dHF, dHE, dBrow, dOcc;  // DIIS history [nhist][Ltot]; new row of B; occupations
    dHF.alloc(sizeof(double) * Ltot * nhist);
    dHE.alloc(sizeof(double) * Ltot * nhist);
    dBrow.alloc(sizeof(double) * nhist);
    dOcc.alloc(sizeof(double) * (size_t)nbf * nspin);
    std::vector<double> Bm((size_t)nhist * nhist, 0.0);  // error overlaps, kept on the host
    Eigh eg;
    const double one = 1.0, zero = 0.0;
    // split-precision exchange needs a float2 copy of the density
    DBuf dP2;
    hfg::DevScratch scr_split = a->scr;
    if (d->split_exchange && kfrac != 0.0) {
      dP2.alloc(sizeof(float2) * nb2);
      scr_split.p2 = dP2.as<float2>();
    }

    // Blocks are kept in the non-orthonormal basis (F_k gathered from the AO
    // matrix); the orthonormal F'_k = (I x X)^T F_k (I x X) is formed only for
    // full eigensolves, and products with F'_k are taken as thin GEMMs.
    auto gather = [&](const double* M, const Block& b, double* out) {
      hfg::k_gather_block(M, nbf, nrad, b.d_ang.as<int>(), b.nk, out, st);
    };
    auto ortho_block = [&](const double* Fk, const Block& b, double* out) {
      const int p = (int)b.ang.size(), nk = b.nk;
      cb(cublasDgemmStridedBatched(hd.bl, CUBLAS_OP_N, CUBLAS_OP_N, nk, nrad, nrad, &one, Fk, nk,
                                   (long long)nrad * nk, dX.as<double>(), nrad, 0, &zero, dT1.as<double>(), nk,
                                   (long long)nrad * nk, p),
         "F X");
      cb(cublasDgemmStridedBatched(hd.bl, CUBLAS_OP_T, CUBLAS_OP_N, nrad, nk, nrad, &one, dX.as<double>(), nrad, 0,
                                   dT1.as<double>(), nk, nrad, &zero, out, nk, nrad, p),
         "X^T F X");
    };
    // out = (I x X) V or (I x X)^T V for an nk x cols block V
    auto x_cols = [&](const Block& b, const double* Vin, int cols, double* out, bool trans) {
      const int p = (int)b.ang.size(), nk = b.nk;
      cb(cublasDgemmStridedBatched(hd.bl, trans ? CUBLAS_OP_T : CUBLAS_OP_N, CUBLAS_OP_N, nrad, cols, nrad, &one,
                                   dX.as<double>(), nrad, 0, Vin, nk, nrad, &zero, out, nk, nrad, p),
         "X V");
    };

    // orbitals: eps (all blocks, per spin), occupations
    std::vector<double> eps((size_t)nbf * nspin);
    std::vector<std::vector<std::vector<double>>> occ(nspin, std::vector<std::vector<double>>(nblk));

    // Eigensolves, grouped by block size into cusolverDnXsyevBatched calls
    // (one call for every block of a size; ~3-7x faster than one syevd per
    // block on GB300). Spherical solves (per-(l,m) blocks with fractional
    // Aufbau) diagonalise one block per l and copy it to the other m.
    const bool spherical = d->symmetry == 2 && ((d->frac_aufbau && !d->fixed_occ) || d->l_occ);
    std::vector<int> rep(nblk);  // block whose eigenpairs block k uses
    for (int k = 0; k < nblk; ++k) {
      rep[k] = k;
      if (spherical)
        for (int q = 0; q < k; ++q)
          if (H.lval[blocks[q].ang[0]] == H.lval[blocks[k].ang[0]]) { rep[k] = q; break; }
    }
    std::vector<size_t> eoff(nblk, 0);
    for (int k = 1; k < nblk; ++k) eoff[k] = eoff[k - 1] + blocks[k - 1].nk;
    std::map<int, std::vector<int>> by_size;  // representative blocks by size
    for (int k = 0; k < nblk; ++k)
      if (rep[k] == k) by_size[blocks[k].nk].push_back(k);
    cusolverDnParams_t sparams = nullptr;
    cs(cusolverDnCreateParams(&sparams), "cusolverDnCreateParams");
    struct ParamsGuard {
      cusolverDnParams_t p;
      ~ParamsGuard() { if (p) cusolverDnDestroyParams(p); }
    } pguard{sparams};
    DBuf dBatch, dBatchW, dWork, dInfo;
    std::vector<char> hwork;
    size_t work_bytes = 0;

    // full eigensolves of the representative blocks selected by `full`
    // (all when empty); results copied to every block they represent
    auto diagonalise = [&](const double* Fo_all, int s, const std::vector<char>& full = {}) {
      double* Vs = dVec.as<double>() + Lblk * s;
      double* Ws = deps.as<double>() + (size_t)nbf * s;
      for (auto& grp0 : by_size) {
        std::pair<int, std::vector<int>> grp{grp0.first, {}};
        for (int k : grp0.second)
          if (full.empty() || full[k]) grp.second.push_back(k);
        if (grp.second.empty()) continue;
        const int n = grp.first, nb = (int)grp.second.size();
        const size_t n2 = (size_t)n * n;
        if (dBatch.n < sizeof(double) * n2 * nb) dBatch.alloc(sizeof(double) * n2 * nb);
        if (dBatchW.n < sizeof(double) * (size_t)n * nb) dBatchW.alloc(sizeof(double) * (size_t)n * nb);
        if (dInfo.n < sizeof(int) * nb) dInfo.alloc(sizeof(int) * nb);
        for (int q = 0; q < nb; ++q)
          ck(cudaMemcpyAsync(dBatch.as<double>() + n2 * q, Fo_all + Lblk * s + blocks[grp.second[q]].off,
                             sizeof(double) * n2, cudaMemcpyDeviceToDevice, st),
             "gather blocks");
        size_t wd = 0, wh = 0;
        cs(cusolverDnXsyevBatched_bufferSize(hd.so, sparams, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n,
                                             CUDA_R_64F, dBatch.p, n, CUDA_R_64F, dBatchW.p, CUDA_R_64F, &wd, &wh, nb),
           "syevBatched buffer size");
        if (wd > work_bytes) {
          dWork.alloc(wd);
          work_bytes = wd;
        }
        if (hwork.size() < wh) hwork.resize(wh);
        cs(cusolverDnXsyevBatched(hd.so, sparams, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, CUDA_R_64F,
                                  dBatch.p, n, CUDA_R_64F, dBatchW.p, CUDA_R_64F, dWork.p, wd,
                                  hwork.empty() ? nullptr : hwork.data(), wh, dInfo.as<int>(), nb),
           "syevBatched");
        for (int k = 0; k < nblk; ++k) {
          const int r = rep[k];
          const auto it = std::find(grp.second.begin(), grp.second.end(), r);
          if (it == grp.second.end()) continue;
          const int q = (int)(it - grp.second.begin());
          ck(cudaMemcpyAsync(Vs + blocks[k].off, dBatch.as<double>() + n2 * q, sizeof(double) * n2,
                             cudaMemcpyDeviceToDevice, st),
             "scatter vectors");
          ck(cudaMemcpyAsync(Ws + eoff[k], dBatchW.as<double>() + (size_t)n * q, sizeof(double) * n,
                             cudaMemcpyDeviceToDevice, st),
             "scatter values");
        }
      }
    };

    auto occupy = [&]() {
      ck(cudaMemcpyAsync(eps.data(), deps.p, sizeof(double) * eps.size(), cudaMemcpyDeviceToHost, st), "D2H eps");
      ck(cudaStreamSynchronize(st), "sync");
      const double maxocc = restricted ? 2.0 : 1.0;
      for (int s = 0; s < nspin; ++s) {
        size_t eo = 0;
        std::vector<std::pair<double, std::pair<int, int>>> all;
        for (int k = 0; k < nblk; ++k) {
          occ[s][k].assign(blocks[k].nk, 0.0);
          for (int i = 0; i < blocks[k].nk; ++i) all.push_back({eps[(size_t)nbf * s + eo + i], {k, i}});
          eo += blocks[k].nk;
        }
        if (d->l_occ) {
          for (int k = 0; k < nblk; ++k) {
            const int l = H.lval[blocks[k].ang[0]];
            double left = 0.0;
            if (l < d->n_l_occ)
              left = (restricted ? d->l_occ[2 * l] + d->l_occ[2 * l + 1] : d->l_occ[2 * l + s]) / (2.0 * l + 1.0);
            for (int i = 0; i < blocks[k].nk && left > 1e-14; ++i) {
              occ[s][k][i] = std::min(maxocc, left);
              left -= occ[s][k][i];
            }
          }
        } else if (d->fixed_occ) {
          for (int k = 0; k < nblk; ++k) {
            double left = restricted ? d->fixed_occ[2 * k] + d->fixed_occ[2 * k + 1] : d->fixed_occ[2 * k + s];
            for (int i = 0; i < blocks[k].nk && left > 0; ++i) {
              occ[s][k][i] = std::min(maxocc, left);
              left -= occ[s][k][i];
            }
          }
        } else {
          std::stable_sort(all.begin(), all.end(), [](auto& x, auto& y) { return x.first < y.first; });
          double left = restricted ? (double)(d->nela + d->nelb) : (s == 0 ? d->nela : d->nelb);
          for (size_t i = 0; i < all.size() && left > 0;) {
            size_t j = i + 1;
            if (d->frac_aufbau)  // degenerate group at this level
              while (j < all.size() && all[j].first - all[i].first < 1e-5 * (1.0 + std::fabs(all[i].first))) ++j;
            const double cap = maxocc * (double)(j - i);
            const double o = (left >= cap) ? maxocc : left / (double)(j - i);
            for (size_t q = i; q < j; ++q) occ[s][all[q].second.first][all[q].second.second] = o;
            left -= o * (double)(j - i);
            i = j;
          }
        }
      }
      // one upload per iteration: [spin][block][orbital]
      std::vector<double> flat((size_t)nbf * nspin, 0.0);
      for (int s = 0; s < nspin; ++s)
        for (int k = 0; k < nblk; ++k)
          std::copy(occ[s][k].begin(), occ[s][k].end(), flat.begin() + (size_t)nbf * s + eoff[k]);
      ck(cudaMemcpyAsync(dOcc.p, flat.data(), sizeof(double) * flat.size(), cudaMemcpyHostToDevice, st), "occ");
    };

    // P_s = sum_k C_occ diag(occ) C_occ^T, C = (I (x) X) V
    auto build_density = [&]() {
      for (int s = 0; s < nspin; ++s) {
        double* P = dPs[s].as<double>();
        ck(cudaMemsetAsync(P, 0, sizeof(double) * nb2, st), "memset");
        for (int k = 0; k < nblk; ++k) {
          const Block& b = blocks[k];
          int nocc = 0;
          while (nocc < b.nk && occ[s][k][nocc] > 0) ++nocc;
          if (nocc == 0) continue;
          const double* Vk = dVec.as<double>() + Lblk * s + b.off;
          const int p = (int)b.ang.size(), nk = b.nk;
          // C_occ = (I x X) V_occ : nk x nocc
          cb(cublasDgemmStridedBatched(hd.bl, CUBLAS_OP_N, CUBLAS_OP_N, nrad, nocc, nrad, &one, dX.as<double>(), nrad,
                                       0, Vk, nk, nrad, &zero, dCo.as<double>(), nk, nrad, p),
             "X V");
          hfg::k_scale_cols(dCo.as<double>(), nk, nocc, dOcc.as<double>() + (size_t)nbf * s + eoff[k], dW.as<double>(),
                            st);
          cb(cublasDgemm(hd.bl, CUBLAS_OP_N, CUBLAS_OP_T, nk, nk, nocc, &one, dW.as<double>(), nk, dCo.as<double>(),
                         nk, &zero, dG.as<double>(), nk),
             "C occ C^T");
          hfg::k_scatter_add_block(P, nbf, nrad, b.d_ang.as<int>(), nk, dG.as<double>(), 1.0, st);
        }
      }
      if (restricted) {
        // P is the total density; the spin density for K is P/2
        ck(cudaMemcpyAsync(dP.p, dPs[0].p, sizeof(double) * nb2, cudaMemcpyDeviceToDevice, st), "copy");
        const double half = 0.5;
        cb(cublasDscal(hd.bl, (int)std::min<size_t>(nb2, 0x7fffffff), &half, dPs[0].as<double>(), 1), "scal");
        if (nb2 > 0x7fffffff) throw std::invalid_argument("basis too large for this driver");
      } else {
        hfg::k_add4(dP.as<double>(), dPs[0].as<double>(), dPs[1].as<double>(), nullptr, nullptr, nb2, st);
      }
    };

    // Eigensolver policy: full batched solves for the first three
    // diagonalisations (and whenever a block has no reference yet), then
    // Davidson refinement of the previous orbitals of each representative
    // block, preconditioned by that block's last full eigendecomposition, to
    // residuals |F'x - theta x| <= dav_tol = 1e-2 x the current orbital
    // gradient, clamped to [1e-8, 1e-4] Eh (the gradient target is 1e-7;
    // early iterations need no more). A block whose refinement does not
    // converge in 12 iterations is solved in full (and becomes the new
    // reference); one that needed 6 or more is solved in full next time.
    // HFG_SCF_EIGENSOLVER=full keeps full solves throughout; HFG_SCF_NFULL
    // sets the number of full solves before the refinement starts.
    const char* eenv = std::getenv("HFG_SCF_EIGENSOLVER");
    const bool use_davidson = !(eenv && std::strcmp(eenv, "full") == 0);
    // Preconditioner of the refinement: the eigenbasis of the block's last
    // full solve. HFG_SCF_PRECOND=banded selects, for runs whose blocks all
    // have one angular function (the spherical, per-(l,m) solves), the banded
    // shift-invert form (S X)^T (band(F_k) - theta S)^-1 (S X) from the
    // current Fock block, with refinement from the second iteration on
    // (measured slower on the batch atoms: the same iteration counts, more
    // fall-backs, and a serial banded solve per Ritz value).
    const char* penv = std::getenv("HFG_SCF_PRECOND");
    const bool band_ok = penv && std::strcmp(penv, "banded") == 0 && H.rad.nn - 1 <= 16;
    bool all_single = true;
    for (const Block& b : blocks) all_single = all_single && b.ang.size() == 1;
    const bool banded = band_ok && all_single;
    const char* nenv = std::getenv("HFG_SCF_NFULL");  // full solves before refinement (default 3; 1 when banded)
    const int n_full_first = (nenv && std::atoi(nenv) > 0) ? std::atoi(nenv) : (banded ? 1 : 3);
    DBuf dSrad, dSX, dZr, dZx, dYt, dBandWork;
    if (banded) {
      dSrad.upload(H.Srad);
      dSX.alloc(sizeof(double) * nr2);
      cb(cublasDgemm(hd.bl, CUBLAS_OP_N, CUBLAS_OP_N, nrad, nrad, nrad, &one, dSrad.as<double>(), nrad,
                     dX.as<double>(), nrad, &zero, dSX.as<double>(), nrad),
         "S X");
    }
    DBuf dVref, dLam, dFx;
    dVref.alloc(sizeof(double) * Ltot);
    dLam.alloc(sizeof(double) * (size_t)nbf * nspin);
    if (orbital_energies) dFx.alloc(sizeof(double) * Ltot);
    std::vector<char> have_ref((size_t)nspin * nblk, 0), want_full((size_t)nspin * nblk, 0);
    hfg::DavidsonWork dav;
    DBuf dFp, dOpA, dOpB, dOpC;  // orthonormal blocks of the full solves; operator temporaries
    dFp.alloc(sizeof(double) * Ltot);
    double shift = 0.0;  // level shift of the virtual space (set by the stabilisation below)
    auto nocc_of = [&](int s, int k) {
      int n = 0;
      while (n < blocks[k].nk && occ[s][k][n] > 0) ++n;
      return n;
    };
    // F'_k (+ the level shift b (1 - V_occ V_occ^T) with the previous
    // occupied orbitals) into dFp, for a full eigensolve
    auto form_ortho = [&](const double* Fo_all, int s, int k) {
      const Block& b = blocks[k];
      double* Fp = dFp.as<double>() + Lblk * s + b.off;
      ortho_block(Fo_all + Lblk * s + b.off, b, Fp);
      if (shift > 0.0) {
        hfg::k_add_diag(Fp, b.nk, shift, st);
        const int nocc = nocc_of(s, k);
        if (nocc > 0) {
          const double* Vk = dVec.as<double>() + Lblk * s + b.off;
          const double mshift = -shift;
          cb(cublasDgemm(hd.bl, CUBLAS_OP_N, CUBLAS_OP_T, b.nk, b.nk, nocc, &mshift, Vk, b.nk, Vk, b.nk, &one, Fp,
                         b.nk),
             "level shift");
        }
      }
    };
    int ndiag = 0;
    double dav_tol = 1e-8;
    bool last_partial = false;
    long dav_iters = 0, dav_solves = 0, dav_fallbacks = 0;
    // verbose only: wall time of the refinements and of the full solves
    double ms_refine = 0.0, ms_full = 0.0;
    auto wall_ms = [&]() {
      ck(cudaStreamSynchronize(st), "sync");
      return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
    };

    auto solve_blocks = [&](const double* Fo_all, int s) {
      std::vector<char> full(nblk, 0);
      bool partial = false;
      const bool aufbau = !d->l_occ && !d->fixed_occ;
      for (int k = 0; k < nblk; ++k) {
        if (rep[k] != k) continue;
        const Block& b = blocks[k];
        const size_t key = (size_t)s * nblk + k;
        bool f = !use_davidson || ndiag < n_full_first || !have_ref[key] || want_full[key] || b.nk < 96;
        if (!f) {
          int nocc = 0;
          while (nocc < b.nk && occ[s][k][nocc] > 0) ++nocc;
          // fixed occupations need the occupied pairs only; the Aufbau order
          // also the lowest virtuals
          const int kconv = std::min(b.nk, std::max(1, nocc + (aufbau ? 3 : 0)));
          const int kk = std::min(b.nk, kconv + 4);
          double* V = dVec.as<double>() + Lblk * s + b.off;
          const double* Fk = Fo_all + Lblk * s + b.off;
          // F' Q = X^T F_k X Q (+ b (Q - V_occ V_occ^T Q)); V keeps the
          // previous orbitals until the refinement succeeds
          const hfg::BlockOperator apply = [&](const double* Q, int c, double* AQ) {
            const size_t need = sizeof(double) * (size_t)b.nk * c;
            if (dOpA.n < need) dOpA.alloc(need);
            if (dOpB.n < need) dOpB.alloc(need);
            x_cols(b, Q, c, dOpA.as<double>(), false);
            cb(cublasDgemm(hd.bl, CUBLAS_OP_N, CUBLAS_OP_N, b.nk, c, b.nk, &one, Fk, b.nk, dOpA.as<double>(), b.nk,
                           &zero, dOpB.as<double>(), b.nk),
               "F (X Q)");
            x_cols(b, dOpB.as<double>(), c, AQ, true);
            if (shift > 0.0) {
              cb(cublasDaxpy(hd.bl, b.nk * c, &shift, Q, 1, AQ, 1), "shift Q");
              if (nocc > 0) {
                if (dOpC.n < sizeof(double) * (size_t)nocc * c) dOpC.alloc(sizeof(double) * (size_t)nocc * c);
                const double mshift = -shift;
                cb(cublasDgemm(hd.bl, CUBLAS_OP_T, CUBLAS_OP_N, nocc, c, b.nk, &one, V, b.nk, Q, b.nk, &zero,
                               dOpC.as<double>(), nocc),
                   "V^T Q");
                cb(cublasDgemm(hd.bl, CUBLAS_OP_N, CUBLAS_OP_N, b.nk, c, nocc, &mshift, V, b.nk, dOpC.as<double>(),
                               nocc, &one, AQ, b.nk),
                   "shift projector");
              }
            }
          };
          // banded shift-invert corrections (one angular function: nk = nrad)
          const hfg::Preconditioner pc = [&](const double* Rg, const double* Xg, const double* thd, int u,
                                             double* Tout) {
            const int n = b.nk, wb = H.rad.nn - 1;
            const size_t need = sizeof(double) * (size_t)n * u;
            if (dZr.n < need) dZr.alloc(need);
            if (dZx.n < need) dZx.alloc(need);
            if (dYt.n < need) dYt.alloc(need);
            const size_t wf = hfg::band_olsen_work_floats(n, wb, u) * sizeof(float);
            if (dBandWork.n < wf) dBandWork.alloc(wf);
            cb(cublasDgemm(hd.bl, CUBLAS_OP_N, CUBLAS_OP_N, n, u, n, &one, dSX.as<double>(), n, Rg, n, &zero,
                           dZr.as<double>(), n),
               "S X r");
            cb(cublasDgemm(hd.bl, CUBLAS_OP_N, CUBLAS_OP_N, n, u, n, &one, dSX.as<double>(), n, Xg, n, &zero,
                           dZx.as<double>(), n),
               "S X x");
            ck(hfg::k_band_olsen(Fk, dSrad.as<double>(), n, wb, thd, dZr.as<double>(), dZx.as<double>(),
                                 dYt.as<double>(), dBandWork.as<float>(), u, st),
               "banded corrections");
            cb(cublasDgemm(hd.bl, CUBLAS_OP_T, CUBLAS_OP_N, n, u, n, &one, dSX.as<double>(), n, dYt.as<double>(), n,
                           &zero, Tout, n),
               "(S X)^T y");
          };
          std::vector<double> th;
          const double t0 = verbose ? wall_ms() : 0.0;
          const int itd = hfg::davidson_lowest(hd.bl, st, apply, b.nk, kk, kconv, V,
                                               dVref.as<double>() + Lblk * s + b.off,
                                               dLam.as<double>() + (size_t)nbf * s + eoff[k], th, dav, 12, dav_tol,
                                               banded ? &pc : nullptr);
          if (verbose) ms_refine += wall_ms() - t0;
          if (itd < 0) {
            f = true;
            ++dav_fallbacks;
          } else {
            ++dav_solves;
            dav_iters += itd;
            want_full[key] = itd >= (banded ? 10 : 6);
            partial = true;
            // the kk Ritz values; the rest out of reach of the Aufbau order
            std::vector<double> ev(b.nk, 1e300);
            std::copy(th.begin(), th.end(), ev.begin());
            for (int q = 0; q < nblk; ++q) {
              if (rep[q] != k) continue;
              ck(cudaMemcpyAsync(deps.as<double>() + (size_t)nbf * s + eoff[q], ev.data(), sizeof(double) * b.nk,
                                 cudaMemcpyHostToDevice, st),
                 "eigenvalues");
              if (q != k)
                ck(cudaMemcpyAsync(dVec.as<double>() + Lblk * s + blocks[q].off, V, sizeof(double) * b.nk * kk,
                                   cudaMemcpyDeviceToDevice, st),
                   "copy vectors");
            }
            ck(cudaStreamSynchronize(st), "sync");
          }
        }
        full[k] = f ? 1 : 0;
      }
      if (std::find(full.begin(), full.end(), 1) != full.end()) {
        const double t0 = verbose ? wall_ms() : 0.0;
        for (int k = 0; k < nblk; ++k)
          if (full[k]) form_ortho(Fo_all, s, k);
        diagonalise(dFp.as<double>(), s, full);
        if (verbose) ms_full += wall_ms() - t0;
        for (int k = 0; k < nblk; ++k) {
          if (!full[k]) continue;
          const Block& b = blocks[k];
          ck(cudaMemcpyAsync(dVref.as<double>() + Lblk * s + b.off, dVec.as<double>() + Lblk * s + b.off,
                             sizeof(double) * b.nk * b.nk, cudaMemcpyDeviceToDevice, st),
             "reference vectors");
          ck(cudaMemcpyAsync(dLam.as<double>() + (size_t)nbf * s + eoff[k], deps.as<double>() + (size_t)nbf * s + eoff[k],
                             sizeof(double) * b.nk, cudaMemcpyDeviceToDevice, st),
             "reference values");
          have_ref[(size_t)s * nblk + k] = 1;
          want_full[(size_t)s * nblk + k] = 0;
        }
      }
      return partial;
    };
    auto solve_all = [&](const double* Fo_all) {
      if (orbital_energies)
        ck(cudaMemcpyAsync(dFx.p, Fo_all, sizeof(double) * Ltot, cudaMemcpyDeviceToDevice, st), "copy F'");
      bool partial = false;
      for (int s = 0; s < nspin; ++s) partial = solve_blocks(Fo_all, s) || partial;
      last_partial = partial;
      ++ndiag;
    };

    auto dot = [&](const double* x, const double* y) {
      double r = 0.0;
      cb(cublasDdot(hd.bl, (int)nb2, x, 1, y, 1, &r), "ddot");
      return r;
    };

    // ---- core-Hamiltonian guess (iguess 0) ----
    ck(cudaMemsetAsync(dFo.p, 0, sizeof(double) * Ltot, st), "memset");
    ck(cudaMemsetAsync(dEo.p, 0, sizeof(double) * Ltot, st), "memset");
    for (int s = 0; s < nspin; ++s)
      for (int k = 0; k < nblk; ++k)
        if (rep[k] == k) gather(dH.as<double>(), blocks[k], dFo.as<double>() + Lblk * s + blocks[k].off);
    solve_all(dFo.as<double>());
    occupy();
    build_density();

    double Eold = 0.0, dEprev = 0.0;
    int it = 0, nh = 0;
    int wcur = 0;  // DIIS ring write cursor: the next (oldest once full) slot
    bool converged = false;
    int n_stable = 0;
    // stabilisation: when the orbital gradient stalls above 1e-5 (DIIS
    // oscillating between states, typical of diffuse anions and near-
    // degenerate open shells) the virtual orbitals are level-shifted,
    // F' += b (1 - Q Q^T) with Q the occupied orbitals of the previous
    // iteration, and the DIIS history restarts
    double emin = 1e300;
    int it_improved = 0;
    // optimal damping (ODA; E. Cances and C. Le Bris, Int. J. Quantum Chem.
    // 79, 82 (2000)) for runs that still stall under the full level shift:
    // the next density is the minimum of the energy on the segment between
    // the damped density P~ and the Aufbau density P of F(P~),
    //   E(lam) = E(P~) + lam s + lam^2 c / 2,  s = sum_s tr(F~_s dP_s).
    // For HF the energy is exactly quadratic there, c = sum_s tr((dJ + dK_s)
    // dP_s), and J, K are linear in P, so the damped J and K are mixed like P
    // with no second build. With an XC functional c comes from the energy at
    // P (the fit through E(0), E'(0) and E(1)) and the XC potential is
    // evaluated again at the damped density. The level shift is off while
    // ODA runs; the run goes back to DIIS (fresh history, no shift) once the
    // gradient has fallen by 100x or the full step is optimal twice in a row.
    // HFG_SCF_ODA=0 turns it off; =first starts it at the first iteration
    const char* oenv = std::getenv("HFG_SCF_ODA");
    const int oda_mode = !oenv ? 0 : std::strcmp(oenv, "0") == 0 ? -1 : std::strcmp(oenv, "first") == 0 ? 1 : 0;
    bool oda = false, oda_have = false;
    double oda_e0 = 0.0, oda_lam = 1.0, oda_Eref = 0.0;  // gradient at the start; E(P~)
    int oda_full = 0;
    DBuf dPt, dPst[2], dJt, dKt[2], dFt[2], dD1, dD2;
    auto oda_alloc = [&]() {
      if (dPt.p) return;
      dPt.alloc(sizeof(double) * nb2);
      dJt.alloc(sizeof(double) * nb2);
      dD1.alloc(sizeof(double) * nb2);
      dD2.alloc(sizeof(double) * nb2);
      for (int s = 0; s < nspin; ++s) {
        dPst[s].alloc(sizeof(double) * nb2);
        dFt[s].alloc(sizeof(double) * nb2);
        if (kfrac != 0.0) dKt[s].alloc(sizeof(double) * nb2);
      }
    };
    auto run_xc = [&]() {
      ck(hfg::launch_xc_fp64(a->dev, a->xc, a->xs, d->x_func, d->c_func,
                             restricted ? dP.as<double>() : dPs[0].as<double>(),
                             restricted ? nullptr : dPs[1].as<double>(), dXC[0].as<double>(),
                             restricted ? nullptr : dXC[1].as<double>(), dE.as<double>(), thr, st),
         "XC");
    };
    // total energy of the current P, J, K (scaled) and XC buffers
    auto energy_now = [&]() {
      double e = dot(dP.as<double>(), T) + dot(dP.as<double>(), V) + 0.5 * dot(dP.as<double>(), dJ.as<double>());
      if (kfrac != 0.0) {
        const double x0 = 0.5 * dot(dPs[0].as<double>(), dK[0].as<double>());
        e += restricted ? 2.0 * x0 : x0 + 0.5 * dot(dPs[1].as<double>(), dK[1].as<double>());
      }
      if (have_xc) {
        double ex[2];
        ck(cudaMemcpyAsync(ex, dE.p, sizeof(ex), cudaMemcpyDeviceToHost, st), "D2H");
        ck(cudaStreamSynchronize(st), "sync");
        e += ex[0];
      }
      return e;
    };
    auto copy_d = [&](DBuf& to, const DBuf& from) {
      ck(cudaMemcpyAsync(to.p, from.p, sizeof(double) * nb2, cudaMemcpyDeviceToDevice, st), "copy");
    };
    double Ekin = 0, Enuc = 0, Ecoul = 0, Exx = 0, Exc = 0, Ngrid = 0, Etot = 0;
    PhaseTimer pt;
    for (it = 1; it <= maxiter; ++it) {
      // ---- Fock build (main.cpp:386-446) ----
      ck(hfg::launch_coulomb_fp64(a->dev, a->scr, dP.as<double>(), dJ.as<double>(), true, st, &a->prof), "J");
      if (kfrac != 0.0)
        for (int s = 0; s < nspin; ++s) {
          if (d->split_exchange)
            ck(hfg::launch_exchange_split(a->dev, scr_split, a->units, dPs[s].as<double>(), dK[s].as<double>(), true,
                                          st, &a->prof, a->tc_for(false), a->side_stream()),
               "K (split)");
          else
            ck(hfg::launch_exchange_fp64(a->dev, a->scr, a->units, dPs[s].as<double>(), dK[s].as<double>(), true,
                                         st, &a->prof),
               "K");
        }
      if (have_xc) run_xc();
      for (int s = 0; s < nspin; ++s)
        if (kfrac != 0.0 && kfrac != 1.0) {
          cb(cublasDscal(hd.bl, (int)nb2, &kfrac, dK[s].as<double>(), 1), "scal K");
        }
      if (oda && oda_have) {
        // line search between P~ (kept with its J, K, F) and the new density
        double s1 = 0.0, c2 = 0.0;
        for (int s = 0; s < nspin; ++s) {
          // restricted: the total density pairs with F, J + K(P/2)
          if (restricted)
            hfg::k_diffsum(dD1.as<double>(), dP.as<double>(), dPt.as<double>(), nullptr, nullptr, nb2, st);
          else
            hfg::k_diffsum(dD1.as<double>(), dPs[s].as<double>(), dPst[s].as<double>(), nullptr, nullptr, nb2, st);
          hfg::k_diffsum(dD2.as<double>(), dJ.as<double>(), dJt.as<double>(),
                         kfrac != 0.0 ? dK[s].as<double>() : nullptr, kfrac != 0.0 ? dKt[s].as<double>() : nullptr,
                         nb2, st);
          s1 += dot(dFt[s].as<double>(), dD1.as<double>());
          c2 += dot(dD2.as<double>(), dD1.as<double>());
        }
        if (have_xc) {
          // the XC energy is not quadratic on the segment: the curvature
          // comes from the energy at the Aufbau density, E(1) = E(P~) + s +
          // c / 2, and the XC potential is recomputed at the damped density
          const double E1 = energy_now();
          c2 = 2.0 * (E1 - oda_Eref - s1);
        }
        double lam = 1.0;
        if (c2 > 0.0) lam = std::min(1.0, std::max(0.0, -s1 / c2));
        else if (s1 > 0.0) lam = 0.0;  // uphill and concave: cannot happen for an Aufbau step; keep P~
        oda_lam = lam;
        oda_full = lam >= 0.999 ? oda_full + 1 : 0;
        if (verbose) std::fprintf(stderr, "hfg_scf it %3d ODA s %.3e c %.3e lambda %.4f\n", it, s1, c2, lam);
        if (lam < 1.0) {
          hfg::k_lerp(dP.as<double>(), dPt.as<double>(), lam, nb2, st);
          hfg::k_lerp(dJ.as<double>(), dJt.as<double>(), lam, nb2, st);
          for (int s = 0; s < nspin; ++s) {
            hfg::k_lerp(dPs[s].as<double>(), dPst[s].as<double>(), lam, nb2, st);
            if (kfrac != 0.0) hfg::k_lerp(dK[s].as<double>(), dKt[s].as<double>(), lam, nb2, st);
          }
          if (have_xc) run_xc();
        }
      }
      for (int s = 0; s < nspin; ++s)
        hfg::k_add4(dF[s].as<double>(), dH.as<double>(), dJ.as<double>(),
                    kfrac != 0.0 ? dK[s].as<double>() : nullptr, have_xc ? dXC[s].as<double>() : nullptr, nb2, st);
      if (oda) {
        // the (damped) state becomes P~ for the next line search
        copy_d(dPt, dP);
        copy_d(dJt, dJ);
        for (int s = 0; s < nspin; ++s) {
          copy_d(dPst[s], dPs[s]);
          copy_d(dFt[s], dF[s]);
          if (kfrac != 0.0) copy_d(dKt[s], dK[s]);
        }
        oda_have = true;
      }
      Ekin = dot(dP.as<double>(), T);
      pt.lap(0);  // Fock build (J, K, XC, assembly) + first blocking dot
      Enuc = dot(dP.as<double>(), V);
      Ecoul = 0.5 * dot(dP.as<double>(), dJ.as<double>());
      Exx = 0.0;
      if (kfrac != 0.0) {
        Exx = 0.5 * dot(dPs[0].as<double>(), dK[0].as<double>());
        Exx = restricted ? 2.0 * Exx : Exx + 0.5 * dot(dPs[1].as<double>(), dK[1].as<double>());
      }
      if (have_xc) {
        double e[2];
        ck(cudaMemcpyAsync(e, dE.p, sizeof(e), cudaMemcpyDeviceToHost, st), "D2H");
        ck(cudaStreamSynchronize(st), "sync");
        Exc = e[0];
        Ngrid = e[1];
      }
      Etot = Ekin + Enuc + Ecoul + Exx + Exc;
      if (oda) oda_Eref = Etot;  // the energy of the state that becomes P~
      pt.lap(1);  // energies

      // ---- Fock blocks and DIIS errors F'D' - D'F' (orthonormal basis) ----
      double emax = 0.0;
      for (int s = 0; s < nspin; ++s)
        for (int k = 0; k < nblk; ++k) {
          if (rep[k] != k) continue;  // identical to its representative (spherical solves)
          const Block& b = blocks[k];
          double* Fo = dFo.as<double>() + Lblk * s + b.off;
          double* Eo = dEo.as<double>() + Lblk * s + b.off;
          gather(dF[s].as<double>(), b, Fo);
          int nocc = 0;
          while (nocc < b.nk && occ[s][k][nocc] > 0) ++nocc;
          if (nocc == 0) {
            ck(cudaMemsetAsync(Eo, 0, sizeof(double) * b.nk * b.nk, st), "memset");
            continue;
          }
          const double* Vk = dVec.as<double>() + Lblk * s + b.off;
          // W = F' V_occ = X^T F_k (X V_occ);  G = W diag(occ) V_occ^T;  E = G - G^T
          x_cols(b, Vk, nocc, dCo.as<double>(), false);
          cb(cublasDgemm(hd.bl, CUBLAS_OP_N, CUBLAS_OP_N, b.nk, nocc, b.nk, &one, Fo, b.nk, dCo.as<double>(), b.nk,
                         &zero, dT1.as<double>(), b.nk),
             "F (X V)");
          x_cols(b, dT1.as<double>(), nocc, dW.as<double>(), true);
          hfg::k_scale_cols(dW.as<double>(), b.nk, nocc, dOcc.as<double>() + (size_t)nbf * s + eoff[k],
                            dCo.as<double>(), st);
          cb(cublasDgemm(hd.bl, CUBLAS_OP_N, CUBLAS_OP_T, b.nk, b.nk, nocc, &one, dCo.as<double>(), b.nk, Vk, b.nk,
                         &zero, dG.as<double>(), b.nk),
             "G");
          hfg::k_antisym(dG.as<double>(), b.nk, Eo, st);
        }
      {
        int imax = 0;
        cb(cublasIdamax(hd.bl, (int)Ltot, dEo.as<double>(), 1, &imax), "idamax");
        ck(cudaMemcpyAsync(&emax, dEo.as<double>() + (imax - 1), sizeof(double), cudaMemcpyDeviceToHost, st), "D2H");
        ck(cudaStreamSynchronize(st), "sync");
        emax = std::fabs(emax);
      }
      pt.lap(2);  // orthonormal blocks + DIIS errors
      dav_tol = std::min(1e-4, std::max(1e-8, 1e-2 * emax));
      if (verbose) std::fprintf(stderr, "hfg_scf it %3d E %.12f dE % .3e diis %.3e\n", it, Etot, Etot - Eold, emax);
      // energy change within etol + 1e-12 |E| (heavy atoms: |E| ~ 1e4 Eh puts
      // the FP64 summation noise of the grid and matrix traces near 1e-9 Eh)
      // Converged: the energy is stable and the orbital gradient (DIIS error)
      // is below dtol; or the energy has been stable for three iterations
      // with the gradient below 1e-5 (the error floor of fractionally
      // occupied spherical shells on fine grids sits at ~1e-7 and stops
      // changing; the energy error is quadratic in it, far below etol)
      const bool estable = it > 1 && std::fabs(Etot - Eold) < etol + 1e-12 * std::fabs(Etot);
      n_stable = estable ? n_stable + 1 : 0;
      // (the stable-energy fallback applies only under the default gradient
      // target; a caller-set diis_tol is a hard requirement)
      // A slow monotone descent also passes the energy test (2e-9 Eh steps
      // at a rate near 1 stopped heavy fractional-occupation atoms 1.4e-7 Eh
      // early), so the fallback also wants the remaining descent,
      // extrapolated geometrically from the last two energy changes (rate
      // capped at 0.999), below 1e-9 Eh; changes of alternating sign (the
      // noise of a gradient floor) or below 1e-11 Eh pass.
      const double dE1 = Etot - Eold;
      double tail = 0.0;
      if (it > 2 && dE1 * dEprev > 0.0 && std::fabs(dE1) > 1e-11) {
        const double rho = std::min(0.999, dE1 / dEprev);
        tail = std::fabs(dE1) * rho / (1.0 - rho);
      }
      dEprev = dE1;
      const bool floor_ok = d->diis_tol <= 0 && n_stable >= 3 && emax < 1e-5 && tail < 1e-9;
      // (a damped step is a fixed point only when it is the full step)
      if (((estable && emax < dtol) || floor_ok) && (!oda || oda_lam >= 0.999)) {
        converged = true;
        break;
      }
      Eold = Etot;
      if (emax < 0.5 * emin) {
        emin = emax;
        it_improved = it;
      }
      if (oda) {
        if (emax < 1e-2 * oda_e0 || oda_full >= 2) {
          // DIIS again without the shift (it slows the last digits down;
          // the stabilisation ladder starts over if DIIS stalls again)
          oda = oda_have = false;
          shift = 0.0;
          it_improved = it;
          emin = emax;
          nh = 0;
          wcur = 0;
          std::fill(Bm.begin(), Bm.end(), 0.0);
          if (verbose) std::fprintf(stderr, "hfg_scf it %3d ODA done, DIIS restart\n", it);
        }
      } else if (emax > std::max(1e-6, 10.0 * dtol) && it >= 12 && it - it_improved >= 6 && shift < 2.0) {
        shift = (shift == 0.0) ? 0.5 : 2.0;
        it_improved = it;
        emin = emax;
        nh = 0;
        wcur = 0;
        std::fill(Bm.begin(), Bm.end(), 0.0);
        if (verbose) std::fprintf(stderr, "hfg_scf it %3d level shift %.2f, DIIS restart\n", it, shift);
      } else if (oda_mode >= 0 && emax > 10.0 * dtol &&
                 ((shift >= 2.0 && it - it_improved >= 10) || (oda_mode == 1 && it == 1))) {
        // still stalled under the full shift (the gradient has not halved in
        // ten iterations): optimal damping from the current (Aufbau) density
        oda_alloc();
        oda = true;
        oda_have = false;
        oda_full = 0;
        oda_lam = 1.0;
        oda_e0 = emax;
        oda_Eref = Etot;
        shift = 0.0;
        it_improved = it;
        emin = emax;
        copy_d(dPt, dP);
        copy_d(dJt, dJ);
        for (int s = 0; s < nspin; ++s) {
          copy_d(dPst[s], dPs[s]);
          copy_d(dFt[s], dF[s]);
          if (kfrac != 0.0) copy_d(dKt[s], dK[s]);
        }
        oda_have = true;
        if (verbose) std::fprintf(stderr, "hfg_scf it %3d optimal damping (ODA)\n", it);
      }

      if (oda) {
        // Roothaan step from F(P~): the blocks gathered above
        pt.lap(3);
        solve_all(dFo.as<double>());
        occupy();
        pt.lap(4);
        build_density();
        ck(cudaStreamSynchronize(st), "sync");
        pt.lap(5);
        continue;
      }

      // ---- DIIS extrapolation ----
      const int slot = wcur;
      wcur = (wcur + 1) % nhist;
      ck(cudaMemcpyAsync(dHF.as<double>() + Ltot * slot, dFo.p, sizeof(double) * Ltot, cudaMemcpyDeviceToDevice, st),
         "copy");
      ck(cudaMemcpyAsync(dHE.as<double>() + Ltot * slot, dEo.p, sizeof(double) * Ltot, cudaMemcpyDeviceToDevice, st),
         "copy");
      if (nh < nhist) ++nh;
      // new row of the error-overlap matrix: one GEMV over the history
      {
        cublasPointerMode_t pm;
        cublasGetPointerMode(hd.bl, &pm);
        cb(cublasDgemv(hd.bl, CUBLAS_OP_T, (int)Ltot, nh, &one, dHE.as<double>(), (int)Ltot,
                       dHE.as<double>() + Ltot * slot, 1, &zero, dBrow.as<double>(), 1),
           "gemv");
        std::vector<double> row(nh);
        ck(cudaMemcpyAsync(row.data(), dBrow.p, sizeof(double) * nh, cudaMemcpyDeviceToHost, st), "D2H");
        ck(cudaStreamSynchronize(st), "sync");
        for (int i = 0; i < nh; ++i) Bm[i + (size_t)slot * nhist] = Bm[slot + (size_t)i * nhist] = row[i];
      }
      std::vector<double> B((size_t)(nh + 1) * (nh + 1), -1.0), rhs(nh + 1, 0.0);
      B[(size_t)nh * (nh + 1) + nh] = 0.0;
      rhs[nh] = -1.0;
      for (int i = 0; i < nh; ++i)
        for (int j = 0; j < nh; ++j) B[i + (size_t)j * (nh + 1)] = Bm[i + (size_t)j * nhist];
      // small dense solve (Gaussian elimination with partial pivoting)
      std::vector<double> c(rhs);
      {
        const int n = nh + 1;
        std::vector<double> M(B);
        bool ok = true;
        for (int col = 0; col < n && ok; ++col) {
          int piv = col;
          for (int r = col + 1; r < n; ++r)
            if (std::fabs(M[r + (size_t)col * n]) > std::fabs(M[piv + (size_t)col * n])) piv = r;
          if (std::fabs(M[piv + (size_t)col * n]) < 1e-300) { ok = false; break; }
          for (int k = 0; k < n; ++k) std::swap(M[col + (size_t)k * n], M[piv + (size_t)k * n]);
          std::swap(c[col], c[piv]);
          for (int r = col + 1; r < n; ++r) {
            const double f = M[r + (size_t)col * n] / M[col + (size_t)col * n];
            for (int k = col; k < n; ++k) M[r + (size_t)k * n] -= f * M[col + (size_t)k * n];
            c[r] -= f * c[col];
          }
        }
        if (ok) {
          for (int r = n - 1; r >= 0; --r) {
            double v = c[r];
            for (int k = r + 1; k < n; ++k) v -= M[r + (size_t)k * n] * c[k];
            c[r] = v / M[r + (size_t)r * n];
          }
        } else {
          std::fill(c.begin(), c.end(), 0.0);
          c[slot] = 1.0;
        }
      }
      ck(cudaMemsetAsync(dFo.p, 0, sizeof(double) * Ltot, st), "memset");
      for (int i = 0; i < nh; ++i)
        cb(cublasDaxpy(hd.bl, (int)Ltot, &c[i], dHF.as<double>() + Ltot * i, 1, dFo.as<double>(), 1), "axpy");
      // (the level shift, if any, is applied when the blocks are solved)
      pt.lap(3);  // DIIS extrapolation
      solve_all(dFo.as<double>());
      occupy();
      pt.lap(4);  // eigensolves + occupations
      build_density();
      ck(cudaStreamSynchronize(st), "sync");
      pt.lap(5);  // density
    }
    if (orbital_energies && last_partial) {
      // the full spectrum of the blocks diagonalised last (refinement gives
      // only the lowest pairs)
      for (int s = 0; s < nspin; ++s) {
        for (int k = 0; k < nblk; ++k)
          if (rep[k] == k) form_ortho(dFx.as<double>(), s, k);
        diagonalise(dFp.as<double>(), s);
      }
      ck(cudaMemcpyAsync(eps.data(), deps.p, sizeof(double) * eps.size(), cudaMemcpyDeviceToHost, st), "D2H eps");
    }
    ck(cudaStreamSynchronize(st), "sync");
    if (verbose)
      std::fprintf(stderr, "hfg_scf eigensolver: %d diagonalisations, %ld refined blocks (%.2f iterations each), "
                           "%ld fell back to full; %.1f ms refining, %.1f ms in full solves\n",
                   ndiag, dav_solves, dav_solves ? (double)dav_iters / dav_solves : 0.0, dav_fallbacks, ms_refine,
                   ms_full);
    a->mark_use(st);
    res->Etot = Etot;
    res->Ekin = Ekin;
    res->Enuc = Enuc;
    res->Ecoul = Ecoul;
    res->Exx = Exx;
    res->Exc = Exc;
    res->Nel_grid = Ngrid;
    res->iterations = std::min(it, maxiter);
    for (int k = 0; k < 6; ++k) res->phase_ms[k] = pt.ms[k];
    res->converged = converged ? 1 : 0;
    if (orbital_energies) std::memcpy(orbital_energies, eps.data(), sizeof(double) * eps.size());
  }
}

extern "C" hfg_status hfg_scf_run(hfg_atom* a, const hfg_scf_desc* d, hfg_scf_result* res, double* orbital_energies,
                                  void* stream) {
  return guard([&] {
    need(a != nullptr, "hfg_scf_run: null argument");
    need(!a->host.spherical, "hfg_scf_run: a spherically averaged handle has no SCF driver (its Fock build is "
                             "hfg_sadatom_coulomb / hfg_sadatom_exchange)");
    a->check_device();
    cudaStream_t st = stream ? (cudaStream_t)stream : a->own_stream;
    Handles hd;
    cb(cublasCreate(&hd.bl), "cublasCreate");
    cb(cublasSetStream(hd.bl, st), "cublasSetStream");
    cs(cusolverDnCreate(&hd.so), "cusolverDnCreate");
    cs(cusolverDnSetStream(hd.so, st), "cusolverDnSetStream");
    hfg_scf_impl(a, d, res, orbital_energies, st, hd.bl, hd.so);
  });
}

// Launchers of the SCF driver's small device kernels (scf_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>

namespace hfg {

void k_gather_block(const double* M, int nbf, int nrad, const int* ang, int nk, double* Mk, cudaStream_t st);
void k_scatter_add_block(double* M, int nbf, int nrad, const int* ang, int nk, const double* Mk, double alpha,
                         cudaStream_t st);
void k_antisym(const double* G, int n, double* E, cudaStream_t st);
void k_add4(double* out, const double* a, const double* b, const double* c, const double* d, size_t n,
            cudaStream_t st);
void k_scale_cols(const double* X, int n, int m, const double* s, double* Y, cudaStream_t st);
// T, V (nbf x nbf, zeroed by the caller) from the radial blocks:
// T = Trad + l(l+1) Tlrad, V = -Z Vrad on the diagonal angular blocks
void k_expand_one_electron(const double* Trad, const double* Tlrad, const double* Vrad, const int* lval, int nang,
                           int nrad, double Z, double* T, double* V, cudaStream_t st);
// X (n x m) rows scaled by d (length n), in place
void k_scale_rows(double* X, int n, int m, const double* d, cudaStream_t st);
// out = (a1 - b1) + (a2 - b2) (a2, b2 may be null)
void k_diffsum(double* out, const double* a1, const double* b1, const double* a2, const double* b2, size_t n,
               cudaStream_t st);
// banded shift-invert Olsen corrections (band_precond.cu): for each of the u
// columns, y = M^-1 zr - eps M^-1 zx with M = band_w(F) - theta S (n x n
// column-major F and S, half-width w <= 16), eps = (zx . M^-1 zr) / (zx . M^-1 zx);
// work holds band_olsen_work_floats(n, w, u) floats
size_t band_olsen_work_floats(int n, int w, int u);
cudaError_t k_band_olsen(const double* F, const double* S, int n, int w, const double* theta, const double* Zr,
                         const double* Zx, double* Y, float* work, int u, cudaStream_t st);
// out = a + lam (out - a)
void k_lerp(double* out, const double* a, double lam, size_t n, cudaStream_t st);
// symmetric n x n test density with every entry nonzero (deterministic)
void fill_test_density(double* P, int n, cudaStream_t st);
// A[i,i] += v, A n x n column-major
void k_add_diag(double* A, int n, double v, cudaStream_t st);
// Davidson steps (n x k column blocks): residuals R = AX - X diag(theta) with
// column norms; reference-preconditioned Olsen corrections in the reference
// eigenbasis (Zr = Vr^T R, Zx = Vr^T X -> Zt)
void k_dav_residual(const double* AX, const double* X, const double* theta, int n, int k, double* R, double* norms,
                    cudaStream_t st);
void k_dav_olsen(const double* Zr, const double* Zx, const double* lam, const double* theta, int n, int k,
                 double floor_, double* Zt, cudaStream_t st);

}  // namespace hfg

// Lowest eigenpairs of the SCF's orthonormal Fock blocks by a
// reference-preconditioned Davidson iteration (device GEMMs, host Rayleigh-Ritz
// on the small projected matrices).
//
// The reference diagonalises every symmetry block in full every iteration
// (src/general/scf_helpers.cpp:41-50 eig_gsym; the driver's eigensolver runs
// dominate an atomic SCF). Only the occupied orbitals (plus a few virtuals for
// the Aufbau order) enter the next density, and the Fock matrix of iteration i
// is close to that of iteration i-1. So after a few full solves the driver
// refines the previous orbitals: Davidson in the span of the previous
// eigenvectors, with the Olsen correction preconditioned by the full
// eigendecomposition of an earlier Fock block, (F_ref - theta)^-1 applied
// exactly in that eigenbasis. Each iteration costs a few n x n x k GEMMs
// instead of an O(n^3) tridiagonalisation.
#pragma once

#include <cublas_v2.h>

#include <functional>
#include <vector>

#include "handle.hpp"

namespace hfg {

// cyclic Jacobi eigensolver for a small symmetric matrix (column-major m x m):
// eigenvalues ascending in w, eigenvectors in the columns of V
void jacobi_eigh(int m, std::vector<double> A, std::vector<double>& w, std::vector<double>& V);

struct DavidsonWork {
  DBuf Q, AQ, X, AX, R, T, Zr, Zx, Zt, sm, sm2, th, nrm;
  std::vector<double> h1, h2;
};

// apply(Q, c, AQ): AQ = F Q for c columns (device, leading dimension n)
using BlockOperator = std::function<void(const double* Q, int cols, double* AQ)>;
// precond(R, X, theta, u, T): the u correction vectors T (device, leading
// dimension n) from the residuals R and Ritz vectors X and the Ritz values
// theta (device); T may alias X
using Preconditioner = std::function<void(const double* R, const double* X, const double* theta, int u, double* T)>;

// Lowest k eigenpairs of the symmetric n x n operator F (applied by `apply`)
// from the k starting columns in V (device, leading dimension n; overwritten
// with the eigenvectors on success); theta (host) receives the eigenvalues.
// Vr (device, n x n) and lam (device, n) are the reference eigenpairs; a
// non-null pc replaces the reference-eigenbasis correction.
// Converged when the residual norms |F x - theta x| of the first kconv pairs
// are <= tol (absolute). Returns the number of iterations, or -1 when not
// converged within maxit (V is then unchanged).
int davidson_lowest(cublasHandle_t bl, cudaStream_t st, const BlockOperator& apply, int n, int k, int kconv,
                    double* V, const double* Vr, const double* lam, std::vector<double>& theta, DavidsonWork& w,
                    int maxit, double tol, const Preconditioner* pc = nullptr);

}  // namespace hfg

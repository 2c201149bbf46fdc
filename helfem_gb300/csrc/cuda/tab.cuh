// Device tabulation of the atomic in-element two-electron tables (launchers
// in tab_fp64.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace hfg {

// All pointers are device pointers.
struct TabInput {
  int nn, nel, NL;
  int no, ni;            // outer / inner Gauss-Legendre orders
  const double* bval;    // [nel+1] element boundaries
  const double* xo;      // [no] outer rule on [-1, 1]
  const double* wo;
  const double* xi;      // [ni] inner rule on [-1, 1]
  const double* wi;
  const double* Bo;      // [p + k*no] LIP values at the outer points
  const double* Bin;     // [(q + p*ni) + k*no*ni] LIP values at the inner points
  const unsigned char* ok;  // [e*nn + k] primitive k of element e is a basis function
  double tol;            // absolute pivoted-Cholesky tolerance
};

size_t tab_t1_doubles(int nn, int nel, int NL);      // pair-packed tensor scratch
size_t tab_factor_doubles(int nn, int nel, int NL);  // factor scratch (nn^2 columns per block)

// T1 (pair-packed in-element tensor) and the pivoted Cholesky factor into
// Lsc [(L*nel+e)*nn^4], ranks into rank [L*nel+e]
cudaError_t launch_tab_factor(const TabInput& in, double* T1, double* Lsc, int* rank, cudaStream_t st);
// padded factor cholp [(L*nel+e)*nn^2*rmax] and exchange-ordered tensor
// tk [(L*nel+e)*nn^4] from the factor
cudaError_t launch_tab_finish(const TabInput& in, const double* Lsc, const int* rank, int rmax, double* cholp,
                              double* tk, cudaStream_t st);
// y[i] = (fl32(x[i]), fl32(x[i] - fl32(x[i])))
cudaError_t launch_split_f2(const double* x, float2* y, size_t n, cudaStream_t st);

}  // namespace hfg

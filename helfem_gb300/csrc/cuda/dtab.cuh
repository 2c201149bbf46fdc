// Device tabulation of the diatomic two-electron primitives (launchers in
// dtab_fp64.cu): the disjoint P/Q integrals and the sign-carrying pivoted
// factor of the two-channel in-element kernel, FP64, with the host
// tabulation's quadrature rules and pivoting rule.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>

namespace hfg {

// All pointers are device pointers.
struct DTabInput {
  int nn, nel, nlm, Lmax, Mtop;  // Legendre tables are (Mtop+1) x (Lmax+1)
  int n1e, no, ni;               // disjoint rule, in-element outer and inner orders
  const double* bval;            // [nel+1] element boundaries in mu (bval[0] = 0)
  const double* xg;              // [n1e] disjoint rule on [-1, 1]
  const double* wg;
  const double* xo;              // [no] outer rule on [-1, 1]
  const double* wo;
  const double* xi;              // [ni] inner rule on [-1, 1]
  const double* wi;
  const double* Bg;              // [q + p*n1e] LIP values at xg
  const double* B1g;             // [q + p*no] LIP values at the outer points (elements e > 0)
  const double* B1z;             //   the same on the first element (mu = mu_1 t^3 map)
  const double* B2g;             // [(q*ni + r) + p*no*ni] LIP values at the inner points
  const double* B2z;
  const unsigned char* ok;       // [e*nn + p] primitive p of element e is a basis function
  const int* lm_L;               // [nlm] multipole list, |M|-major
  const int* lm_M;
  const int* lmidx;              // [M*(Lmax+1) + L] -> ilm, or -1
  double thresh;                 // relative pivot threshold of the factor
};

// Legendre P and Q at every disjoint and outer quadrature point:
// PQ[((e*(n1e+no) + q)*2 + {0: P, 1: Q})*(Mtop+1)*(Lmax+1) + M*(Lmax+1) + L]
size_t dtab_pq_doubles(const DTabInput& in);
cudaError_t launch_dtab_pq(const DTabInput& in, double* PQ, cudaStream_t st);

// the disjoint integrals p0, p2, q0, q2 [(ilm*nel + e)*nn^2 + a + b*nn]
cudaError_t launch_dtab_disjoint(const DTabInput& in, const double* PQ, double* p0, double* p2, double* q0,
                                 double* q2, cudaStream_t st);

// Scratch of one group of ne elements (tiles g = el*nlm + ilm, el = e - e0)
size_t dtab_group_doubles(const DTabInput& in, int ne, int capR);

// In-element kernel of elements e0 .. e0+ne-1 and its sign-carrying pivoted
// factor: factor columns into Bsc [g*N*capR + i + k*N] (N = 2 nn^2), signs
// into ssc [g*capR + k], ranks into rank [g] (-1: the rank exceeds capR).
// scratch holds dtab_group_doubles(in, ne, capR) doubles.
cudaError_t launch_dtab_factor(const DTabInput& in, const double* PQ, int e0, int ne, int capR, double* scratch,
                               double* Bsc, double* ssc, int* rank, cudaStream_t st);

// Repack ng factors from a source of column capacity capS into the
// destination layout with column capacity capD: source tile g goes to
// destination tile dst_tile(g) = (g % nlm)*nel + e0 + g / nlm when
// scatter != 0, else to tile g. Columns at and beyond the rank are zeroed.
cudaError_t launch_dtab_pack(int N, int ng, int nlm, int nel, int e0, int scatter, int capS, int capD,
                             const double* Bs, const double* ss, const int* rank, double* Bd, double* sd,
                             cudaStream_t st);

}  // namespace hfg

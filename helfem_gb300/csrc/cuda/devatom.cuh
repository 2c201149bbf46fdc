// Device-resident atom context shared by the Fock-build kernels.
//
// Radial layout: element e owns an nn x nn primitive tile; primitive p is the
// global radial function g(e,p) = e*(nn-1) + p - 1, valid for 0 <= g < nrad.
// AO index = iang*nrad + irad; matrices are column-major FP64 (nbf x nbf).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace hfg {

struct DevAtom {
  int nn, nel, nrad, nang, nbf, NL, rmax;
  // per (L,e) padded tiles
  const double* rs;     // [(L*nel+e)*nn*nn]
  const double* rb;     // [(L*nel+e)*nn*nn] (zero for e = 0)
  const double* cholp;  // [(L*nel+e)*nn*nn*rmax]
  const int* rank;      // [L*nel+e]
  const double* tk;     // [(L*nel+e)*(nn*nn)^2] exchange-ordered in-element tensor
  // Coulomb coupling lists
  int nchan;
  const int* chanL;     // [nchan]
  const int* jket_ptr;  // [nchan+1]
  const int* jket_blk;
  const double* jket_coef;
  const int* jbra_ptr;  // [nang*nang+1]
  const int* jbra_chan;
  const double* jbra_coef;
  // exchange recoupling lists
  const int* kjk_ptr;   // [nang*nang+1] -> entries
  const int* kent_L;
  const int* kent_ptr;  // [nent+1] -> terms
  const int* kterm_blk;
  const int* kterm_off;  // density offset of the term's block: l*nrad*nbf + i*nrad
  const double* kterm_coef;
  int nent;
  int max_terms_per_jk; // bound on terms of one output block
  // split-precision copies: every FP64 value v stored as float2 (hi, lo) with
  // hi = fl32(v), lo = fl32(v - hi)
  const float2* rs2 = nullptr;
  const float2* rb2 = nullptr;
  const float2* tk2 = nullptr;
  const float2* kterm_coef2 = nullptr;
  // split form of the Coulomb build (float-pair copies of the coupling
  // coefficients and of the in-element factor, made on first use)
  const float2* jket_coef2 = nullptr;
  const float2* jbra_coef2 = nullptr;
  const float2* cholp2 = nullptr;
};

// Scratch owned by the atom handle (sizes fixed at creation)
struct DevScratch {
  double* jin;          // [nchan*nel*nn*nn]
  double* jscal;        // [nchan*nel*2]
  double* khalo;        // [nel*nel*nang*nang*(2nn-1)]
  double* bnorm;        // [nang*nang*NORM_SPLIT] partial squared block norms
  unsigned char* act;   // [nang*nang] density block above the screen
  unsigned char* ent_act;  // [nent] exchange entry with an active term
  float2* p2;           // [nbf*nbf] split copy of the density (split path)
};

// Column bands per angular block in the density-norm pass
#define NORM_SPLIT 16

// Exchange work units (int4: a, b, lo, hi), built once per atom on the host.
// a != b: element pair, output blocks jk in [lo, hi) (natural order);
// a == b: diagonal element, output blocks diag_jk[lo..hi).
struct KUnits {
  const int4* all = nullptr;   // every ordered pair and every jk
  int n_all = 0;
  const int4* sym = nullptr;   // a < b pairs, j <= k diagonal blocks
  int n_sym = 0;
  int n_off_all = 0, n_off_sym = 0;  // off-diagonal units come first
  const int* diag_all = nullptr;  // 0..nang^2-1
  const int* diag_sym = nullptr;  // jk with j <= k
  const int* diag_jk_src(bool symmetric) const { return symmetric ? diag_sym : diag_all; }
};

__host__ __device__ inline int gfun(const DevAtom& A, int e, int p) { return e * (A.nn - 1) + p - 1; }

// Tensor-core split-precision exchange (k_tc.cu): the radial tables as
// balanced base-256 digit planes (bf16, 16 x 16 in the no-swizzle K-major
// operand layout) with one power-of-two scale per row, the output blocks in
// groups of up to 8, and the work units (a, b, range of groups).
#define TC_NDIGITS 7
#define TC_TPLANE 512
struct DevTC {
  const unsigned char* digits = nullptr;  // [kind (0 r_small, 1 r_big)][L][e][TC_NDIGITS][TC_TPLANE]
  const int* rowexp = nullptr;            // [kind][L][e][16]
  const int* group_jk = nullptr;          // [ngroups][8], -1: empty slot
  const int* group_ent = nullptr;         // [ngroups][8][NL], -1: no entry with that L
  int ngroups = 0;
  const int4* units_sym = nullptr;        // (a, b, first group, end group), a < b
  int n_sym = 0;
  const int4* units_all = nullptr;        // (a, b, first group, end group), a != b
  int n_all = 0;
  int* err = nullptr;                     // set when a completion wait ran out
  // diagonal element tiles: the exchange-ordered tensor as digit planes
  // [L][e][row tile][K step][digit][128 x 16], per-row exponents, groups of
  // up to 16 output blocks (j <= k in symmetric mode), units (a, group, row tile)
  const unsigned char* tk_digits = nullptr;
  const int* tk_rowexp = nullptr;         // [L][e][row tile][128]
  int dmtiles = 0, dksteps = 0;
  const int* dgroup_jk_sym = nullptr;     // [groups][16]
  const int* dgroup_ent_sym = nullptr;    // [groups][16][NL]
  const int* dgroup_jk_all = nullptr;
  const int* dgroup_ent_all = nullptr;
  const int4* dunits_sym = nullptr;
  int n_dsym = 0;
  const int4* dunits_all = nullptr;
  int n_dall = 0;
};

#ifdef __CUDACC__
__device__ __forceinline__ size_t k_halo_idx(const DevAtom& A, int a, int b, int jk, int h) {
  return ((size_t)(a * A.nel + b) * (A.nang * A.nang) + jk) * (2 * A.nn - 1) + h;
}
// store the finished contribution y of tile (a,b), angular block jk, at
// local position (p,q): owned entries go to K, the shared last row/column to
// the halo buffer (added by the boundary fix-up in a fixed order)
__device__ __forceinline__ void k_store_tile(const DevAtom& A, const DevScratch& S, double* K, int a, int b, int jk,
                                             int p, int q, double y) {
  const int nn = A.nn;
  if (p >= nn || q >= nn) return;
  const int gp = gfun(A, a, p), gq = gfun(A, b, q);
  if (gp < 0 || gp >= A.nrad || gq < 0 || gq >= A.nrad) return;
  const int j = jk % A.nang, k = jk / A.nang;
  if (p <= nn - 2 && q <= nn - 2)
    K[(size_t)(k * A.nrad + gq) * A.nbf + (size_t)j * A.nrad + gp] = y;
  else if (p == nn - 1)
    S.khalo[k_halo_idx(A, a, b, jk, q)] = y;
  else
    S.khalo[k_halo_idx(A, a, b, jk, nn + p)] = y;
}
#endif

// Optional per-kernel timing (the engine's counterpart of the reference's
// FockTimer): when enabled, every kernel launch is bracketed by a pair of
// pre-created events on its stream; records are read back after the work.
enum KernelClass { KC_J_CONTRACT = 0, KC_J_SCATTER, KC_K_NORMS, KC_K_TILES, KC_K_FIXUP, KC_COUNT };
struct Profiler {
  bool on = false;
  unsigned mask = ~0u;  // classes that are bracketed (bit KC_*)
  int cap = 0, n = 0;
  cudaEvent_t* ev = nullptr;  // [2*cap]
  int* cls = nullptr;         // [cap]
};

// Device tables of the atomic DFT grid (host layout in host/atom.hpp)
struct DevXC {
  int nquad = 0, nap = 0;
  const double* wang = nullptr;  // [nap]
  const double* isin = nullptr;  // [nap]
  const double* W = nullptr;     // [(alpha + beta*nang)*nap + a]
  const double* Wt = nullptr;
  const double* Wp = nullptr;
  const double* r = nullptr;     // [e*nquad + q]
  const double* wr = nullptr;    // radial weight times r^2
  const double* R = nullptr;     // [(e*nquad + q)*nn + p]
  const double* dR = nullptr;
};
struct XcScratch {
  double* D;      // [2][nel][nang^2][nquad]
  double* Dr;     // same
  double* F;      // [2][4][nel][nquad][nap]
  double* U;      // [2][4][nel][nang^2][nquad]
  double* epart;  // [nel*nquad][2]
};
bool xc_func_supported(int id);
bool xc_func_is_gga(int id);
// Pb == nullptr: restricted (Pa is the total density, Ha the potential);
// energies (device, may be null) receives {Exc, Nel}
cudaError_t launch_xc_fp64(const DevAtom& A, const DevXC& X, const XcScratch& S, int xid, int cid,
                           const double* Pa, const double* Pb, double* Ha, double* Hb, double* energies,
                           double thr, cudaStream_t st);

// Capacity of the static scratch behind hfg_coulomb_noalloc (4 MiB).
#define HFG_NOALLOC_SCRATCH_DOUBLES (512 * 1024)
// Device address of that scratch on the current device; resolved once per
// device (coulomb_noalloc.cu). cudaErrorInvalidValue if doubles_needed
// exceeds the capacity.
cudaError_t noalloc_coulomb_scratch(size_t doubles_needed, double** out);
// tensor-core exchange tiles (k_tc.cu): off-diagonal element pairs only
cudaError_t launch_k_tiles_tc(const DevAtom& A, const DevScratch& S, const DevTC& T, bool symmetric, double* K,
                              cudaStream_t st);
cudaError_t launch_k_diag_tc(const DevAtom& A, const DevScratch& S, const DevTC& T, bool symmetric, double* K,
                             cudaStream_t st);
cudaError_t launch_tk_digits(const DevAtom& A, int mtiles, int ksteps, unsigned char* out, int* rowexp,
                             cudaStream_t st);
// tensor-core probe (tc_probe.cu)
cudaError_t tc_selftest(const float* A, const float* B, float* D, int N, int ksteps, int a_mn, int b_mn, int swap,
                        int* timed_out);
cudaError_t tc_peak(int ctas_per_sm, int iters, double* tflops, double* ms, int* timed_out);

// launchers (jk_fp64.cu)
cudaError_t launch_coulomb_fp64(const DevAtom& A, const DevScratch& S, const double* P, double* J,
                                bool zero_output, cudaStream_t st, Profiler* prof = nullptr);
// range-separated exchange with the erfc kernel: tk = the pair tables
// [((L*nel + a)*nel + b)*n2*n2 + t + v*n2] (general mode, every pair)
cudaError_t launch_exchange_erfc(const DevAtom& A, const DevScratch& S, const double* tk, const double* P, double* K,
                                 cudaStream_t st, Profiler* prof = nullptr);
// the same J in float pairs (needs jket_coef2, jbra_coef2, cholp2, rs2, rb2)
// P(r, c) = P(c, r) wherever r / bw < c / bw (upper part of a symmetric
// matrix from its lower column blocks of width bw)
cudaError_t launch_mirror_blocks(double* P, int n, int bw, cudaStream_t st);
cudaError_t launch_coulomb_split(const DevAtom& A, const DevScratch& S, const double* P, double* J,
                                bool zero_output, cudaStream_t st, Profiler* prof = nullptr);
cudaError_t launch_exchange_fp64(const DevAtom& A, const DevScratch& S, const KUnits& U, const double* P,
                                 double* K, bool symmetric, cudaStream_t st, Profiler* prof = nullptr);
// split-precision exchange (float-float on the FP32 pipe, FP64 recombination)
// tc != nullptr: the off-diagonal element pairs run on the tensor cores (k_tc.cu)
// a second stream with a fork and a join event (owned by the caller)
struct SideStream {
  cudaStream_t s = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
};
// side (tensor-core form only): the diagonal tiles run on side->s,
// concurrently with the off-diagonal ones, joined back before the fix-up
cudaError_t launch_exchange_split(const DevAtom& A, const DevScratch& S, const KUnits& U, const double* P,
                                  double* K, bool symmetric, cudaStream_t st, Profiler* prof = nullptr,
                                  const DevTC* tc = nullptr, const SideStream* side = nullptr);

}  // namespace hfg

/*
 * helfem_gb300 — C ABI of the GB300 Fock-build engine for HelFEM's atomic
 * finite-element basis.
 *
 * This is the drop-in boundary. The reference exposes the path as C++ member
 * functions (no plugin ABI); each entry point below names the reference
 * interface it replaces. include/helfem_gb300/TwoDBasis.hpp re-exposes the
 * reference's C++ signatures on top of these calls.
 *
 * Conventions
 *   - Matrices are FP64, column-major, nbf x nbf, AO index = iang*Nrad + irad
 *     with the angular order of the reference's angular_basis
 *     (src/atomic/basis.cpp:179-203: |m| outer, l inner, +m before -m).
 *   - Functions return 0 (HFG_OK) or an error code and never throw or abort.
 *     hfg_last_error() returns a message for the last failure on the calling
 *     thread.
 *   - Entry points taking a `stream` expect DEVICE pointers on the current
 *     CUDA device and enqueue work on `stream` (a cudaStream_t; NULL is the
 *     legacy default stream). They return without synchronising.
 *   - The *_host variants take HOST pointers, copy in and out through the
 *     handle's own stream and return after the result is on the host (the
 *     reference's value semantics).
 *   - A handle keeps per-handle device scratch: calls on one handle must not
 *     overlap in time (issue them on one stream or serialise them). Distinct
 *     handles are independent.
 */
#ifndef HELFEM_GB300_H
#define HELFEM_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int hfg_status;
enum {
  HFG_OK = 0,
  HFG_ERR_ARG = 1,       /* invalid argument (shape, range, null pointer)  */
  HFG_ERR_CUDA = 2,      /* CUDA runtime / driver failure                   */
  HFG_ERR_STATE = 3,     /* handle not ready (e.g. integrals not computed)  */
  HFG_ERR_NOMEM = 4,     /* host or device allocation failed                */
  HFG_ERR_INTERNAL = 5   /* anything else                                   */
};

typedef struct hfg_atom hfg_atom;

/* Description of an atomic basis. Mirrors the arguments of the reference's
 * TwoDBasisT constructor (src/atomic/TwoDBasis.h:135-142; TwoDBasis.cpp:66-94)
 * for a point nucleus and LIP elements on Gauss-Lobatto nodes (primbas 4,
 * libhelfem/src/PolynomialBasis.cpp:51-59). */
typedef struct {
  int Z;               /* nuclear charge                                    */
  int nnodes;          /* LIP nodes per element, 3..17                       */
  int nquad;           /* radial DFT points per element; 0 -> 5*nnodes       */
  int nelem;           /* number of radial elements                          */
  const double* bval;  /* nelem+1 element boundaries, bval[0] = 0            */
  int nang;            /* number of angular functions                        */
  const int* lval;     /* [nang] l of each angular function                  */
  const int* mval;     /* [nang] m of each angular function                  */
  double chol_tol;     /* pivoted-Cholesky tolerance; 0 -> 1e-12 (reference) */
  int host_only;       /* 0: device handle; the in-element two-electron
                             factors and exchange tensor are tabulated on
                             the GPU (rs/rb, one-electron and coupling
                             tables on the host);
                          1: tabulate on the host only and never touch a GPU;
                             the device entry points then fail with
                             HFG_ERR_STATE (for CPU-side checks);
                          2: device handle with every table tabulated on
                             the host and uploaded                          */
} hfg_atom_desc;

typedef struct {
  int nrad;   /* radial functions: nelem*(nnodes-1)-1 */
  int nang;
  int nbf;    /* nang*nrad */
  int nelem;
  int nnodes;
  int NL;     /* multipoles L = 0..NL-1, NL = 2*max(l)+1 */
  int rmax;   /* largest in-element Cholesky rank */
} hfg_atom_dims_t;

/* Message for the last failure on the calling thread ("" if none). */
const char* hfg_last_error(void);

/* Fill bval with grid::get_grid (libhelfem/include/grid.h:37-101): igrid
 * 1 linear, 2 quadratic, 3 polynomial, 4 exponential, 5 geometric.
 * bval has nelem+1 entries. */
hfg_status hfg_grid(double rmax, int nelem, int igrid, double zexp, double* bval);

/* Angular basis of the reference (src/atomic/basis.cpp:179-203). Call with
 * lval = mval = NULL to get the count in *nang. */
hfg_status hfg_angular_basis(int lmax, int mmax, int* nang, int* lval, int* mval);

/* Build the basis and its two-electron integral caches on the host in FP64
 * and upload them to the current device. Replaces the TwoDBasisT
 * constructor followed by compute_tei(bool) (src/atomic/TwoDBasis.h:180-181,
 * TwoDBasis.cpp:708-735): disjoint r^L / r^-L-1 factors
 * (libhelfemqc/include/CoulombExchangeFE.h:180-217) and pivoted-Cholesky
 * factors of the in-element tensors (libhelfem/src/RadialBasis.cpp:643-716). */
hfg_status hfg_atom_create(const hfg_atom_desc* desc, hfg_atom** out);
hfg_status hfg_atom_destroy(hfg_atom* atom);
hfg_status hfg_atom_get_dims(const hfg_atom* atom, hfg_atom_dims_t* dims);

/* One-electron matrices, host output nbf x nbf. Replace TwoDBasisT::overlap,
 * kinetic, nuclear (src/atomic/TwoDBasis.h:201-207; point nucleus). */
hfg_status hfg_overlap(const hfg_atom* atom, double* S);
hfg_status hfg_kinetic(const hfg_atom* atom, double* T);
hfg_status hfg_nuclear(const hfg_atom* atom, double* V);
/* Cached radial tables of multipole L and element iel, in the reference's
 * compact layout (Ni x Ni; Cholesky factor Ni^2 x rank, pair index a + b*Ni,
 * CoulombExchangeFE.h:471-477). Any output may be NULL; rbig is zero for
 * iel = 0 (never used there). For checking against an independent
 * tabulation. On a device-tabulated handle the factors are copied from the
 * device on the first call. */
hfg_status hfg_atom_radial_tables(const hfg_atom* atom, int L, int iel, int* ni, double* rsmall,
                                  double* rbig, int* rank, double* chol);

/* Gaunt coefficient coeff(L,M,l,m,lp) = int Y_L^M* Y_l^m Y_lp^(M-m), the
 * value of GauntT<double>::coeff (src/general/gaunt.cpp:201-251). */
hfg_status hfg_gaunt(int L, int M, int l, int m, int lp, double* value);

/* ---- Fock-build hot path (device pointers, asynchronous on `stream`) ---- */

/* J(P): replaces TwoDBasisT::coulomb (src/atomic/TwoDBasis.cpp:773-877).
 * J is overwritten (zero outside the element-diagonal tiles). */
hfg_status hfg_coulomb(hfg_atom* atom, const double* P, double* J, void* stream);

/* hfg_coulomb with options. HFG_COULOMB_SPLIT: the same J in float pairs
 * (the FP64 pipe bounds the FP64 form on GB300): the density is split into
 * hi + lo with integer operations, the in-element factor and the radial
 * tables are float-pair copies (the factor's copy is made on the first
 * call), products are error-free, long sums renormalised every step, one FP64
 * conversion per output element; relative error ~1e-14 against FP64,
 * reported by the tests and the benchmark. */
#define HFG_COULOMB_SPLIT 4
hfg_status hfg_coulomb_ex(hfg_atom* atom, const double* P, double* J, int flags, void* stream);

/* F += J(P): the same build accumulated into an existing matrix, for
 * Fock assembly without a separate J buffer. */
hfg_status hfg_coulomb_acc(hfg_atom* atom, const double* P, double* F, void* stream);

/* K(P) for a spin density P, returned with the reference's sign (the matrix
 * that is ADDED to the Fock matrix): replaces TwoDBasisT::exchange
 * (src/atomic/TwoDBasis.cpp:879-999), including its density-block screening
 * (blocks with Frobenius norm < 10*DBL_EPSILON are skipped). K is
 * overwritten. */
hfg_status hfg_exchange(hfg_atom* atom, const double* P, double* K, void* stream);

/* hfg_exchange with options. HFG_EXCHANGE_SYMMETRIC: the caller guarantees
 * P = P^T (every density matrix is); K is then symmetric and only half of
 * the element-pair tiles are computed, each written with its transposed
 * partner (about half the FP64 work). The result for a non-symmetric P is
 * undefined under this flag. */
#define HFG_EXCHANGE_SYMMETRIC 1
/* HFG_EXCHANGE_SPLIT: split-precision form. Each FP64 density element and
 * integral is split into two FP32 pieces (hi + lo, ~48 significant bits);
 * the contractions run on the FP32 pipe with error-free products and sums
 * and are recombined in FP64 (relative error ~1e-14 against FP64; reported
 * by the tests and the benchmark). Allocates an nbf^2 float2 density copy
 * on the first call. */
#define HFG_EXCHANGE_SPLIT 2
hfg_status hfg_exchange_ex(hfg_atom* atom, const double* P, double* K, int flags, void* stream);

/* Autotuner of the exchange work partition: times the tile kernels (form
 * given by flags) on a synthetic density with every block active for
 * candidate partitions and keeps the fastest for the later calls of this
 * handle: output-block ranges per element pair (plain and float-pair
 * forms), or groups of 8 output blocks per element-pair unit (the
 * tensor-core split form). Synchronous; K does not change, bit for bit. */
hfg_status hfg_atom_autotune(hfg_atom* atom, int flags, int* best_nsplit, double* best_ms);
/* Set the exchange work partition directly (the value hfg_atom_autotune
 * picks; it sets both partitions): 0 = automatic. */
hfg_status hfg_atom_set_partition(hfg_atom* atom, int nsplit);

/* Range-separated exchange with the Yukawa kernel e^{-lambda r12}/r12.
 * hfg_atom_compute_yukawa replaces TwoDBasisT::compute_yukawa
 * (src/atomic/TwoDBasis.cpp:736-758): the screened disjoint factors
 * int B B i_L(lambda r), int B B k_L(lambda r) (modified spherical Bessel
 * functions, libhelfem/include/math.h:48-110) and the pivoted-Cholesky
 * in-element tensors of the screened kernel, built on the host in FP64 and
 * uploaded; calling it again replaces lambda. hfg_rs_exchange replaces
 * TwoDBasisT::rs_exchange (src/atomic/TwoDBasis.cpp:1001-1131) for that
 * kernel: the same sign, screening and flags as hfg_exchange_ex; before
 * compute_yukawa it fails with HFG_ERR_STATE. (The erfc kernel of
 * compute_erfc: hfg_atom_compute_erfc below.) */
hfg_status hfg_atom_compute_yukawa(hfg_atom* atom, double lambda);
/* The screened tables of multipole L and element iel as stored (padded
 * nnodes x nnodes; r_small carries (2L+1) lambda so that the bare coupling
 * factor 4 pi/(2L+1) becomes 4 pi lambda; tk is the exchange-ordered
 * in-element tensor nnodes^2 x nnodes^2, same factor). Any output may be
 * NULL. Works on host-only handles (for checking). */
hfg_status hfg_atom_yukawa_tables(const hfg_atom* atom, int L, int iel, double* rsmall, double* rbig, double* tk);
hfg_status hfg_rs_exchange(hfg_atom* atom, const double* P, double* K, int flags, void* stream);
hfg_status hfg_rs_exchange_host(hfg_atom* atom, const double* P, double* K, int flags);

/* Range-separated exchange with the erfc kernel: hfg_atom_compute_erfc
 * replaces TwoDBasisT::compute_erfc (src/atomic/TwoDBasis.cpp:760-771,
 * CoulombExchangeFE.h:275-295): erfc(mu r12)/r12 expanded in Legendre
 * polynomials after Angyan, Gerber and Marsman (libhelfem/src/erfc_expn.cpp)
 * and integrated on the radial basis's Gauss-Chebyshev rule, one dense table
 * per element pair and multipole (RadialBasis.cpp:742-811), formed on the
 * host and kept on the device (NL nel^2 nn^4 doubles). After it,
 * hfg_rs_exchange / hfg_rs_exchange_host evaluate the erfc-kernel exchange
 * (same sign and spin-density convention as hfg_exchange; FP64;
 * HFG_EXCHANGE_SPLIT is refused) until hfg_atom_compute_yukawa is called.
 * flags: HFG_ERFC_EXACT_BINOMIAL uses the generalised binomial coefficient
 * in the short-range series of the expansion instead of the reference's
 * rule for negative arguments (which deviates from the exact Legendre
 * coefficients by up to ~1.5e-6 relative at arguments below 1 and ~1e-3 at
 * mu r> = 5-6 with mu r< near 0.4, where the kernel is small); the default
 * keeps the reference's numbers.
 * hfg_atom_erfc_table copies the nn^2 x nn^2 table of (L, iel, kel):
 * out[t + v nn^2] = mu (ij|kl), t = j + k nn, v = i + l nn. */
#define HFG_ERFC_EXACT_BINOMIAL 1
hfg_status hfg_atom_compute_erfc(hfg_atom* atom, double mu, int flags);
hfg_status hfg_atom_erfc_table(const hfg_atom* atom, int L, int iel, int kel, double* out);

/* Spherically averaged atom: replaces sadatom::basis::TwoDBasis
 * (src/sadatom/basis.h:25-130) for its Fock build. The basis is the radial
 * FE basis with one channel per l = 0..lmax; densities and results are
 * l-channel matrices, nrad x nrad column-major, one slice per channel one
 * after the other ((lmax+1) nrad^2 doubles), host or device pointers.
 *   hfg_sadatom_coulomb:  J = 4 pi J_0[P] for the radial density P (one
 *                         slice in, one out; basis.cpp:186-207)
 *   hfg_sadatom_exchange: K[l_out] = -sum_L K_L[sum_l_in (4 pi/(2L+1))
 *                         c(l_out, l_in, L) P[l_in]], c = (2 l_out + 1)^-1
 *                         sum_{m_out, m_in} Gaunt(l_out, m_out, L,
 *                         m_out - m_in, l_in)^2 (basis.cpp:209-312); flags
 *                         as hfg_exchange_ex
 *   hfg_sadatom_rs_exchange: the same with the range-separated kernel of
 *                         hfg_atom_compute_yukawa / hfg_atom_compute_erfc on
 *                         this handle (basis.cpp:314-429)
 * The caller scales densities as the reference's SCF does
 * (src/sadatom/scf.cpp:199-233). The handle is an hfg_atom (dims, destroy,
 * compute_yukawa / compute_erfc work as for atoms, its full-matrix J/K
 * entries act on the block-diagonal (l, 0) matrix); hfg_scf_run and the
 * atomic XC grid refuse it (its XC is hfg_sadatom_xc below). */
typedef struct {
  int Z;               /* nuclear charge                                    */
  int nnodes;          /* LIP nodes per element, 3..17                       */
  int nquad;           /* radial quadrature points per element; 0 -> 5*nnodes */
  int nelem;           /* number of radial elements                          */
  const double* bval;  /* nelem+1 element boundaries, bval[0] = 0            */
  int lmax;            /* highest channel, 0..3                              */
  double chol_tol;     /* pivoted-Cholesky tolerance; 0 -> 1e-12             */
  int host_only;       /* as hfg_atom_desc                                   */
} hfg_sadatom_desc;
hfg_status hfg_sadatom_create(const hfg_sadatom_desc* desc, hfg_atom** out);
hfg_status hfg_sadatom_coulomb(hfg_atom* atom, const double* P, double* J, void* stream);
hfg_status hfg_sadatom_exchange(hfg_atom* atom, const double* P, double* K, int flags, void* stream);
hfg_status hfg_sadatom_rs_exchange(hfg_atom* atom, const double* P, double* K, int flags, void* stream);
hfg_status hfg_sadatom_coulomb_host(hfg_atom* atom, const double* P, double* J);
hfg_status hfg_sadatom_exchange_host(hfg_atom* atom, const double* P, double* K, int flags);
hfg_status hfg_sadatom_rs_exchange_host(hfg_atom* atom, const double* P, double* K, int flags);
/* XC of the spherically averaged atom (src/sadatom/dftgrid.cpp:256-459 with
 * the SCF's scaling, scf.cpp:163-192): Pa (Pb) the radial density matrix,
 * nrad x nrad, total (Pb NULL) or per spin; Ha (Hb) receives the XC block
 * every channel adds to its Fock matrix, int B_a B_b v_xc(r) dr, the block
 * that makes a closed-shell atom's spherically averaged and m-resolved
 * solutions coincide. Functionals, energies and thr as hfg_xc. Evaluated on
 * an s-only basis over the same radial grid, built on first use. */
hfg_status hfg_sadatom_xc(hfg_atom* atom, int x_func, int c_func, const double* Pa, const double* Pb, double* Ha,
                          double* Hb, double* energies, double thr, void* stream);
hfg_status hfg_sadatom_xc_host(hfg_atom* atom, int x_func, int c_func, const double* Pa, const double* Pb,
                               double* Ha, double* Hb, double* Exc, double* Nel, double thr);

/* J(P) like hfg_coulomb, but allocation-free at every call: its scratch is a
 * fixed 4 MiB array in the library's static device memory rather than the
 * handle's buffers. No counterpart in the reference; it exists for callers
 * whose per-call path cannot allocate device memory (a host framework that
 * owns every device allocation and hands the library a fixed budget, or a
 * loop that must not risk an allocation's implicit synchronisation or its
 * failure).
 * Atoms needing more than 4 MiB of Coulomb scratch
 * (channels * elements * (nnodes^2 + 2) doubles) are rejected with
 * HFG_ERR_ARG. All calls share the one array: calls that overlap on the GPU
 * race and must be serialised by the caller. The first call on each device
 * resolves the array's device address; make it before any stream capture. */
hfg_status hfg_coulomb_noalloc(hfg_atom* atom, const double* P, double* J, void* stream);

/* ---- tensor-core probe (no counterpart in the reference) ----
 * hfg_tc_selftest: D (128 x N, row-major, host) = A B^T with A 128 x K and
 * B N x K (row-major host floats, K = 16 ksteps, 1 <= ksteps <= 8,
 * N in 16..256 step 16), the operands rounded to bf16 and staged in shared
 * memory in this library's tcgen05 operand layouts (a_mn_major /
 * b_mn_major: MN-major instead of K-major), accumulated in FP32 in tensor
 * memory. swap_offsets exchanges the two core-matrix strides of the
 * descriptors (a diagnostic: the product is then wrong). For integer
 * operands with exactly representable sums the result is exact.
 * hfg_tc_peak: dense bf16 MMA rate (M = 128, N = 256, K = 16 back to back
 * on resident operands, ctas_per_sm in 1..2), TFLOP/s and milliseconds. */
hfg_status hfg_tc_selftest(const float* A, const float* B, float* D, int N, int ksteps, int a_mn_major,
                           int b_mn_major, int swap_offsets);
hfg_status hfg_tc_peak(int ctas_per_sm, int iters, double* tflops, double* ms);

/* ---- XC potential on the atomic DFT grid ----
 * Replaces DFTGrid::eval_Fxc (src/atomic/dftgrid.h:156-159,
 * src/atomic/dftgrid.cpp:591-712) with functionals restated from the papers
 * (libxc ids: 1 lda_x, 7 lda_c_vwn (VWN5), 12 lda_c_pw (PW92), 101 gga_x_pbe,
 * 130 gga_c_pbe; 0 = none). External functional parameters are not
 * supported. Restricted: Pb == NULL, Pa is the total density and Ha the XC
 * potential matrix. Unrestricted: spin densities Pa, Pb -> Ha, Hb. Ha/Hb are
 * overwritten. `energies` (device, 2 doubles, may be NULL) receives
 * {Exc, electron count on the grid}. thr is the density threshold
 * (reference default 1e-12). */
/* (Re)build the grid: ldft cos(theta) points x mdft phi points per element
 * (0 -> the reference defaults 4*lmax+12, 4*mmax+12; src/atomic/main.cpp:329-331).
 * Called implicitly with the defaults by the first XC call. */
hfg_status hfg_dft_grid(hfg_atom* atom, int ldft, int mdft);
hfg_status hfg_xc(hfg_atom* atom, int x_func, int c_func, const double* Pa, const double* Pb, double* Ha,
                  double* Hb, double* energies, double thr, void* stream);
hfg_status hfg_xc_host(hfg_atom* atom, int x_func, int c_func, const double* Pa, const double* Pb, double* Ha,
                       double* Hb, double* Exc, double* Nel, double thr);

/* ---- Fock diagonalisation step ----
 * Per symmetry block (symmetry 1: one block per m, unique m ascending;
 * 2: one block per angular function) the orthonormal Fock block
 * F'_k = X_k^T F X_k with the reference's symmetric orthonormaliser
 * (scf_driver_common.h:176-187, 432-445; utils.cpp:120-159), its eigenpairs
 * and the AO coefficients C_k = X_k V (scf_helpers.cpp:41-50 eig_gsym).
 * F, C (nbf x nbf) and eps (nbf) are device pointers; eps holds the blocks'
 * eigenvalues in block order, ascending within a block, and column j of C is
 * the orbital of eps[j] (zero outside its block's rows). C^T S C = 1. */
hfg_status hfg_fock_diag(hfg_atom* atom, const double* F, int symmetry, double* C, double* eps, void* stream);

/* J(PJ) and K(PK) on the device in one call (the Fock builder's pair of
 * calls, src/atomic/main.cpp:424-443): the Coulomb build runs on a second
 * stream of the handle, forked from `stream` after the work already queued
 * there and joined back into it, concurrently with the exchange build on
 * `stream`; when the call returns, work queued later on `stream` sees both
 * results. flags: HFG_EXCHANGE_SYMMETRIC and HFG_EXCHANGE_SPLIT for K,
 * HFG_COULOMB_SPLIT for J. PJ and PK may be the same pointer; J and K must
 * not overlap. Calls on one handle must not overlap in time (the second
 * stream and the scratch are per handle). */
hfg_status hfg_jk(hfg_atom* atom, const double* PJ, const double* PK, double* J, double* K, int flags, void* stream);

/* ---- host-pointer drop-ins (value semantics, synchronous) ----
 * Under HFG_EXCHANGE_SYMMETRIC a density is read from the host as its lower
 * column blocks only (16 blocks of columns, each from its first column's
 * row down: about 53 % of the matrix) and the rest is mirrored on the
 * device: the flag already promises P = P^T. In hfg_jk_host that applies to
 * PJ only when it is the same pointer as PK. */
hfg_status hfg_coulomb_host(hfg_atom* atom, const double* P, double* J);
hfg_status hfg_exchange_host(hfg_atom* atom, const double* P, double* K);
/* hfg_exchange_host with the hfg_exchange_ex flags (symmetric / split). */
hfg_status hfg_exchange_host_ex(hfg_atom* atom, const double* P, double* K, int flags);
/* J(PJ) and K(PK) in one call (the Fock builder's pair of calls,
 * src/atomic/main.cpp:424-443): the density is staged once when PK == PJ
 * (same pointer), and J is copied back on a second stream while K is built.
 * flags as hfg_exchange_ex for K, plus HFG_COULOMB_SPLIT for J. */
hfg_status hfg_jk_host(hfg_atom* atom, const double* PJ, const double* PK, double* J, double* K, int flags);
/* Bytes the last host-pointer J/K call on this handle copied host to device
 * and device to host. */
hfg_status hfg_host_copy_bytes(const hfg_atom* atom, size_t* h2d, size_t* d2h);

/* Algorithmic work of one J and one K build on this basis with every density
 * block active (the unit counts behind roofline figures). FLOPs count one
 * fused multiply-add as two; recoupling FLOPs are the Gaunt-weighted sums of
 * density tiles, transform FLOPs the r_small/r_big products (off-diagonal
 * element pairs) and the in-element tensor contraction (diagonal elements).
 * Bytes are the minimal HBM traffic: read P, write the output. */
typedef struct {
  double k_offdiag_flops;  /* element pairs a != b: recoupling + A X B^T     */
  double k_diag_flops;     /* element pairs a == b: recoupling + tensor      */
  double k_offdiag_sym_flops; /* the same under HFG_EXCHANGE_SYMMETRIC       */
  double k_diag_sym_flops;
  double k_bytes;          /* 8*nbf^2 (read P) + 8*nbf^2 (write K)           */
  double j_flops;
  double j_bytes;          /* element-diagonal tiles of P read, J band written */
  int n_k_entries;         /* (jang,kang,L) transforms                        */
  int n_k_terms;           /* recoupling terms over all entries               */
} hfg_work_t;
hfg_status hfg_atom_work(const hfg_atom* atom, hfg_work_t* work);
/* bf16 tensor-core FLOPs (digit-plane MMAs) one split-precision exchange
 * issues with every exchange entry active: the executed tensor work that the
 * roofline of the split form is measured against (0 when the handle runs the
 * float-pair form). No counterpart in the reference. */
hfg_status hfg_atom_tc_work(const hfg_atom* atom, int symmetric, double* mma_flops);

/* ---- atomic SCF on the device ----
 * The Fock-builder loop of the reference's atomic driver
 * (src/atomic/main.cpp:369-470) with per-symmetry-block orthonormalisation
 * and diagonalisation (src/general/scf_driver_common.h:176-187, 406-520) and
 * the energy decomposition (main.cpp:410-446). Convergence: Pulay DIIS in
 * the orthonormal basis (the reference delegates to OpenOrbitalOptimizer;
 * converged energies do not depend on the accelerator). Core-Hamiltonian
 * guess. Energies in hartree. */
typedef struct {
  int nela, nelb;          /* alpha / beta electrons                          */
  int restricted;          /* 1: closed-shell P (max occupation 2)            */
  int symmetry;            /* 1: blocks per m (reference default), 2: per (l,m) */
  int x_func, c_func;      /* XC functional ids (0, 0 = Hartree-Fock)         */
  double kfrac;            /* exact-exchange fraction; < 0 -> 1 for HF, 0 for DFT */
  int maxiter;             /* 0 -> 200                                        */
  double e_tol;            /* |dE| convergence; 0 -> 1e-10                    */
  double diis_tol;         /* max |F'D' - D'F'|; 0 -> 1e-7, or below 1e-5 with
                              the energy stable for three iterations; > 0:
                              required as given                            */
  const int* fixed_occ;    /* NULL: Aufbau; else [n_fixed_blocks][2] (alpha, beta)
                              electrons per block, blocks in ascending m (the
                              reference's --readocc)                           */
  int n_fixed_blocks;
  double dftthr;           /* density threshold; 0 -> 1e-12                   */
  int frac_aufbau;         /* 1: electrons that only partly fill a degenerate
                              frontier shell are shared equally over it
                              (spherically averaged open shells); 0: integer
                              Aufbau as the reference                         */
  int split_exchange;      /* 1: exchange in the split-precision form          */
  const double* l_occ;     /* NULL, or (symmetry 2) [n_l_occ][2] alpha/beta
                              electrons per l, shared equally over its 2l+1
                              m blocks and filled lowest-first within a block
                              (spherically averaged fixed occupations)      */
  int n_l_occ;
} hfg_scf_desc;
typedef struct {
  double Etot, Ekin, Enuc, Ecoul, Exx, Exc, Nel_grid;
  int iterations, converged;
  /* wall milliseconds per phase over all iterations: 0 Fock build, 1 energies,
   * 2 orthonormal blocks + DIIS errors, 3 DIIS extrapolation,
   * 4 eigensolves + occupations, 5 density */
  double phase_ms[6];
} hfg_scf_result;
/* orbital_energies (host, may be NULL): nbf per spin, blocks concatenated in
 * block order, ascending within a block. Runs on `stream` (NULL: the
 * handle's stream) and returns when converged or out of iterations. */
hfg_status hfg_scf_run(hfg_atom* atom, const hfg_scf_desc* desc, hfg_scf_result* result,
                       double* orbital_energies, void* stream);

/* ---- batched / serving runtime ----
 * Many atomic SCF solves on one GPU: worker threads, one CUDA stream each,
 * run whole solves (tabulation, upload, device SCF) concurrently.
 * A queued job starts when its estimated device footprint fits in the HBM
 * budget still free (first fitting job in arrival order). The reference has
 * no counterpart (one atom per process); this serves the batched and
 * streaming configurations. */
typedef struct hfg_engine hfg_engine;
typedef struct {
  int status;               /* 0 queued, 1 running, 2 done (converged),
                               3 failed: an error, or an SCF that did not
                               converge (scf then holds its last iterate)  */
  hfg_scf_result scf;
  double queue_ms;          /* submit -> start                                 */
  double setup_ms;          /* host tabulation + upload                        */
  double scf_ms;            /* device SCF                                      */
  double total_ms;          /* submit -> result                                */
  double footprint_bytes;   /* admission estimate                              */
  char error[256];          /* failure message (status 3)                      */
} hfg_job_result;
hfg_status hfg_engine_create(int n_workers, double hbm_budget_gb, hfg_engine** out);
/* copies the descriptions (and their arrays); returns at once */
hfg_status hfg_engine_submit(hfg_engine* e, const hfg_atom_desc* atom, const hfg_scf_desc* scf,
                             unsigned long long* job_id);
/* waits up to timeout_s (< 0: no limit); a finished job's result is returned
 * once and then forgotten; status < 2 means it is still pending. Several
 * threads may wait on the same id: one receives the result, the others an
 * error. */
hfg_status hfg_engine_wait(hfg_engine* e, unsigned long long job_id, double timeout_s, hfg_job_result* out);
hfg_status hfg_engine_stats(hfg_engine* e, int* queued, int* running, double* in_use_gb);
/* cancels queued jobs, waits for running ones and for every thread inside
 * hfg_engine_wait to return, then frees the engine */
hfg_status hfg_engine_destroy(hfg_engine* e);

/* ---- per-kernel timing (counterpart of the reference's scf_driver::FockTimer,
 * src/general/scf_driver_common.h:69-170) ----
 * Kernel classes: 0 J contraction, 1 J scatter, 2 K block norms,
 * 3 K element-pair tiles, 4 K boundary fix-up.
 * hfg_profile_enable(atom, capacity) brackets each of the next `capacity`
 * launches on this handle with CUDA events on the launch stream (0 turns
 * timing off). hfg_profile_read waits for the recorded events and returns
 * per-class launch counts and total milliseconds; reset != 0 clears them. */
#define HFG_NUM_KERNEL_CLASSES 5
typedef struct {
  int launches[HFG_NUM_KERNEL_CLASSES];
  double ms[HFG_NUM_KERNEL_CLASSES];
} hfg_profile_t;
hfg_status hfg_profile_enable(hfg_atom* atom, int capacity);
/* Only the kernel classes whose bit (1 << class, the hfg_profile_t order) is
 * set in mask are bracketed from now on (default: all); fewer events on the
 * stream between the launches of a timed region. */
hfg_status hfg_profile_classes(hfg_atom* atom, unsigned mask);
hfg_status hfg_profile_read(hfg_atom* atom, hfg_profile_t* out, int reset);

/* ======================================================================
 * Diatomic molecules (prolate spheroidal coordinates mu, nu, phi):
 * src/diatomic/basis.{h,cpp}. Matrices are over the PURE basis (the
 * reference's Nbf(): every m != 0 shell drops its mu = 0 radial function,
 * basis.cpp:712-736), FP64 column-major, with the angular order of
 * lm_to_l_m (basis.cpp:456-471: |m| outer, l inner, +m before -m).
 * ====================================================================== */
typedef struct hfg_diatomic hfg_diatomic;

typedef struct {
  int Z1, Z2;            /* nuclear charges (Z2 = 0: a dummy centre)       */
  double Rhalf;          /* half bond length, bohr                         */
  int nnodes;            /* LIP nodes per mu element (3..17)               */
  int nelem;             /* mu elements                                    */
  const double* bval;    /* nelem+1 boundaries in mu, bval[0] = 0          */
  int nang;              /* angular functions                              */
  const int* lval;       /* [nang]                                         */
  const int* mval;       /* [nang]                                         */
  double cd_thresh;      /* in-element factor threshold (<= 0: 1e-12)      */
  int host_only;         /* 0: device handle, two-electron primitives      *
                          *    tabulated on the device; 1: host tables      *
                          *    only, no device state; 2: device handle,     *
                          *    host tabulation uploaded                     */
} hfg_diatomic_desc;

typedef struct {
  int nrad, nang, nel, nnodes, ndummy, nbf, nlm, Lmax, rmax, nchan, nent;
} hfg_diatomic_dims_t;

/* Replaces the TwoDBasis constructor + compute_tei (basis.cpp:522-645,
 * 1382-1548): tabulates the disjoint P/Q integrals and the sign-carrying
 * factor of the 2-channel in-element kernel, on the device (host_only 0)
 * or on the host with an upload (host_only 2). The two agree to rounding;
 * a device-tabulated factor stays on the device (hfg_diatomic_tables
 * copies the requested one back). */
hfg_status hfg_diatomic_create(const hfg_diatomic_desc* desc, hfg_diatomic** out);
hfg_status hfg_diatomic_destroy(hfg_diatomic* d);
hfg_status hfg_diatomic_get_dims(const hfg_diatomic* d, hfg_diatomic_dims_t* dims);
/* dummy index (iang*Nrad + irad) of each pure function, [nbf] */
hfg_status hfg_diatomic_pure_indices(const hfg_diatomic* d, int* idx);

/* One-electron matrices (host, nbf x nbf): overlap, kinetic, nuclear
 * (basis.cpp:1033-1140, point nuclei). */
hfg_status hfg_diatomic_overlap(const hfg_diatomic* d, double* S);
hfg_status hfg_diatomic_kinetic(const hfg_diatomic* d, double* T);
hfg_status hfg_diatomic_nuclear(const hfg_diatomic* d, double* V);
/* The same restricted to one symmetry block (the pure functions with
 * m == mblock, in pure order): which 0 = S, 1 = T, 2 = V. *n receives the
 * block size; out may be NULL to query it. */
hfg_status hfg_diatomic_one_electron_block(const hfg_diatomic* d, int which, int mblock, double* out, int* n);

/* Cached tables of multipole index ilm (the (L,|M|) list, |M|-major) and
 * element iel, padded nnodes x nnodes column-major (which 0..3 = P0, P2, Q0,
 * Q2: int B_a B_b sinh cosh^k P_L^|M|(cosh mu), k = 0, 2, and the same with
 * Q), or the in-element factor (which 4: (2 nnodes^2 x rank) with its signs
 * in sigma). L, M, rank and sigma may be NULL. For checking against an
 * independent tabulation. */
hfg_status hfg_diatomic_tables(const hfg_diatomic* d, int which, int ilm, int iel, int* L, int* M, int* rank,
                               double* out, double* sigma);

/* Associated Legendre functions P_L^M(cosh mu), Q_L^M(cosh mu) (Hobson
 * convention, src/legendre/Legendre.h), out[M*(Lmax+1) + L]. */
hfg_status hfg_legendre_pq(int Lmax, int Mmax, double mu, double* P, double* Q);
/* mod_coeff(lj,mj,L,M,li,mi) = int Y_lj^mj* cos^2(nu) Y_L^M Y_li^mi
 * (src/general/gaunt.cpp:254-275). */
hfg_status hfg_gaunt_mod(int lj, int mj, int L, int M, int li, int mi, double* value);

/* J(P) over the pure basis: replaces diatomic TwoDBasis::coulomb
 * (basis.cpp:1621-1815, boundary expansion and removal included). */
hfg_status hfg_diatomic_coulomb(hfg_diatomic* d, const double* P, double* J, void* stream);
/* K(P) for a spin density, with the reference's sign (added to F): replaces
 * diatomic TwoDBasis::exchange (basis.cpp:1817-2061), including its
 * density-block screening. flags: HFG_EXCHANGE_SYMMETRIC (P = P^T),
 * HFG_EXCHANGE_SPLIT (split precision as for atoms; the first split call
 * allocates float-pair copies of the tables and an ndummy^2 density copy),
 * HFG_EXCHANGE_ITEMWISE (split form only: the diagonal element tiles one
 * output block per work item inside the tile kernel, instead of in groups of
 * output blocks sharing each in-element kernel-table pass; the same K bit
 * for bit, slower; kept for comparison). */
#define HFG_EXCHANGE_ITEMWISE 4
hfg_status hfg_diatomic_exchange(hfg_diatomic* d, const double* P, double* K, int flags, void* stream);
/* host-pointer value-semantics variants */
hfg_status hfg_diatomic_coulomb_host(hfg_diatomic* d, const double* P, double* J);
hfg_status hfg_diatomic_exchange_host(hfg_diatomic* d, const double* P, double* K, int flags);

/* Algorithmic work of one exchange build given the density-block activity
 * (act[i + l*nang] != 0 for blocks above the screen; NULL = all active),
 * restricted to the output blocks with jk_mask[j + k*nang] != 0 (NULL = all):
 * FP64 flops of the off-diagonal element-pair contractions, of the in-element
 * blocks and of the recoupling, and the number of (output block, multipole)
 * entries evaluated. */
typedef struct {
  double k_offdiag_flops, k_diag_flops, k_recouple_flops, n_entries;
  double k_offdiag_sym_flops, k_diag_sym_flops, k_recouple_sym_flops, n_entries_sym;
} hfg_diatomic_work_t;
hfg_status hfg_diatomic_work(const hfg_diatomic* d, const unsigned char* act, const unsigned char* jk_mask,
                             hfg_diatomic_work_t* w);

/* XC potential on the pure-m diatomic DFT grid: replaces
 * helfem::diatomic::dftgrid_purem::PureMDFTGrid::eval_Fxc (both overloads,
 * src/diatomic/dftgrid_purem.h:154-161, dftgrid_purem.cpp:668-742), the XC
 * path the reference takes when the orbitals do not mix m (symmetry >= 1,
 * src/diatomic/main.cpp:319-330): the phi integral is analytic and only the
 * (m, m) blocks of the density and the potential enter. Functional ids, the
 * restricted/unrestricted convention, `energies` and thr are as in hfg_xc;
 * densities and potentials are in the pure basis (nbf x nbf, column-major)
 * and Ha/Hb are overwritten. */
/* (Re)build the grid: lang Chebyshev points in cos(nu) (0 -> 4*lmax+12,
 * src/diatomic/main.cpp:316) and 5*nnodes Chebyshev points in mu per
 * element (main.cpp:191). Called implicitly by the first XC call. */
hfg_status hfg_diatomic_dft_grid(hfg_diatomic* d, int lang);
hfg_status hfg_diatomic_xc(hfg_diatomic* d, int x_func, int c_func, const double* Pa, const double* Pb, double* Ha,
                           double* Hb, double* energies, double thr, void* stream);
hfg_status hfg_diatomic_xc_host(hfg_diatomic* d, int x_func, int c_func, const double* Pa, const double* Pb,
                                double* Ha, double* Hb, double* Exc, double* Nel, double thr);

#ifdef __cplusplus
}
#endif

#endif /* HELFEM_GB300_H */

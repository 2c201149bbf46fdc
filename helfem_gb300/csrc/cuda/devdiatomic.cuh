// Device-resident diatomic context shared by the diatomic Fock-build kernels.
//
// Radial layout: element e owns an nn x nn primitive tile; primitive p is the
// global function g(e,p) = e*(nn-1) + p, valid for g < nrad. Dummy AO index
// = iang*nrad + irad (nd = nang*nrad); the pure index of (s, g) is
// poff[s] + g - pstart[s] for g >= pstart[s] (m != 0 shells drop g = 0).
// Matrices are column-major FP64.
#pragma once

#include <cuda_runtime.h>

namespace hfg {

struct DevDiatomic {
  int nn, nel, nrad, nang, nd, nlm, rmax, Lmax, mmax, nM, nbf;
  const int* poff;       // [nang] pure index of (s, pstart[s])
  const int* pstart;     // [nang] first radial function of shell s in the pure basis
  // per (ilm, e) padded nn x nn tiles
  const double* p0;
  const double* p2;
  const double* q0;
  const double* q2;
  const double* cdB;     // [(ilm*nel+e)*2nn^2*rmax]
  const double* cds;     // [(ilm*nel+e)*rmax]
  const int* cdrank;     // [ilm*nel+e]
  const double* tx;      // [((ilm*nel+e)*4 + ab)*(nn^2)^2] exchange-ordered in-element kernel
  const double* lmfac;   // [ilm] 4 pi Rhalf^5 (L-|M|)!/(L+|M|)! (sign (-1)^M applied at use)
  // angular coupling table: (a, L, M) -> (b, c0 = cos^2 coupling, c2 = Gaunt)
  const int* al_ptr;
  const int* al_b;
  const double* al_c0;
  const double* al_c2;
  // Coulomb channels and bra lists
  int nchan;
  const int* ch_L;
  const int* ch_M;
  const int* ch_ilm;
  const double* ch_fac;
  const int* jbra_ptr;
  const int* jbra_chan;
  const double* jbra_c0;
  const double* jbra_c2;
  // exchange entries
  int nent;
  const int* kjk_ptr;    // [nang^2+1]
  const int* kent_L;
  const int* kent_Ma;
  const int* kent_ilm;
  const int* kent_jk;    // [nent] owning output block
  // element pairs: off-diagonal ordered pairs (a != b) and a < b pairs
  const int2* pairs_all;
  int npairs_all;
  const int2* pairs_sym;
  int npairs_sym;
  // split-precision copies: each FP64 value v as float2 (hi, lo), hi = fl32(v)
  const float2* p0s = nullptr;
  const float2* p2s = nullptr;
  const float2* q0s = nullptr;
  const float2* q2s = nullptr;
  const float2* txs = nullptr;
  const float2* al_c0s = nullptr;
  const float2* al_c2s = nullptr;
  const float2* lmfacs = nullptr;
  // P_L^|M| grows as e^{L mu} and Q_L^|M| decays as e^{-(L+1) mu}: beyond the
  // FP32 range at large L and mu. The split tables hold P * 2^-k and
  // Q * 2^+k with k = kexp[ilm*nel+e] (the exponent of the element's largest
  // P entry); an element pair (inner a, outer b) restores 2^(k_a - k_b) <= 1.
  const int* kexp = nullptr;
};

struct DevDiatomicScratch {
  double* jin;            // [nchan*nel*2*nn^2] in-element channel tiles, then the full channel tiles
  double* jscal;          // [nchan*nel*4]
  double* khalo;          // [nel*nel*nang^2*(2nn-1)]
  double* bnorm;          // [nang^2*DNORM_SPLIT]
  unsigned char* act;     // [nang^2] density block above the screen
  unsigned char* ent_act; // [nent]
  unsigned char* jk_act;  // [nang^2]
  int* jk_list;           // [2*nang^2]: active output blocks, then those with j <= k
  int* counts;            // [2]
  float2* pd2;            // [nd*nd] split copy of the density (split path)
};

#define DNORM_SPLIT 8

// pure-m DFT grid: nq mu points per element, na nu points, npair same-m
// unordered angular pairs (s <= t)
struct DevDiatomicXC {
  int nq = 0, na = 0, npair = 0;
  const int* ps = nullptr;     // [npair]
  const int* pt = nullptr;
  const double* mult = nullptr;  // 2 (s != t) or 1
  const double* W = nullptr;   // [k*na + a]: Y_s Y_t
  const double* Wt = nullptr;  //             Y_s' Y_t + Y_s Y_t'
  const double* R = nullptr;   // [(e*nq + q)*nn + p]
  const double* dR = nullptr;
  const double* w = nullptr;   // [(e*nq + q)*na + a]
  const double* hinv = nullptr;
  // Fock-side pairs: tiles built for pairs fk[0..nfock), each also written to
  // the mirror shells (fms, fmt) of opposite m when fms >= 0
  int nfock = 0;
  const int* fk = nullptr;
  const int* fms = nullptr;
  const int* fmt = nullptr;
};
struct DiatomicXcScratch {
  double* D;      // [nsd][nel][nq][npair]  mult * B^T P_st B
  double* Dr;     // same                   mult/2 * (dB^T P_st B + B^T P_st dB)
  double* F;      // [nout][3][nel][nq][na]
  double* U;      // [nout][3][nel][npair][nq]
  double* epart;  // [nel*nq][2]
};
// Pb == nullptr: restricted (Pa is the total density, Ha the potential).
// Densities and potentials are in the pure basis (nbf x nbf, column-major);
// H is overwritten. energies (device, may be null) receives {Exc, Nel}.
cudaError_t launch_diatomic_xc(const DevDiatomic& D, const DevDiatomicXC& X, const DiatomicXcScratch& S, int xid,
                               int cid, const double* Pa, const double* Pb, double* Ha, double* Hb, double* energies,
                               double thr, cudaStream_t st);

cudaError_t launch_diatomic_expand(const double* P, int nbf, const int* pure, double* Pd, int nd, cudaStream_t st);
cudaError_t launch_diatomic_gather(const double* Fd, int nd, const int* pure, int nbf, double* F, cudaStream_t st);
cudaError_t launch_diatomic_tx(const DevDiatomic& D, double* tx, cudaStream_t st);
// J of a pure-basis density, written to the pure-basis J (overwritten)
cudaError_t launch_diatomic_coulomb(const DevDiatomic& D, const DevDiatomicScratch& S, const double* P, double* J,
                                    cudaStream_t st);
cudaError_t launch_diatomic_exchange(const DevDiatomic& D, const DevDiatomicScratch& S, const double* Pd,
                                     double* Kd, bool symmetric, cudaStream_t st);
// split-precision exchange (float-float on the FP32 pipe, FP64 recombination);
// inline_diag: diagonal element tiles item by item inside the tile kernel
// instead of the grouped kernel (bitwise the same K)
cudaError_t launch_diatomic_exchange_split(const DevDiatomic& D, const DevDiatomicScratch& S, const double* Pd,
                                           double* Kd, bool symmetric, cudaStream_t st, bool inline_diag = false);
// txs[i] = split(tx[i])
cudaError_t launch_diatomic_split_tx(const double* tx, float2* txs, size_t n, cudaStream_t st);

}  // namespace hfg

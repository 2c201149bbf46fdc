// Plain-FP64 Coulomb (J) and exchange (K) builds for the atomic FE basis.
//
// J restates TwoDBasisT::coulomb (src/atomic/TwoDBasis.cpp:773-877) with the
// per-multipole FE assembly of assemble_J_FE_one_multipole_cached_chol
// (libhelfemqc/include/CoulombExchangeFE.h:432-482):
//   j_contract : per (L,M) channel and element, the Gaunt-weighted ket
//                contraction restricted to the element-diagonal tile (the only
//                part of Paux the assembly reads), the two disjoint traces
//                and the in-element Cholesky contraction L (L^T vec P).
//   j_scatter  : per output angular block and element, the O(Nel) prefix
//                sums of the disjoint traces (the reference's O(Nel^2) double
//                loop) and the Gaunt-weighted bra scatter.
// K restates TwoDBasisT::exchange (TwoDBasis.cpp:879-999) with
// assemble_K_FE_one_multipole_cached_chol (CoulombExchangeFE.h:484-530):
//   k_block_norms : density-block screening, ||P_il||_F < 10 eps skipped.
//   k_tiles       : work units of (element pair, range of output angular
//                   blocks). Off-diagonal pairs: recouple the (a,b) tiles of
//                   P, then A_L X B_L^T with A/B = r_small/r_big by element
//                   order. Diagonal elements: the exchange-ordered
//                   in-element tensor (equal to sum_p M_p X M_p^T). With a
//                   symmetric density only half of the tiles are computed and
//                   each is also written transposed (K_kj(b,a) = K_jk(a,b)^T).
//   k_fixup       : adds the contributions of neighbouring tiles on the
//                   shared boundary functions, in a fixed order (no atomics,
//                   bitwise reproducible).
#include <algorithm>
#include <cfloat>

#include "devatom.cuh"
#include "ff.cuh"
#include "smem_limit.hpp"

namespace hfg {
namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide sum, result valid in every thread; red needs >= 32 doubles
__device__ double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < nw; ++i) s += red[i];
  return s;
}

__device__ __forceinline__ bool gvalid(const DevAtom& A, int g) { return g >= 0 && g < A.nrad; }

// ------------------------------------------------------------------ Coulomb
__global__ void j_contract(DevAtom A, DevScratch S, const double* __restrict__ P) {
  const int ch = blockIdx.x, e = blockIdx.y;
  const int nn = A.nn, n2 = nn * nn, L = A.chanL[ch];
  extern __shared__ double sm[];
  double* X = sm;
  double* sc = X + n2;
  double* red = sc + A.rmax;
  const int k0 = A.jket_ptr[ch], k1 = A.jket_ptr[ch + 1];
  for (int idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    const int p = idx % nn, q = idx / nn;
    const int gp = gfun(A, e, p), gq = gfun(A, e, q);
    double x = 0.0;
    if (gvalid(A, gp) && gvalid(A, gq))
      for (int u = k0; u < k1; ++u) {
        const int blk = A.jket_blk[u], k = blk % A.nang, l = blk / A.nang;
        x += A.jket_coef[u] * P[(size_t)(l * A.nrad + gq) * A.nbf + (size_t)k * A.nrad + gp];
      }
    X[idx] = x;
  }
  __syncthreads();
  const size_t le = (size_t)L * A.nel + e;
  const double* rs = A.rs + le * n2;
  const double* rb = A.rb + le * n2;
  double ts = 0.0, tb = 0.0;
  for (int idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    const int p = idx % nn, q = idx / nn;
    const double xt = X[q + p * nn];
    ts += rs[idx] * xt;
    tb += rb[idx] * xt;
  }
  ts = block_sum(ts, red);
  tb = block_sum(tb, red);
  if (threadIdx.x == 0) {
    S.jscal[((size_t)ch * A.nel + e) * 2 + 0] = ts;
    S.jscal[((size_t)ch * A.nel + e) * 2 + 1] = tb;
  }
  const int r = A.rank[le];
  const double* C = A.cholp + le * n2 * A.rmax;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  for (int j = w; j < r; j += nw) {
    double s = 0.0;
    for (int q = lane; q < n2; q += 32) s += C[q + (size_t)j * n2] * X[q];
    s = warp_sum(s);
    if (lane == 0) sc[j] = s;
  }
  __syncthreads();
  double* jin = S.jin + ((size_t)ch * A.nel + e) * n2;
  for (int idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < r; ++j) s += C[idx + (size_t)j * n2] * sc[j];
    jin[idx] = s;
  }
}

constexpr int JMAXTERMS = 64;

// ---- Coulomb, split form: the contraction above in float pairs (the FP64
// pipe bounds the FP64 form on GB300: 2 n2 r multiply-adds per channel and
// element for the in-element factor alone). The density is split with
// integer operations, the in-element factor and the radial tables come as
// float-pair copies, sums of n2 or r terms are renormalised every step; the
// in-element part goes to the scratch as float pairs, the two scalars per
// (channel, element) as FP64.
__device__ __forceinline__ ffv ff_warp_sum(ffv v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v = ff_add(v, ffv{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)});
  return v;
}

// block-wide float-pair sum, valid in thread 0; red needs >= 32 entries
__device__ ffv ff_block_sum(ffv v, ffv* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = ff_warp_sum(v);
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  ffv s{0.f, 0.f};
  if (threadIdx.x == 0)
    for (int i = 0; i < nw; ++i) s = ff_add(s, red[i]);
  return s;
}

__global__ void j_contract_split(DevAtom A, DevScratch S, const double* __restrict__ P,
                                 const float2* __restrict__ C2) {
  const int ch = blockIdx.x, e = blockIdx.y;
  const int nn = A.nn, n2 = nn * nn, L = A.chanL[ch];
  extern __shared__ float2 smf[];
  float2* X = smf;       // [n2]
  float2* sc = X + n2;   // [rmax]
  __shared__ ffv red[32];
  const int k0 = A.jket_ptr[ch], k1 = A.jket_ptr[ch + 1];
  for (int idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    const int p = idx % nn, q = idx / nn;
    const int gp = gfun(A, e, p), gq = gfun(A, e, q);
    ffv x{0.f, 0.f};
    if (gvalid(A, gp) && gvalid(A, gq))
      for (int u = k0; u < k1; ++u) {
        const int blk = A.jket_blk[u], k = blk % A.nang, l = blk / A.nang;
        x = ff_fma(x, A.jket_coef2[u], split_bits(P[(size_t)(l * A.nrad + gq) * A.nbf + (size_t)k * A.nrad + gp]));
      }
    X[idx] = ff2(x);
  }
  __syncthreads();
  const size_t le = (size_t)L * A.nel + e;
  const float2* rs = A.rs2 + le * n2;
  const float2* rb = A.rb2 + le * n2;
  ffv ts{0.f, 0.f}, tb{0.f, 0.f};
  for (int idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    const int p = idx % nn, q = idx / nn;
    const float2 xt = X[q + p * nn];
    ts = ff_fma_n(ts, rs[idx], xt);
    tb = ff_fma_n(tb, rb[idx], xt);
  }
  ts = ff_block_sum(ts, red);
  tb = ff_block_sum(tb, red);
  if (threadIdx.x == 0) {
    S.jscal[((size_t)ch * A.nel + e) * 2 + 0] = ff_to_d(ts);
    S.jscal[((size_t)ch * A.nel + e) * 2 + 1] = ff_to_d(tb);
  }
  const int r = A.rank[le];
  const float2* C = C2 + le * n2 * A.rmax;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  for (int j = w; j < r; j += nw) {
    ffv v{0.f, 0.f};
    for (int q = lane; q < n2; q += 32) v = ff_fma_n(v, C[q + (size_t)j * n2], X[q]);
    v = ff_warp_sum(v);
    if (lane == 0) sc[j] = make_float2(v.hi, v.lo);
  }
  __syncthreads();
  float2* jin = reinterpret_cast<float2*>(S.jin) + ((size_t)ch * A.nel + e) * n2;
  for (int idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    ffv v{0.f, 0.f};
    for (int j = 0; j < r; ++j) v = ff_fma_n(v, C[idx + (size_t)j * n2], sc[j]);
    jin[idx] = ff2(v);
  }
}

__global__ void j_scatter_split(DevAtom A, DevScratch S, double* __restrict__ J, int accumulate) {
  const int ij = blockIdx.x, e = blockIdx.y;
  const int i = ij % A.nang, j = ij / A.nang;
  const int b0 = A.jbra_ptr[ij], b1 = A.jbra_ptr[ij + 1];
  const int nt = b1 - b0;
  if (nt == 0) return;
  const int nn = A.nn, n2 = nn * nn;
  __shared__ float2 Ab[JMAXTERMS], As[JMAXTERMS], Ab1[JMAXTERMS], As1[JMAXTERMS];
  for (int u = threadIdx.x; u < nt; u += blockDim.x) {
    const int ch = A.jbra_chan[b0 + u];
    const double* sc = S.jscal + (size_t)ch * A.nel * 2;
    double big = 0.0, small = 0.0;
    for (int e2 = e + 1; e2 < A.nel; ++e2) big += sc[2 * e2 + 1];
    for (int e2 = 0; e2 < e; ++e2) small += sc[2 * e2 + 0];
    Ab[u] = split_bits(big);
    As[u] = split_bits(small);
    if (e > 0) {
      Ab1[u] = split_bits(big + sc[2 * e + 1]);
      As1[u] = split_bits(small - sc[2 * (e - 1) + 0]);
    }
  }
  __syncthreads();
  const float2* jin2 = reinterpret_cast<const float2*>(S.jin);
  for (int idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    const int p = idx % nn, q = idx / nn;
    // J has element-diagonal tiles only: the single entry two tiles share is
    // the corner on the common boundary function, owned by the later tile
    if (p == nn - 1 && q == nn - 1) continue;
    const int gp = gfun(A, e, p), gq = gfun(A, e, q);
    if (!gvalid(A, gp) || !gvalid(A, gq)) continue;
    ffv v{0.f, 0.f};
    for (int u = 0; u < nt; ++u) {
      const int ch = A.jbra_chan[b0 + u], L = A.chanL[ch];
      const size_t le = (size_t)L * A.nel + e;
      ffv t{0.f, 0.f};
      t = ff_fma(t, Ab[u], A.rs2[le * n2 + idx]);
      t = ff_fma(t, As[u], A.rb2[le * n2 + idx]);
      const float2 ji = jin2[((size_t)ch * A.nel + e) * n2 + idx];
      t = ff_add(t, ffv{ji.x, ji.y});
      v = ff_fma_n(v, A.jbra_coef2[b0 + u], ff2(t));
    }
    if (p == 0 && q == 0 && e > 0) {
      const int c = (nn - 1) + (nn - 1) * nn;
      for (int u = 0; u < nt; ++u) {
        const int ch = A.jbra_chan[b0 + u], L = A.chanL[ch];
        const size_t le = (size_t)L * A.nel + (e - 1);
        ffv t{0.f, 0.f};
        t = ff_fma(t, Ab1[u], A.rs2[le * n2 + c]);
        t = ff_fma(t, As1[u], A.rb2[le * n2 + c]);
        const float2 ji = jin2[((size_t)ch * A.nel + (e - 1)) * n2 + c];
        t = ff_add(t, ffv{ji.x, ji.y});
        v = ff_fma_n(v, A.jbra_coef2[b0 + u], ff2(t));
      }
    }
    double* out = J + (size_t)(j * A.nrad + gq) * A.nbf + (size_t)i * A.nrad + gp;
    const double y = ff_to_d(v);
    if (accumulate) *out += y; else *out = y;
  }
}

__global__ void j_scatter(DevAtom A, DevScratch S, double* __restrict__ J, int accumulate) {
  const int ij = blockIdx.x, e = blockIdx.y;
  const int i = ij % A.nang, j = ij / A.nang;
  const int b0 = A.jbra_ptr[ij], b1 = A.jbra_ptr[ij + 1];
  const int nt = b1 - b0;
  if (nt == 0) return;
  const int nn = A.nn, n2 = nn * nn;
  __shared__ double Ab[JMAXTERMS], As[JMAXTERMS], Ab1[JMAXTERMS], As1[JMAXTERMS];
  for (int u = threadIdx.x; u < nt; u += blockDim.x) {
    const int ch = A.jbra_chan[b0 + u];
    const double* sc = S.jscal + (size_t)ch * A.nel * 2;
    double big = 0.0, small = 0.0;
    for (int e2 = e + 1; e2 < A.nel; ++e2) big += sc[2 * e2 + 1];
    for (int e2 = 0; e2 < e; ++e2) small += sc[2 * e2 + 0];
    Ab[u] = big;
    As[u] = small;
    if (e > 0) {
      Ab1[u] = big + sc[2 * e + 1];
      As1[u] = small - sc[2 * (e - 1) + 0];
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < n2; idx += blockDim.x) {
    const int p = idx % nn, q = idx / nn;
    // J has element-diagonal tiles only: the single entry two tiles share is
    // the corner on the common boundary function, owned by the later tile
    if (p == nn - 1 && q == nn - 1) continue;
    const int gp = gfun(A, e, p), gq = gfun(A, e, q);
    if (!gvalid(A, gp) || !gvalid(A, gq)) continue;
    double v = 0.0;
    for (int u = 0; u < nt; ++u) {
      const int ch = A.jbra_chan[b0 + u], L = A.chanL[ch];
      const size_t le = (size_t)L * A.nel + e;
      const double* jin = S.jin + ((size_t)ch * A.nel + e) * n2;
      v += A.jbra_coef[b0 + u] * (Ab[u] * A.rs[le * n2 + idx] + As[u] * A.rb[le * n2 + idx] + jin[idx]);
    }
    if (p == 0 && q == 0 && e > 0) {
      const int c = (nn - 1) + (nn - 1) * nn;
      for (int u = 0; u < nt; ++u) {
        const int ch = A.jbra_chan[b0 + u], L = A.chanL[ch];
        const size_t le = (size_t)L * A.nel + (e - 1);
        const double* jin = S.jin + ((size_t)ch * A.nel + (e - 1)) * n2;
        v += A.jbra_coef[b0 + u] * (Ab1[u] * A.rs[le * n2 + c] + As1[u] * A.rb[le * n2 + c] + jin[c]);
      }
    }
    double* out = J + (size_t)(j * A.nrad + gq) * A.nbf + (size_t)i * A.nrad + gp;
    if (accumulate) *out += v; else *out = v;
  }
}

// ----------------------------------------------------------------- exchange
// Partial Frobenius norms of the angular blocks of P: grid (nang^2, NORM_SPLIT),
// each CTA sums a band of columns; consumers add the partials in a fixed
// order and apply the reference's 10*DBL_EPSILON screen.
__global__ void k_block_norms(DevAtom A, const double* __restrict__ P, double* __restrict__ part,
                              float2* __restrict__ p2) {
  __shared__ double red[32];
  const int blk = blockIdx.x, i = blk % A.nang, l = blk / A.nang;
  const int c0 = (int)((long)A.nrad * blockIdx.y / NORM_SPLIT);
  const int c1 = (int)((long)A.nrad * (blockIdx.y + 1) / NORM_SPLIT);
  double s = 0.0;
  float sf = 0.f;
  // the band's elements in column order (32-bit index arithmetic); four
  // loads in flight per thread (one at a time left the pass latency-bound
  // at half the HBM rate; eight measured the same as four), summed in the
  // same order as one at a time
  constexpr int NU = 4;
  const int n = A.nrad * (c1 - c0), bd = blockDim.x;
  for (int base = threadIdx.x; base < n; base += NU * bd) {
    double v[NU];
    size_t o[NU];
#pragma unroll
    for (int u = 0; u < NU; ++u) {
      const int idx = base + u * bd;
      const int r = idx % A.nrad, c = c0 + idx / A.nrad;
      o[u] = (size_t)(l * A.nrad + c) * A.nbf + (size_t)i * A.nrad + r;
      v[u] = idx < n ? P[o[u]] : 0.0;
    }
#pragma unroll
    for (int u = 0; u < NU; ++u) {
      if (base + u * bd >= n) break;
      if (p2) {
        // split path: integer-only split (no FP64-pipe instructions) and an
        // FP32 norm of the high words for the screen
        const float2 h = split_bits(v[u]);
        p2[o[u]] = h;
        sf = fmaf(h.x, h.x, sf);
      } else {
        s += v[u] * v[u];
      }
    }
  }
  if (p2) s = (double)sf;
  s = block_sum(s, red);
  if (threadIdx.x == 0) part[blk * NORM_SPLIT + blockIdx.y] = s;
}

// density-block screen (10*DBL_EPSILON, the reference's threshold) and the
// exchange entries that see an active block, once per build
__global__ void k_flags(DevAtom A, DevScratch S) {
  const int nang2 = A.nang * A.nang;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  for (int idx = tid; idx < nang2; idx += nth) {
    double s = 0.0;
    for (int c = 0; c < NORM_SPLIT; ++c) s += S.bnorm[idx * NORM_SPLIT + c];
    S.act[idx] = !(sqrt(s) < 10.0 * DBL_EPSILON);
  }
  // every thread recomputes the block flags its entries need (no grid sync)
  for (int ent = tid; ent < A.nent; ent += nth) {
    bool any = false;
    for (int u = A.kent_ptr[ent]; u < A.kent_ptr[ent + 1] && !any; ++u) {
      const int blk = A.kterm_blk[u];
      double s = 0.0;
      for (int c = 0; c < NORM_SPLIT; ++c) s += S.bnorm[blk * NORM_SPLIT + c];
      any = !(sqrt(s) < 10.0 * DBL_EPSILON);
    }
    S.ent_act[ent] = any ? 1 : 0;
  }
}

__device__ __forceinline__ void load_active(const DevAtom& A, const DevScratch& S, unsigned char* act) {
  const int nang2 = A.nang * A.nang;
  for (int idx = threadIdx.x; idx < nang2; idx += blockDim.x) act[idx] = S.act[idx];
}

__device__ __forceinline__ size_t halo_idx(const DevAtom& A, int a, int b, int jk, int h) {
  return ((size_t)(a * A.nel + b) * (A.nang * A.nang) + jk) * (2 * A.nn - 1) + h;
}

// store the finished contribution y of tile (a,b), angular block jk, at
// local position (p,q): owned entries go to K, the shared last row/column to
// the halo buffer (added by k_fixup)
__device__ __forceinline__ void k_store(const DevAtom& A, const DevScratch& S, double* K, int a, int b,
                                        int jk, int p, int q, double y) {
  const int nn = A.nn;
  const int gp = gfun(A, a, p), gq = gfun(A, b, q);
  if (!gvalid(A, gp) || !gvalid(A, gq)) return;
  const int j = jk % A.nang, k = jk / A.nang;
  if (p <= nn - 2 && q <= nn - 2)
    K[(size_t)(k * A.nrad + gq) * A.nbf + (size_t)j * A.nrad + gp] = y;
  else if (p == nn - 1)
    S.khalo[halo_idx(A, a, b, jk, q)] = y;
  else
    S.khalo[halo_idx(A, a, b, jk, nn + p)] = y;
}

// recoupled tile value for thread (p,q) of element pair (a,b), entry ent
// P_base = P + gq*nbf + gp for this thread's tile entry
__device__ __forceinline__ double k_recouple(const DevAtom& A, const double* __restrict__ Pbase,
                                             const unsigned char* act, int ent) {
  double x = 0.0;
  const int u0 = A.kent_ptr[ent], u1 = A.kent_ptr[ent + 1];
  for (int u = u0; u < u1; ++u) {
    if (!act[A.kterm_blk[u]]) continue;
    x += A.kterm_coef[u] * Pbase[A.kterm_off[u]];
  }
  return x;
}

// Range-separated exchange with the erfc kernel (TwoDBasisT::rs_exchange,
// src/atomic/TwoDBasis.cpp:1001-1131, with the pairwise assembly of
// CoulombExchangeFE.h:396-422): the kernel does not separate into r< / r>
// factors, so every element pair (a,b) carries a dense exchange-ordered
// table per multipole, K_jk(a,b)[t] = -sum_L sum_v T_L(a,b)[t, v] X_L(a,b)[v]
// (t = p + q nn, v = p' + q' nn). One CTA per (element pair, output block),
// one thread per tile entry t; FP64.
__global__ void k_erfc_tiles(DevAtom A, DevScratch S, const double* __restrict__ tk,
                             const double* __restrict__ P, double* __restrict__ K) {
  const int a = blockIdx.x % A.nel, b = blockIdx.x / A.nel, jk = blockIdx.y;
  const int nn = A.nn, n2 = nn * nn, t = threadIdx.x;
  extern __shared__ double xs[];  // [n2]
  unsigned char* act = reinterpret_cast<unsigned char*>(xs + n2);
  for (int idx = t; idx < A.nang * A.nang; idx += blockDim.x) act[idx] = S.act[idx];
  __syncthreads();
  double y = 0.0;
  for (int e = A.kjk_ptr[jk]; e < A.kjk_ptr[jk + 1]; ++e) {
    if (!S.ent_act[e]) continue;  // uniform over the CTA
    for (int v = t; v < n2; v += blockDim.x) {
      const int gp = gfun(A, a, v % nn), gq = gfun(A, b, v / nn);
      xs[v] = (gvalid(A, gp) && gvalid(A, gq)) ? k_recouple(A, P + (size_t)gq * A.nbf + gp, act, e) : 0.0;
    }
    __syncthreads();
    if (t < n2) {
      const double* T = tk + (((size_t)A.kent_L[e] * A.nel + a) * A.nel + b) * n2 * n2;
      for (int v = 0; v < n2; ++v) y += T[t + (size_t)v * n2] * xs[v];
    }
    __syncthreads();
  }
  if (t < n2) k_store(A, S, K, a, b, jk, t % nn, t / nn, -y);
}

// One work unit = one element pair (a,b) and a range of output angular
// blocks. a != b: off-diagonal pair, jk over [lo,hi) in natural order,
// contribution A_L X B_L^T. a == b: diagonal element, jk = diag_jk[lo..hi),
// contribution Tk X. In symmetric mode (P = P^T) only a < b pairs and j <= k
// diagonal blocks are units; each also writes the transposed partner tile
// (k,j,b,a), since K_kj(b,a) = K_jk(a,b)^T.
__global__ void __launch_bounds__(320) k_tiles(DevAtom A, DevScratch S, const int4* __restrict__ units,
                                               const int* __restrict__ diag_jk, int symmetric,
                                               const double* __restrict__ P, double* __restrict__ K) {
  const int4 u = units[blockIdx.x];
  const int a = u.x, b = u.y;
  const int nn = A.nn, n2 = nn * nn, NL = A.NL, nang2 = A.nang * A.nang;
  extern __shared__ double sm[];
  double* X = sm;
  double* T = X + n2;
  double* Am = T + n2;
  double* Bm = Am + NL * n2;
  unsigned char* act = reinterpret_cast<unsigned char*>(Bm + NL * n2);
  const bool diag = (a == b);
  if (!diag) {
    const double* srcA = (a < b) ? A.rs : A.rb;
    const double* srcB = (a < b) ? A.rb : A.rs;
    for (int idx = threadIdx.x; idx < NL * n2; idx += blockDim.x) {
      const int L = idx / n2, o = idx % n2;
      Am[idx] = srcA[((size_t)L * A.nel + a) * n2 + o];
      Bm[idx] = srcB[((size_t)L * A.nel + b) * n2 + o];
    }
  }
  load_active(A, S, act);
  __syncthreads();
  const int t = threadIdx.x;
  const bool live = t < n2;
  const int p = live ? t % nn : 0, q = live ? t / nn : 0;
  const int gp = gfun(A, a, p), gq = gfun(A, b, q);
  const bool vpq = live && gvalid(A, gp) && gvalid(A, gq);
  for (int w = u.z; w < u.w; ++w) {
    const int jk = diag ? diag_jk[w] : w;
    double y = 0.0;
    const double* Pbase = P + (size_t)gq * A.nbf + gp;
    for (int ent = A.kjk_ptr[jk]; ent < A.kjk_ptr[jk + 1]; ++ent) {
      if (!S.ent_act[ent]) continue;  // uniform over the CTA
      const int L = A.kent_L[ent];
      if (live) X[t] = vpq ? k_recouple(A, Pbase, act, ent) : 0.0;
      __syncthreads();
      if (diag) {
        if (live) {
          const double* Tk = A.tk + ((size_t)L * A.nel + a) * n2 * n2;
          double s = 0.0;
          for (int v = 0; v < n2; ++v) s += Tk[t + (size_t)v * n2] * X[v];
          y += s;
        }
      } else {
        if (live) {
          const double* Bl = Bm + L * n2;
          double s = 0.0;
          for (int c = 0; c < nn; ++c) s += X[p + c * nn] * Bl[q + c * nn];
          T[t] = s;
        }
        __syncthreads();
        if (live) {
          const double* Al = Am + L * n2;
          double s = 0.0;
          for (int c = 0; c < nn; ++c) s += Al[p + c * nn] * T[c + q * nn];
          y += s;
        }
      }
      __syncthreads();
    }
    if (live) k_store(A, S, K, a, b, jk, p, q, -y);
    const int j = jk % A.nang, k = jk / A.nang;
    if (symmetric && (!diag || j != k)) {
      // transposed partner: stage through shared memory so that consecutive
      // threads write consecutive rows of the column-major output
      if (live) X[t] = -y;
      __syncthreads();
      if (live) k_store(A, S, K, b, a, k + j * A.nang, p, q, X[q + p * nn]);
      __syncthreads();
    }
  }
}

// p2base = S.p2 + gq*nbf + gp for this thread's tile entry
__device__ __forceinline__ ffv k_recouple_ff(const DevAtom& A, const float2* __restrict__ p2base,
                                             const unsigned char* act, int ent) {
  ffv x = {0.f, 0.f};
  const int u0 = A.kent_ptr[ent], u1 = A.kent_ptr[ent + 1];
  for (int u = u0; u < u1; ++u) {
    if (!act[A.kterm_blk[u]]) continue;
    x = ff_fma(x, A.kterm_coef2[u], p2base[A.kterm_off[u]]);
  }
  return x;
}


// NN > 0: element order fixed at compile time (the element-pair contractions
// unroll with immediate shared-memory offsets); NN = 0: any order
template <int NN>
__global__ void __launch_bounds__(320) k_tiles_split(DevAtom A, DevScratch S, const int4* __restrict__ units,
                                                     const int* __restrict__ diag_jk, int symmetric,
                                                     double* __restrict__ K) {
  const int4 u = units[blockIdx.x];
  const int a = u.x, b = u.y;
  const int nn = NN > 0 ? NN : A.nn, n2 = nn * nn, NL = A.NL;
  extern __shared__ float2 sm2[];
  float2* X = sm2;
  float2* T = X + n2;
  float2* Am = T + n2;
  float2* Bm = Am + NL * n2;
  double* Y = reinterpret_cast<double*>(Bm + NL * n2);
  unsigned char* act = reinterpret_cast<unsigned char*>(Y + n2);
  const bool diag = (a == b);
  if (!diag) {
    const float2* srcA = (a < b) ? A.rs2 : A.rb2;
    const float2* srcB = (a < b) ? A.rb2 : A.rs2;
    for (int idx = threadIdx.x; idx < NL * n2; idx += blockDim.x) {
      const int L = idx / n2, o = idx % n2;
      Am[idx] = srcA[((size_t)L * A.nel + a) * n2 + o];
      Bm[idx] = srcB[((size_t)L * A.nel + b) * n2 + o];
    }
  }
  load_active(A, S, act);
  __syncthreads();
  const int t = threadIdx.x;
  const bool live = t < n2;
  const int p = live ? t % nn : 0, q = live ? t / nn : 0;
  const int gp = gfun(A, a, p), gq = gfun(A, b, q);
  const bool vpq = live && gvalid(A, gp) && gvalid(A, gq);
  const float2* p2base = S.p2 + (size_t)gq * A.nbf + gp;
  for (int w = u.z; w < u.w; ++w) {
    const int jk = diag ? diag_jk[w] : w;
    ffv yacc = {0.f, 0.f};
    // the recoupled density tile of the next active entry is loaded while the
    // current one is contracted (its global loads overlap the FP32 work)
    const int ent_end = A.kjk_ptr[jk + 1];
    int ent = A.kjk_ptr[jk];
    while (ent < ent_end && !S.ent_act[ent]) ++ent;  // uniform over the CTA
    float2 xcur = make_float2(0.f, 0.f);
    if (ent < ent_end && vpq) xcur = ff2(k_recouple_ff(A, p2base, act, ent));
    while (ent < ent_end) {
      const int L = A.kent_L[ent];
      if (live) X[t] = xcur;
      __syncthreads();
      int ent_next = ent + 1;
      while (ent_next < ent_end && !S.ent_act[ent_next]) ++ent_next;
      float2 xnext = make_float2(0.f, 0.f);
      if (ent_next < ent_end && vpq) xnext = ff2(k_recouple_ff(A, p2base, act, ent_next));
      ffv acc = {0.f, 0.f};
      if (diag) {
        if (live) {
          // lazy low-word accumulation, renormalised every nn terms
          const float2* Tk = A.tk2 + ((size_t)L * A.nel + a) * n2 * n2;
          for (int v0 = 0; v0 < n2; v0 += nn) {
#pragma unroll
            for (int c = 0; c < (NN > 0 ? NN : 1); ++c) {
              if (NN == 0) break;
              acc = ff_fma(acc, Tk[t + (size_t)(v0 + c) * n2], X[v0 + c]);
            }
            if (NN == 0)
              for (int v = v0; v < v0 + nn; ++v) acc = ff_fma(acc, Tk[t + (size_t)v * n2], X[v]);
            acc = ff_norm(acc.hi, acc.lo);
          }
        }
      } else {
        if (live) {
          const float2* Bl = Bm + L * n2;
          ffv s = {0.f, 0.f};
          if (NN > 0) {
#pragma unroll
            for (int c = 0; c < (NN > 0 ? NN : 1); ++c) s = ff_fma(s, X[p + c * nn], Bl[q + c * nn]);
          } else {
            for (int c = 0; c < nn; ++c) s = ff_fma(s, X[p + c * nn], Bl[q + c * nn]);
          }
          T[t] = ff2(s);
        }
        __syncthreads();
        if (live) {
          const float2* Al = Am + L * n2;
          if (NN > 0) {
#pragma unroll
            for (int c = 0; c < (NN > 0 ? NN : 1); ++c) acc = ff_fma(acc, Al[p + c * nn], T[c + q * nn]);
          } else {
            for (int c = 0; c < nn; ++c) acc = ff_fma(acc, Al[p + c * nn], T[c + q * nn]);
          }
        }
      }
      yacc = ff_add(yacc, ff_norm(acc.hi, acc.lo));
      __syncthreads();
      ent = ent_next;
      xcur = xnext;
    }
    const double y = ff_to_d(yacc);  // FP64 recombination, once per output element
    if (live) k_store(A, S, K, a, b, jk, p, q, -y);
    const int j = jk % A.nang, k = jk / A.nang;
    if (symmetric && (!diag || j != k)) {
      if (live) Y[t] = -y;
      __syncthreads();
      if (live) k_store(A, S, K, b, a, k + j * A.nang, p, q, Y[q + p * nn]);
      __syncthreads();
    }
  }
}

// one CTA per element pair (a,b), all output blocks: the first row/column of
// each tile receives its neighbours' halo entries in a fixed order
__global__ void k_fixup(DevAtom A, DevScratch S, double* __restrict__ K) {
  const int a = blockIdx.x % A.nel, b = blockIdx.x / A.nel;
  const int nn = A.nn, per = 2 * nn - 3, nang2 = A.nang * A.nang;
  for (int w = threadIdx.x; w < per * nang2; w += blockDim.x) {
    const int idx = w % per, jk = w / per;
    const int j = jk % A.nang, k = jk / A.nang;
    int p, q;
    double v;
    if (idx < nn - 1) {  // first row of tile (a,b), q in [0, nn-2]
      if (a == 0) continue;
      p = 0;
      q = idx;
      v = S.khalo[halo_idx(A, a - 1, b, jk, q)];
      if (q == 0) {
        if (b == 0) continue;
        v += S.khalo[halo_idx(A, a, b - 1, jk, nn + 0)];
        v += S.khalo[halo_idx(A, a - 1, b - 1, jk, nn - 1)];
      }
    } else {  // first column, p in [1, nn-2]
      if (b == 0) continue;
      p = idx - (nn - 1) + 1;
      q = 0;
      v = S.khalo[halo_idx(A, a, b - 1, jk, nn + p)];
    }
    const int gp = gfun(A, a, p), gq = gfun(A, b, q);
    if (!gvalid(A, gp) || !gvalid(A, gq)) continue;
    K[(size_t)(k * A.nrad + gq) * A.nbf + (size_t)j * A.nrad + gp] += v;
  }
}

inline int threads_for(int n2) { return ((n2 + 31) / 32) * 32; }

struct Mark {
  Profiler* p;
  int slot = -1;
  cudaStream_t s;
  Mark(Profiler* p_, int k, cudaStream_t s_) : p(p_), s(s_) {
    if (p && p->on && ((p->mask >> k) & 1u) && p->n < p->cap) {
      slot = p->n++;
      p->cls[slot] = k;
      cudaEventRecord(p->ev[2 * slot], s);
    }
  }
  ~Mark() {
    if (slot >= 0) cudaEventRecord(p->ev[2 * slot + 1], s);
  }
};

}  // namespace

cudaError_t launch_coulomb_fp64(const DevAtom& A, const DevScratch& S, const double* P, double* J,
                                bool zero_output, cudaStream_t st, Profiler* prof) {
  const int n2 = A.nn * A.nn, th = threads_for(n2);
  if (zero_output) {
    cudaError_t err = cudaMemsetAsync(J, 0, sizeof(double) * (size_t)A.nbf * A.nbf, st);
    if (err != cudaSuccess) return err;
  }
  const size_t sm1 = sizeof(double) * (n2 + A.rmax + 32);
  {
    Mark m(prof, KC_J_CONTRACT, st);
    j_contract<<<dim3(A.nchan, A.nel), th, sm1, st>>>(A, S, P);
  }
  {
    Mark m(prof, KC_J_SCATTER, st);
    j_scatter<<<dim3(A.nang * A.nang, A.nel), th, 0, st>>>(A, S, J, zero_output ? 0 : 1);
  }
  return cudaGetLastError();
}

cudaError_t launch_coulomb_split(const DevAtom& A, const DevScratch& S, const double* P, double* J,
                                 bool zero_output, cudaStream_t st, Profiler* prof) {
  if (!A.cholp2 || !A.jket_coef2 || !A.jbra_coef2 || !A.rs2 || !A.rb2) return cudaErrorInvalidValue;
  const int n2 = A.nn * A.nn, th = threads_for(n2);
  if (zero_output) {
    cudaError_t err = cudaMemsetAsync(J, 0, sizeof(double) * (size_t)A.nbf * A.nbf, st);
    if (err != cudaSuccess) return err;
  }
  const size_t sm1 = sizeof(float2) * (n2 + A.rmax);
  {
    Mark m(prof, KC_J_CONTRACT, st);
    const cudaError_t e = smem_limit(j_contract_split, sm1);
    if (e != cudaSuccess) return e;
    j_contract_split<<<dim3(A.nchan, A.nel), th, sm1, st>>>(A, S, P, A.cholp2);
  }
  {
    Mark m(prof, KC_J_SCATTER, st);
    j_scatter_split<<<dim3(A.nang * A.nang, A.nel), th, 0, st>>>(A, S, J, zero_output ? 0 : 1);
  }
  return cudaGetLastError();
}

cudaError_t launch_exchange_erfc(const DevAtom& A, const DevScratch& S, const double* tk, const double* P, double* K,
                                 cudaStream_t st, Profiler* prof) {
  const int n2 = A.nn * A.nn, nang2 = A.nang * A.nang;
  {
    Mark m(prof, KC_K_NORMS, st);
    k_block_norms<<<dim3(nang2, NORM_SPLIT), 256, 0, st>>>(A, P, S.bnorm, nullptr);
    k_flags<<<std::max(1, std::min(152, (A.nent + 255) / 256)), 256, 0, st>>>(A, S);
  }
  {
    Mark m(prof, KC_K_TILES, st);
    const size_t smem = sizeof(double) * n2 + nang2;
    const cudaError_t e = smem_limit(k_erfc_tiles, smem);
    if (e != cudaSuccess) return e;
    k_erfc_tiles<<<dim3(A.nel * A.nel, nang2), threads_for(n2), smem, st>>>(A, S, tk, P, K);
  }
  {
    Mark m(prof, KC_K_FIXUP, st);
    k_fixup<<<A.nel * A.nel, 256, 0, st>>>(A, S, K);
  }
  return cudaGetLastError();
}

cudaError_t launch_exchange_fp64(const DevAtom& A, const DevScratch& S, const KUnits& U, const double* P,
                                 double* K, bool symmetric, cudaStream_t st, Profiler* prof) {
  const int n2 = A.nn * A.nn, th = threads_for(n2), nang2 = A.nang * A.nang;
  {
    Mark m(prof, KC_K_NORMS, st);
    k_block_norms<<<dim3(nang2, NORM_SPLIT), 256, 0, st>>>(A, P, S.bnorm, nullptr);
    k_flags<<<std::max(1, std::min(152, (A.nent + 255) / 256)), 256, 0, st>>>(A, S);
  }
  {
    Mark m(prof, KC_K_TILES, st);
    const size_t smem = sizeof(double) * (2 * n2 + 2 * A.NL * n2) + nang2;
    const int nunits = symmetric ? U.n_sym : U.n_all;
    const cudaError_t e = smem_limit(k_tiles, smem);
    if (e != cudaSuccess) return e;
    k_tiles<<<nunits, th, smem, st>>>(A, S, symmetric ? U.sym : U.all, U.diag_jk_src(symmetric), symmetric ? 1 : 0,
                                      P, K);
  }
  {
    Mark m(prof, KC_K_FIXUP, st);
    k_fixup<<<A.nel * A.nel, 256, 0, st>>>(A, S, K);
  }
  return cudaGetLastError();
}

cudaError_t launch_exchange_split(const DevAtom& A, const DevScratch& S, const KUnits& U, const double* P,
                                  double* K, bool symmetric, cudaStream_t st, Profiler* prof, const DevTC* tc,
                                  const SideStream* side) {
  const int n2 = A.nn * A.nn, th = threads_for(n2), nang2 = A.nang * A.nang;
  {
    Mark m(prof, KC_K_NORMS, st);
    k_block_norms<<<dim3(nang2, NORM_SPLIT), 256, 0, st>>>(A, P, S.bnorm, S.p2);
    k_flags<<<std::max(1, std::min(152, (A.nent + 255) / 256)), 256, 0, st>>>(A, S);
  }
  {
    Mark m(prof, KC_K_TILES, st);
    const size_t smem = sizeof(float2) * (2 * n2 + 2 * A.NL * n2) + sizeof(double) * n2 + nang2;
    int nunits = symmetric ? U.n_sym : U.n_all;
    const int4* units = symmetric ? U.sym : U.all;
    if (tc) {
      // every element pair on the tensor cores: the off-diagonal tiles and
      // the diagonal ones through the exchange-ordered tensor
      cudaError_t e = cudaSuccess;
      if (side && side->s) {
        // the diagonal stage (a chain of dependent steps in 0.8 of a wave)
        // beside the issue-bound off-diagonal tiles, joined before the fix-up
        e = cudaEventRecord(side->fork, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(side->s, side->fork, 0);
        if (e == cudaSuccess) e = launch_k_diag_tc(A, S, *tc, symmetric, K, side->s);
        if (e == cudaSuccess) e = cudaEventRecord(side->join, side->s);
        if (e == cudaSuccess) e = launch_k_tiles_tc(A, S, *tc, symmetric, K, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, side->join, 0);
      } else {
        e = launch_k_tiles_tc(A, S, *tc, symmetric, K, st);
        if (e == cudaSuccess) e = launch_k_diag_tc(A, S, *tc, symmetric, K, st);
      }
      if (e != cudaSuccess) return e;
      nunits = 0;
    }
    auto kern = (A.nn == 15) ? k_tiles_split<15> : k_tiles_split<0>;
    if (nunits > 0) {
      const cudaError_t e = smem_limit(kern, smem);
      if (e != cudaSuccess) return e;
    }
    if (nunits > 0)
      kern<<<nunits, th, smem, st>>>(A, S, units, U.diag_jk_src(symmetric), symmetric ? 1 : 0, K);
  }
  {
    Mark m(prof, KC_K_FIXUP, st);
    k_fixup<<<A.nel * A.nel, 256, 0, st>>>(A, S, K);
  }
  return cudaGetLastError();
}

// Upper part of a symmetric column-major n x n matrix from its lower
// column blocks: for blocks of bw columns, P(r, c) = P(c, r) wherever
// r / bw < c / bw (block c holds rows >= its first column, so the source
// is always present). 32 x 32 tiles through shared memory.
__global__ void k_mirror_blocks(double* __restrict__ P, int n, int bw) {
  __shared__ double t[32][33];
  const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  if (r0 / bw >= min(c0 + 31, n - 1) / bw) return;  // no element of the tile is mirrored
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int k = ty; k < 32; k += 8) {
    const int r = r0 + k, c = c0 + tx;
    if (r < n && c < n && r / bw < c / bw) t[k][tx] = P[c + (size_t)r * n];
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int c = c0 + k, r = r0 + tx;
    if (r < n && c < n && r / bw < c / bw) P[r + (size_t)c * n] = t[tx][k];
  }
}

cudaError_t launch_mirror_blocks(double* P, int n, int bw, cudaStream_t st) {
  if (n < 1 || bw < 1) return cudaErrorInvalidValue;
  const int nt = (n + 31) / 32;
  k_mirror_blocks<<<dim3(nt, nt), dim3(32, 8), 0, st>>>(P, n, bw);
  return cudaGetLastError();
}

}  // namespace hfg

// Plain-FP64 Coulomb (J) and exchange (K) builds for the diatomic basis.
//
// J restates diatomic TwoDBasis::coulomb (src/diatomic/basis.cpp:1621-1815):
//   dj_contract : per signed (L,M) channel and element, the two Gaunt-weighted
//                 ket sums over the element-diagonal tile (channel 0 with the
//                 cos^2-weighted coupling, channel 2 with the plain one), the
//                 four disjoint traces tr(P0 X0), tr(Q0 X0), tr(P2 X2),
//                 tr(Q2 X2) times LMfac, and the in-element contraction
//                 LMfac B diag(sigma) B' [x0; x2].
//   dj_scatter  : per output angular block and element, the O(Nel) prefix
//                 sums of the traces (the reference's O(Nel^2) loop) with the
//                 channel signs (+ for 00, 22; - for 02, 20) and the bra sum.
// K restates diatomic TwoDBasis::exchange (basis.cpp:1817-2061):
//   dk_norms / dk_act : density-block screening (||P_il|| < 10 eps skipped).
//   dk_entry_act      : which (output block, (L,|M|)) entries see an active
//                       density block; dk_compact lists the active output
//                       blocks on the device.
//   dk_tiles          : persistent CTAs over (element pair, active output
//                       block) items. Each entry recouples the four radial
//                       matrices R00, R02, R20, R22 from the density with the
//                       product couplings (the j-side coupling times the
//                       k-side one, summed in that order), then
//                       off-diagonal pairs: K -= I0 (R00 J0' + R02 J2') +
//                       I2 (R20 J0' + R22 J2') with I/J the P- or Q-type
//                       integrals by element order; in-element blocks: the
//                       exchange-ordered kernel rebuilt from the factor.
//   dk_fixup          : the shared-boundary contributions of neighbouring
//                       tiles, added in a fixed order (bitwise reproducible).
#include <algorithm>
#include <cfloat>

#include "devdiatomic.cuh"
#include "ff.cuh"
#include "smem_limit.hpp"

namespace hfg {
namespace {

__device__ __forceinline__ double dwarp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ double dblock_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = dwarp_sum(v);
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int i = 0; i < nw; ++i) s += red[i];
  __syncthreads();
  return s;
}

__device__ __forceinline__ int dgf(const DevDiatomic& D, int e, int p) { return e * (D.nn - 1) + p; }

// pure index of radial function g of shell s, or -1 where it is not in the
// pure basis (g = 0 of an m != 0 shell, or g >= nrad)
__device__ __forceinline__ int dpure_idx(const DevDiatomic& D, int s, int g) {
  const int st = D.pstart[s];
  return (g >= st && g < D.nrad) ? D.poff[s] + g - st : -1;
}
__device__ __forceinline__ int al_idx(const DevDiatomic& D, int a, int L, int M) {
  return (a * (D.Lmax + 1) + L) * D.nM + M + 2 * D.mmax;
}

// ------------------------------------------------------- boundary handling
__global__ void d_expand(const double* __restrict__ P, int nbf, const int* __restrict__ pure, double* __restrict__ Pd,
                         int nd) {
  const size_t n = (size_t)nbf * nbf;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(idx % nbf), c = (int)(idx / nbf);
    Pd[(size_t)pure[r] + (size_t)pure[c] * nd] = P[idx];
  }
}

__global__ void d_gather(const double* __restrict__ Fd, int nd, const int* __restrict__ pure, int nbf,
                         double* __restrict__ F) {
  const size_t n = (size_t)nbf * nbf;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(idx % nbf), c = (int)(idx / nbf);
    F[idx] = Fd[(size_t)pure[r] + (size_t)pure[c] * nd];
  }
}

// exchange-ordered in-element kernel from the sign-carrying factor:
//   tx_ab[(p,q),(i,l)] = s_ab sum_r sigma_r M_a^r(i,p) M_b^r(q,l),
// M_a^r the channel-a half of factor column r as an nn x nn matrix and
// s_ab = +1 for 00, 22 and -1 for 02, 20
__global__ void d_build_tx(DevDiatomic D, double* __restrict__ tx) {
  const int blk = blockIdx.x, ab = blk & 3, le = blk >> 2;
  const int a = ab >> 1, b = ab & 1;
  const double sgn = (a == b) ? 1.0 : -1.0;
  const int nn = D.nn, n2 = nn * nn, N = 2 * n2;
  const int r = D.cdrank[le];
  const double* B = D.cdB + (size_t)le * N * D.rmax;
  const double* s = D.cds + (size_t)le * D.rmax;
  double* out = tx + (size_t)blk * n2 * n2;
  for (int idx = threadIdx.x; idx < n2 * n2; idx += blockDim.x) {
    const int t = idx % n2, v = idx / n2;
    const int p = t % nn, q = t / nn, i = v % nn, l = v / nn;
    const int ra = a * n2 + i + p * nn, rb = b * n2 + q + l * nn;
    double acc = 0.0;
    for (int k = 0; k < r; ++k) acc += s[k] * B[ra + (size_t)k * N] * B[rb + (size_t)k * N];
    out[idx] = sgn * acc;
  }
}

// ------------------------------------------------------------------ Coulomb
__global__ void dj_contract(DevDiatomic D, DevDiatomicScratch S, const double* __restrict__ P) {
  const int ch = blockIdx.x, e = blockIdx.y;
  const int nn = D.nn, n2 = nn * nn, L = D.ch_L[ch], M = D.ch_M[ch], ilm = D.ch_ilm[ch];
  const double fac = D.ch_fac[ch];
  extern __shared__ double sm[];
  double* X = sm;             // [2*n2]
  double* cv = X + 2 * n2;    // [rmax]
  double* red = cv + D.rmax;  // [32]
  for (int t = threadIdx.x; t < n2; t += blockDim.x) {
    const int p = t % nn, q = t / nn;
    const int gp = dgf(D, e, p), gq = dgf(D, e, q);
    double x0 = 0.0, x2 = 0.0;
    if (gp < D.nrad && gq < D.nrad)
      for (int k = 0; k < D.nang; ++k) {
        const int pk = dpure_idx(D, k, gp);
        if (pk < 0) continue;
        const int ix = al_idx(D, k, L, M);
        for (int u = D.al_ptr[ix]; u < D.al_ptr[ix + 1]; ++u) {
          const int pl = dpure_idx(D, D.al_b[u], gq);
          if (pl < 0) continue;
          const double v = P[(size_t)pl * D.nbf + pk];
          x0 += D.al_c0[u] * v;
          x2 += D.al_c2[u] * v;
        }
      }
    X[t] = x0;
    X[n2 + t] = x2;
  }
  __syncthreads();
  const size_t le = (size_t)ilm * D.nel + e;
  const double* P0 = D.p0 + le * n2;
  const double* P2 = D.p2 + le * n2;
  const double* Q0 = D.q0 + le * n2;
  const double* Q2 = D.q2 + le * n2;
  double ts0 = 0.0, tb0 = 0.0, ts2 = 0.0, tb2 = 0.0;
  for (int t = threadIdx.x; t < n2; t += blockDim.x) {
    const int p = t % nn, q = t / nn, tt = q + p * nn;  // tr(A X) = sum A(p,q) X(q,p)
    ts0 += P0[t] * X[tt];
    tb0 += Q0[t] * X[tt];
    ts2 += P2[t] * X[n2 + tt];
    tb2 += Q2[t] * X[n2 + tt];
  }
  ts0 = dblock_sum(ts0, red);
  tb0 = dblock_sum(tb0, red);
  ts2 = dblock_sum(ts2, red);
  tb2 = dblock_sum(tb2, red);
  if (threadIdx.x == 0) {
    double* sc = S.jscal + ((size_t)ch * D.nel + e) * 4;
    sc[0] = fac * ts0;
    sc[1] = fac * tb0;
    sc[2] = fac * ts2;
    sc[3] = fac * tb2;
  }
  const int r = D.cdrank[le], N = 2 * n2;
  const double* B = D.cdB + le * N * D.rmax;
  const double* sg = D.cds + le * D.rmax;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  for (int j = w; j < r; j += nw) {
    double s = 0.0;
    for (int v = lane; v < N; v += 32) s += B[v + (size_t)j * N] * X[v];
    s = dwarp_sum(s);
    if (lane == 0) cv[j] = s * sg[j];
  }
  __syncthreads();
  double* jin = S.jin + ((size_t)ch * D.nel + e) * N;
  for (int v = threadIdx.x; v < N; v += blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < r; ++j) s += B[v + (size_t)j * N] * cv[j];
    jin[v] = fac * s;
  }
}

// The full potential tiles of channel ch on element e (both multipole
// channels), in place over the in-element part:
//   T0 = big_e P0 + small_e Q0 + jin0,  T2 = -big_e P2 - small_e Q2 + jin2,
// big_e / small_e the traces of the outer / inner elements with the channel
// signs. grid (nchan, nel)
__global__ void dj_tiles(DevDiatomic D, DevDiatomicScratch S) {
  const int ch = blockIdx.x, e = blockIdx.y;
  const int n2 = D.nn * D.nn;
  __shared__ double bs[2];
  if (threadIdx.x == 0) {
    const double* sc = S.jscal + (size_t)ch * D.nel * 4;
    double big = 0.0, small = 0.0;
    for (int e2 = e + 1; e2 < D.nel; ++e2) big += sc[4 * e2 + 1] - sc[4 * e2 + 3];
    for (int e2 = 0; e2 < e; ++e2) small += sc[4 * e2 + 0] - sc[4 * e2 + 2];
    bs[0] = big;
    bs[1] = small;
  }
  __syncthreads();
  const double big = bs[0], small = bs[1];
  const size_t le = (size_t)D.ch_ilm[ch] * D.nel + e;
  double* jt = S.jin + ((size_t)ch * D.nel + e) * 2 * n2;
  for (int t = threadIdx.x; t < n2; t += blockDim.x) {
    jt[t] += big * D.p0[le * n2 + t] + small * D.q0[le * n2 + t];
    jt[n2 + t] += -big * D.p2[le * n2 + t] - small * D.q2[le * n2 + t];
  }
}

// J tile of output block (i, j) on element e = the bra sum of the channel
// tiles; the shared first function adds element e-1's corner. Written to the
// pure-basis J. grid (nang^2, nel)
__global__ void dj_scatter(DevDiatomic D, DevDiatomicScratch S, double* __restrict__ J) {
  const int ij = blockIdx.x, e = blockIdx.y;
  const int i = ij % D.nang, j = ij / D.nang;
  const int b0 = D.jbra_ptr[ij], b1 = D.jbra_ptr[ij + 1];
  const int nt = b1 - b0;
  if (nt == 0) return;
  const int nn = D.nn, n2 = nn * nn;
  for (int t = threadIdx.x; t < n2; t += blockDim.x) {
    const int p = t % nn, q = t / nn;
    // the corner on the boundary function shared with the next element is
    // owned by that element's tile
    if (p == nn - 1 && q == nn - 1) continue;
    const int pp = dpure_idx(D, i, dgf(D, e, p)), pq = dpure_idx(D, j, dgf(D, e, q));
    if (pp < 0 || pq < 0) continue;
    double v = 0.0;
    for (int u = b0; u < b1; ++u) {
      const double* jt = S.jin + ((size_t)D.jbra_chan[u] * D.nel + e) * 2 * n2;
      v += D.jbra_c0[u] * jt[t] + D.jbra_c2[u] * jt[n2 + t];
    }
    if (p == 0 && q == 0 && e > 0) {
      const int c = (nn - 1) + (nn - 1) * nn;
      for (int u = b0; u < b1; ++u) {
        const double* jt = S.jin + ((size_t)D.jbra_chan[u] * D.nel + (e - 1)) * 2 * n2;
        v += D.jbra_c0[u] * jt[c] + D.jbra_c2[u] * jt[n2 + c];
      }
    }
    J[(size_t)pq * D.nbf + pp] = v;
  }
}

// ----------------------------------------------------------------- exchange
__global__ void dk_norms(DevDiatomic D, const double* __restrict__ Pd, double* __restrict__ part,
                         float2* __restrict__ pd2) {
  __shared__ double red[32];
  const int blk = blockIdx.x, i = blk % D.nang, l = blk / D.nang;
  const int c0 = (int)((long)D.nrad * blockIdx.y / DNORM_SPLIT);
  const int c1 = (int)((long)D.nrad * (blockIdx.y + 1) / DNORM_SPLIT);
  double s = 0.0;
  const size_t n = (size_t)D.nrad * (c1 - c0);
  for (size_t idx = threadIdx.x; idx < n; idx += blockDim.x) {
    const size_t r = idx % D.nrad, c = c0 + idx / D.nrad;
    const size_t o = (size_t)(l * D.nrad + c) * D.nd + (size_t)i * D.nrad + r;
    const double v = Pd[o];
    s += v * v;
    if (pd2) pd2[o] = split_bits(v);
  }
  s = dblock_sum(s, red);
  if (threadIdx.x == 0) part[blk * DNORM_SPLIT + blockIdx.y] = s;
}

__global__ void dk_act(DevDiatomic D, DevDiatomicScratch S) {
  const int n = D.nang * D.nang;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < DNORM_SPLIT; ++c) s += S.bnorm[idx * DNORM_SPLIT + c];
    S.act[idx] = !(sqrt(s) < 10.0 * DBL_EPSILON);
  }
}

__global__ void dk_entry_act(DevDiatomic D, DevDiatomicScratch S) {
  for (int ent = blockIdx.x * blockDim.x + threadIdx.x; ent < D.nent; ent += gridDim.x * blockDim.x) {
    const int jk = D.kent_jk[ent], j = jk % D.nang, k = jk / D.nang;
    const int L = D.kent_L[ent], Ma = D.kent_Ma[ent];
    bool any = false;
    for (int sgn = 0; sgn < (Ma ? 2 : 1) && !any; ++sgn) {
      const int M = sgn ? -Ma : Ma;
      const int xj = al_idx(D, j, L, M), xk = al_idx(D, k, L, M);
      for (int uj = D.al_ptr[xj]; uj < D.al_ptr[xj + 1] && !any; ++uj) {
        const int i = D.al_b[uj];
        for (int uk = D.al_ptr[xk]; uk < D.al_ptr[xk + 1]; ++uk)
          if (S.act[i + D.al_b[uk] * D.nang]) { any = true; break; }
      }
    }
    S.ent_act[ent] = any ? 1 : 0;
  }
}

// one CTA: flags and compacted lists of the active output blocks (all, and
// those with j <= k for the symmetric mode), in ascending jk order
__global__ void dk_compact(DevDiatomic D, DevDiatomicScratch S) {
  __shared__ int ca[1024], cs[1024];
  const int n = D.nang * D.nang, nt = blockDim.x;
  const int chunk = (n + nt - 1) / nt;
  const int lo = min(n, (int)threadIdx.x * chunk), hi = min(n, lo + chunk);
  int na = 0, ns = 0;
  for (int jk = lo; jk < hi; ++jk) {
    bool a = false;
    for (int ent = D.kjk_ptr[jk]; ent < D.kjk_ptr[jk + 1]; ++ent)
      if (S.ent_act[ent]) { a = true; break; }
    S.jk_act[jk] = a ? 1 : 0;
    if (a) {
      ++na;
      if (jk % D.nang <= jk / D.nang) ++ns;
    }
  }
  ca[threadIdx.x] = na;
  cs[threadIdx.x] = ns;
  __syncthreads();
  if (threadIdx.x == 0) {
    int sa = 0, ss = 0;
    for (int t = 0; t < nt; ++t) {
      const int a = ca[t], s = cs[t];
      ca[t] = sa;
      cs[t] = ss;
      sa += a;
      ss += s;
    }
    S.counts[0] = sa;
    S.counts[1] = ss;
  }
  __syncthreads();
  int oa = ca[threadIdx.x], os = cs[threadIdx.x];
  for (int jk = lo; jk < hi; ++jk)
    if (S.jk_act[jk]) {
      S.jk_list[oa++] = jk;
      if (jk % D.nang <= jk / D.nang) S.jk_list[n + os++] = jk;
    }
}

__device__ __forceinline__ size_t dhalo_idx(const DevDiatomic& D, int a, int b, int jk, int h) {
  return ((size_t)(a * D.nel + b) * (D.nang * D.nang) + jk) * (2 * D.nn - 1) + h;
}

__device__ __forceinline__ void dk_store(const DevDiatomic& D, const DevDiatomicScratch& S, double* Kd, int a, int b,
                                         int jk, int p, int q, double y) {
  const int nn = D.nn;
  const int gp = dgf(D, a, p), gq = dgf(D, b, q);
  if (gp >= D.nrad || gq >= D.nrad) return;
  const int j = jk % D.nang, k = jk / D.nang;
  if (p <= nn - 2 && q <= nn - 2)
    Kd[(size_t)(k * D.nrad + gq) * D.nd + (size_t)j * D.nrad + gp] = y;
  else if (p == nn - 1)
    S.khalo[dhalo_idx(D, a, b, jk, q)] = y;
  else
    S.khalo[dhalo_idx(D, a, b, jk, nn + p)] = y;
}

// Persistent CTAs over work items. Item w < n_off: element pair
// pairs[w / n_act], output block jk_list[w % n_act]; the rest: diagonal
// element e, output block from the (symmetric: j <= k) list. In symmetric
// mode (P = P^T) only a < b pairs are items and each also writes the
// transposed partner tile, K_kj(b,a) = K_jk(a,b)^T.
__global__ void __launch_bounds__(320) dk_tiles(DevDiatomic D, DevDiatomicScratch S, const double* __restrict__ Pd,
                                                double* __restrict__ Kd, int symmetric) {
  const int nn = D.nn, n2 = nn * nn, nang2 = D.nang * D.nang;
  const int n_act = S.counts[0], n_dact = symmetric ? S.counts[1] : S.counts[0];
  const int* dlist = symmetric ? S.jk_list + nang2 : S.jk_list;
  const int2* pairs = symmetric ? D.pairs_sym : D.pairs_all;
  const long npairs = symmetric ? D.npairs_sym : D.npairs_all;
  const long n_off = npairs * n_act, total = n_off + (long)D.nel * n_dact;
  extern __shared__ double sm[];
  double* X = sm;            // [4*n2]: R00, R02, R20, R22 tiles
  double* T = X + 4 * n2;    // [2*n2]
  double* Im = T + 2 * n2;   // [2*n2] row-element integrals (channel 0, 2)
  double* Jm = Im + 2 * n2;  // [2*n2] column-element integrals
  unsigned char* act = reinterpret_cast<unsigned char*>(Jm + 2 * n2);
  for (int idx = threadIdx.x; idx < nang2; idx += blockDim.x) act[idx] = S.act[idx];
  __syncthreads();
  const int t = threadIdx.x;
  const bool live = t < n2;
  const int p = live ? t % nn : 0, q = live ? t / nn : 0;
  for (long w = blockIdx.x; w < total; w += gridDim.x) {
    int a, b, jk;
    if (w < n_off) {
      const int2 pr = pairs[w / n_act];
      a = pr.x;
      b = pr.y;
      jk = S.jk_list[w % n_act];
    } else {
      const long w2 = w - n_off;
      a = b = (int)(w2 / n_dact);
      jk = dlist[w2 % n_dact];
    }
    const bool diag = (a == b);
    const int j = jk % D.nang, k = jk / D.nang;
    const int gp = dgf(D, a, p), gq = dgf(D, b, q);
    const bool vpq = live && gp < D.nrad && gq < D.nrad;
    double y = 0.0;
    for (int ent = D.kjk_ptr[jk]; ent < D.kjk_ptr[jk + 1]; ++ent) {
      if (!S.ent_act[ent]) continue;  // uniform over the CTA
      const int L = D.kent_L[ent], Ma = D.kent_Ma[ent], ilm = D.kent_ilm[ent];
      double x00 = 0.0, x02 = 0.0, x20 = 0.0, x22 = 0.0;
      if (vpq) {
        for (int sgn = 0; sgn < (Ma ? 2 : 1); ++sgn) {
          const int M = sgn ? -Ma : Ma;
          const int xj = al_idx(D, j, L, M), xk = al_idx(D, k, L, M);
          const int k0 = D.al_ptr[xk], k1 = D.al_ptr[xk + 1];
          for (int uj = D.al_ptr[xj]; uj < D.al_ptr[xj + 1]; ++uj) {
            const int i = D.al_b[uj];
            const double* Pi = Pd + (size_t)i * D.nrad + gp;
            double u0 = 0.0, u2 = 0.0;
            for (int uk = k0; uk < k1; ++uk) {
              const int l = D.al_b[uk];
              if (!act[i + l * D.nang]) continue;
              const double v = Pi[(size_t)(l * D.nrad + gq) * D.nd];
              u0 += D.al_c0[uk] * v;
              u2 += D.al_c2[uk] * v;
            }
            const double c0 = D.al_c0[uj], c2 = D.al_c2[uj];
            x00 += c0 * u0;
            x02 += c0 * u2;
            x20 += c2 * u0;
            x22 += c2 * u2;
          }
        }
      }
      const double fac = (Ma & 1) ? -D.lmfac[ilm] : D.lmfac[ilm];
      if (live) {
        X[t] = fac * x00;
        X[n2 + t] = -fac * x02;
        X[2 * n2 + t] = -fac * x20;
        X[3 * n2 + t] = fac * x22;
        if (!diag) {
          const size_t la = ((size_t)ilm * D.nel + a) * n2 + t, lb = ((size_t)ilm * D.nel + b) * n2 + t;
          Im[t] = (a < b) ? D.p0[la] : D.q0[la];
          Im[n2 + t] = (a < b) ? D.p2[la] : D.q2[la];
          Jm[t] = (a < b) ? D.q0[lb] : D.p0[lb];
          Jm[n2 + t] = (a < b) ? D.q2[lb] : D.p2[lb];
        }
      }
      __syncthreads();
      if (diag) {
        if (live) {
          const double* tx = D.tx + ((size_t)ilm * D.nel + a) * 4 * n2 * n2;
          double s = 0.0;
          for (int ab = 0; ab < 4; ++ab) {
            const double* txb = tx + (size_t)ab * n2 * n2;
            const double* Xb = X + ab * n2;
            for (int v = 0; v < n2; ++v) s += txb[t + (size_t)v * n2] * Xb[v];
          }
          y += s;
        }
      } else {
        if (live) {
          double s0 = 0.0, s2 = 0.0;
          for (int c = 0; c < nn; ++c) {
            const double j0 = Jm[q + c * nn], j2 = Jm[n2 + q + c * nn];
            s0 += X[p + c * nn] * j0 + X[n2 + p + c * nn] * j2;
            s2 += X[2 * n2 + p + c * nn] * j0 + X[3 * n2 + p + c * nn] * j2;
          }
          T[t] = s0;
          T[n2 + t] = s2;
        }
        __syncthreads();
        if (live) {
          double s = 0.0;
          for (int c = 0; c < nn; ++c) s += Im[p + c * nn] * T[c + q * nn] + Im[n2 + p + c * nn] * T[n2 + c + q * nn];
          y += s;
        }
      }
      __syncthreads();
    }
    if (live) dk_store(D, S, Kd, a, b, jk, p, q, -y);
    if (symmetric && (!diag || j != k)) {
      if (live) X[t] = -y;
      __syncthreads();
      if (live) dk_store(D, S, Kd, b, a, k + j * D.nang, p, q, X[q + p * nn]);
      __syncthreads();
    }
  }
}

// Split-precision tiles: dk_tiles with every operand a (hi, lo) float pair,
// TwoProd/TwoSum products on the FP32 pipe, the per-multipole results summed
// as float pairs and recombined in FP64 once per output element.
template <int NN>
// 15-node elements: 256 threads, at most 51 registers so that five CTAs share an SM
__global__ void __launch_bounds__(NN == 15 ? 256 : 320, NN == 15 ? 5 : 1) dk_tiles_split(DevDiatomic D, DevDiatomicScratch S, double* __restrict__ Kd,
                                                      int symmetric, int with_diag) {
  const int nn = NN > 0 ? NN : D.nn, n2 = nn * nn, nang2 = D.nang * D.nang;
  const int n_act = S.counts[0], n_dact = symmetric ? S.counts[1] : S.counts[0];
  const int* dlist = symmetric ? S.jk_list + nang2 : S.jk_list;
  const int2* pairs = symmetric ? D.pairs_sym : D.pairs_all;
  const long npairs = symmetric ? D.npairs_sym : D.npairs_all;
  const long n_off = npairs * n_act, total = n_off + (with_diag ? (long)D.nel * n_dact : 0L);
  extern __shared__ float2 sm2[];
  float2* X = sm2;           // [4*n2]
  float2* T = X + 4 * n2;    // [2*n2]
  float2* Im = T + 2 * n2;   // [2*n2]
  float2* Jm = Im + 2 * n2;  // [2*n2]
  double* Y = reinterpret_cast<double*>(Jm + 2 * n2);
  unsigned char* act = reinterpret_cast<unsigned char*>(Y + n2);
  for (int idx = threadIdx.x; idx < nang2; idx += blockDim.x) act[idx] = S.act[idx];
  __syncthreads();
  const int t = threadIdx.x;
  const bool live = t < n2;
  const int p = live ? t % nn : 0, q = live ? t / nn : 0;
  for (long w = blockIdx.x; w < total; w += gridDim.x) {
    int a, b, jk;
    if (w < n_off) {
      const int2 pr = pairs[w / n_act];
      a = pr.x;
      b = pr.y;
      jk = S.jk_list[w % n_act];
    } else {
      const long w2 = w - n_off;
      a = b = (int)(w2 / n_dact);
      jk = dlist[w2 % n_dact];
    }
    const bool diag = (a == b);
    const int j = jk % D.nang, k = jk / D.nang;
    const int gp = dgf(D, a, p), gq = dgf(D, b, q);
    const bool vpq = live && gp < D.nrad && gq < D.nrad;
    const float2* pbase = S.pd2 + (size_t)gq * D.nd + gp;
    ffv yacc = {0.f, 0.f};
    for (int ent = D.kjk_ptr[jk]; ent < D.kjk_ptr[jk + 1]; ++ent) {
      if (!S.ent_act[ent]) continue;  // uniform over the CTA
      const int L = D.kent_L[ent], Ma = D.kent_Ma[ent], ilm = D.kent_ilm[ent];
      ffv x00 = {0.f, 0.f}, x02 = {0.f, 0.f}, x20 = {0.f, 0.f}, x22 = {0.f, 0.f};
      if (vpq) {
        for (int sgn = 0; sgn < (Ma ? 2 : 1); ++sgn) {
          const int M = sgn ? -Ma : Ma;
          const int xj = al_idx(D, j, L, M), xk = al_idx(D, k, L, M);
          const int k0 = D.al_ptr[xk], k1 = D.al_ptr[xk + 1];
          for (int uj = D.al_ptr[xj]; uj < D.al_ptr[xj + 1]; ++uj) {
            const int i = D.al_b[uj];
            ffv u0 = {0.f, 0.f}, u2 = {0.f, 0.f};
            for (int uk = k0; uk < k1; ++uk) {
              const int l = D.al_b[uk];
              if (!act[i + l * D.nang]) continue;
              const float2 v = pbase[(size_t)(l * D.nrad) * D.nd + (size_t)i * D.nrad];
              u0 = ff_fma(u0, D.al_c0s[uk], v);
              u2 = ff_fma(u2, D.al_c2s[uk], v);
            }
            const float2 U0 = ff2(u0), U2 = ff2(u2), c0 = D.al_c0s[uj], c2 = D.al_c2s[uj];
            x00 = ff_fma(x00, c0, U0);
            x02 = ff_fma(x02, c0, U2);
            x20 = ff_fma(x20, c2, U0);
            x22 = ff_fma(x22, c2, U2);
          }
        }
      }
      if (live) {
        float2 fac = D.lmfacs[ilm];
        if (Ma & 1) fac = make_float2(-fac.x, -fac.y);
        const ffv z = {0.f, 0.f};
        const float2 f00 = ff2(ff_fma(z, fac, ff2(x00))), f02 = ff2(ff_fma(z, fac, ff2(x02)));
        const float2 f20 = ff2(ff_fma(z, fac, ff2(x20))), f22 = ff2(ff_fma(z, fac, ff2(x22)));
        X[t] = f00;
        X[n2 + t] = make_float2(-f02.x, -f02.y);
        X[2 * n2 + t] = make_float2(-f20.x, -f20.y);
        X[3 * n2 + t] = f22;
        if (!diag) {
          const size_t la = ((size_t)ilm * D.nel + a) * n2 + t, lb = ((size_t)ilm * D.nel + b) * n2 + t;
          Im[t] = (a < b) ? D.p0s[la] : D.q0s[la];
          Im[n2 + t] = (a < b) ? D.p2s[la] : D.q2s[la];
          Jm[t] = (a < b) ? D.q0s[lb] : D.p0s[lb];
          Jm[n2 + t] = (a < b) ? D.q2s[lb] : D.p2s[lb];
        }
      }
      __syncthreads();
      ffv acc = {0.f, 0.f};
      if (diag) {
        if (live) {
          const float2* tx = D.txs + ((size_t)ilm * D.nel + a) * 4 * n2 * n2;
          for (int ab = 0; ab < 4; ++ab) {
            const float2* txb = tx + (size_t)ab * n2 * n2;
            const float2* Xb = X + ab * n2;
            for (int v0 = 0; v0 < n2; v0 += nn) {
              if (NN > 0) {  // unrolled: the nn table loads are issued together
#pragma unroll
                for (int c = 0; c < (NN > 0 ? NN : 1); ++c)
                  acc = ff_fma(acc, txb[t + (size_t)(v0 + c) * n2], Xb[v0 + c]);
              } else {
                for (int v = v0; v < v0 + nn; ++v) acc = ff_fma(acc, txb[t + (size_t)v * n2], Xb[v]);
              }
              acc = ff_norm(acc.hi, acc.lo);
            }
          }
        }
      } else {
        if (live) {
          ffv s0 = {0.f, 0.f}, s2 = {0.f, 0.f};
#pragma unroll
          for (int c = 0; c < (NN > 0 ? NN : 17); ++c) {
            if (NN == 0 && c >= nn) break;
            const float2 j0 = Jm[q + c * nn], j2 = Jm[n2 + q + c * nn];
            s0 = ff_fma(s0, X[p + c * nn], j0);
            s0 = ff_fma(s0, X[n2 + p + c * nn], j2);
            s2 = ff_fma(s2, X[2 * n2 + p + c * nn], j0);
            s2 = ff_fma(s2, X[3 * n2 + p + c * nn], j2);
          }
          T[t] = ff2(s0);
          T[n2 + t] = ff2(s2);
        }
        __syncthreads();
        if (live) {
#pragma unroll
          for (int c = 0; c < (NN > 0 ? NN : 17); ++c) {
            if (NN == 0 && c >= nn) break;
            acc = ff_fma(acc, Im[p + c * nn], T[c + q * nn]);
            acc = ff_fma(acc, Im[n2 + p + c * nn], T[n2 + c + q * nn]);
          }
          // undo the tables' power-of-two scaling: 2^(k_inner - k_outer) <= 1
          const int ka = D.kexp[(size_t)ilm * D.nel + a], kb = D.kexp[(size_t)ilm * D.nel + b];
          const int dk = (a < b) ? ka - kb : kb - ka;
          acc.hi = ldexpf(acc.hi, dk);
          acc.lo = ldexpf(acc.lo, dk);
        }
      }
      yacc = ff_add(yacc, ff_norm(acc.hi, acc.lo));
      __syncthreads();
    }
    const double y = ff_to_d(yacc);
    if (live) dk_store(D, S, Kd, a, b, jk, p, q, -y);
    if (symmetric && (!diag || j != k)) {
      if (live) Y[t] = -y;
      __syncthreads();
      if (live) dk_store(D, S, Kd, b, a, k + j * D.nang, p, q, Y[q + p * nn]);
      __syncthreads();
    }
  }
}

// Diagonal element tiles of the split exchange, G output blocks per item.
// Item w: element e = w / ngroups, the active output blocks
// dlist[G*(w % ngroups) ...]. The members' entry lists (ascending multipole
// index ilm) are merged: per multipole present in any member, the members
// holding it recouple their density tiles into shared memory, then one pass
// over the exchange-ordered kernel table of (ilm, e) feeds all of them, so
// each table element is loaded once per item instead of once per member.
// Per member the operations and their order are those of the item-by-item
// schedule in dk_tiles_split, so K is bitwise the same.
constexpr int DIAG_GROUP = 8;

template <int NN, int G>
__global__ void __launch_bounds__(NN == 15 ? 256 : 320, NN == 15 ? 3 : 1) dk_diag_split(DevDiatomic D, DevDiatomicScratch S, double* __restrict__ Kd,
                                                         int symmetric) {
  const int nn = NN > 0 ? NN : D.nn, n2 = nn * nn, nang2 = D.nang * D.nang;
  const int n_dact = symmetric ? S.counts[1] : S.counts[0];
  const int* dlist = symmetric ? S.jk_list + nang2 : S.jk_list;
  const int ngrp = (n_dact + G - 1) / G;
  const long total = (long)D.nel * ngrp;
  extern __shared__ float2 sm2[];
  float2* X = sm2;  // [G][4*n2]
  double* Y = reinterpret_cast<double*>(X + (size_t)G * 4 * n2);
  unsigned char* act = reinterpret_cast<unsigned char*>(Y + n2);
  __shared__ int s_ptr[G], s_end[G], s_jk[G], s_has[G];
  __shared__ int s_ilm;
  for (int idx = threadIdx.x; idx < nang2; idx += blockDim.x) act[idx] = S.act[idx];
  __syncthreads();
  const int t = threadIdx.x;
  const bool live = t < n2;
  const int p = live ? t % nn : 0, q = live ? t / nn : 0;
  for (long w = blockIdx.x; w < total; w += gridDim.x) {
    const int e = (int)(w / ngrp), g0 = (int)(w % ngrp) * G;
    const int ng = min(G, n_dact - g0);
    if (t < G) {
      if (t < ng) {
        const int jk = dlist[g0 + t];
        s_jk[t] = jk;
        s_ptr[t] = D.kjk_ptr[jk];
        s_end[t] = D.kjk_ptr[jk + 1];
      } else {
        s_jk[t] = -1;
        s_ptr[t] = s_end[t] = 0;
      }
    }
    __syncthreads();
    const int gp = dgf(D, e, p), gq = dgf(D, e, q);
    const bool vpq = live && gp < D.nrad && gq < D.nrad;
    const float2* pbase = S.pd2 + (size_t)gq * D.nd + gp;
    ffv yacc[G];
#pragma unroll
    for (int g = 0; g < G; ++g) yacc[g] = {0.f, 0.f};
    for (;;) {
      if (t < 32) {  // warp 0: skip inactive entries, smallest pending multipole
        int pt = 0, me = 0x7fffffff;
        if (t < G) {
          pt = s_ptr[t];
          while (pt < s_end[t] && !S.ent_act[pt]) ++pt;
          s_ptr[t] = pt;
          if (pt < s_end[t]) me = D.kent_ilm[pt];
        }
        int m = me;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (t < G) s_has[t] = (me == m && m != 0x7fffffff) ? 1 : 0;
        if (t == 0) s_ilm = m;
      }
      __syncthreads();
      const int ilm = s_ilm;
      if (ilm == 0x7fffffff) break;
#pragma unroll 1
      for (int g = 0; g < G; ++g) {
        float2* Xg = X + (size_t)g * 4 * n2;
        if (!s_has[g]) {  // uniform over the CTA
          if (live) Xg[t] = Xg[n2 + t] = Xg[2 * n2 + t] = Xg[3 * n2 + t] = make_float2(0.f, 0.f);
          continue;
        }
        const int ent = s_ptr[g], jk = s_jk[g];
        const int j = jk % D.nang, k = jk / D.nang;
        const int L = D.kent_L[ent], Ma = D.kent_Ma[ent];
        ffv x00 = {0.f, 0.f}, x02 = {0.f, 0.f}, x20 = {0.f, 0.f}, x22 = {0.f, 0.f};
        if (vpq) {
          for (int sgn = 0; sgn < (Ma ? 2 : 1); ++sgn) {
            const int M = sgn ? -Ma : Ma;
            const int xj = al_idx(D, j, L, M), xk = al_idx(D, k, L, M);
            const int k0 = D.al_ptr[xk], k1 = D.al_ptr[xk + 1];
            for (int uj = D.al_ptr[xj]; uj < D.al_ptr[xj + 1]; ++uj) {
              const int i = D.al_b[uj];
              ffv u0 = {0.f, 0.f}, u2 = {0.f, 0.f};
              for (int uk = k0; uk < k1; ++uk) {
                const int l = D.al_b[uk];
                if (!act[i + l * D.nang]) continue;
                const float2 v = pbase[(size_t)(l * D.nrad) * D.nd + (size_t)i * D.nrad];
                u0 = ff_fma(u0, D.al_c0s[uk], v);
                u2 = ff_fma(u2, D.al_c2s[uk], v);
              }
              const float2 U0 = ff2(u0), U2 = ff2(u2), c0 = D.al_c0s[uj], c2 = D.al_c2s[uj];
              x00 = ff_fma(x00, c0, U0);
              x02 = ff_fma(x02, c0, U2);
              x20 = ff_fma(x20, c2, U0);
              x22 = ff_fma(x22, c2, U2);
            }
          }
        }
        if (live) {
          float2 fac = D.lmfacs[ilm];
          if (Ma & 1) fac = make_float2(-fac.x, -fac.y);
          const ffv z = {0.f, 0.f};
          const float2 f00 = ff2(ff_fma(z, fac, ff2(x00))), f02 = ff2(ff_fma(z, fac, ff2(x02)));
          const float2 f20 = ff2(ff_fma(z, fac, ff2(x20))), f22 = ff2(ff_fma(z, fac, ff2(x22)));
          Xg[t] = f00;
          Xg[n2 + t] = make_float2(-f02.x, -f02.y);
          Xg[2 * n2 + t] = make_float2(-f20.x, -f20.y);
          Xg[3 * n2 + t] = f22;
        }
      }
      __syncthreads();
      if (live) {
        ffv acc[G];
#pragma unroll
        for (int g = 0; g < G; ++g) acc[g] = {0.f, 0.f};
        const float2* tx = D.txs + ((size_t)ilm * D.nel + e) * 4 * n2 * n2;
        for (int ab = 0; ab < 4; ++ab) {
          const float2* txb = tx + (size_t)ab * n2 * n2;
          for (int v0 = 0; v0 < n2; v0 += nn) {
            if (NN > 0) {
#pragma unroll
              for (int c = 0; c < (NN > 0 ? NN : 1); ++c) {
                const float2 tv = txb[t + (size_t)(v0 + c) * n2];
#pragma unroll
                for (int g = 0; g < G; ++g) acc[g] = ff_fma(acc[g], tv, X[(size_t)g * 4 * n2 + ab * n2 + v0 + c]);
              }
            } else {
              for (int v = v0; v < v0 + nn; ++v) {
                const float2 tv = txb[t + (size_t)v * n2];
#pragma unroll
                for (int g = 0; g < G; ++g) acc[g] = ff_fma(acc[g], tv, X[(size_t)g * 4 * n2 + ab * n2 + v]);
              }
            }
#pragma unroll
            for (int g = 0; g < G; ++g) acc[g] = ff_norm(acc[g].hi, acc[g].lo);
          }
        }
#pragma unroll
        for (int g = 0; g < G; ++g)
          if (s_has[g]) yacc[g] = ff_add(yacc[g], ff_norm(acc[g].hi, acc[g].lo));
      }
      __syncthreads();
      if (t < G && s_has[t]) ++s_ptr[t];
    }
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (g >= ng) break;  // uniform over the CTA
      const int jk = s_jk[g], j = jk % D.nang, k = jk / D.nang;
      const double y = ff_to_d(yacc[g]);
      if (live) dk_store(D, S, Kd, e, e, jk, p, q, -y);
      if (symmetric && j != k) {
        if (live) Y[t] = -y;
        __syncthreads();
        if (live) dk_store(D, S, Kd, e, e, k + j * D.nang, p, q, Y[q + p * nn]);
      }
      __syncthreads();
    }
  }
}

__global__ void d_split(const double* __restrict__ x, float2* __restrict__ y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = split_bits(x[i]);
}

// Shared-boundary fix-up: entry (p,q) of tile (a,b) in its first row or
// column also receives the last row of the tile above (a-1,b), the last
// column of the tile to the left (a,b-1) and, at the corner, the last corner
// of (a-1,b-1). Unlike the atomic basis, element 0 keeps its first function
// (mu = 0), so the first row of a = 0 tiles and the first column of b = 0
// tiles are real entries too.
__global__ void dk_fixup(DevDiatomic D, DevDiatomicScratch S, double* __restrict__ Kd) {
  const int a = blockIdx.x % D.nel, b = blockIdx.x / D.nel;
  const int nn = D.nn, per = 2 * nn - 3, n_act = S.counts[0];
  for (long w = threadIdx.x; w < (long)per * n_act; w += blockDim.x) {
    const int idx = (int)(w % per), jk = S.jk_list[w / per];
    const int j = jk % D.nang, k = jk / D.nang;
    const int p = idx < nn - 1 ? 0 : idx - (nn - 1) + 1;  // first row q in [0, nn-2], then first column
    const int q = idx < nn - 1 ? idx : 0;
    double v = 0.0;
    bool any = false;
    if (p == 0 && a > 0) {
      v += S.khalo[dhalo_idx(D, a - 1, b, jk, q)];
      any = true;
    }
    if (q == 0 && b > 0) {
      v += S.khalo[dhalo_idx(D, a, b - 1, jk, nn + p)];
      any = true;
    }
    if (p == 0 && q == 0 && a > 0 && b > 0) v += S.khalo[dhalo_idx(D, a - 1, b - 1, jk, nn - 1)];
    if (!any) continue;
    const int gp = dgf(D, a, p), gq = dgf(D, b, q);
    if (gp >= D.nrad || gq >= D.nrad) continue;
    Kd[(size_t)(k * D.nrad + gq) * D.nd + (size_t)j * D.nrad + gp] += v;
  }
}

inline int dthreads(int n2) { return ((n2 + 31) / 32) * 32; }
inline int dgrid(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 32); }

}  // namespace

cudaError_t launch_diatomic_expand(const double* P, int nbf, const int* pure, double* Pd, int nd, cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(Pd, 0, sizeof(double) * (size_t)nd * nd, st);
  if (e != cudaSuccess) return e;
  d_expand<<<dgrid((size_t)nbf * nbf), 256, 0, st>>>(P, nbf, pure, Pd, nd);
  return cudaGetLastError();
}

cudaError_t launch_diatomic_gather(const double* Fd, int nd, const int* pure, int nbf, double* F, cudaStream_t st) {
  d_gather<<<dgrid((size_t)nbf * nbf), 256, 0, st>>>(Fd, nd, pure, nbf, F);
  return cudaGetLastError();
}

cudaError_t launch_diatomic_tx(const DevDiatomic& D, double* tx, cudaStream_t st) {
  d_build_tx<<<D.nlm * D.nel * 4, 256, 0, st>>>(D, tx);
  return cudaGetLastError();
}

cudaError_t launch_diatomic_coulomb(const DevDiatomic& D, const DevDiatomicScratch& S, const double* P, double* J,
                                    cudaStream_t st) {
  const int n2 = D.nn * D.nn, th = dthreads(n2);
  cudaError_t e = cudaMemsetAsync(J, 0, sizeof(double) * (size_t)D.nbf * D.nbf, st);
  if (e != cudaSuccess) return e;
  const size_t sm1 = sizeof(double) * (2 * n2 + D.rmax + 32);
  dj_contract<<<dim3(D.nchan, D.nel), th, sm1, st>>>(D, S, P);
  dj_tiles<<<dim3(D.nchan, D.nel), th, 0, st>>>(D, S);
  dj_scatter<<<dim3(D.nang * D.nang, D.nel), th, 0, st>>>(D, S, J);
  return cudaGetLastError();
}

cudaError_t launch_diatomic_exchange(const DevDiatomic& D, const DevDiatomicScratch& S, const double* Pd, double* Kd,
                                     bool symmetric, cudaStream_t st) {
  const int n2 = D.nn * D.nn, th = dthreads(n2), nang2 = D.nang * D.nang;
  cudaError_t e = cudaMemsetAsync(Kd, 0, sizeof(double) * (size_t)D.nd * D.nd, st);
  if (e != cudaSuccess) return e;
  dk_norms<<<dim3(nang2, DNORM_SPLIT), 256, 0, st>>>(D, Pd, S.bnorm, nullptr);
  dk_act<<<(nang2 + 255) / 256, 256, 0, st>>>(D, S);
  dk_entry_act<<<(D.nent + 127) / 128 > 0 ? (D.nent + 127) / 128 : 1, 128, 0, st>>>(D, S);
  dk_compact<<<1, 1024, 0, st>>>(D, S);
  int dev = 0, nsm = 152, per = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = sizeof(double) * 10 * n2 + nang2;
  e = smem_limit(dk_tiles, smem);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, dk_tiles, th, smem);
  if (e != cudaSuccess) return e;
  const int grid = nsm * std::max(per, 1);
  dk_tiles<<<grid, th, smem, st>>>(D, S, Pd, Kd, symmetric ? 1 : 0);
  dk_fixup<<<D.nel * D.nel, 256, 0, st>>>(D, S, Kd);
  return cudaGetLastError();
}

cudaError_t launch_diatomic_split_tx(const double* tx, float2* txs, size_t n, cudaStream_t st) {
  d_split<<<dgrid(n), 256, 0, st>>>(tx, txs, n);
  return cudaGetLastError();
}

cudaError_t launch_diatomic_exchange_split(const DevDiatomic& D, const DevDiatomicScratch& S, const double* Pd,
                                           double* Kd, bool symmetric, cudaStream_t st, bool inline_diag) {
  const int n2 = D.nn * D.nn, th = dthreads(n2), nang2 = D.nang * D.nang;
  cudaError_t e = cudaMemsetAsync(Kd, 0, sizeof(double) * (size_t)D.nd * D.nd, st);
  if (e != cudaSuccess) return e;
  dk_norms<<<dim3(nang2, DNORM_SPLIT), 256, 0, st>>>(D, Pd, S.bnorm, S.pd2);
  dk_act<<<(nang2 + 255) / 256, 256, 0, st>>>(D, S);
  dk_entry_act<<<(D.nent + 127) / 128 > 0 ? (D.nent + 127) / 128 : 1, 128, 0, st>>>(D, S);
  dk_compact<<<1, 1024, 0, st>>>(D, S);
  int dev = 0, nsm = 152, per = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = sizeof(float2) * 10 * n2 + sizeof(double) * n2 + nang2;
  auto kern = (D.nn == 15) ? dk_tiles_split<15> : dk_tiles_split<0>;
  e = smem_limit(kern, smem);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, th, smem);
  if (e != cudaSuccess) return e;
  kern<<<nsm * std::max(per, 1), th, smem, st>>>(D, S, Kd, symmetric ? 1 : 0, inline_diag ? 1 : 0);
  if (!inline_diag) {
    constexpr int G = DIAG_GROUP;
    const size_t smd = sizeof(float2) * (size_t)G * 4 * n2 + sizeof(double) * n2 + nang2;
    auto dkern = (D.nn == 15) ? dk_diag_split<15, G> : dk_diag_split<0, G>;
    e = smem_limit(dkern, smd);
    if (e != cudaSuccess) return e;
    int dper = 1;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&dper, dkern, th, smd);
    if (e != cudaSuccess) return e;
    dkern<<<nsm * std::max(dper, 1), th, smd, st>>>(D, S, Kd, symmetric ? 1 : 0);
  }
  dk_fixup<<<D.nel * D.nel, 256, 0, st>>>(D, S, Kd);
  return cudaGetLastError();
}

}  // namespace hfg

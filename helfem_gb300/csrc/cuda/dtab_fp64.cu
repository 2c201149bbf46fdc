// Device tabulation of the diatomic two-electron primitives, FP64.
//
// Follows src/diatomic/basis.cpp:1382-1547 (compute_tei: the disjoint
// Plm/Qlm integrals of every (L,|M|) and element, and the in-element
// two-channel kernel of src/diatomic/quadrature.cpp:175-255 with its
// sign-carrying pivoted factor) with the host tabulation's fixed
// Gauss-Legendre rules, its map mu = mu_1 t^3 on the first element and its
// pivoting rule, so that the two tabulations agree to rounding:
//
//   dtab_pq           Legendre P_L^M, Q_L^M(cosh mu) at every disjoint and
//                     outer point, one thread per point (upward recurrence
//                     for P; Q_0 and Q^1 in closed form near mu = 0, else by
//                     a normalised backward recurrence; upward in M)
//   dtab_disjoint     p0/p2/q0/q2 tiles, one CTA per (element, multipole)
//   dtab_inner_outer  per (outer point, element, 32 multipoles): the inner
//                     integrals int_{mu_s}^{mu_1} B_a B_b sinh cosh^k P over
//                     the 64 inner points, and the outer weights with Q
//   dtab_gemm         R = O^T I per (multipole, element): the in-element
//                     kernel before symmetrisation, (2 np)^2 entries
//   dtab_chol         the sign-carrying pivoted factor of the two-channel
//                     kernel W, one CTA per tile, W read from R on the fly
//   dtab_pack         factor columns into a padded layout
#include <algorithm>
#include <cfloat>
#include <climits>

#include "dtab.cuh"
#include "smem_limit.hpp"

namespace hfg {
namespace {

constexpr int DT_LMC = 32;     // multipoles per inner/outer CTA
constexpr int DT_THREADS = 256;
constexpr int DCHOL = 640;     // factor CTA: one thread per row of W (2 nn^2 <= 578)

__device__ __forceinline__ double clean(double v) {
  return (!isfinite(v) || (v != 0.0 && fabs(v) < DBL_MIN)) ? 0.0 : v;
}

// pair index k = a + b (b + 1) / 2 (a <= b) -> (a, b)
__device__ __forceinline__ void pair_of(int k, int& a, int& b) {
  b = 0;
  while ((b + 1) * (b + 2) / 2 <= k) ++b;
  a = k - b * (b + 1) / 2;
}

// P_L^M(x), x = cosh(mu), w = sinh(mu), Hobson convention: emit(M, L, P)
// for M <= min(Mmax, Lmax), M <= L <= Lmax
template <class F>
__device__ void leg_p(int Lmax, int Mmax, double x, double w, F emit) {
  double diag = 1.0;
  for (int M = 0; M <= Mmax && M <= Lmax; ++M) {
    if (M > 0) diag *= (2 * M - 1) * w;
    emit(M, M, diag);
    if (M + 1 <= Lmax) {
      double prev = diag, cur = (2 * M + 1) * x * diag;
      emit(M, M + 1, cur);
      for (int L = M + 1; L < Lmax; ++L) {
        const double nxt = ((2 * L + 1) * x * cur - (L + M) * prev) / (L + 1 - M);
        emit(M, L + 1, nxt);
        prev = cur;
        cur = nxt;
      }
    }
  }
}

// Q_L^M(cosh mu) into Q[M*(Lmax+1) + L], M <= Mmax (entries with no value
// stay 0)
__device__ void leg_q(int Lmax, int Mmax, double mu, double x, double w, double* Q) {
  const int NLs = Lmax + 1;
  for (int i = 0; i < (Mmax + 1) * NLs; ++i) Q[i] = 0.0;
  const double q00 = -log(tanh(0.5 * mu));
  if (mu < 1.0 / max(Lmax, 1)) {
    // Q_L = P_L Q_0 - W_L (W_0 = 0, W_1 = 1, Legendre recurrence); Q_L^1
    // from the x-derivative times w
    double pl0 = 1.0, pl1 = x, wl0 = 0.0, wl1 = 1.0, dp0 = 0.0, dp1 = 1.0, dw0 = 0.0, dw1 = 0.0;
    Q[0] = q00;
    if (Mmax >= 1) Q[NLs] = -1.0 / w;
    if (Lmax >= 1) {
      Q[1] = pl1 * q00 - wl1;
      if (Mmax >= 1) Q[NLs + 1] = w * dp1 * q00 - pl1 / w - w * dw1;
    }
    for (int k = 1; k < Lmax; ++k) {
      const double pl2 = ((2 * k + 1) * x * pl1 - k * pl0) / (k + 1);
      const double wl2 = ((2 * k + 1) * x * wl1 - k * wl0) / (k + 1);
      const double dp2 = ((2 * k + 1) * (pl1 + x * dp1) - k * dp0) / (k + 1);
      const double dw2 = ((2 * k + 1) * (wl1 + x * dw1) - k * dw0) / (k + 1);
      Q[k + 1] = pl2 * q00 - wl2;
      if (Mmax >= 1) Q[NLs + k + 1] = w * dp2 * q00 - pl2 / w - w * dw2;
      pl0 = pl1; pl1 = pl2; wl0 = wl1; wl1 = wl2; dp0 = dp1; dp1 = dp2; dw0 = dw1; dw1 = dw2;
    }
  } else {
    // backward recurrence from well past Lmax (the minimal solution
    // dominates), normalised on Q_0^0 and Q_0^1 = -1/w
    const int N = Lmax + (int)ceil(37.0 / mu) + 20;
    for (int M = 0; M <= min(Mmax, 1); ++M) {
      double* qm = Q + M * NLs;
      double nxt = 0.0, cur = 1e-280;
      for (int L = N; L >= 1; --L) {
        const double prev = ((2 * L + 1) * x * cur - (L - M + 1) * nxt) / (L + M);
        nxt = cur;
        cur = prev;
        if (L - 1 <= Lmax) qm[L - 1] = cur;
        if (fabs(cur) > 1e250) {
          cur *= 1e-250;
          nxt *= 1e-250;
          for (int l = L - 1; l <= Lmax; ++l) qm[l] *= 1e-250;
        }
      }
      const double s = (M == 0 ? q00 : -1.0 / w) / qm[0];
      for (int l = 0; l <= Lmax; ++l) qm[l] *= s;
    }
  }
  for (int M = 1; M < Mmax; ++M)
    for (int L = 0; L <= Lmax; ++L)
      Q[(M + 1) * NLs + L] =
          -2.0 * M * x / w * Q[M * NLs + L] + (double)(L + M) * (L - M + 1) * Q[(M - 1) * NLs + L];
  for (int i = 0; i < (Mmax + 1) * NLs; ++i) Q[i] = clean(Q[i]);
}

// outer point q of element e and its weight (the first element maps
// mu = mu_1 t^3, which makes the Q-weighted integrand smooth at mu = 0)
__device__ __forceinline__ void outer_point(const DTabInput& in, int e, int q, double& mu1, double& w1) {
  const double mus = in.bval[e], mue = in.bval[e + 1];
  if (e == 0) {
    const double t = 0.5 * (in.xo[q] + 1.0);
    mu1 = mus + (mue - mus) * t * t * t;
    w1 = 0.5 * in.wo[q] * 3.0 * (mue - mus) * t * t;
  } else {
    const double sf = 0.5 * (mue - mus), mid = 0.5 * (mue + mus);
    mu1 = mid + sf * in.xo[q];
    w1 = sf * in.wo[q];
  }
}

__global__ void dtab_pq(DTabInput in, double* __restrict__ PQ) {
  const int npe = in.n1e + in.no, total = in.nel * npe;
  const int NLs = in.Lmax + 1, NLM = (in.Mtop + 1) * NLs;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
    const int e = t / npe, q = t % npe;
    double mu;
    if (q < in.n1e) {
      const double mus = in.bval[e], mue = in.bval[e + 1];
      mu = 0.5 * (mue + mus) + 0.5 * (mue - mus) * in.xg[q];
    } else {
      double w1;
      outer_point(in, e, q - in.n1e, mu, w1);
    }
    double* P = PQ + (size_t)t * 2 * NLM;
    double* Q = P + NLM;
    const double x = cosh(mu), w = sinh(mu);
    for (int i = 0; i < NLM; ++i) P[i] = 0.0;
    leg_p(in.Lmax, in.Mtop, x, w, [&](int M, int L, double v) { P[M * NLs + L] = clean(v); });
    leg_q(in.Lmax, in.Mtop, mu, x, w, Q);
  }
}

__global__ void __launch_bounds__(DT_THREADS) dtab_disjoint(DTabInput in, const double* __restrict__ PQ,
                                                            double* __restrict__ p0, double* __restrict__ p2,
                                                            double* __restrict__ q0, double* __restrict__ q2) {
  __shared__ double s_pv[DT_THREADS], s_qv[DT_THREADS], s_ch[DT_THREADS];
  const int e = blockIdx.x, ilm = blockIdx.y;
  const int nn = in.nn, n2 = nn * nn, n1e = in.n1e;
  const int NLs = in.Lmax + 1, NLM = (in.Mtop + 1) * NLs;
  const int lo = in.lm_M[ilm] * NLs + in.lm_L[ilm];
  const double mus = in.bval[e], mue = in.bval[e + 1];
  const double sf = 0.5 * (mue - mus), mid = 0.5 * (mue + mus);
  for (int q = threadIdx.x; q < n1e; q += blockDim.x) {
    const double mu = mid + sf * in.xg[q], wq = in.wg[q] * sf, sh = sinh(mu), ch = cosh(mu);
    const double* P = PQ + ((size_t)e * (n1e + in.no) + q) * 2 * NLM;
    s_pv[q] = P[lo] * wq * sh;
    s_qv[q] = P[NLM + lo] * wq * sh;
    s_ch[q] = ch;
  }
  __syncthreads();
  const unsigned char* ok = in.ok + (size_t)e * nn;
  const size_t base = ((size_t)ilm * in.nel + e) * n2;
  for (int t = threadIdx.x; t < n2; t += blockDim.x) {
    const int a = t % nn, b = t / nn;
    double v0 = 0.0, v2 = 0.0, u0 = 0.0, u2 = 0.0;
    if (ok[a] && ok[b]) {
      for (int q = 0; q < n1e; ++q) {
        const double bb = in.Bg[q + (size_t)a * n1e] * in.Bg[q + (size_t)b * n1e];
        const double pv = s_pv[q], qv = s_qv[q], ch = s_ch[q];
        v0 += bb * pv;
        v2 += bb * pv * ch * ch;
        u0 += bb * qv;
        u2 += bb * qv * ch * ch;
      }
    }
    p0[base + t] = v0;
    p2[base + t] = v2;
    q0[base + t] = u0;
    q2[base + t] = u2;
  }
}

// Per (outer point q, element e0 + el, multipoles lm0 .. lm0+31):
//   It[(g*no + q)*2np + l*np + k] = sum_r w_r sinh cosh^{2l} P_L^M (mu_r) B_a B_b (mu_r)
//   Ot[(g*no + q)*2np + l*np + k] = w_q sinh cosh^{2l} Q_L^M (mu_q) B_a B_b (mu_q)
// over the unique pairs k = (a <= b), g = el*nlm + ilm; the inner points
// run over [mu_s, mu_q].
__global__ void __launch_bounds__(DT_THREADS) dtab_inner_outer(DTabInput in, const double* __restrict__ PQ,
                                                               int e0, double* __restrict__ Ot,
                                                               double* __restrict__ It) {
  extern __shared__ double sm[];
  const int q = blockIdx.x, el = blockIdx.y, e = e0 + el, lm0 = blockIdx.z * DT_LMC;
  const int nn = in.nn, np = nn * (nn + 1) / 2, ni = in.ni, no = in.no, M2 = 2 * np;
  const int NLs = in.Lmax + 1, NLM = (in.Mtop + 1) * NLs;
  const int nlc = min(DT_LMC, in.nlm - lm0);
  double* s_P = sm;                         // [ni][DT_LMC]
  double* s_BB = s_P + (size_t)ni * DT_LMC;  // [ni][np]
  double* s_c = s_BB + (size_t)ni * np;      // [ni]
  const double mus = in.bval[e];
  double mu1, w1;
  outer_point(in, e, q, mu1, w1);
  const double h = 0.5 * (mu1 - mus);
  for (int r = threadIdx.x; r < ni; r += blockDim.x) {
    const double mu2 = mus + h * (in.xi[r] + 1.0), w2 = h * in.wi[r];
    const double sh = sinh(mu2), ch = cosh(mu2), ws = w2 * sh;
    s_c[r] = ch;
    double* Pr = s_P + (size_t)r * DT_LMC;
    for (int c = 0; c < DT_LMC; ++c) Pr[c] = 0.0;
    leg_p(in.Lmax, in.Mtop, ch, sh, [&](int M, int L, double v) {
      const int ilm = in.lmidx[M * NLs + L];
      if (ilm >= lm0 && ilm < lm0 + DT_LMC) Pr[ilm - lm0] = ws * clean(v);
    });
  }
  const double* B2 = e == 0 ? in.B2z : in.B2g;
  const unsigned char* ok = in.ok + (size_t)e * nn;
  const size_t s2 = (size_t)no * ni;
  for (int t = threadIdx.x; t < ni * np; t += blockDim.x) {
    const int r = t / np, k = t % np;
    int a, b;
    pair_of(k, a, b);
    const size_t i = (size_t)q * ni + r;
    s_BB[t] = (ok[a] && ok[b]) ? B2[i + a * s2] * B2[i + b * s2] : 0.0;
  }
  __syncthreads();
  for (int o = threadIdx.x; o < nlc * np; o += blockDim.x) {
    const int c = o / np, k = o % np;
    double i0 = 0.0, i2 = 0.0;
    for (int r = 0; r < ni; ++r) {
      const double bb = s_BB[(size_t)r * np + k], wr0 = s_P[(size_t)r * DT_LMC + c], cr = s_c[r];
      const double wr2 = wr0 * cr * cr;
      i0 += wr0 * bb;
      i2 += wr2 * bb;
    }
    double* dst = It + ((size_t)(el * in.nlm + lm0 + c) * no + q) * M2;
    dst[k] = i0;
    dst[np + k] = i2;
  }
  // outer weights
  const double* B1 = e == 0 ? in.B1z : in.B1g;
  const double sh1 = sinh(mu1), ch1 = cosh(mu1);
  const double* Qp = PQ + (((size_t)e * (in.n1e + no) + in.n1e + q) * 2 + 1) * NLM;
  for (int o = threadIdx.x; o < nlc * np; o += blockDim.x) {
    const int c = o / np, k = o % np, ilm = lm0 + c;
    int a, b;
    pair_of(k, a, b);
    const double wq0 = w1 * sh1 * Qp[in.lm_M[ilm] * NLs + in.lm_L[ilm]];
    const double bb = (ok[a] && ok[b]) ? B1[q + (size_t)a * no] * B1[q + (size_t)b * no] : 0.0;
    double* dst = Ot + ((size_t)(el * in.nlm + ilm) * no + q) * M2;
    dst[k] = wq0 * bb;
    dst[np + k] = wq0 * ch1 * ch1 * bb;
  }
}

// R[g*M2*M2 + c + d*M2] = sum_q Ot[(g*no + q)*M2 + c] It[(g*no + q)*M2 + d],
// q ascending; 64 x 64 output tile per CTA, 4 x 4 per thread
__global__ void __launch_bounds__(256) dtab_gemm(int M2, int no, int tilesM, const double* __restrict__ Ot,
                                                 const double* __restrict__ It, double* __restrict__ R) {
  __shared__ double sA[16][64], sB[16][64];
  const size_t g = blockIdx.y;
  const int c0 = (blockIdx.x % tilesM) * 64, d0 = (blockIdx.x / tilesM) * 64;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const double* A = Ot + g * no * M2;
  const double* B = It + g * no * M2;
  double acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.0;
  for (int q0 = 0; q0 < no; q0 += 16) {
    for (int t = threadIdx.x; t < 16 * 64; t += 256) {
      const int qq = t / 64, cc = t % 64, q = q0 + qq;
      sA[qq][cc] = (q < no && c0 + cc < M2) ? A[(size_t)q * M2 + c0 + cc] : 0.0;
      sB[qq][cc] = (q < no && d0 + cc < M2) ? B[(size_t)q * M2 + d0 + cc] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int qq = 0; qq < 16; ++qq) {
      double av[4], bv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        av[u] = sA[qq][tx + 16 * u];
        bv[u] = sB[qq][ty + 16 * u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[u][v] += av[u] * bv[v];
    }
    __syncthreads();
  }
  double* Rg = R + g * M2 * M2;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int c = c0 + tx + 16 * u, d = d0 + ty + 16 * v;
      if (c < M2 && d < M2) Rg[c + (size_t)d * M2] = acc[u][v];
    }
}

// row i of W (channel bi = i / n2, primitive pair (a, b) = i % n2) -> its
// index c' = pair(a, b) + bi*np in R
__device__ __forceinline__ int w_index(int i, int nn, int n2, int np, int& ch) {
  ch = i / n2;
  const int ab = i % n2, a = ab % nn, b = ab / nn, lo = min(a, b), hi = max(a, b);
  return lo + hi * (hi + 1) / 2 + ch * np;
}

// Sign-carrying pivoted factor of the symmetric two-channel kernel
//   W(i, j) = s_ij (R(c_i, c_j) + R(c_j, c_i)),  s_ij = -1 across channels,
// W ~ B diag(sigma) B^T: pivot on the largest |residual diagonal| (lowest
// row on ties), stop at thresh * max|diag W| or after N steps; ranks above
// capR are reported as -1.
__global__ void __launch_bounds__(DCHOL) dtab_chol(int nn, int capR, double thresh, const double* __restrict__ R,
                                                   double* __restrict__ Bsc, double* __restrict__ ssc,
                                                   int* __restrict__ rank) {
  __shared__ double s_f[DCHOL];
  __shared__ double wv[DCHOL / 32];
  __shared__ int wi[DCHOL / 32];
  __shared__ double s_dp, s_dmax;
  __shared__ int s_piv;
  const int g = blockIdx.x;
  const int n2 = nn * nn, np = nn * (nn + 1) / 2, N = 2 * n2, M2 = 2 * np;
  const int i = threadIdx.x, lane = i & 31, warp = i >> 5;
  const double* Rg = R + (size_t)g * M2 * M2;
  double* B = Bsc + (size_t)g * N * capR;
  double* sgn = ssc + (size_t)g * capR;
  int chi = 0;
  const int ci = i < N ? w_index(i, nn, n2, np, chi) : 0;
  double d = i < N ? Rg[ci + (size_t)ci * M2] + Rg[ci + (size_t)ci * M2] : 0.0;
  {
    double v = fabs(d);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) wv[warp] = v;
    __syncthreads();
    if (i == 0) {
      double m = wv[0];
      for (int w = 1; w < DCHOL / 32; ++w) m = fmax(m, wv[w]);
      s_dmax = m;
    }
    __syncthreads();
  }
  const double dmax0 = s_dmax;
  int r = 0;
  bool overflow = false;
  for (int it = 0; it < N; ++it) {
    double v = i < N ? fabs(d) : -1.0;
    int idx = i < N ? i : INT_MAX;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double v2 = __shfl_down_sync(0xffffffffu, v, o);
      const int i2 = __shfl_down_sync(0xffffffffu, idx, o);
      if (v2 > v || (v2 == v && i2 < idx)) { v = v2; idx = i2; }
    }
    if (lane == 0) { wv[warp] = v; wi[warp] = idx; }
    __syncthreads();
    if (i == 0) {
      double bv = wv[0];
      int bi = wi[0];
      for (int w = 1; w < DCHOL / 32; ++w)
        if (wv[w] > bv || (wv[w] == bv && wi[w] < bi)) { bv = wv[w]; bi = wi[w]; }
      s_piv = bi;
    }
    __syncthreads();
    const int piv = s_piv;
    if (i == piv) s_dp = d;
    __syncthreads();
    const double dp = s_dp;
    if (dmax0 <= 0.0 || fabs(dp) <= thresh * dmax0) break;
    if (r == capR) { overflow = true; break; }
    const double sg = dp >= 0.0 ? 1.0 : -1.0;
    if (i < r) s_f[i] = sgn[i] * B[piv + (size_t)i * N];
    __syncthreads();
    if (i < N) {
      int chp;
      const int cp = w_index(piv, nn, n2, np, chp);
      double col = Rg[ci + (size_t)cp * M2] + Rg[cp + (size_t)ci * M2];
      if (chi != chp) col = -col;
      for (int k = 0; k < r; ++k) {
        const double f = s_f[k];
        if (f != 0.0) col -= f * B[i + (size_t)k * N];
      }
      const double inv = 1.0 / sqrt(fabs(dp));
      col *= inv;
      d -= sg * col * col;
      if (i == piv) d = 0.0;
      B[i + (size_t)r * N] = col;
    }
    if (i == 0) sgn[r] = sg;
    ++r;
    __syncthreads();
  }
  if (i == 0) rank[g] = overflow ? -1 : r;
}

__global__ void dtab_pack(int N, int ng, int nlm, int nel, int e0, int scatter, int capS, int capD,
                          const double* __restrict__ Bs, const double* __restrict__ ss, const int* __restrict__ rank,
                          double* __restrict__ Bd, double* __restrict__ sd) {
  const size_t per = (size_t)N * capD, total = (size_t)ng * per;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const int g = (int)(t / per);
    const size_t rem = t % per;
    const int k = (int)(rem / N), i = (int)(rem % N);
    const size_t dt = scatter ? (size_t)(g % nlm) * nel + e0 + g / nlm : (size_t)g;
    const int rk = rank[g];
    Bd[dt * per + rem] = k < rk ? Bs[(size_t)g * N * capS + i + (size_t)k * N] : 0.0;
    if (i == 0) sd[dt * capD + k] = k < rk ? ss[(size_t)g * capS + k] : 0.0;
  }
}

size_t inner_smem(const DTabInput& in) {
  const size_t np = (size_t)in.nn * (in.nn + 1) / 2;
  return sizeof(double) * ((size_t)in.ni * DT_LMC + (size_t)in.ni * np + in.ni);
}

bool valid_input(const DTabInput& in) {
  return in.nn >= 3 && 2 * in.nn * in.nn <= DCHOL && in.nel >= 1 && in.nlm >= 1 && in.Lmax >= 0 && in.Mtop >= 0 &&
         in.n1e >= 1 && in.n1e <= DT_THREADS && in.no >= 1 && in.ni >= 1 && inner_smem(in) <= 227 * 1024;
}

}  // namespace

size_t dtab_pq_doubles(const DTabInput& in) {
  return (size_t)in.nel * (in.n1e + in.no) * 2 * (in.Mtop + 1) * (in.Lmax + 1);
}

cudaError_t launch_dtab_pq(const DTabInput& in, double* PQ, cudaStream_t st) {
  if (!valid_input(in)) return cudaErrorInvalidValue;
  const int total = in.nel * (in.n1e + in.no);
  dtab_pq<<<(total + 127) / 128, 128, 0, st>>>(in, PQ);
  return cudaGetLastError();
}

cudaError_t launch_dtab_disjoint(const DTabInput& in, const double* PQ, double* p0, double* p2, double* q0,
                                 double* q2, cudaStream_t st) {
  if (!valid_input(in) || in.nlm > 65535) return cudaErrorInvalidValue;
  dtab_disjoint<<<dim3(in.nel, in.nlm), DT_THREADS, 0, st>>>(in, PQ, p0, p2, q0, q2);
  return cudaGetLastError();
}

size_t dtab_group_doubles(const DTabInput& in, int ne, int capR) {
  (void)capR;
  const size_t np = (size_t)in.nn * (in.nn + 1) / 2, M2 = 2 * np, ng = (size_t)ne * in.nlm;
  return ng * (2 * (size_t)in.no * M2 + M2 * M2);
}

cudaError_t launch_dtab_factor(const DTabInput& in, const double* PQ, int e0, int ne, int capR, double* scratch,
                               double* Bsc, double* ssc, int* rank, cudaStream_t st) {
  const int np = in.nn * (in.nn + 1) / 2, M2 = 2 * np, N = 2 * in.nn * in.nn;
  const size_t ng = (size_t)ne * in.nlm;
  if (!valid_input(in) || e0 < 0 || ne < 1 || e0 + ne > in.nel || capR < 1 || capR > N || ng > 65535 ||
      in.no > 65535 || ne > 65535)
    return cudaErrorInvalidValue;
  double* Ot = scratch;
  double* It = Ot + ng * in.no * M2;
  double* R = It + ng * in.no * M2;
  const size_t smem = inner_smem(in);
  {
    const cudaError_t e = smem_limit(dtab_inner_outer, smem);
    if (e != cudaSuccess) return e;
  }
  dtab_inner_outer<<<dim3(in.no, ne, (in.nlm + DT_LMC - 1) / DT_LMC), DT_THREADS, smem, st>>>(in, PQ, e0, Ot, It);
  const int tilesM = (M2 + 63) / 64;
  dtab_gemm<<<dim3(tilesM * tilesM, (unsigned)ng), 256, 0, st>>>(M2, in.no, tilesM, Ot, It, R);
  dtab_chol<<<(unsigned)ng, DCHOL, 0, st>>>(in.nn, capR, in.thresh, R, Bsc, ssc, rank);
  return cudaGetLastError();
}

cudaError_t launch_dtab_pack(int N, int ng, int nlm, int nel, int e0, int scatter, int capS, int capD,
                             const double* Bs, const double* ss, const int* rank, double* Bd, double* sd,
                             cudaStream_t st) {
  if (N < 1 || ng < 1 || capS < 1 || capD < 1) return cudaErrorInvalidValue;
  const size_t total = (size_t)ng * N * capD;
  const int grid = (int)std::min<size_t>((total + 255) / 256, 152 * 16);
  dtab_pack<<<grid, 256, 0, st>>>(N, ng, nlm, nel, e0, scatter, capS, capD, Bs, ss, rank, Bd, sd);
  return cudaGetLastError();
}

}  // namespace hfg

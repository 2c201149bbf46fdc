// Device tabulation of the atomic in-element two-electron tables (FP64):
// the in-element tensor of the bare kernel r<^L / r>^(L+1), its pivoted
// Cholesky factor and the exchange-ordered tensor rebuilt from the factor.
//
// Follows what HelFEM's compute_tei computes per (L, element)
// (src/atomic/TwoDBasis.cpp:708-735 -> RadialBasis::twoe_integral /
// twoe_integral_cholesky, libhelfem/src/RadialBasis.cpp:643-716;
// quadrature::twoe_integral, libhelfem/src/quadrature.cpp:36-161), with the
// quadrature of the host tabulation (Gauss-Legendre outer rule of TWOE_NO
// points, inner rule of TWOE_NI points on [r_min, r]):
//   G_kl(r_p)  = sum_q win(p, q) B_k B_l (r_pq)                   (inner)
//   T1[ij, kl] = sum_p wout(p) B_i B_j (r_p) G_kl(r_p)            (outer)
//   T = T1 + T1^T,  T = L L^T (greedy pivoted Cholesky, absolute tolerance)
//   Tk[(a + c nn) + (b + d nn) nn^2] = sum_p L(a + b nn, p) L(c + d nn, p)
// T1 is symmetric under i <-> j and k <-> l, so it is formed over the pairs
// i <= j only (a = i + j (j + 1) / 2) and expanded on the fly.
//
// Kernels
//   tab_t1    grid (tiles^2, nel, NL), 256 threads: one 64 x 64 tile of T1;
//             per outer point the block forms the inner integrals of its 64
//             ket pairs and the outer weights of its 64 bra pairs in shared
//             memory and adds their outer product (p ascending).
//   tab_chol  grid (nel, NL), one thread per row of T: the pivoted Cholesky
//             (block argmax with the lowest index on ties, as the host loop).
//   tab_pack  the factor into the padded J layout (nn^2 x rmax, zero columns).
//   tab_tk    grid (nn^2 (b, d) columns, nel, NL): column (b, d) of Tk is
//             L_b L_d^T with L_b = rows (a + b nn) of the factor.
//   split_f2  float-pair copies for the split-precision exchange.
#include <cuda_runtime.h>

#include <algorithm>

#include "smem_limit.hpp"
#include "tab.cuh"

namespace hfg {

namespace {

constexpr int T1_TILE = 64;
constexpr int T1_THREADS = 256;
constexpr int CHOL_THREADS = 320;  // >= nn^2 for nn <= 17

__device__ __forceinline__ int pair_index(int i, int j) {
  const int lo = i < j ? i : j, hi = i < j ? j : i;
  return lo + hi * (hi + 1) / 2;
}

__device__ __forceinline__ double ipow(double r, int n) {
  double v = 1.0;
  for (int k = 0; k < n; ++k) v *= r;
  return v;
}

__global__ void __launch_bounds__(T1_THREADS) tab_t1(TabInput in, double* __restrict__ T1) {
  const int nn = in.nn, np = nn * (nn + 1) / 2, nt = (np + T1_TILE - 1) / T1_TILE;
  const int e = blockIdx.y, L = blockIdx.z, le = L * in.nel + e;
  const int ta = blockIdx.x % nt, tb = blockIdx.x / nt;
  const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
  __shared__ double win[64];
  __shared__ double Gs[T1_TILE], Ws[T1_TILE];
  __shared__ int pk[T1_TILE], pl[T1_TILE], pi_[T1_TILE], pj_[T1_TILE];
  const double rmin = in.bval[e], rmax = in.bval[e + 1];
  const double sf = 0.5 * (rmax - rmin), mid = 0.5 * (rmax + rmin);
  const unsigned char* ok = in.ok + (size_t)e * nn;
  if (tid < T1_TILE) {
    // pair a <-> (i, j), i <= j, from a = i + j (j + 1) / 2
    const int a = ta * T1_TILE + tid, b = tb * T1_TILE + tid;
    int i = -1, j = -1, k = -1, l = -1;
    if (a < np) {
      j = 0;
      while ((j + 1) * (j + 2) / 2 <= a) ++j;
      i = a - j * (j + 1) / 2;
      if (!ok[i] || !ok[j]) i = j = -1;
    }
    if (b < np) {
      l = 0;
      while ((l + 1) * (l + 2) / 2 <= b) ++l;
      k = b - l * (l + 1) / 2;
      if (!ok[k] || !ok[l]) k = l = -1;
    }
    pi_[tid] = i; pj_[tid] = j; pk[tid] = k; pl[tid] = l;
  }
  double acc[4][4];
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc[u][v] = 0.0;
  const size_t npin = (size_t)in.no * in.ni;
  for (int p = 0; p < in.no; ++p) {
    const double ro = mid + sf * in.xo[p];
    const double half = 0.5 * (ro - rmin);
    if (tid < in.ni) {
      const double r = rmin + half * (in.xi[tid] + 1.0);
      win[tid] = half * in.wi[tid] * ipow(r, L);
    }
    __syncthreads();
    if (tid < T1_TILE) {
      const int k = pk[tid], l = pl[tid];
      double s = 0.0;
      if (k >= 0) {
        const double* bk = in.Bin + (size_t)p * in.ni + (size_t)k * npin;
        const double* bl = in.Bin + (size_t)p * in.ni + (size_t)l * npin;
        for (int q = 0; q < in.ni; ++q) s += win[q] * bk[q] * bl[q];
      }
      Gs[tid] = s;
    } else if (tid < 2 * T1_TILE) {
      const int t = tid - T1_TILE, i = pi_[t], j = pj_[t];
      double w = 0.0;
      if (i >= 0) {
        const double wp = in.wo[p] * sf / ipow(ro, L + 1);
        w = wp * in.Bo[p + (size_t)i * in.no] * in.Bo[p + (size_t)j * in.no];
      }
      Ws[t] = w;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const double wa = Ws[tx + 16 * u];
#pragma unroll
      for (int v = 0; v < 4; ++v) acc[u][v] += wa * Gs[ty + 16 * v];
    }
  }
  double* out = T1 + (size_t)le * np * np;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int a = ta * T1_TILE + tx + 16 * u, b = tb * T1_TILE + ty + 16 * v;
      if (a < np && b < np) out[a + (size_t)b * np] = acc[u][v];
    }
}

// T[x, y] of the expanded tensor from the pair-packed T1
__device__ __forceinline__ double t_entry(const double* T1, int np, int pa, int pb) {
  return pa == pb ? 2.0 * T1[pa + (size_t)pa * np] : T1[pa + (size_t)pb * np] + T1[pb + (size_t)pa * np];
}

__global__ void __launch_bounds__(CHOL_THREADS) tab_chol(TabInput in, const double* __restrict__ T1,
                                                          double* __restrict__ Lsc, int* __restrict__ rank) {
  const int nn = in.nn, n2 = nn * nn, np = nn * (nn + 1) / 2;
  const int e = blockIdx.x, L = blockIdx.y, le = L * in.nel + e;
  const int i = threadIdx.x, lane = i & 31, warp = i >> 5;
  __shared__ double Lp[CHOL_THREADS];
  __shared__ double wv[CHOL_THREADS / 32];
  __shared__ int wi[CHOL_THREADS / 32];
  __shared__ double s_pv;
  __shared__ int s_piv;
  const double* T = T1 + (size_t)le * np * np;
  double* Lf = Lsc + (size_t)le * n2 * n2;
  const unsigned char* ok = in.ok + (size_t)e * nn;
  int pa = -1;
  if (i < n2) {
    const int a = i % nn, b = i / nn;
    if (ok[a] && ok[b]) pa = pair_index(a, b);
  }
  double D = pa >= 0 ? t_entry(T, np, pa, pa) : 0.0;
  bool done = false;
  int k = 0;
  for (; k < n2; ++k) {
    // argmax of the residual diagonal over rows not yet pivoted and above
    // the tolerance; equal values go to the lowest row
    double v = (i < n2 && !done && D > in.tol) ? D : -1.0;
    int idx = (v >= 0.0) ? i : 0x7fffffff;
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
      for (int w = 1; w < CHOL_THREADS / 32; ++w)
        if (wv[w] > bv || (wv[w] == bv && wi[w] < bi)) { bv = wv[w]; bi = wi[w]; }
      s_pv = bv;
      s_piv = bv >= 0.0 ? bi : -1;
    }
    __syncthreads();
    const int piv = s_piv;
    if (piv < 0) break;
    const double pv = s_pv;
    if (i == piv) done = true;
    const double s = sqrt(pv);
    if (i < k) Lp[i] = Lf[piv + (size_t)i * n2];
    __syncthreads();
    if (i < n2) {
      double col;
      if (i == piv) {
        col = s;
      } else if (done) {
        col = 0.0;
      } else {
        const int pp = pair_index(piv % nn, piv / nn);
        double x = pa >= 0 ? t_entry(T, np, pa, pp) : 0.0;
        for (int j = 0; j < k; ++j) x -= Lf[i + (size_t)j * n2] * Lp[j];
        col = x / s;
      }
      Lf[i + (size_t)k * n2] = col;
      if (!done) D -= col * col;
    }
    __syncthreads();
  }
  if (i == 0) rank[le] = k;
}

__global__ void tab_pack(int nn, int nblk, int rmax, const double* __restrict__ Lsc, const int* __restrict__ rank,
                         double* __restrict__ cholp) {
  const int n2 = nn * nn;
  const size_t total = (size_t)nblk * n2 * rmax;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(t % n2);
    const size_t rest = t / n2;
    const int p = (int)(rest % rmax);
    const int le = (int)(rest / rmax);
    cholp[t] = p < rank[le] ? Lsc[(size_t)le * n2 * n2 + x + (size_t)p * n2] : 0.0;
  }
}

__global__ void tab_tk(TabInput in, int rmax, const double* __restrict__ Lsc, const int* __restrict__ rank,
                       double* __restrict__ tk) {
  extern __shared__ double sm[];
  const int nn = in.nn, n2 = nn * nn;
  const int bd = blockIdx.x, e = blockIdx.y, L = blockIdx.z, le = L * in.nel + e;
  const int b = bd % nn, d = bd / nn;
  const int r = rank[le];
  double* Lb = sm;            // [a + p*nn]
  double* Ld = sm + nn * rmax;
  const double* Lf = Lsc + (size_t)le * n2 * n2;
  for (int t = threadIdx.x; t < nn * r; t += blockDim.x) {
    const int a = t % nn, p = t / nn;
    Lb[t] = Lf[(a + b * nn) + (size_t)p * n2];
    Ld[t] = Lf[(a + d * nn) + (size_t)p * n2];
  }
  __syncthreads();
  double* out = tk + (size_t)le * n2 * n2 + (size_t)(b + d * nn) * n2;
  for (int t = threadIdx.x; t < n2; t += blockDim.x) {
    const int a = t % nn, c = t / nn;
    double s = 0.0;
    for (int p = 0; p < r; ++p) s += Lb[a + p * nn] * Ld[c + p * nn];
    out[t] = s;
  }
}

__global__ void split_f2_kernel(const double* __restrict__ x, float2* __restrict__ y, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const double v = x[t];
    const float hi = (float)v;
    y[t] = make_float2(hi, (float)(v - (double)hi));
  }
}

}  // namespace

size_t tab_t1_doubles(int nn, int nel, int NL) {
  const size_t np = (size_t)nn * (nn + 1) / 2;
  return (size_t)NL * nel * np * np;
}

size_t tab_factor_doubles(int nn, int nel, int NL) {
  const size_t n2 = (size_t)nn * nn;
  return (size_t)NL * nel * n2 * n2;
}

cudaError_t launch_tab_factor(const TabInput& in, double* T1, double* Lsc, int* rank, cudaStream_t st) {
  if (in.nn < 3 || in.nn * in.nn > CHOL_THREADS || in.ni > 64) return cudaErrorInvalidValue;
  const int np = in.nn * (in.nn + 1) / 2, nt = (np + T1_TILE - 1) / T1_TILE;
  tab_t1<<<dim3(nt * nt, in.nel, in.NL), T1_THREADS, 0, st>>>(in, T1);
  tab_chol<<<dim3(in.nel, in.NL), CHOL_THREADS, 0, st>>>(in, T1, Lsc, rank);
  return cudaGetLastError();
}

cudaError_t launch_tab_finish(const TabInput& in, const double* Lsc, const int* rank, int rmax, double* cholp,
                              double* tk, cudaStream_t st) {
  const int n2 = in.nn * in.nn;
  if (rmax < 1 || rmax > n2) return cudaErrorInvalidValue;
  const int nblk = in.NL * in.nel;
  const size_t total = (size_t)nblk * n2 * rmax;
  const int grid = (int)std::min<size_t>((total + 255) / 256, 152 * 16);
  tab_pack<<<grid, 256, 0, st>>>(in.nn, nblk, rmax, Lsc, rank, cholp);
  const size_t smem = sizeof(double) * 2 * in.nn * rmax;
  {
    const cudaError_t e = smem_limit(tab_tk, smem);
    if (e != cudaSuccess) return e;
  }
  tab_tk<<<dim3(n2, in.nel, in.NL), n2 <= 128 ? 128 : 320, smem, st>>>(in, rmax, Lsc, rank, tk);
  return cudaGetLastError();
}

cudaError_t launch_split_f2(const double* x, float2* y, size_t n, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const int grid = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  split_f2_kernel<<<grid, 256, 0, st>>>(x, y, n);
  return cudaGetLastError();
}

}  // namespace hfg

// Banded shift-invert preconditioner of the SCF's Davidson refinement.
//
// In the finite-element basis every term of a Fock block but the exchange
// couples only functions that share an element (T, V, J, V_xc; the overlap
// S too), so the band part of F_k with half-width w = nn - 1 holds most of
// it. The correction equation (F' - theta) t' = -r' of the orthonormal block
// F' = X^T F_k X (X^T S X = 1) is preconditioned by
//     t' = (S X)^T M^-1 (S X) r',   M = band(F_k) - theta S,
// one banded solve per Ritz value (instead of an eigendecomposition of an
// earlier Fock block). Here: Olsen's form of it,
//     y = M^-1 z_r - eps M^-1 z_x,  eps = (z_x . M^-1 z_r) / (z_x . M^-1 z_x),
// with z_r = S X r', z_x = S X x' given, so that the correction is
// orthogonal to the Ritz vector in the preconditioner's metric.
//
// One warp per Ritz value: Gaussian elimination with partial pivoting on the
// band (LAPACK gbtrf's scheme: the pivot search runs over the w rows below
// the diagonal, U keeps an upper bandwidth of 2w), both right-hand sides
// eliminated on the way, the active (w+1) x (2w+1) window in shared memory
// with circular row and column slots, U's rows to a global scratch, then
// back substitution. FP32: a preconditioner needs no more, and the FP32 pipe
// is 64x the FP64 one on GB300; the Davidson residuals stay FP64.
#include <cuda_runtime.h>

#include <cmath>

#include "scf_kernels.cuh"

namespace hfg {
namespace {

constexpr int WMAX = 16;             // half-bandwidth limit (nn <= 17)
constexpr int RMAX = WMAX + 1;       // window rows
constexpr int CMAX = 2 * WMAX + 1;   // window columns

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(32) band_olsen(const double* __restrict__ F, const double* __restrict__ S, int n,
                                                 int w, const double* __restrict__ theta,
                                                 const double* __restrict__ Zr, const double* __restrict__ Zx,
                                                 double* __restrict__ Y, float* __restrict__ work) {
  const int col = blockIdx.x, lane = threadIdx.x;
  const int R = w + 1, C = 2 * w + 1;
  const float th = (float)theta[col];
  const double* zr = Zr + (size_t)col * n;
  const double* zx = Zx + (size_t)col * n;
  double* y = Y + (size_t)col * n;
  float* U = work + (size_t)col * ((size_t)n * C + 2 * (size_t)n);  // row j: C values from column j
  float* bU = U + (size_t)n * C;                                       // eliminated right-hand sides
  __shared__ float A[RMAX][CMAX];
  __shared__ float br[RMAX], bx[RMAX];
  __shared__ float yr[CMAX], yx[CMAX];

  auto m_at = [&](int r, int c) -> float {  // M(r, c) of the original band
    const size_t o = (size_t)r + (size_t)c * n;
    return (float)(F[o] - (double)th * S[o]);
  };
  // load row r (its slot zeroed first) with columns [r - w, r + w] inside [lo, n)
  auto load_row = [&](int r, int lo) {
    const int s = r % R;
    for (int k = lane; k < C; k += 32) A[s][k] = 0.f;
    __syncwarp();
    for (int c = max(lo, r - w) + lane; c <= min(n - 1, r + w); c += 32) A[s][c % C] = m_at(r, c);
    if (lane == 0) {
      br[s] = (float)zr[r];
      bx[s] = (float)zx[r];
    }
  };
  for (int r = 0; r < min(R, n); ++r) load_row(r, 0);
  __syncwarp();

  for (int j = 0; j < n; ++j) {
    const int rows = min(R, n - j);  // candidate rows j .. j + rows - 1
    // pivot: the largest |M(r, j)| among the candidates (first on ties)
    float v = -1.f;
    int pr = j;
    if (lane < rows) {
      v = fabsf(A[(j + lane) % R][j % C]);
      pr = j + lane;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float v2 = __shfl_xor_sync(0xffffffffu, v, o);
      const int p2 = __shfl_xor_sync(0xffffffffu, pr, o);
      if (v2 > v || (v2 == v && p2 < pr)) {
        v = v2;
        pr = p2;
      }
    }
    const int sj = j % R, sp = pr % R;
    if (pr != j) {
      for (int k = lane; k < C; k += 32) {
        const float t = A[sj][k];
        A[sj][k] = A[sp][k];
        A[sp][k] = t;
      }
      if (lane == 0) {
        float t = br[sj];
        br[sj] = br[sp];
        br[sp] = t;
        t = bx[sj];
        bx[sj] = bx[sp];
        bx[sp] = t;
      }
    }
    __syncwarp();
    float piv = A[sj][j % C];
    if (fabsf(piv) < 1e-30f) piv = 1e-30f;  // singular band: keep the solve finite
    // U row j (columns j .. j + 2w) and the eliminated right-hand sides
    for (int k = lane; k < C; k += 32) U[(size_t)j * C + k] = (k == 0) ? piv : A[sj][(j + k) % C];
    if (lane == 0) {
      bU[2 * (size_t)j] = br[sj];
      bU[2 * (size_t)j + 1] = bx[sj];
    }
    // eliminate column j from rows j+1 .. j+rows-1 over columns j+1 .. j+2w
    const int nr = rows - 1, nc = 2 * w;
    for (int q = lane; q < nr * nc; q += 32) {
      const int r = j + 1 + q / nc, c = j + 1 + q % nc;
      const float f = A[r % R][j % C] / piv;
      A[r % R][c % C] = fmaf(-f, A[sj][c % C], A[r % R][c % C]);
    }
    if (lane < nr) {
      const int r = j + 1 + lane;
      const float f = A[r % R][j % C] / piv;
      br[r % R] = fmaf(-f, br[sj], br[r % R]);
      bx[r % R] = fmaf(-f, bx[sj], bx[r % R]);
    }
    __syncwarp();
    // column slot j % C now holds column j + C = j + 2w + 1: clear it for
    // the rows that stay; row j's slot takes the next row
    for (int k = lane; k < R; k += 32) A[k][j % C] = 0.f;
    __syncwarp();
    if (j + R < n) load_row(j + R, j + 1);
    __syncwarp();
  }

  // back substitution, both right-hand sides; y of the last 2w rows in a
  // circular buffer
  for (int k = lane; k < C; k += 32) {
    yr[k] = 0.f;
    yx[k] = 0.f;
  }
  __syncwarp();
  double dot_r = 0.0, dot_x = 0.0, dot_xx = 0.0;
  for (int j = n - 1; j >= 0; --j) {
    float sr = 0.f, sx = 0.f;
    for (int k = 1 + lane; k < C; k += 32) {
      if (j + k >= n) continue;
      const float u = U[(size_t)j * C + k];
      sr = fmaf(u, yr[(j + k) % C], sr);
      sx = fmaf(u, yx[(j + k) % C], sx);
    }
    sr = warp_sum_f(sr);
    sx = warp_sum_f(sx);
    const float d = U[(size_t)j * C];
    const float vr = (bU[2 * (size_t)j] - sr) / d, vx = (bU[2 * (size_t)j + 1] - sx) / d;
    __syncwarp();
    if (lane == 0) {
      yr[j % C] = vr;
      yx[j % C] = vx;
      // y holds M^-1 z_r for now; the Olsen combination follows
      y[j] = (double)vr;
      U[(size_t)j * C] = vx;  // M^-1 z_x kept in U's diagonal slot (row j is done)
    }
    __syncwarp();
  }
  __syncwarp();
  for (int i = lane; i < n; i += 32) {
    const double a = y[i], b = (double)U[(size_t)i * C], z = zx[i];
    dot_r += z * a;
    dot_x += z * b;
  }
  dot_r = warp_sum_d(dot_r);
  dot_x = warp_sum_d(dot_x);
  (void)dot_xx;
  const double eps = (dot_x != 0.0) ? dot_r / dot_x : 0.0;
  for (int i = lane; i < n; i += 32) y[i] = y[i] - eps * (double)U[(size_t)i * C];
}

}  // namespace

size_t band_olsen_work_floats(int n, int w, int u) {
  return (size_t)u * ((size_t)n * (2 * w + 1) + 2 * (size_t)n);
}

cudaError_t k_band_olsen(const double* F, const double* S, int n, int w, const double* theta, const double* Zr,
                         const double* Zx, double* Y, float* work, int u, cudaStream_t st) {
  if (w < 1 || w > WMAX) return cudaErrorInvalidValue;
  if (u <= 0) return cudaSuccess;
  band_olsen<<<u, 32, 0, st>>>(F, S, n, w, theta, Zr, Zx, Y, work);
  return cudaGetLastError();
}

}  // namespace hfg

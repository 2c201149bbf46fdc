// Small device kernels of the SCF driver: gathering a symmetry block out of
// an AO matrix, scattering a block density back, the DIIS commutator in the
// orthonormal basis and elementwise Fock assembly.
#include "scf_kernels.cuh"

namespace hfg {
namespace {

// angular-block indexed gather: Mk[r + c*nk] = M[ang[r/nrad]*nrad + r%nrad, ang[c/nrad]*nrad + c%nrad]
__global__ void gather_block(const double* __restrict__ M, int nbf, int nrad, const int* __restrict__ ang, int nk,
                             double* __restrict__ Mk) {
  const size_t n = (size_t)nk * nk;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(idx % nk), c = (int)(idx / nk);
    const size_t R = (size_t)ang[r / nrad] * nrad + r % nrad;
    const size_t C = (size_t)ang[c / nrad] * nrad + c % nrad;
    Mk[idx] = M[R + C * nbf];
  }
}

__global__ void scatter_add_block(double* __restrict__ M, int nbf, int nrad, const int* __restrict__ ang, int nk,
                                  const double* __restrict__ Mk, double alpha) {
  const size_t n = (size_t)nk * nk;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n; idx += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(idx % nk), c = (int)(idx / nk);
    const size_t R = (size_t)ang[r / nrad] * nrad + r % nrad;
    const size_t C = (size_t)ang[c / nrad] * nrad + c % nrad;
    M[R + C * nbf] += alpha * Mk[idx];
  }
}

// E = G - G^T where G = W diag(occ) V^T  (W = F' V_occ): the commutator F'D' - D'F'
__global__ void antisym(const double* __restrict__ G, int n, double* __restrict__ E) {
  const size_t nn = (size_t)n * n;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < nn; idx += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(idx % n), c = (int)(idx / n);
    E[idx] = G[idx] - G[c + (size_t)r * n];
  }
}

// out = a + b + c (+ d), any of c, d may be null
__global__ void add4(double* __restrict__ out, const double* __restrict__ a, const double* __restrict__ b,
                     const double* __restrict__ c, const double* __restrict__ d, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    double v = a[i] + b[i];
    if (c) v += c[i];
    if (d) v += d[i];
    out[i] = v;
  }
}

// columns scaled: Y[:, j] = X[:, j] * s[j]
__global__ void scale_cols(const double* __restrict__ X, int n, int m, const double* __restrict__ s,
                           double* __restrict__ Y) {
  const size_t nn = (size_t)n * m;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < nn; idx += (size_t)gridDim.x * blockDim.x)
    Y[idx] = X[idx] * s[idx / n];
}

__global__ void add_diag(double* __restrict__ A, int n, double v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) A[i + (size_t)i * n] += v;
}

__global__ void test_density(double* __restrict__ P, int n) {
  const size_t nn = (size_t)n * n;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < nn; idx += (size_t)gridDim.x * blockDim.x) {
    const unsigned r = (unsigned)(idx % n), c = (unsigned)(idx / n);
    const unsigned lo = r < c ? r : c, hi = r < c ? c : r;
    unsigned h = lo * 2654435761u ^ (hi * 40503u + 0x9e3779b9u);
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    P[idx] = 1e-3 * ((double)(h & 0xFFFFFF) / 16777216.0 - 0.5);
  }
}

// Davidson residuals: R[:, j] = AX[:, j] - theta[j] X[:, j] and their norms;
// one block per column
__global__ void dav_residual(const double* __restrict__ AX, const double* __restrict__ X,
                             const double* __restrict__ theta, int n, double* __restrict__ R,
                             double* __restrict__ norms) {
  const int j = blockIdx.x;
  const double t = theta[j];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double r = AX[i + (size_t)j * n] - t * X[i + (size_t)j * n];
    R[i + (size_t)j * n] = r;
    s += r * r;
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w];
    norms[j] = sqrt(v);
  }
}

// Olsen-corrected, reference-preconditioned Davidson update in the reference
// eigenbasis: with d_i = 1/(lam_i - theta_j),
//   eps = (zx . d zr) / (zx . d zx),  zt = d (zr - eps zx),
// which makes the correction orthogonal to the Ritz vector; one block per
// column. |lam_i - theta_j| is kept above floor.
__global__ void dav_olsen(const double* __restrict__ Zr, const double* __restrict__ Zx,
                          const double* __restrict__ lam, const double* __restrict__ theta, int n, double floor_,
                          double* __restrict__ Zt) {
  const int j = blockIdx.x;
  const double t = theta[j];
  const double* zr = Zr + (size_t)j * n;
  const double* zx = Zx + (size_t)j * n;
  auto dinv = [&](int i) {
    double g = lam[i] - t;
    if (fabs(g) < floor_) g = (g < 0.0) ? -floor_ : floor_;
    return 1.0 / g;
  };
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double d = dinv(i);
    a += zx[i] * d * zr[i];
    b += zx[i] * d * zx[i];
  }
  __shared__ double ra[32], rb[32], e;
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if ((threadIdx.x & 31) == 0) {
    ra[threadIdx.x >> 5] = a;
    rb[threadIdx.x >> 5] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double sa = 0.0, sb = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      sa += ra[w];
      sb += rb[w];
    }
    e = (sb != 0.0) ? sa / sb : 0.0;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) Zt[i + (size_t)j * n] = dinv(i) * (zr[i] - e * zx[i]);
}

inline int grid_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

}  // namespace

void k_gather_block(const double* M, int nbf, int nrad, const int* ang, int nk, double* Mk, cudaStream_t st) {
  gather_block<<<grid_for((size_t)nk * nk), 256, 0, st>>>(M, nbf, nrad, ang, nk, Mk);
}
void k_scatter_add_block(double* M, int nbf, int nrad, const int* ang, int nk, const double* Mk, double alpha,
                         cudaStream_t st) {
  scatter_add_block<<<grid_for((size_t)nk * nk), 256, 0, st>>>(M, nbf, nrad, ang, nk, Mk, alpha);
}
void k_antisym(const double* G, int n, double* E, cudaStream_t st) {
  antisym<<<grid_for((size_t)n * n), 256, 0, st>>>(G, n, E);
}
namespace {
__global__ void diffsum(double* __restrict__ out, const double* a1, const double* b1, const double* a2,
                        const double* b2, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (a1[i] - b1[i]) + (a2 ? a2[i] - b2[i] : 0.0);
}
__global__ void lerp(double* out, const double* a, double lam, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = a[i] + lam * (out[i] - a[i]);
}
}  // namespace

namespace {
// T and V of the AO basis from the radial blocks: only the diagonal angular
// blocks are nonzero (the caller zeroes the rest)
__global__ void expand_one_electron(const double* __restrict__ Trad, const double* __restrict__ Tlrad,
                                    const double* __restrict__ Vrad, const int* __restrict__ lval, int nang,
                                    int nrad, double Z, double* __restrict__ T, double* __restrict__ V) {
  const size_t nr2 = (size_t)nrad * nrad, nbf = (size_t)nang * nrad, tot = nr2 * nang;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < tot; idx += (size_t)gridDim.x * blockDim.x) {
    const int ia = (int)(idx / nr2);
    const size_t q = idx % nr2;
    const size_t r = q % nrad, c = q / nrad;
    const double lf = (double)lval[ia] * (lval[ia] + 1);
    const size_t o = ((size_t)ia * nrad + c) * nbf + (size_t)ia * nrad + r;
    T[o] = Trad[q] + lf * Tlrad[q];
    V[o] = -Z * Vrad[q];
  }
}
// Y[r + c n] = d[r] X[r + c n]
__global__ void scale_rows(double* __restrict__ X, int n, int m, const double* __restrict__ d) {
  const size_t nn = (size_t)n * m;
  for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < nn; idx += (size_t)gridDim.x * blockDim.x)
    X[idx] *= d[idx % n];
}
}  // namespace

void k_expand_one_electron(const double* Trad, const double* Tlrad, const double* Vrad, const int* lval, int nang,
                           int nrad, double Z, double* T, double* V, cudaStream_t st) {
  const size_t tot = (size_t)nrad * nrad * nang;
  expand_one_electron<<<grid_for(tot), 256, 0, st>>>(Trad, Tlrad, Vrad, lval, nang, nrad, Z, T, V);
}
void k_scale_rows(double* X, int n, int m, const double* d, cudaStream_t st) {
  scale_rows<<<grid_for((size_t)n * m), 256, 0, st>>>(X, n, m, d);
}

void k_diffsum(double* out, const double* a1, const double* b1, const double* a2, const double* b2, size_t n,
               cudaStream_t st) {
  diffsum<<<grid_for(n), 256, 0, st>>>(out, a1, b1, a2, b2, n);
}
void k_lerp(double* out, const double* a, double lam, size_t n, cudaStream_t st) {
  lerp<<<grid_for(n), 256, 0, st>>>(out, a, lam, n);
}

void k_add4(double* out, const double* a, const double* b, const double* c, const double* d, size_t n,
            cudaStream_t st) {
  add4<<<grid_for(n), 256, 0, st>>>(out, a, b, c, d, n);
}
void k_scale_cols(const double* X, int n, int m, const double* s, double* Y, cudaStream_t st) {
  scale_cols<<<grid_for((size_t)n * m), 256, 0, st>>>(X, n, m, s, Y);
}

void fill_test_density(double* P, int n, cudaStream_t st) {
  test_density<<<grid_for((size_t)n * n), 256, 0, st>>>(P, n);
}

void k_dav_residual(const double* AX, const double* X, const double* theta, int n, int k, double* R, double* norms,
                    cudaStream_t st) {
  dav_residual<<<k, 256, 0, st>>>(AX, X, theta, n, R, norms);
}

void k_dav_olsen(const double* Zr, const double* Zx, const double* lam, const double* theta, int n, int k,
                 double floor_, double* Zt, cudaStream_t st) {
  dav_olsen<<<k, 256, 0, st>>>(Zr, Zx, lam, theta, n, floor_, Zt);
}

void k_add_diag(double* A, int n, double v, cudaStream_t st) {
  add_diag<<<(n + 255) / 256, 256, 0, st>>>(A, n, v);
}

}  // namespace hfg

// XC potential on the pure-m diatomic DFT grid, plain FP64.
//
// Restates PureMDFTGrid::eval_Fxc and its worker
// (src/diatomic/dftgrid_purem.cpp:83-199 basis values and weights, 213-291
// and 306-369 density and gradient, 480-530 and 575-650 Fock increments,
// 668-712 element loop) in separable form. On mu element e, at mu point q and
// nu point a, the dummy function (s, p) has the value Y_s(a) B_p(q); only
// same-m angular pairs k = (s, t) couple. With
//   D_k(q)  = B(q)^T P_st B(q),   Dr_k(q) = dB(q)^T P_st B(q)
// the density and its gradient components along mu and nu are
//   rho(q,a) = sum_k D_k(q) W_k(a),        W_k  = Y_s Y_t
//   g_mu     = 2/h sum_k Dr_k(q) W_k(a)
//   g_nu     = 2/h sum_k D_k(q) Wt_k(a),   Wt_k = (dY_s/dnu) Y_t
// and the Fock tile of pair k on element e is
//   V_{(s,i),(t,j)} = sum_q B_i B_j U0_k(q) + X + X^T,
//   X_{(s,i),(t,j)} = sum_q [dB_i B_j Umu_k(q) + B_i B_j Unu_k(q)],
//   Uc_k(q) = sum_a f_c(q,a) Wc_k(a)
// with f_0 = w v_rho and f_c = w (2 v_ss g_c,s + v_ab g_c,s') / h
// (dftgrid_purem.cpp:509-528, 594-615). The same quadrature sums as the
// reference.
//
// Kernels: dxc_rad (D, Dr), dxc_point (density, functional, point weights,
// energy partials), dxc_ang (U), dxc_fock (tiles, shared-boundary corner),
// dxc_energy (fixed-order reduction).
#include "devatom.cuh"  // xc_func_is_gga
#include "devdiatomic.cuh"
#include "xc_func.cuh"

namespace hfg {
namespace {

constexpr int PAIR_CHUNK = 512;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

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

__device__ __forceinline__ int dgfun(const DevDiatomic& D, int e, int p) { return e * (D.nn - 1) + p; }

// D[s][e][q][k], Dr likewise; grid (nel, npair, nsd)
__global__ void dxc_rad(DevDiatomic D, DevDiatomicXC X, DiatomicXcScratch S, const double* __restrict__ P0,
                        const double* __restrict__ P1) {
  const int e = blockIdx.x, k = blockIdx.y, s = blockIdx.z;
  const int nn = D.nn, nq = X.nq;
  const int sa = X.ps[k], ta = X.pt[k];
  const double* P = s ? P1 : P0;
  extern __shared__ double sm[];
  double* Pt = sm;            // nn*nn
  double* R = Pt + nn * nn;   // nq*nn
  double* dR = R + nq * nn;   // nq*nn
  for (int idx = threadIdx.x; idx < nn * nn; idx += blockDim.x) {
    const int i = idx % nn, j = idx / nn;
    const int gi = dgfun(D, e, i), gj = dgfun(D, e, j);
    Pt[idx] = (gi < D.nrad && gj < D.nrad) ? P[(size_t)(ta * D.nrad + gj) * D.nd + (size_t)sa * D.nrad + gi] : 0.0;
  }
  for (int idx = threadIdx.x; idx < nq * nn; idx += blockDim.x) {
    R[idx] = X.R[(size_t)e * nq * nn + idx];
    dR[idx] = X.dR[(size_t)e * nq * nn + idx];
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    const double* Rq = R + q * nn;
    const double* dRq = dR + q * nn;
    double d = 0.0, dr = 0.0;
    for (int j = 0; j < nn; ++j) {
      double t = 0.0, td = 0.0;
      for (int i = 0; i < nn; ++i) {
        const double p = Pt[i + j * nn];
        t += Rq[i] * p;
        td += dRq[i] * p;
      }
      d += t * Rq[j];
      dr += td * Rq[j];
    }
    const size_t o = (((size_t)s * D.nel + e) * nq + q) * X.npair + k;
    S.D[o] = d;
    S.Dr[o] = dr;
  }
}

// grid (nel, nq); one thread per nu point (blockDim >= na)
__global__ void dxc_point(DevDiatomic D, DevDiatomicXC X, DiatomicXcScratch S, int xid, int cid, int gga, int nsd,
                          int polarized, double thr) {
  const int e = blockIdx.x, q = blockIdx.y;
  const int nq = X.nq, na = X.na, np = X.npair;
  __shared__ double Dq[2][PAIR_CHUNK];
  __shared__ double Drq[2][PAIR_CHUNK];
  __shared__ double red[32];
  const int a = threadIdx.x;
  const bool live = a < na;
  double rho[2] = {0.0, 0.0}, gm[2] = {0.0, 0.0}, gn[2] = {0.0, 0.0};
  for (int c0 = 0; c0 < np; c0 += PAIR_CHUNK) {
    const int nc = min(PAIR_CHUNK, np - c0);
    __syncthreads();
    for (int idx = threadIdx.x; idx < nsd * nc; idx += blockDim.x) {
      const int s = idx / nc, kk = idx % nc;
      const size_t o = (((size_t)s * D.nel + e) * nq + q) * np + c0 + kk;
      Dq[s][kk] = S.D[o];
      Drq[s][kk] = S.Dr[o];
    }
    __syncthreads();
    if (live) {
      for (int s = 0; s < nsd; ++s) {
        double rs = rho[s], mr = gm[s], nr = gn[s];
        for (int kk = 0; kk < nc; ++kk) {
          const double w = X.W[(size_t)(c0 + kk) * na + a];
          const double d = Dq[s][kk];
          rs += d * w;
          if (gga) {
            mr += Drq[s][kk] * w;
            nr += d * X.Wt[(size_t)(c0 + kk) * na + a];
          }
        }
        rho[s] = rs;
        gm[s] = mr;
        gn[s] = nr;
      }
    }
  }
  double esum = 0.0, nsum = 0.0;
  if (live) {
    const size_t pq = ((size_t)e * nq + q) * na + a;
    const double w = X.w[pq], hinv = X.hinv[pq];
    double g[2][2];
    for (int s = 0; s < 2; ++s) {
      g[s][0] = 2.0 * gm[s] * hinv;
      g[s][1] = 2.0 * gn[s] * hinv;
    }
    if (!polarized) {  // restricted: equal spin densities from the total P
      rho[0] *= 0.5;
      rho[1] = rho[0];
      for (int c = 0; c < 2; ++c) {
        g[0][c] *= 0.5;
        g[1][c] = g[0][c];
      }
    }
    double ra = rho[0], rb = rho[1];
    const double n = ra + rb;
    double ev = 0.0, v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (n >= thr) {  // density threshold: below it the point contributes nothing
      ra = fmax(ra, 0.5 * thr);
      rb = fmax(rb, 0.5 * thr);
      const double saa = g[0][0] * g[0][0] + g[0][1] * g[0][1];
      const double sab = g[0][0] * g[1][0] + g[0][1] * g[1][1];
      const double sbb = g[1][0] * g[1][0] + g[1][1] * g[1][1];
      if (gga) eval_func<5>(xid, cid, ra, rb, saa, sab, sbb, ev, v);
      else eval_func<2>(xid, cid, ra, rb, 0.0, 0.0, 0.0, ev, v);
    }
    esum = w * ev;
    nsum = w * n;
    const int nout = polarized ? 2 : 1;
    for (int s = 0; s < nout; ++s) {
      const size_t cstride = (size_t)D.nel * nq * na;
      const size_t base = (size_t)s * 3 * cstride + ((size_t)e * nq + q) * na + a;
      S.F[base] = w * v[s];
      if (gga) {
        const double vss = v[s == 0 ? 2 : 4], vab = v[3];
        for (int c = 0; c < 2; ++c)
          S.F[base + (size_t)(c + 1) * cstride] = w * (2.0 * vss * g[s][c] + vab * g[1 - s][c]) * hinv;
      }
    }
  }
  esum = block_sum(esum, red);
  nsum = block_sum(nsum, red);
  if (threadIdx.x == 0) {
    S.epart[((size_t)e * nq + q) * 2 + 0] = esum;
    S.epart[((size_t)e * nq + q) * 2 + 1] = nsum;
  }
}

// U[o][c][e][k][q] = sum_a F[o][c][e][q][a] Wc[k][a]; grid (nel, nq, nout)
__global__ void dxc_ang(DevDiatomic D, DevDiatomicXC X, DiatomicXcScratch S, int ncomp) {
  const int e = blockIdx.x, q = blockIdx.y, o = blockIdx.z;
  const int nq = X.nq, na = X.na, np = X.npair;
  extern __shared__ double Fq[];  // [ncomp][na]
  const size_t cstride = (size_t)D.nel * nq * na;
  for (int idx = threadIdx.x; idx < ncomp * na; idx += blockDim.x) {
    const int c = idx / na, a = idx % na;
    Fq[idx] = S.F[((size_t)o * 3 + c) * cstride + ((size_t)e * nq + q) * na + a];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int row = w; row < ncomp * np; row += nw) {
    const int c = row / np, k = row % np;
    const double* Wc = (c == 2) ? X.Wt : X.W;
    double acc = 0.0;
    for (int a = lane; a < na; a += 32) acc += Fq[c * na + a] * Wc[(size_t)k * na + a];
    acc = warp_sum(acc);
    if (lane == 0) S.U[((((size_t)o * 3 + c) * D.nel + e) * np + k) * nq + q] = acc;
  }
}

__device__ __forceinline__ double dfock_value(const DevDiatomic& D, const DevDiatomicXC& X,
                                              const DiatomicXcScratch& S, int o, int e, int k, int i, int j,
                                              int gga) {
  const int nq = X.nq, nn = D.nn, np = X.npair;
  const double* R = X.R + (size_t)e * nq * nn;
  const double* dR = X.dR + (size_t)e * nq * nn;
  auto U = [&](int c, int kk) { return S.U + ((((size_t)o * 3 + c) * D.nel + e) * np + kk) * nq; };
  const double* U0 = U(0, k);
  double v = 0.0;
  for (int q = 0; q < nq; ++q) v += R[q * nn + i] * R[q * nn + j] * U0[q];
  if (gga) {
    const int kr = X.prev[k];
    const double *Um = U(1, k), *Un = U(2, k), *Vm = U(1, kr), *Vn = U(2, kr);
    for (int q = 0; q < nq; ++q) {
      const double Ri = R[q * nn + i], Rj = R[q * nn + j];
      v += dR[q * nn + i] * Rj * Um[q] + Ri * Rj * Un[q];  // X
      v += dR[q * nn + j] * Ri * Vm[q] + Ri * Rj * Vn[q];  // X^T
    }
  }
  return v;
}

// grid (npair, nel, nout); H written on the element-diagonal tiles of the
// same-m blocks (the rest of H is zero)
__global__ void dxc_fock(DevDiatomic D, DevDiatomicXC X, DiatomicXcScratch S, int gga, double* __restrict__ H0,
                         double* __restrict__ H1) {
  const int k = blockIdx.x, e = blockIdx.y, o = blockIdx.z;
  const int nn = D.nn, sa = X.ps[k], ta = X.pt[k];
  double* H = o ? H1 : H0;
  for (int idx = threadIdx.x; idx < nn * nn; idx += blockDim.x) {
    const int i = idx % nn, j = idx / nn;
    if (i == nn - 1 && j == nn - 1) continue;  // owned by the next element (or dropped)
    const int gi = dgfun(D, e, i), gj = dgfun(D, e, j);
    if (gi >= D.nrad || gj >= D.nrad) continue;
    double v = dfock_value(D, X, S, o, e, k, i, j, gga);
    if (i == 0 && j == 0 && e > 0) v += dfock_value(D, X, S, o, e - 1, k, nn - 1, nn - 1, gga);
    H[(size_t)(ta * D.nrad + gj) * D.nd + (size_t)sa * D.nrad + gi] = v;
  }
}

__global__ void dxc_energy(const double* __restrict__ part, int n, double* out) {
  __shared__ double red[32];
  double e = 0.0, nel = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    e += part[2 * i];
    nel += part[2 * i + 1];
  }
  e = block_sum(e, red);
  nel = block_sum(nel, red);
  if (threadIdx.x == 0) {
    out[0] = e;
    out[1] = nel;
  }
}

}  // namespace

cudaError_t launch_diatomic_xc(const DevDiatomic& D, const DevDiatomicXC& X, const DiatomicXcScratch& S, int xid,
                               int cid, const double* Pa, const double* Pb, double* Ha, double* Hb, double* energies,
                               double thr, cudaStream_t st) {
  const bool polarized = Pb != nullptr;
  const int nsd = polarized ? 2 : 1, nout = nsd;
  const bool gga = xc_func_is_gga(xid) || xc_func_is_gga(cid);
  const int ncomp = gga ? 3 : 1;
  if (X.na > 1024 || X.npair <= 0) return cudaErrorInvalidValue;
  const size_t bytes = sizeof(double) * (size_t)D.nd * D.nd;
  cudaError_t err = cudaMemsetAsync(Ha, 0, bytes, st);
  if (err == cudaSuccess && polarized) err = cudaMemsetAsync(Hb, 0, bytes, st);
  if (err != cudaSuccess) return err;
  dxc_rad<<<dim3(D.nel, X.npair, nsd), 128, sizeof(double) * (D.nn * D.nn + 2 * X.nq * D.nn), st>>>(D, X, S, Pa,
                                                                                                   Pb);
  const int tp = ((X.na + 31) / 32) * 32;
  dxc_point<<<dim3(D.nel, X.nq), tp, 0, st>>>(D, X, S, xid, cid, gga ? 1 : 0, nsd, polarized ? 1 : 0, thr);
  dxc_ang<<<dim3(D.nel, X.nq, nout), 256, sizeof(double) * ncomp * X.na, st>>>(D, X, S, ncomp);
  dxc_fock<<<dim3(X.npair, D.nel, nout), ((D.nn * D.nn + 31) / 32) * 32, 0, st>>>(D, X, S, gga ? 1 : 0, Ha, Hb);
  if (energies) dxc_energy<<<1, 512, 0, st>>>(S.epart, D.nel * X.nq, energies);
  return cudaGetLastError();
}

}  // namespace hfg

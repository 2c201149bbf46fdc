// XC potential on the pure-m diatomic DFT grid, plain FP64.
//
// Restates PureMDFTGrid::eval_Fxc and its worker
// (src/diatomic/dftgrid_purem.cpp:83-199 basis values and weights, 213-291
// and 306-369 density and gradient, 480-530 and 575-650 Fock increments,
// 668-712 element loop) in separable form. On mu element e, at mu point q and
// nu point a, the dummy function (s, p) has the value Y_s(a) B_p(q); only
// same-m angular pairs couple. Everything is symmetric under s <-> t, so the
// sums run over unordered pairs k = (s <= t) with multiplicity c_k = 2 (s != t)
// or 1. With
//   D_k(q)  = c_k B(q)^T P_st B(q)
//   Dr_k(q) = c_k/2 [dB(q)^T P_st B(q) + B(q)^T P_st dB(q)]
// the density and its gradient components along mu and nu are
//   rho(q,a) = sum_k D_k(q) W_k(a),          W_k  = Y_s Y_t
//   g_mu     = 2/h sum_k Dr_k(q) W_k(a)
//   g_nu     = 1/h sum_k D_k(q) Wt_k(a),     Wt_k = Y_s' Y_t + Y_s Y_t'
// and the Fock tile of pair k on element e (the X + X^T of the reference
// summed over both orders of the pair) is the symmetric nn x nn matrix
//   V_ij = sum_q B_i B_j (U0_k + Unu_k) + (dB_i B_j + B_i dB_j) Umu_k,
//   U0_k = sum_a f_0 W_k,  Umu_k = sum_a f_mu W_k,  Unu_k = sum_a f_nu Wt_k
// with f_0 = w v_rho and f_c = w (2 v_ss g_c,s + v_ab g_c,s') / h
// (dftgrid_purem.cpp:509-528, 594-615). The same quadrature sums as the
// reference. Densities are read and potentials written in the pure basis
// directly (the mu = 0 function of an m != 0 shell is absent).
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

// pure index of radial function g of shell s, or -1 where the function is
// not in the pure basis
__device__ __forceinline__ int dpure(const DevDiatomic& D, int s, int g) {
  const int st = D.pstart[s];
  return (g >= st && g < D.nrad) ? D.poff[s] + g - st : -1;
}

// D[s][e][q][k], Dr likewise; grid (nel, npair, nsd)
__global__ void dxc_rad(DevDiatomic D, DevDiatomicXC X, DiatomicXcScratch S, const double* __restrict__ P0,
                        const double* __restrict__ P1) {
  const int e = blockIdx.x, k = blockIdx.y, s = blockIdx.z;
  const int nn = D.nn, nq = X.nq;
  const int sa = X.ps[k], ta = X.pt[k];
  const double c = X.mult[k];
  const double* P = s ? P1 : P0;
  extern __shared__ double sm[];
  double* Pt = sm;            // nn*nn, rows (sa, i), columns (ta, j)
  double* R = Pt + nn * nn;   // nq*nn
  double* dR = R + nq * nn;   // nq*nn
  for (int idx = threadIdx.x; idx < nn * nn; idx += blockDim.x) {
    const int i = idx % nn, j = idx / nn;
    const int pi = dpure(D, sa, dgfun(D, e, i)), pj = dpure(D, ta, dgfun(D, e, j));
    Pt[idx] = (pi >= 0 && pj >= 0) ? P[(size_t)pj * D.nbf + pi] : 0.0;
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
      double t = 0.0, u = 0.0;  // (P R)_j-column partials: t = sum_i R_i P_ij, u = sum_i dR_i P_ij
      for (int i = 0; i < nn; ++i) {
        const double p = Pt[i + j * nn];
        t += Rq[i] * p;
        u += dRq[i] * p;
      }
      d += t * Rq[j];
      dr += u * Rq[j] + t * dRq[j];
    }
    const size_t o = (((size_t)s * D.nel + e) * nq + q) * X.npair + k;
    S.D[o] = c * d;
    S.Dr[o] = 0.5 * c * dr;
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
      g[s][1] = gn[s] * hinv;
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

// U[o][c][e][k][q] = sum_a F[o][c][e][q][a] Wc[k][a] for the Fock-side pairs k;
// grid (nel, nq, nout)
__global__ void dxc_ang(DevDiatomic D, DevDiatomicXC X, DiatomicXcScratch S, int ncomp) {
  const int e = blockIdx.x, q = blockIdx.y, o = blockIdx.z;
  const int nq = X.nq, na = X.na, np = X.npair, nf = X.nfock;
  extern __shared__ double Fq[];  // [ncomp][na]
  const size_t cstride = (size_t)D.nel * nq * na;
  for (int idx = threadIdx.x; idx < ncomp * na; idx += blockDim.x) {
    const int c = idx / na, a = idx % na;
    Fq[idx] = S.F[((size_t)o * 3 + c) * cstride + ((size_t)e * nq + q) * na + a];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int row = w; row < ncomp * nf; row += nw) {
    const int c = row / nf, k = X.fk[row % nf];
    const double* Wc = (c == 2) ? X.Wt : X.W;
    double acc = 0.0;
    for (int a = lane; a < na; a += 32) acc += Fq[c * na + a] * Wc[(size_t)k * na + a];
    acc = warp_sum(acc);
    if (lane == 0) S.U[((((size_t)o * 3 + c) * D.nel + e) * np + k) * nq + q] = acc;
  }
}

// value v at row (a, gi), column (b, gj) of the pure H and at the transposed
// position, where both functions are in the pure basis
__device__ __forceinline__ void dxc_put(const DevDiatomic& D, double* H, int a, int gi, int b, int gj, double v) {
  const int pi = dpure(D, a, gi), pj = dpure(D, b, gj);
  if (pi < 0 || pj < 0) return;
  H[(size_t)pj * D.nbf + pi] = v;
  H[(size_t)pi * D.nbf + pj] = v;
}

// grid (nfock, nel, nout). The tile of a pair is symmetric in (i, j): each
// thread builds one i <= j entry and writes it to the (s, t) and (t, s)
// blocks at both (i, j) and (j, i), and to the mirror blocks of opposite m.
// The rest of H is zero.
__global__ void dxc_fock(DevDiatomic D, DevDiatomicXC X, DiatomicXcScratch S, int gga, double* __restrict__ H0,
                         double* __restrict__ H1) {
  const int kf = blockIdx.x, e = blockIdx.y, o = blockIdx.z;
  const int nn = D.nn, nq = X.nq, np = X.npair;
  const int k = X.fk[kf], sa = X.ps[k], ta = X.pt[k], ms = X.fms[kf], mt = X.fmt[kf];
  double* H = o ? H1 : H0;
  extern __shared__ double sm[];
  double* R = sm;             // nq*nn
  double* dR = R + nq * nn;   // nq*nn
  double* Us = dR + nq * nn;  // nq: U0 + Unu
  double* Um = Us + nq;       // nq: Umu
  __shared__ double corner;
  auto U = [&](int c, int ee) { return S.U + ((((size_t)o * 3 + c) * D.nel + ee) * np + k) * nq; };
  for (int idx = threadIdx.x; idx < nq * nn; idx += blockDim.x) {
    R[idx] = X.R[(size_t)e * nq * nn + idx];
    dR[idx] = X.dR[(size_t)e * nq * nn + idx];
  }
  for (int q = threadIdx.x; q < nq; q += blockDim.x) {
    Us[q] = U(0, e)[q] + (gga ? U(2, e)[q] : 0.0);
    Um[q] = gga ? U(1, e)[q] : 0.0;
  }
  // the first function of element e is the last of element e-1: its diagonal
  // value there, V_{nn-1,nn-1}(e-1)
  if (threadIdx.x < 32) {
    double c = 0.0;
    if (e > 0) {
      const double* Rp = X.R + (size_t)(e - 1) * nq * nn;
      const double* dRp = X.dR + (size_t)(e - 1) * nq * nn;
      for (int q = threadIdx.x; q < nq; q += 32) {
        const double r = Rp[q * nn + nn - 1], dr = dRp[q * nn + nn - 1];
        c += r * r * (U(0, e - 1)[q] + (gga ? U(2, e - 1)[q] : 0.0)) + (gga ? 2.0 * dr * r * U(1, e - 1)[q] : 0.0);
      }
    }
    c = warp_sum(c);
    if (threadIdx.x == 0) corner = c;
  }
  __syncthreads();
  const int ntri = nn * (nn + 1) / 2;
  for (int idx = threadIdx.x; idx < ntri; idx += blockDim.x) {
    // idx -> (i <= j), j-major
    int j = (int)((sqrtf(8.0f * idx + 1.0f) - 1.0f) * 0.5f);
    while (j * (j + 1) / 2 > idx) --j;
    while ((j + 1) * (j + 2) / 2 <= idx) ++j;
    const int i = idx - j * (j + 1) / 2;
    if (i == nn - 1 && j == nn - 1) continue;  // owned by the next element (or dropped)
    const int gi = dgfun(D, e, i), gj = dgfun(D, e, j);
    if (gi >= D.nrad || gj >= D.nrad) continue;
    double v = 0.0;
    for (int q = 0; q < nq; ++q) {
      const double Ri = R[q * nn + i], Rj = R[q * nn + j];
      v += Ri * (Rj * Us[q] + dR[q * nn + j] * Um[q]) + dR[q * nn + i] * Rj * Um[q];
    }
    if (i == 0 && j == 0) v += corner;
    dxc_put(D, H, sa, gi, ta, gj, v);
    dxc_put(D, H, sa, gj, ta, gi, v);
    if (ms >= 0) {
      dxc_put(D, H, ms, gi, mt, gj, v);
      dxc_put(D, H, ms, gj, mt, gi, v);
    }
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
  if (X.na > 1024 || X.npair <= 0 || X.nfock <= 0) return cudaErrorInvalidValue;
  const size_t bytes = sizeof(double) * (size_t)D.nbf * D.nbf;
  cudaError_t err = cudaMemsetAsync(Ha, 0, bytes, st);
  if (err == cudaSuccess && polarized) err = cudaMemsetAsync(Hb, 0, bytes, st);
  if (err != cudaSuccess) return err;
  const int tq = ((X.nq + 31) / 32) * 32;
  dxc_rad<<<dim3(D.nel, X.npair, nsd), tq, sizeof(double) * (D.nn * D.nn + 2 * X.nq * D.nn), st>>>(D, X, S, Pa,
                                                                                                  Pb);
  const int tp = ((X.na + 31) / 32) * 32;
  dxc_point<<<dim3(D.nel, X.nq), tp, 0, st>>>(D, X, S, xid, cid, gga ? 1 : 0, nsd, polarized ? 1 : 0, thr);
  dxc_ang<<<dim3(D.nel, X.nq, nout), 256, sizeof(double) * ncomp * X.na, st>>>(D, X, S, ncomp);
  const int ntri = D.nn * (D.nn + 1) / 2;
  dxc_fock<<<dim3(X.nfock, D.nel, nout), ((ntri + 31) / 32) * 32, sizeof(double) * (2 * X.nq * D.nn + 2 * X.nq),
             st>>>(D, X, S, gga ? 1 : 0, Ha, Hb);
  if (energies) dxc_energy<<<1, 512, 0, st>>>(S.epart, D.nel * X.nq, energies);
  return cudaGetLastError();
}

}  // namespace hfg

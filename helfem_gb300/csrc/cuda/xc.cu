// XC potential on the atomic DFT grid, plain FP64.
//
// Restates DFTGrid::eval_Fxc and its worker (src/atomic/dftgrid.cpp:51-128,
// 304-359, 470-576, 591-712) and the split real/imaginary accumulations of
// src/general/dftgrid_common.h:128-217, in separable form. On element e with
// radial points q and angular points a (a product rule), the basis functions
// are phi_{alpha i} = R_i(r_q) Y_alpha(Omega_a). Every quantity the reference
// forms from dense (functions x points) matrices factorises:
//   rho(q,a)      = sum_{alpha beta} D_ab(q) W_ab(a),  D_ab(q) = R(q)^T P_ab R(q)
//   grad_r rho    = 2 sum Dr_ab(q) W_ab(a),           Dr_ab(q) = dR(q)^T P_ab R(q)
//   grad_th rho   = (2/r) sum D_ab(q) Wt_ab(a)
//   grad_ph rho   = (2/(r sin th)) sum D_ab(q) Wp_ab(a)
// and the Fock matrix
//   V_{ai,bj} = sum_q R_i R_j U0_ab(q) + X + X^T,
//   X_{ai,bj} = sum_q [dR_i R_j Ur_ab(q) + R_i R_j (Ut_ab(q) + Up_ab(q))],
//   Uc_ab(q)  = sum_a f_c(q,a) Wc_ab(a)
// with per-point weights f_0 = w v_rho, f_c = w (2 v_ss grad_c rho_s +
// v_ab grad_c rho_s') / scale_c (dftgrid.cpp:321-334). The same quadrature sums
// as the reference, about a hundred times fewer operations.
//
// Kernels: xc_rad (D, Dr), xc_point (density, functional, point weights,
// energy partials), xc_ang (U), xc_fock (V, shared-boundary corner as in J),
// xc_energy (fixed-order reduction).
#include <cfloat>

#include "devatom.cuh"
#include "xc_func.cuh"

namespace hfg {
namespace {

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

__device__ __forceinline__ bool gvalid(const DevAtom& A, int g) { return g >= 0 && g < A.nrad; }

// D[s][e][ab][q], Dr likewise; grid (nel, nang^2, nsd)
__global__ void xc_rad(DevAtom A, DevXC X, XcScratch S, const double* __restrict__ P0,
                       const double* __restrict__ P1) {
  const int e = blockIdx.x, ab = blockIdx.y, s = blockIdx.z;
  const int nn = A.nn, nq = X.nquad;
  const int al = ab % A.nang, be = ab / A.nang;
  const double* P = s ? P1 : P0;
  extern __shared__ double sm[];
  double* Pt = sm;                 // nn*nn
  double* R = Pt + nn * nn;        // nq*nn
  double* dR = R + nq * nn;        // nq*nn
  for (int idx = threadIdx.x; idx < nn * nn; idx += blockDim.x) {
    const int i = idx % nn, j = idx / nn;
    const int gi = gfun(A, e, i), gj = gfun(A, e, j);
    Pt[idx] = (gvalid(A, gi) && gvalid(A, gj))
                  ? P[(size_t)(be * A.nrad + gj) * A.nbf + (size_t)al * A.nrad + gi]
                  : 0.0;
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
    const size_t o = (((size_t)s * A.nel + e) * (A.nang * A.nang) + ab) * nq + q;
    S.D[o] = d;
    S.Dr[o] = dr;
  }
}

// grid (nel, nquad); threads over angular points
__global__ void xc_point(DevAtom A, DevXC X, XcScratch S, int xid, int cid, int gga, int nsd, int polarized,
                         double thr) {
  const int e = blockIdx.x, q = blockIdx.y;
  const int nq = X.nquad, nap = X.nap, nab = A.nang * A.nang;
  extern __shared__ double sm[];
  double* Dq = sm;              // [nsd][nab]
  double* Drq = Dq + nsd * nab; // [nsd][nab]
  __shared__ double red[32];
  for (int idx = threadIdx.x; idx < nsd * nab; idx += blockDim.x) {
    const int s = idx / nab, ab = idx % nab;
    const size_t o = (((size_t)s * A.nel + e) * nab + ab) * nq + q;
    Dq[idx] = S.D[o];
    Drq[idx] = S.Dr[o];
  }
  __syncthreads();
  const double r = X.r[(size_t)e * nq + q];
  const double wr = X.wr[(size_t)e * nq + q];
  double esum = 0.0, nsum = 0.0;
  for (int a = threadIdx.x; a < nap; a += blockDim.x) {
    double rho[2] = {0.0, 0.0}, g[2][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
    for (int s = 0; s < nsd; ++s) {
      double rs = 0.0, gr = 0.0, gt = 0.0, gp = 0.0;
      for (int ab = 0; ab < nab; ++ab) {
        const double w = X.W[(size_t)ab * nap + a];
        const double d = Dq[s * nab + ab];
        rs += d * w;
        if (gga) {
          gr += Drq[s * nab + ab] * w;
          gt += d * X.Wt[(size_t)ab * nap + a];
          gp += d * X.Wp[(size_t)ab * nap + a];
        }
      }
      rho[s] = rs;
      g[s][0] = 2.0 * gr;
      g[s][1] = 2.0 * gt / r;
      g[s][2] = 2.0 * gp / r * X.isin[a];
    }
    if (!polarized) {  // restricted: equal spin densities from the total P
      rho[0] *= 0.5;
      rho[1] = rho[0];
      for (int c = 0; c < 3; ++c) { g[0][c] *= 0.5; g[1][c] = g[0][c]; }
    }
    const double w = X.wang[a] * wr;
    double ra = rho[0], rb = rho[1];
    const double n = ra + rb;
    double ev = 0.0, v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (n >= thr) {  // libxc density threshold: below it the point contributes nothing
      ra = fmax(ra, 0.5 * thr);
      rb = fmax(rb, 0.5 * thr);
      const double saa = g[0][0] * g[0][0] + g[0][1] * g[0][1] + g[0][2] * g[0][2];
      const double sab = g[0][0] * g[1][0] + g[0][1] * g[1][1] + g[0][2] * g[1][2];
      const double sbb = g[1][0] * g[1][0] + g[1][1] * g[1][1] + g[1][2] * g[1][2];
      if (gga) eval_func<5>(xid, cid, ra, rb, saa, sab, sbb, ev, v);
      else eval_func<2>(xid, cid, ra, rb, 0.0, 0.0, 0.0, ev, v);
    }
    esum += w * ev;
    nsum += w * n;
    const double scale[3] = {1.0, 1.0 / r, X.isin[a] / r};
    const int nout = polarized ? 2 : 1;
    for (int s = 0; s < nout; ++s) {
      const size_t base = (((size_t)s * 4) * A.nel + e) * nq + q;  // comp stride nel*nq
      S.F[(base + 0) * nap + a] = w * v[s];
      if (gga) {
        const double vss = v[s == 0 ? 2 : 4], vab = v[3];
        for (int c = 0; c < 3; ++c) {
          const double f = w * (2.0 * vss * g[s][c] + vab * g[1 - s][c]) * scale[c];
          S.F[(base + (size_t)(c + 1) * A.nel * nq) * nap + a] = f;
        }
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

// U[s][c][e][ab][q] = sum_a F[s][c][e][q][a] Wc[ab][a]; grid (nel, nquad, nout)
__global__ void xc_ang(DevAtom A, DevXC X, XcScratch S, int ncomp) {
  const int e = blockIdx.x, q = blockIdx.y, s = blockIdx.z;
  const int nq = X.nquad, nap = X.nap, nab = A.nang * A.nang;
  extern __shared__ double Fq[];  // [ncomp][nap]
  for (int idx = threadIdx.x; idx < ncomp * nap; idx += blockDim.x) {
    const int c = idx / nap, a = idx % nap;
    Fq[idx] = S.F[(((((size_t)s * 4) + c) * A.nel + e) * nq + q) * nap + a];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int row = w; row < ncomp * nab; row += nw) {
    const int c = row / nab, ab = row % nab;
    const double* Wc = (c == 2) ? X.Wt : (c == 3) ? X.Wp : X.W;
    double acc = 0.0;
    for (int a = lane; a < nap; a += 32) acc += Fq[c * nap + a] * Wc[(size_t)ab * nap + a];
    acc = warp_sum(acc);
    if (lane == 0) S.U[(((((size_t)s * 4) + c) * A.nel + e) * nab + ab) * nq + q] = acc;
  }
}

// tile value V_{(al,i),(be,j)} of element e
__device__ __forceinline__ double fock_value(const DevAtom& A, const DevXC& X, const XcScratch& S, int s, int e,
                                             int al, int be, int i, int j, int gga) {
  const int nq = X.nquad, nn = A.nn, nab = A.nang * A.nang;
  const int ab = al + be * A.nang, ba = be + al * A.nang;
  const double* R = X.R + (size_t)e * nq * nn;
  const double* dR = X.dR + (size_t)e * nq * nn;
  auto U = [&](int c, int idx) { return S.U + (((((size_t)s * 4) + c) * A.nel + e) * nab + idx) * nq; };
  const double* U0 = U(0, ab);
  double v = 0.0;
  for (int q = 0; q < nq; ++q) v += R[q * nn + i] * R[q * nn + j] * U0[q];
  if (gga) {
    const double *Ur = U(1, ab), *Ut = U(2, ab), *Up = U(3, ab);
    const double *Vr = U(1, ba), *Vt = U(2, ba), *Vp = U(3, ba);
    for (int q = 0; q < nq; ++q) {
      const double Ri = R[q * nn + i], Rj = R[q * nn + j];
      v += dR[q * nn + i] * Rj * Ur[q] + Ri * Rj * (Ut[q] + Up[q]);  // X
      v += dR[q * nn + j] * Ri * Vr[q] + Ri * Rj * (Vt[q] + Vp[q]);  // X^T
    }
  }
  return v;
}

// grid (nang^2, nel, nout); H overwritten on the element-diagonal tiles
__global__ void xc_fock(DevAtom A, DevXC X, XcScratch S, int gga, double* __restrict__ H0, double* __restrict__ H1) {
  const int ab = blockIdx.x, e = blockIdx.y, s = blockIdx.z;
  const int nn = A.nn, al = ab % A.nang, be = ab / A.nang;
  double* H = s ? H1 : H0;
  for (int idx = threadIdx.x; idx < nn * nn; idx += blockDim.x) {
    const int i = idx % nn, j = idx / nn;
    if (i == nn - 1 && j == nn - 1) continue;  // owned by the next element
    const int gi = gfun(A, e, i), gj = gfun(A, e, j);
    if (!gvalid(A, gi) || !gvalid(A, gj)) continue;
    double v = fock_value(A, X, S, s, e, al, be, i, j, gga);
    if (i == 0 && j == 0 && e > 0) v += fock_value(A, X, S, s, e - 1, al, be, nn - 1, nn - 1, gga);
    H[(size_t)(be * A.nrad + gj) * A.nbf + (size_t)al * A.nrad + gi] = v;
  }
}

__global__ void xc_energy(const double* __restrict__ part, int n, double* out) {
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

bool xc_func_supported(int id) { return id == 0 || id == 1 || id == 7 || id == 12 || id == 101 || id == 130; }
bool xc_func_is_gga(int id) { return id == 101 || id == 130; }

cudaError_t launch_xc_fp64(const DevAtom& A, const DevXC& X, const XcScratch& S, int xid, int cid,
                           const double* Pa, const double* Pb, double* Ha, double* Hb, double* energies,
                           double thr, cudaStream_t st) {
  const bool polarized = Pb != nullptr;
  const int nsd = polarized ? 2 : 1, nout = nsd;
  const bool gga = xc_func_is_gga(xid) || xc_func_is_gga(cid);
  const int ncomp = gga ? 4 : 1;
  const size_t bytes = sizeof(double) * (size_t)A.nbf * A.nbf;
  cudaError_t err = cudaMemsetAsync(Ha, 0, bytes, st);
  if (err == cudaSuccess && polarized) err = cudaMemsetAsync(Hb, 0, bytes, st);
  if (err != cudaSuccess) return err;
  const int nab = A.nang * A.nang;
  xc_rad<<<dim3(A.nel, nab, nsd), 128, sizeof(double) * (A.nn * A.nn + 2 * X.nquad * A.nn), st>>>(A, X, S, Pa, Pb);
  xc_point<<<dim3(A.nel, X.nquad), 256, sizeof(double) * 2 * nsd * nab, st>>>(A, X, S, xid, cid, gga ? 1 : 0, nsd,
                                                                           polarized ? 1 : 0, thr);
  xc_ang<<<dim3(A.nel, X.nquad, nout), 256, sizeof(double) * ncomp * X.nap, st>>>(A, X, S, ncomp);
  xc_fock<<<dim3(nab, A.nel, nout), ((A.nn * A.nn + 31) / 32) * 32, 0, st>>>(A, X, S, gga ? 1 : 0, Ha, Hb);
  if (energies) xc_energy<<<1, 512, 0, st>>>(S.epart, A.nel * X.nquad, energies);
  return cudaGetLastError();
}

}  // namespace hfg

// Exchange-correlation energy densities (per volume) in spin-resolved form,
// written once as templates and differentiated exactly by forward-mode dual
// numbers: slot 0..4 = d/d(rho_a, rho_b, sigma_aa, sigma_ab, sigma_bb).
//
// Restated from the published papers (the reference evaluates them through
// libxc, src/general/dftgrid_common.cpp:98-255; libxc is not used here):
//   Slater/Dirac exchange                                   (libxc id 1)
//   VWN5 correlation, Vosko-Wilk-Nusair, CJP 58, 1200 (1980)      (id 7)
//   PW92 correlation, Perdew-Wang, PRB 45, 13244 (1992)            (id 12)
//   PBE exchange / correlation, Perdew-Burke-Ernzerhof, PRL 77, 3865
//   (1996); correlation built on PW92 with the more precise constants   (101, 130)
#pragma once

#include <cuda_runtime.h>

namespace hfg {
namespace xcf {

template <int N>
struct Dual {
  double v;
  double d[N];
};

template <int N>
__device__ __forceinline__ Dual<N> cst(double x) {
  Dual<N> r;
  r.v = x;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = 0.0;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> var(double x, int slot) {
  Dual<N> r = cst<N>(x);
  if (slot < N) r.d[slot] = 1.0;
  return r;
}
// chain rule helper: f(a) with f'(a) = g
template <int N>
__device__ __forceinline__ Dual<N> chain(const Dual<N>& a, double f, double g) {
  Dual<N> r;
  r.v = f;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = g * a.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v + b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v - b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r;
  r.v = -a.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  r.v = a.v * b.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r;
  const double ib = 1.0 / b.v;
  r.v = a.v * ib;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator+(const Dual<N>& a, double b) { Dual<N> r = a; r.v += b; return r; }
template <int N>
__device__ __forceinline__ Dual<N> operator+(double b, const Dual<N>& a) { return a + b; }
template <int N>
__device__ __forceinline__ Dual<N> operator-(const Dual<N>& a, double b) { Dual<N> r = a; r.v -= b; return r; }
template <int N>
__device__ __forceinline__ Dual<N> operator-(double b, const Dual<N>& a) { return (-a) + b; }
template <int N>
__device__ __forceinline__ Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r;
  r.v = a.v * b;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <int N>
__device__ __forceinline__ Dual<N> operator*(double b, const Dual<N>& a) { return a * b; }
template <int N>
__device__ __forceinline__ Dual<N> operator/(const Dual<N>& a, double b) { return a * (1.0 / b); }
template <int N>
__device__ __forceinline__ Dual<N> operator/(double a, const Dual<N>& b) {
  const double ib = 1.0 / b.v;
  return chain(b, a * ib, -a * ib * ib);
}
template <int N>
__device__ __forceinline__ Dual<N> log(const Dual<N>& a) { return chain(a, ::log(a.v), 1.0 / a.v); }
template <int N>
__device__ __forceinline__ Dual<N> exp(const Dual<N>& a) { const double e = ::exp(a.v); return chain(a, e, e); }
template <int N>
__device__ __forceinline__ Dual<N> sqrt(const Dual<N>& a) { const double s = ::sqrt(a.v); return chain(a, s, 0.5 / s); }
template <int N>
__device__ __forceinline__ Dual<N> atan(const Dual<N>& a) { return chain(a, ::atan(a.v), 1.0 / (1.0 + a.v * a.v)); }
template <int N>
__device__ __forceinline__ Dual<N> pow(const Dual<N>& a, double p) {
  const double f = ::pow(a.v, p);
  return chain(a, f, p * f / a.v);
}

constexpr double PI = 3.14159265358979323846;

// f(zeta) from opz = 1 + zeta = 2 rho_a / n and omz = 1 - zeta = 2 rho_b / n,
// formed from the spin densities rather than by subtracting zeta from one
// (which loses the relative precision of a minority spin density)
template <class T>
__device__ __forceinline__ T fzeta(const T& opz, const T& omz) {
  const double den = 1.0 / (2.5198420997897464 - 2.0);  // 2^{4/3} - 2
  return (pow(opz, 4.0 / 3.0) + pow(omz, 4.0 / 3.0) - 2.0) * den;
}

// ---------------------------------------------------------------- Slater x
template <class T>
__device__ __forceinline__ T slater_x(const T& ra, const T& rb) {
  const double c = -0.75 * 1.2407009817988531;  // (6/pi)^{1/3}
  return c * (pow(ra, 4.0 / 3.0) + pow(rb, 4.0 / 3.0));
}

// ------------------------------------------------------------------- VWN5
template <class T>
__device__ __forceinline__ T vwn_eps(const T& x, double A, double b, double c, double x0) {
  const T X = x * x + b * x + c;
  const double X0 = x0 * x0 + b * x0 + c;
  const double Q = ::sqrt(4.0 * c - b * b);
  const T at = atan(Q / (2.0 * x + b));
  return A * (log(x * x / X) + (2.0 * b / Q) * at -
              (b * x0 / X0) * (log((x - x0) * (x - x0) / X) + (2.0 * (b + 2.0 * x0) / Q) * at));
}

template <class T>
__device__ __forceinline__ T vwn5_c(const T& ra, const T& rb) {
  const T n = ra + rb;
  const T z = (ra - rb) / n;
  const T rs = pow((3.0 / (4.0 * PI)) / n, 1.0 / 3.0);
  const T x = sqrt(rs);
  const T opz = 2.0 * ra / n, omz = 2.0 * rb / n;
  const T eP = vwn_eps(x, 0.0310907, 3.72744, 12.9352, -0.10498);
  const T eF = vwn_eps(x, 0.01554535, 7.06042, 18.0578, -0.32500);
  const T ac = vwn_eps(x, -1.0 / (6.0 * PI * PI), 1.13107, 13.0045, -0.0047584);
  const double fpp = 4.0 / (9.0 * (1.2599210498948732 - 1.0));
  const T f = fzeta(opz, omz);
  const T z2 = z * z;
  const T z4 = z2 * z2;
  return n * (eP + ac * f * (1.0 / fpp) * (1.0 - z4) + (eF - eP) * f * z4);
}

// ------------------------------------------------------------------- PW92
struct PWPar { double A, a1, b1, b2, b3, b4; };

template <class T>
__device__ __forceinline__ T pw_G(const T& rs, const PWPar& p) {
  const T srs = sqrt(rs);
  const T den = 2.0 * p.A * (p.b1 * srs + p.b2 * rs + p.b3 * rs * srs + p.b4 * rs * rs);
  return -2.0 * p.A * (1.0 + p.a1 * rs) * log(1.0 + 1.0 / den);
}

template <class T>
__device__ __forceinline__ T pw_eps(const T& n, const T& z, const T& opz, const T& omz, bool mod) {
  const PWPar P = {mod ? 0.0310907 : 0.031091, 0.21370, 7.5957, 3.5876, 1.6382, 0.49294};
  const PWPar F = {mod ? 0.01554535 : 0.015545, 0.20548, 14.1189, 6.1977, 3.3662, 0.62517};
  const PWPar Ap = {mod ? 0.0168869 : 0.016887, 0.11125, 10.357, 3.6231, 0.88026, 0.49671};
  const double fpp = mod ? 1.709920934161365617563962776245 : 1.709921;
  const T rs = pow((3.0 / (4.0 * PI)) / n, 1.0 / 3.0);
  const T eP = pw_G(rs, P);
  const T eF = pw_G(rs, F);
  const T ac = -pw_G(rs, Ap);
  const T f = fzeta(opz, omz);
  const T z2 = z * z;
  const T z4 = z2 * z2;
  return eP + ac * f * (1.0 / fpp) * (1.0 - z4) + (eF - eP) * f * z4;
}

template <class T>
__device__ __forceinline__ T pw92_c(const T& ra, const T& rb) {
  const T n = ra + rb;
  return n * pw_eps(n, (ra - rb) / n, 2.0 * ra / n, 2.0 * rb / n, false);
}

// -------------------------------------------------------------------- PBE
constexpr double PBE_KAPPA = 0.804;
constexpr double PBE_MU = 0.2195149727645171;
constexpr double PBE_BETA = 0.06672455060314922;
constexpr double PBE_GAMMA = 0.031090690869654895;  // (1 - ln 2) / pi^2

template <class T>
__device__ __forceinline__ T pbe_x_unpol(const T& n, const T& s2n) {
  const T kf = pow(3.0 * PI * PI * n, 1.0 / 3.0);
  const T exu = (-0.75 / PI) * kf * n;
  const T d = 2.0 * kf * n;
  const T s2 = s2n / (d * d);
  const T Fx = (1.0 + PBE_KAPPA) - PBE_KAPPA / (1.0 + (PBE_MU / PBE_KAPPA) * s2);
  return exu * Fx;
}

template <class T>
__device__ __forceinline__ T pbe_x(const T& ra, const T& rb, const T& saa, const T& sbb) {
  return 0.5 * (pbe_x_unpol(2.0 * ra, 4.0 * saa) + pbe_x_unpol(2.0 * rb, 4.0 * sbb));
}

template <class T>
__device__ __forceinline__ T pbe_c(const T& ra, const T& rb, const T& saa, const T& sab, const T& sbb) {
  const T n = ra + rb;
  const T z = (ra - rb) / n;
  const T opz = 2.0 * ra / n, omz = 2.0 * rb / n;
  const T ec = pw_eps(n, z, opz, omz, true);
  const T phi = 0.5 * (pow(opz, 2.0 / 3.0) + pow(omz, 2.0 / 3.0));
  const T kf = pow(3.0 * PI * PI * n, 1.0 / 3.0);
  const T ks = sqrt((4.0 / PI) * kf);
  const T sig = saa + 2.0 * sab + sbb;
  const T d = 2.0 * phi * ks * n;
  const T t2 = sig / (d * d);
  const T g3 = PBE_GAMMA * phi * phi * phi;
  const T A = (PBE_BETA / PBE_GAMMA) / (exp(-ec / g3) - 1.0);
  const T At2 = A * t2;
  const T H = g3 * log(1.0 + (PBE_BETA / PBE_GAMMA) * t2 * (1.0 + At2) / (1.0 + At2 + At2 * At2));
  return n * (ec + H);
}

}  // namespace xcf

// energy density and its partial derivatives (v_a, v_b, v_aa, v_ab, v_bb)
// of the exchange + correlation pair at one point; ids as in hfg_xc
template <int N>
__device__ inline void eval_func(int xid, int cid, double ra, double rb, double saa, double sab, double sbb,
                                 double& e, double* v) {
  using namespace xcf;
  const Dual<N> a = var<N>(ra, 0), b = var<N>(rb, 1);
  const Dual<N> xaa = var<N>(saa, 2), xab = var<N>(sab, 3), xbb = var<N>(sbb, 4);
  Dual<N> tot = cst<N>(0.0);
  const int ids[2] = {xid, cid};
  for (int k = 0; k < 2; ++k) {
    switch (ids[k]) {
      case 1: tot = tot + slater_x(a, b); break;
      case 7: tot = tot + vwn5_c(a, b); break;
      case 12: tot = tot + pw92_c(a, b); break;
      case 101: tot = tot + pbe_x(a, b, xaa, xbb); break;
      case 130: tot = tot + pbe_c(a, b, xaa, xab, xbb); break;
      default: break;
    }
  }
  e = tot.v;
#pragma unroll
  for (int i = 0; i < N; ++i) v[i] = tot.d[i];
}

}  // namespace hfg

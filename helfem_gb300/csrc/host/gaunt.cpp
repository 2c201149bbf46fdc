// Gaunt coefficients  coeff(L,M,l,m,lp) = int Y_L^M* Y_l^m Y_lp^(M-m) dOmega,
// the quantity HelFEM's GauntT<T>::coeff returns (src/general/gaunt.cpp:77-84,
// 201-251) and that its tests pin to DBL_EPSILON (src/general/gaunt_test.cpp).
//
// Evaluated from Racah's closed form for the two Wigner 3j symbols. The
// alternating Racah sum is formed EXACTLY as a big integer (every term is an
// integer once multiplied by a common factorial product), so there is no
// cancellation error; the remaining products of factorials are formed in
// long double and the result is rounded once to double.
#include "atom.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <vector>

namespace hfg {
namespace {

// Little-endian base-2^32 unsigned big integer: only what the Racah sum needs.
struct BigU {
  std::vector<uint32_t> d;  // empty == 0
  static BigU one() { BigU b; b.d.push_back(1u); return b; }
  void mul(uint32_t m) {
    uint64_t carry = 0;
    for (auto& x : d) {
      uint64_t t = (uint64_t)x * m + carry;
      x = (uint32_t)t;
      carry = t >> 32;
    }
    if (carry) d.push_back((uint32_t)carry);
    trim();
  }
  void trim() { while (!d.empty() && d.back() == 0) d.pop_back(); }
  bool zero() const { return d.empty(); }
};

int cmp(const BigU& a, const BigU& b) {
  if (a.d.size() != b.d.size()) return a.d.size() < b.d.size() ? -1 : 1;
  for (size_t i = a.d.size(); i-- > 0;)
    if (a.d[i] != b.d[i]) return a.d[i] < b.d[i] ? -1 : 1;
  return 0;
}

BigU add(const BigU& a, const BigU& b) {
  BigU r;
  const size_t n = std::max(a.d.size(), b.d.size());
  r.d.resize(n + 1, 0u);
  uint64_t carry = 0;
  for (size_t i = 0; i < n; ++i) {
    uint64_t t = carry;
    if (i < a.d.size()) t += a.d[i];
    if (i < b.d.size()) t += b.d[i];
    r.d[i] = (uint32_t)t;
    carry = t >> 32;
  }
  r.d[n] = (uint32_t)carry;
  r.trim();
  return r;
}

// a - b, requires a >= b
BigU sub(const BigU& a, const BigU& b) {
  BigU r;
  r.d.resize(a.d.size(), 0u);
  int64_t borrow = 0;
  for (size_t i = 0; i < a.d.size(); ++i) {
    int64_t t = (int64_t)a.d[i] - borrow - (i < b.d.size() ? (int64_t)b.d[i] : 0);
    borrow = 0;
    if (t < 0) { t += ((int64_t)1 << 32); borrow = 1; }
    r.d[i] = (uint32_t)t;
  }
  r.trim();
  return r;
}

long double to_ld(const BigU& a) {
  long double r = 0.0L;
  for (size_t i = a.d.size(); i-- > 0;) r = r * 4294967296.0L + (long double)a.d[i];
  return r;
}

long double lfact(int n) {
  long double r = 1.0L;
  for (int i = 2; i <= n; ++i) r *= (long double)i;
  return r;
}

// (j1 j2 j3; m1 m2 m3) in long double, exact Racah sum.
long double threej(int j1, int j2, int j3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0) return 0.0L;
  if (j3 < std::abs(j1 - j2) || j3 > j1 + j2) return 0.0L;
  if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0.0L;
  const int kmin = std::max({0, j2 - j3 - m1, j1 - j3 + m2});
  const int kmax = std::min({j1 + j2 - j3, j1 - m1, j2 + m2});
  if (kmax < kmin) return 0.0L;
  // six factorial arguments a_i + s_i k
  const int base[6] = {0, j3 - j2 + m1, j3 - j1 - m2, j1 + j2 - j3, j1 - m1, j2 + m2};
  const int sgn[6] = {+1, +1, +1, -1, -1, -1};
  int mx[6];
  for (int i = 0; i < 6; ++i) mx[i] = std::max(base[i] + sgn[i] * kmin, base[i] + sgn[i] * kmax);
  BigU pos, neg;
  for (int k = kmin; k <= kmax; ++k) {
    BigU t = BigU::one();
    for (int i = 0; i < 6; ++i)
      for (int x = base[i] + sgn[i] * k + 1; x <= mx[i]; ++x) t.mul((uint32_t)x);
    if (k & 1) neg = add(neg, t); else pos = add(pos, t);
  }
  long double S;
  if (cmp(pos, neg) >= 0) S = to_ld(sub(pos, neg));
  else S = -to_ld(sub(neg, pos));
  long double C = 1.0L;
  for (int i = 0; i < 6; ++i) C *= lfact(mx[i]);
  const long double pre = lfact(j1 + j2 - j3) * lfact(j1 - j2 + j3) * lfact(-j1 + j2 + j3) /
                          lfact(j1 + j2 + j3 + 1) * lfact(j1 + m1) * lfact(j1 - m1) *
                          lfact(j2 + m2) * lfact(j2 - m2) * lfact(j3 + m3) * lfact(j3 - m3);
  const int ph = ((j1 - j2 - m3) % 2 + 2) % 2 ? -1 : 1;
  return ph * std::sqrt(pre) * (S / C);
}

}  // namespace

double gaunt_coeff(int L, int M, int l, int m, int lp) {
  const int mp = M - m;
  if (L < 0 || l < 0 || lp < 0) return 0.0;
  if (std::abs(M) > L || std::abs(m) > l || std::abs(mp) > lp) return 0.0;
  if ((L + l + lp) % 2 || lp < std::abs(L - l) || lp > L + l) return 0.0;
  // Y_L^M* = (-1)^M Y_L^-M
  const long double a = threej(L, l, lp, 0, 0, 0);
  const long double b = threej(L, l, lp, -M, m, mp);
  const long double pi = 3.141592653589793238462643383279502884L;
  const long double nrm = std::sqrt((long double)((2 * L + 1) * (2 * l + 1) * (2 * lp + 1)) / (4.0L * pi));
  const long double s = (M & 1) ? -1.0L : 1.0L;
  return (double)(s * nrm * a * b);
}

}  // namespace hfg

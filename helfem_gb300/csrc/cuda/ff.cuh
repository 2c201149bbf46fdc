// Split-precision helpers shared by the exchange kernels.
//
// Every FP64 operand is held as an unevaluated sum of two floats (hi + lo,
// ~48 significant bits). Products are made exact with an FMA (TwoProd), sums
// carry their rounding error (TwoSum), so the FP32 pipe - 64x the FP64 pipe
// on GB300 - does the contraction; results are recombined in FP64 once per
// output element.
#pragma once

#include <cuda_runtime.h>

namespace hfg {

// Split an FP64 value into float hi + lo using integer operations only (the
// FP64 pipe is the scarce unit on GB300): hi carries the top 24 significand
// bits (truncated), lo the next 29 bits rounded to 24; |hi + lo - v| <=
// 2^-47 |v|. Values below 2^-126 and non-finite inputs map to (0, 0) and
// (v, 0) respectively.
static __device__ __forceinline__ float2 split_bits(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e == 0x7FF) return make_float2((float)v, 0.f);
  const int E = e - 1023;
  if (E < -126) return make_float2(0.f, 0.f);
  const unsigned long long S = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const float sgn = (b >> 63) ? -1.f : 1.f;
  const float hi = sgn * ldexpf(__uint2float_rn((unsigned)(S >> 29)), E - 23);
  const float lo = sgn * ldexpf(__uint2float_rn((unsigned)(S & 0x1FFFFFFFull)), E - 52);
  return make_float2(hi, lo);
}


struct ffv {
  float hi, lo;
};



// The explicitly rounded intrinsics keep the compiler from contracting the
// error-free transformations into FMAs (which would break their exactness).
static __device__ __forceinline__ ffv ff_norm(float s, float e) {  // fast two-sum, |s| >= |e|
  const float t = __fadd_rn(s, e);
  return {t, __fsub_rn(e, __fsub_rn(t, s))};
}

// acc + x*y: TwoProd via FMA, TwoSum for the high words; the low words
// (product and sum errors) accumulate in acc.lo, which stays small against
// acc.hi over the short contractions here and is renormalised on read
static __device__ __forceinline__ ffv ff_fma(ffv acc, float2 x, float2 y) {
  const float p = __fmul_rn(x.x, y.x);
  float pe = fmaf(x.x, y.x, -p);
  pe = fmaf(x.x, y.y, pe);
  pe = fmaf(x.y, y.x, pe);
  const float s = __fadd_rn(acc.hi, p);
  const float bb = __fsub_rn(s, acc.hi);
  const float e = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  return {s, __fadd_rn(acc.lo, __fadd_rn(e, pe))};
}

// normalised every call: for the long (nn^2-term) in-element contraction
static __device__ __forceinline__ ffv ff_fma_n(ffv acc, float2 x, float2 y) {
  const ffv r = ff_fma(acc, x, y);
  return ff_norm(r.hi, r.lo);
}

static __device__ __forceinline__ float2 ff2(ffv v) {
  const ffv n = ff_norm(v.hi, v.lo);
  return make_float2(n.hi, n.lo);
}
static __device__ __forceinline__ double ff_to_d(ffv v) { return (double)v.hi + (double)v.lo; }


// (hi, lo) + (hi, lo), renormalised: accumulates the per-multipole results
// of one output block before the single FP64 recombination
static __device__ __forceinline__ ffv ff_add(ffv a, ffv b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return ff_norm(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}


}  // namespace hfg

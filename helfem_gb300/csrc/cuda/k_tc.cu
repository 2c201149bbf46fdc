// Split-precision exchange on the tensor cores: the element-pair tiles of
// TwoDBasisT::exchange (src/atomic/TwoDBasis.cpp:879-999) with the FE
// assembly of assemble_K_FE_one_multipole_cached_chol
// (libhelfemqc/include/CoulombExchangeFE.h:484-530).
//
//   off-diagonal pairs a != b:  K_jk(a,b) -= sum_L A_L(a) X_jkL(a,b) B_L(b)^T,
//                               A/B = r_small/r_big by element order;
//   diagonal elements:          K_jk(a,a) -= sum_L Tk_L(a) vec X_jkL(a,a),
//                               Tk the exchange-ordered in-element tensor
//                               (the reference's sum_p M_p X M_p^T).
// X is the recoupled density tile.
//
// Arithmetic (an Ozaki-style slicing with exact integer sums):
//  * every operand is a fixed-point number below 1 written as balanced
//    base-256 digits: x = sum_k d_k 256^-(k+1), |d_0| <= 256, |d_k| <= 128
//    (k >= 1, the 4th digit of a density tile may reach 256); digits are
//    integers, exact in bf16;
//  * the radial tables and Tk are digitised once per atom with one
//    power-of-two scale per row (row sum of |values| <= 1 after scaling); a
//    density tile X (recoupled on the CUDA cores in float pairs) gets one
//    scale per tile;
//  * the tensor core forms the digit products level by level,
//    acc_d = sum_{k+l=d} sum_p a_k b_l (d = 0..6), in FP32 in tensor memory;
//    for the 16-term products of the off-diagonal tiles every acc_d is an
//    integer below 2^23, so the FP32 sums are exact;
//  * the levels are carried into balanced digits again on the CUDA cores:
//    the first product (Y = A X, 128 rows = 8 output blocks x 16) becomes the
//    digit operand of the second (Y B^T), whose levels are turned into a
//    float pair, scaled, and accumulated over the multipoles of the output
//    block; one FP64 conversion per output element at the end.
// Truncation (levels above 6 dropped, 48-bit density tiles) leaves ~1e-14 of
// max|K| against the FP64 result.
//
// Off-diagonal work unit = one element pair (a,b) and a range of groups of
// up to 8 output angular blocks; per group and multipole L the group's
// entries with that L form one batch of M = 128 rows. For density digit kx
// the table planes kt = 0..6-kx are consecutive in shared memory and form one
// operand of N = 16 (7 - kx) rows whose block kt lands on the tensor-memory
// columns of level kx + kt, so a batch is 6 + 7 MMAs. 256 threads: 8 warps
// recouple one block each (the next batch's while the tensor core works on
// the current one); warps w and w+4 read the same tensor-memory lanes and
// split the columns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>

#include "devatom.cuh"
#include "smem_limit.hpp"
#include "ff.cuh"
#include "tc.cuh"

namespace hfg {
namespace {

constexpr int ND = TC_NDIGITS;  // digits per table / intermediate operand
constexpr int NDX = 6;          // digits of a float-pair density tile (48 bits)
constexpr int APLANE = 4096;    // bytes of one 128 x 16 bf16 operand plane
constexpr int TPLANE = 512;     // bytes of one 16 x 16 bf16 table plane

constexpr float kMagic = 12582912.0f;  // 1.5 * 2^23: x + M - M rounds |x| < 2^22 to an integer

__device__ __forceinline__ float rnd(float x) { return __fsub_rn(__fadd_rn(x, kMagic), kMagic); }
// rint(x * s) with one rounding of the product
__device__ __forceinline__ float rnd_mul(float x, float s) { return __fsub_rn(__fmaf_rn(x, s, kMagic), kMagic); }
__device__ __forceinline__ float exp2i(int k) {  // 2^k, k clamped to the normal range
  k = k < -126 ? -126 : (k > 127 ? 127 : k);
  return __int_as_float((k + 127) << 23);
}
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

// all 7 levels (16 columns apart) of 8 consecutive columns, one wait
__device__ __forceinline__ void tmem_ld_levels(uint32_t taddr, float (&v)[ND][8]) {
  static_assert(ND == 7, "level count of the load below");
  uint32_t r[56];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%56];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%57];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16,%17,%18,%19,%20,%21,%22,%23}, [%58];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%24,%25,%26,%27,%28,%29,%30,%31}, [%59];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%32,%33,%34,%35,%36,%37,%38,%39}, [%60];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%40,%41,%42,%43,%44,%45,%46,%47}, [%61];\n"
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%48,%49,%50,%51,%52,%53,%54,%55}, [%62];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
        "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
        "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
        "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55])
      : "r"(taddr), "r"(taddr + 16), "r"(taddr + 32), "r"(taddr + 48), "r"(taddr + 64), "r"(taddr + 80),
        "r"(taddr + 96)
      : "memory");
#pragma unroll
  for (int d = 0; d < ND; ++d)
#pragma unroll
    for (int j = 0; j < 8; ++j) v[d][j] = __uint_as_float(r[8 * d + j]);
}

// carry the level sums (weights 256^-(d+2)) into balanced digits
// y_0..y_{ND-1} (weights 256^-(k+1)); the remainder of the last level is
// rounded into its neighbour and dropped
__device__ __forceinline__ void carry(float (&acc)[ND], float (&y)[ND]) {
#pragma unroll
  for (int d = ND - 1; d >= 1; --d) {
    const float c = rnd_mul(acc[d], 1.0f / 256.0f);
    acc[d] = __fmaf_rn(c, -256.0f, acc[d]);
    acc[d - 1] = __fadd_rn(acc[d - 1], c);
  }
  const float c0 = rnd_mul(acc[0], 1.0f / 256.0f);
  y[0] = c0;
  y[1] = __fmaf_rn(c0, -256.0f, acc[0]);
#pragma unroll
  for (int k = 2; k < ND; ++k) y[k] = acc[k - 1];
}

// the value of level sums as a float pair scaled by sc: carried into digits,
// an exact head and a rounded tail
__device__ __forceinline__ ffv levels_to_pair(float (&lv)[ND], float sc) {
  float z[ND];
  carry(lv, z);
  const float h = __fmaf_rn(z[1], 1.0f / 65536.0f, __fmul_rn(z[0], 1.0f / 256.0f));
  const float m2 = __fmul_rn(z[2], 1.0f / 16777216.0f);
  const float sh = __fadd_rn(h, m2);
  const float bb = __fsub_rn(sh, h);
  const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(sh, bb)), __fsub_rn(m2, bb));
  float tail = 0.f;
#pragma unroll
  for (int k = ND - 1; k >= 3; --k) tail = __fmaf_rn(tail, 1.0f / 256.0f, z[k]);
  tail = __fmul_rn(tail, 1.0f / 4294967296.0f);  // z_3 weight 2^-32
  return {__fmul_rn(sh, sc), __fmul_rn(__fadd_rn(e, tail), sc)};
}

// the 6 balanced digits of 8 float-pair values against |X| < 2^E, packed in
// bf16 pairs: pk[k][j/2] holds elements j, j+1 of digit plane k
__device__ __forceinline__ void digits_of(const ffv (&x)[8], int E, uint32_t (&pk)[NDX][4]) {
  const float s = exp2i(24 - E);
#pragma unroll
  for (int jj = 0; jj < 8; jj += 2) {
    float dg[NDX][2];
#pragma unroll
    for (int w = 0; w < 2; ++w) {
      const int j = jj + w;
      const float h = __fmul_rn(x[j].hi, s);
      const float d0 = rnd_mul(h, 1.0f / 65536.0f);
      const float t1 = __fmaf_rn(d0, -65536.0f, h);
      const float d1 = rnd_mul(t1, 1.0f / 256.0f);
      const float t2 = __fmaf_rn(d1, -256.0f, t1);
      const float d2 = rnd(t2);
      float r = __fmaf_rn(x[j].lo, s, __fsub_rn(t2, d2));
      const float d3 = rnd_mul(r, 256.0f);
      r = __fmaf_rn(r, 256.0f, -d3);
      const float d4 = rnd_mul(r, 256.0f);
      r = __fmaf_rn(r, 256.0f, -d4);
      dg[0][w] = d0;
      dg[1][w] = d1;
      dg[2][w] = d2;
      dg[3][w] = d3;
      dg[4][w] = d4;
      dg[5][w] = rnd_mul(r, 256.0f);
    }
#pragma unroll
    for (int k = 0; k < NDX; ++k) pk[k][jj / 2] = pack_bf16(dg[k][0], dg[k][1]);
  }
}

// tile exponent from the biased float exponent of the largest high word:
// |X| < 2^E; tiles below 2^-100 keep fewer digits (their contribution is
// negligible)
__device__ __forceinline__ int tile_exponent(unsigned eb) { return max((int)max(eb, 1u) - 126, -100); }

// exact float -> double through the bit pattern (no FP64-pipe conversion);
// zero and subnormal floats map to zero
__device__ __forceinline__ double f2d_bits(float f) {
  const uint32_t bits = __float_as_uint(f);
  const uint32_t e = (bits >> 23) & 0xFFu;
  if (e == 0) return 0.0;
  const unsigned long long r = ((unsigned long long)(bits >> 31) << 63) | ((unsigned long long)(e + 896u) << 52) |
                               ((unsigned long long)(bits & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)r);
}
__device__ __forceinline__ double pair_to_d(ffv a) {
  const ffv n = ff_norm(a.hi, a.lo);
  return f2d_bits(n.hi) + f2d_bits(n.lo);
}

// recoupled density tile of (slot = warp, entry ent) for this lane's 8
// elements (rows p = 8 ph + j, column q), float pairs; the loads of two
// terms are in flight together
__device__ __forceinline__ void recouple(const DevAtom& A, const unsigned char* act, int ent, const float2* base,
                                         const bool (&vp)[8], ffv (&x)[8]) {
#pragma unroll
  for (int j = 0; j < 8; ++j) x[j] = {0.f, 0.f};
  const int u1 = A.kent_ptr[ent + 1];
  for (int uu = A.kent_ptr[ent]; uu < u1; uu += 2) {
    float2 c[2], pv[2][8];
#pragma unroll
    for (int w = 0; w < 2; ++w) {
      const bool on = uu + w < u1 && act[A.kterm_blk[uu + w]];
      c[w] = on ? A.kterm_coef2[uu + w] : make_float2(0.f, 0.f);
      const float2* pb = base + (on ? A.kterm_off[uu + w] : 0);
#pragma unroll
      for (int j = 0; j < 8; ++j) pv[w][j] = (on && vp[j]) ? pb[j] : make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int w = 0; w < 2; ++w)
#pragma unroll
      for (int j = 0; j < 8; ++j) x[j] = ff_fma(x[j], c[w], pv[w][j]);
  }
}

// digits of the recoupled tile written as rows (slot, q), K = p of the first
// product's operand; returns the tile exponent (warp-wide maximum)
__device__ __forceinline__ int digitise(ffv (&x)[8], unsigned char* A1, int row, int k0) {
  unsigned eb = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    x[j] = ff_norm(x[j].hi, x[j].lo);
    eb = max(eb, (__float_as_uint(x[j].hi) >> 23) & 0xFFu);
  }
  const int E = tile_exponent(__reduce_max_sync(0xffffffffu, eb));
  uint32_t pk[NDX][4];
  digits_of(x, E, pk);
  const uint32_t off = tc::off_kmajor(row, k0);
#pragma unroll
  for (int k = 0; k < NDX; ++k)
    *reinterpret_cast<uint4*>(A1 + k * APLANE + off) = make_uint4(pk[k][0], pk[k][1], pk[k][2], pk[k][3]);
  return E;
}

// the 8 values y[j] of tile (a,b), block jk, at row p and columns q0 + j:
// one pass over the columns with the block's base address computed once;
// owned entries go to K, the shared last row / column to the halo buffer
__device__ __forceinline__ void store_rows(const DevAtom& A, const DevScratch& S, double* K, int a, int b, int jk,
                                           int p, int q0, const double (&y)[8]) {
  const int nn = A.nn;
  const int gp = gfun(A, a, p);
  if (p >= nn || gp < 0 || gp >= A.nrad) return;
  const int j = jk % A.nang, k = jk / A.nang;
  double* base = K + (size_t)k * A.nrad * A.nbf + (size_t)j * A.nrad + gp;
  double* halo = S.khalo + ((size_t)(a * A.nel + b) * (A.nang * A.nang) + jk) * (2 * nn - 1);
#pragma unroll
  for (int jj = 0; jj < 8; ++jj) {
    const int q = q0 + jj, gq = gfun(A, b, q);
    if (q >= nn || gq < 0 || gq >= A.nrad) continue;
    if (p <= nn - 2 && q <= nn - 2)
      base[(size_t)gq * A.nbf] = y[jj];
    else if (p == nn - 1)
      halo[q] = y[jj];
    else
      halo[nn + p] = y[jj];
  }
}

struct Smem {
  unsigned char* A1;  // NDX planes: rows (slot, q), K = p (K-major)
  unsigned char* A2;  // ND planes: rows (slot, i), K = q (MN-major)
  unsigned char* T1;  // NL * ND planes of the left tables of element a
  unsigned char* T2;  // NL * ND planes of the right tables of element b
  int* alpha;         // [NL][16] row exponents of the left tables
  int* beta;          // [NL][16] row exponents of the right tables
  int* ex;            // [2][8] tile exponents, by batch parity
  int* sact;          // [NL][8] slot active in the batch of multipole L
  int* gent;          // [8][NL] entry of (slot, L) or -1
  int* gjk;           // [8] output block of the slot or -1
  unsigned char* act; // [nang^2] density block above the screen
  uint64_t* mbar;
  uint32_t* tslot;
  int* fail;
};

}  // namespace

__global__ void __launch_bounds__(256, 2) k_tiles_tc(DevAtom A, DevScratch S, DevTC T, const int4* __restrict__ units,
                                                     int symmetric, double* __restrict__ K) {
  const int4 u = units[blockIdx.x];
  const int a = u.x, b = u.y;
  const int nn = A.nn, NL = A.NL, nang2 = A.nang * A.nang;
  extern __shared__ __align__(1024) unsigned char smraw[];
  Smem sm;
  {
    unsigned char* p = smraw;
    sm.A1 = p;
    p += NDX * APLANE;
    sm.A2 = p;
    p += ND * APLANE;
    sm.T1 = p;
    p += NL * ND * TPLANE;
    sm.T2 = p;
    p += NL * ND * TPLANE;
    int* ip = reinterpret_cast<int*>(p);
    sm.alpha = ip;
    ip += NL * 16;
    sm.beta = ip;
    ip += NL * 16;
    sm.ex = ip;
    ip += 16;
    sm.sact = ip;
    ip += 8 * NL;
    sm.gent = ip;
    ip += 8 * NL;
    sm.gjk = ip;
    ip += 8;
    sm.fail = ip;
    ip += 2;
    sm.mbar = reinterpret_cast<uint64_t*>(ip);
    sm.tslot = reinterpret_cast<uint32_t*>(sm.mbar + 1);
    sm.act = reinterpret_cast<unsigned char*>(sm.tslot + 2);
  }
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int qw = warp & 3, half = warp >> 2;

  // ---- set-up once per unit: tables of this element pair, block flags ----
  {
    const int kl = (a < b) ? 0 : 1, kr = (a < b) ? 1 : 0;  // left: r_small(a) if a < b
    const uint4* s1 = reinterpret_cast<const uint4*>(T.digits) + (size_t)(kl * NL * A.nel) * (ND * TPLANE / 16);
    const uint4* s2 = reinterpret_cast<const uint4*>(T.digits) + (size_t)(kr * NL * A.nel) * (ND * TPLANE / 16);
    const int per = ND * TPLANE / 16;  // uint4 per (L, e)
    for (int idx = t; idx < NL * per; idx += blockDim.x) {
      const int L = idx / per, o = idx % per;
      reinterpret_cast<uint4*>(sm.T1)[idx] = s1[((size_t)L * A.nel + a) * per + o];
      reinterpret_cast<uint4*>(sm.T2)[idx] = s2[((size_t)L * A.nel + b) * per + o];
    }
    for (int idx = t; idx < NL * 16; idx += blockDim.x) {
      const int L = idx / 16, r = idx % 16;
      sm.alpha[idx] = T.rowexp[((size_t)(kl * NL + L) * A.nel + a) * 16 + r];
      sm.beta[idx] = T.rowexp[((size_t)(kr * NL + L) * A.nel + b) * 16 + r];
    }
    for (int idx = t; idx < nang2; idx += blockDim.x) sm.act[idx] = S.act[idx];
    if (t == 0) sm.fail[0] = 0;
  }
  // operand rows of an idle slot are never cleared: a tensor-core row only
  // feeds the same row of the result, and idle rows are never read back
  if (warp == 0) {
    tc::tmem_alloc(sm.tslot, 256);
    tc::tmem_relinquish();
  }
  if (t == 0) tc::mbar_init(sm.mbar, 1);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = *sm.tslot;
  const uint32_t tD1 = tbase, tD2 = tbase + 128;
  const uint32_t lane_off = (uint32_t)(32 * qw) << 16;
  uint32_t phase = 0;
  const uint64_t dA1 = tc::smem_desc(tc::smem_u32(sm.A1)), dA2 = tc::smem_desc(tc::smem_u32(sm.A2));
  const uint64_t dT1 = tc::smem_desc(tc::smem_u32(sm.T1)), dT2 = tc::smem_desc(tc::smem_u32(sm.T2));

  // this thread's tensor-memory lane (slot, row) and columns [8 half, 8 half + 8)
  const int m_out = 32 * qw + lane;
  const int oslot = m_out >> 4, oi = m_out & 15;
  const int pslot = 2 * qw + ((lane >> 4) ^ 1);  // the other slot of this warp's lanes

  // recoupling layout: warp = slot, lane = (q, p-half)
  const int rq = lane & 15, rph = lane >> 4;
  const int gq = gfun(A, b, rq);
  const bool vq = rq < nn && gq >= 0 && gq < A.nrad;
  const int gp0 = gfun(A, a, 8 * rph);
  bool vp[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int p = 8 * rph + j, gp = gp0 + j;
    vp[j] = vq && p < nn && gp >= 0 && gp < A.nrad;
  }
  const float2* pbase = S.p2 + (size_t)(vq ? gq : 0) * A.nbf + gp0;

  auto next_active = [&](int L0) {
    for (int L = L0; L < NL; ++L) {
      int any = 0;
#pragma unroll
      for (int s = 0; s < 8; ++s) any |= sm.sact[L * 8 + s];
      if (any) return L;
    }
    return -1;
  };

  for (int g = u.z; g < u.w; ++g) {
    // ---- the group's entries and their activity ----
    for (int idx = t; idx < 8 * NL; idx += blockDim.x) {
      const int e = T.group_ent[(size_t)g * 8 * NL + idx];  // idx = slot * NL + L
      sm.gent[idx] = e;
      sm.sact[(idx % NL) * 8 + idx / NL] = (e >= 0 && S.ent_act[e]) ? 1 : 0;
    }
    if (t < 8) sm.gjk[t] = T.group_jk[g * 8 + t];
    __syncthreads();

    ffv acc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] = {0.f, 0.f};

    // prologue: the first active batch's density tiles
    int L = next_active(0);
    int par = 0;
    if (L >= 0 && sm.sact[L * 8 + warp]) {
      ffv x[8];
      recouple(A, sm.act, sm.gent[warp * NL + L], pbase, vp, x);
      const int E = digitise(x, sm.A1, warp * 16 + rq, 8 * rph);
      if (lane == 0) sm.ex[par * 8 + warp] = E;
    }

    while (L >= 0) {
      const int Ln = next_active(L + 1);
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
      if (sm.fail[0]) break;  // read after the barrier: uniform over the CTA
      // ---- first product: D1[(slot,q), 16 level + i] ----
      if (t == 0) {
#pragma unroll 1
        for (int kx = 0; kx < NDX; ++kx)
          tc::mma_bf16(tD1 + 16 * kx, dA1 + (uint64_t)(kx * APLANE >> 4), dT1 + (uint64_t)(L * ND * TPLANE >> 4),
                       tc::idesc_bf16(128, 16 * (ND - kx), 0, 0), kx > 0 ? 1u : 0u);
        tc::mma_commit(sm.mbar);
      }
      // the next batch's recoupling (global loads) overlaps the tensor core
      ffv xn[8];
      const bool nact = Ln >= 0 && sm.sact[Ln * 8 + warp];
      if (nact) recouple(A, sm.act, sm.gent[warp * NL + Ln], pbase, vp, xn);
      if (!__all_sync(0xffffffffu, tc::mbar_wait(sm.mbar, phase)) && lane == 0) atomicExch(sm.fail, 1);
      phase ^= 1u;
      tc::fence_after_sync();

      // ---- levels -> balanced digits of Y = A X, the second product's
      // MN-major operand: rows (slot, i), K = q (lane = (slot, q)) ----
      if (sm.sact[L * 8 + oslot] | sm.sact[L * 8 + pslot]) {
        float v[ND][8];
        tmem_ld_levels(tD1 + lane_off + 8 * half, v);
        uint32_t pk[ND][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          float lv[ND], y[ND];
#pragma unroll
          for (int d = 0; d < ND; ++d) lv[d] = v[d][j];
          carry(lv, y);
#pragma unroll
          for (int k = 0; k < ND; ++k) v[k][j] = y[k];
        }
#pragma unroll
        for (int k = 0; k < ND; ++k)
#pragma unroll
          for (int jj = 0; jj < 4; ++jj) pk[k][jj] = pack_bf16(v[k][2 * jj], v[k][2 * jj + 1]);
        const uint32_t off = tc::off_mnmajor(oslot * 16 + 8 * half, oi);
#pragma unroll
        for (int k = 0; k < ND; ++k)
          *reinterpret_cast<uint4*>(sm.A2 + k * APLANE + off) = make_uint4(pk[k][0], pk[k][1], pk[k][2], pk[k][3]);
      }
      tc::fence_async_smem();
      tc::fence_before_sync();
      __syncthreads();
      tc::fence_after_sync();
      if (sm.fail[0]) break;

      // ---- second product: D2[(slot,i), 16 level + r], issued from another
      // warp than the first product so that the issue cost is shared ----
      if (t == 128) {
#pragma unroll 1
        for (int ky = 0; ky < ND; ++ky)
          tc::mma_bf16(tD2 + 16 * ky, dA2 + (uint64_t)(ky * APLANE >> 4), dT2 + (uint64_t)(L * ND * TPLANE >> 4),
                       tc::idesc_bf16(128, 16 * (ND - ky), 1, 0), ky > 0 ? 1u : 0u);
        tc::mma_commit(sm.mbar);
      }
      // the next batch's digits go to the first operand (its MMAs are done)
      if (nact) {
        const int E = digitise(xn, sm.A1, warp * 16 + rq, 8 * rph);
        if (lane == 0) sm.ex[(par ^ 1) * 8 + warp] = E;
      }
      if (!__all_sync(0xffffffffu, tc::mbar_wait(sm.mbar, phase)) && lane == 0) atomicExch(sm.fail, 1);
      phase ^= 1u;
      tc::fence_after_sync();

      // ---- levels -> float pairs, scaled, accumulated over the multipoles ----
      if (sm.sact[L * 8 + oslot] | sm.sact[L * 8 + pslot]) {
        float v[ND][8];
        tmem_ld_levels(tD2 + lane_off + 8 * half, v);
        if (sm.sact[L * 8 + oslot]) {
          const int ea = sm.alpha[L * 16 + oi] + sm.ex[par * 8 + oslot];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            float lv[ND];
#pragma unroll
            for (int d = 0; d < ND; ++d) lv[d] = v[d][j];
            acc[j] = ff_add(acc[j], levels_to_pair(lv, exp2i(ea + sm.beta[L * 16 + 8 * half + j])));
          }
        }
      }
      tc::fence_before_sync();
      L = Ln;
      par ^= 1;
    }
    __syncthreads();

    // ---- store: K_jk(a,b) rows p = oi, columns q = 8 half + j; the
    // transposed partner K_kj(b,a) through shared memory ----
    const bool failed = sm.fail[0] != 0;
    const int jk = sm.gjk[oslot];
    double y[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) y[j] = failed ? __longlong_as_double(0x7ff8000000000000ll) : -pair_to_d(acc[j]);
    if (jk >= 0) store_rows(A, S, K, a, b, jk, oi, 8 * half, y);
    if (symmetric) {
      double* stage = reinterpret_cast<double*>(sm.A1);  // 8 x 16 x 16 doubles; every MMA has completed
#pragma unroll
      for (int j = 0; j < 8; ++j) stage[(oslot * 16 + oi) * 16 + 8 * half + j] = y[j];
      __syncthreads();
      if (jk >= 0) {
        // partner row p' = oi, columns q' = 8 half + j
#pragma unroll
        for (int j = 0; j < 8; ++j) y[j] = stage[(oslot * 16 + 8 * half + j) * 16 + oi];
        store_rows(A, S, K, b, a, (jk / A.nang) + (jk % A.nang) * A.nang, oi, 8 * half, y);
      }
    }
    __syncthreads();  // the stage (first operand) and the group tables are reused
    if (failed) break;
  }

  if (sm.fail[0] && t == 0) {
    atomicExch(T.err, 1);
    // the MMAs of the abandoned batch may still be running: give them one
    // more bounded wait before the tensor memory is released
    tc::mbar_wait(sm.mbar, phase ^ 1u);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, 256);
}

// ------------------------------------------------------------------------
// Diagonal element tiles. Per element a, group of up to 16 output blocks
// and row tile of 128 rows t of Tk, one batch per multipole L:
//     D[t, 16 level + slot] = sum_{kt+kx=level} sum_v Tk_kt[t, v] X_kx[slot, v],
// v = p + q nn. Tk's digit planes are streamed through shared memory one K
// step (16 columns v) at a time by bulk asynchronous copies,
// double-buffered; the density digits of all 16 slots are resident. For
// table digit kt the density planes kx = 0..6-kt are consecutive and form
// one operand of N = 16 (7 - kt). The level sums here run over up to nn^2
// products: the leading levels stay exact, and a rounding in the deepest
// ones is below 2^-60 of max|K|.

namespace {
constexpr int DSLOT = 16;  // output blocks per diagonal group
}

__global__ void tc_tk_digits_kernel(const double* __restrict__ tk, int NL, int nel, int n2, int mtiles, int ksteps,
                                    unsigned char* __restrict__ out, int* __restrict__ rowexp) {
  const int mt = blockIdx.x, le = blockIdx.y, m = threadIdx.x;  // le = L * nel + e
  const int t = 128 * mt + m;
  const double* Tm = tk + (size_t)le * n2 * n2;
  int ex = 0;
  if (t < n2) {
    double rs = 0.0;
    for (int v = 0; v < n2; ++v) rs += fabs(Tm[t + (size_t)v * n2]);
    if (rs > 0.0) frexp(rs, &ex);  // rs <= 2^ex
  }
  rowexp[((size_t)le * mtiles + mt) * 128 + m] = ex;
  unsigned char* base = out + ((size_t)le * mtiles + mt) * ksteps * ND * APLANE;
  for (int v = 0; v < 16 * ksteps; ++v) {
    double r = (t < n2 && v < n2) ? ldexp(Tm[t + (size_t)v * n2], -ex) : 0.0;
    unsigned char* plane = base + (size_t)(v >> 4) * ND * APLANE;
    const uint32_t off = tc::off_kmajor(m, v & 15);
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      r *= 256.0;
      const double dg = rint(r);
      r -= dg;
      *reinterpret_cast<__nv_bfloat16*>(plane + k * APLANE + off) = __float2bfloat16_rn((float)dg);
    }
  }
}

__global__ void __launch_bounds__(256, 2) k_diag_tc(DevAtom A, DevScratch S, DevTC T, int symmetric,
                                                    double* __restrict__ K) {
  const int4 u = (symmetric ? T.dunits_sym : T.dunits_all)[blockIdx.x];
  const int a = u.x, g = u.y, mt = u.z;
  const int nn = A.nn, n2 = nn * nn, NL = A.NL, nang2 = A.nang * A.nang;
  const int ksteps = T.dksteps, mtiles = T.dmtiles;
  const int* gjk_all = symmetric ? T.dgroup_jk_sym : T.dgroup_jk_all;
  const int* gent_all = symmetric ? T.dgroup_ent_sym : T.dgroup_ent_all;
  extern __shared__ __align__(1024) unsigned char smraw[];
  unsigned char* Abuf = smraw;                                             // 2 x ND planes of 128 x 16
  unsigned char* Bx = Abuf + 2 * ND * APLANE;                              // ksteps x ND planes of 16 x 16
  int* alpha = reinterpret_cast<int*>(Bx + (size_t)ksteps * ND * TPLANE);  // [128]
  int* exs = alpha + 128;                                                  // [16] slot exponents (float bits)
  int* sact = exs + DSLOT;                                                 // [NL][16]
  int* gent = sact + NL * DSLOT;                                           // [16][NL]
  int* gjk = gent + NL * DSLOT;                                            // [16]
  int* fail = gjk + DSLOT;                                                 // [2]
  uint64_t* mb = reinterpret_cast<uint64_t*>(fail + 2);                    // full[2], empty[2], done
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mb + 5);
  unsigned char* act = reinterpret_cast<unsigned char*>(tslot + 2);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int qw = warp & 3, half = warp >> 2;

  for (int idx = t; idx < DSLOT * NL; idx += blockDim.x) {
    const int e = gent_all[(size_t)g * DSLOT * NL + idx];  // idx = slot * NL + L
    gent[idx] = e;
    sact[(idx % NL) * DSLOT + idx / NL] = (e >= 0 && S.ent_act[e]) ? 1 : 0;
  }
  if (t < DSLOT) gjk[t] = gjk_all[g * DSLOT + t];
  for (int idx = t; idx < nang2; idx += blockDim.x) act[idx] = S.act[idx];
  // the zero seventh density plane of every K step (operands of N = 112)
  for (int idx = t; idx < ksteps * (TPLANE / 16); idx += blockDim.x) {
    const int ks = idx / (TPLANE / 16), o = idx % (TPLANE / 16);
    reinterpret_cast<uint4*>(Bx + ((size_t)ks * ND + NDX) * TPLANE)[o] = make_uint4(0, 0, 0, 0);
  }
  if (t == 0) {
    fail[0] = 0;
    for (int i = 0; i < 5; ++i) tc::mbar_init(&mb[i], 1);
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, 128);
    tc::tmem_relinquish();
  }
  tc::fence_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tD = *tslot;
  const uint32_t lane_off = (uint32_t)(32 * qw) << 16;
  uint32_t nfull[2] = {0, 0}, nempty[2] = {0, 0}, ndone = 0;
  const uint64_t dA = tc::smem_desc(tc::smem_u32(Abuf)), dB = tc::smem_desc(tc::smem_u32(Bx));
  const int row = 32 * qw + lane, trow = 128 * mt + row;  // this thread's tensor-memory lane
  const int nchunk = DSLOT * 2 * ksteps;                  // chunks of 8 consecutive v per slot
  ffv acc[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j] = {0.f, 0.f};

  for (int L = 0; L < NL; ++L) {
    int any = 0;
    for (int s = 0; s < DSLOT; ++s) any |= sact[L * DSLOT + s];
    if (!any) continue;  // uniform: sact is written before the first barrier
    const size_t tslice = ((size_t)L * A.nel + a) * mtiles + mt;
    const unsigned char* Ag = T.tk_digits + tslice * ksteps * ND * APLANE;
    // the producer starts streaming the first two K steps of the table
    if (t == 0) {
      for (int ks = 0; ks < 2 && ks < ksteps; ++ks) {
        tc::mbar_expect_tx(&mb[ks], ND * APLANE);
        tc::bulk_g2s(Abuf + ks * ND * APLANE, Ag + (size_t)ks * ND * APLANE, ND * APLANE, &mb[ks]);
      }
    }
    for (int idx = t; idx < 128; idx += blockDim.x) alpha[idx] = T.tk_rowexp[tslice * 128 + idx];
    if (t < DSLOT) exs[t] = 0;
    __syncthreads();
    // ---- recouple the 16 density vectors and take each slot's exponent ----
    ffv xs[2][8];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int ch = t + c * 256;
#pragma unroll
      for (int j = 0; j < 8; ++j) xs[c][j] = {0.f, 0.f};
      if (ch >= nchunk) continue;
      const int s = ch / (2 * ksteps), v0 = 8 * (ch % (2 * ksteps));
      if (!sact[L * DSLOT + s]) continue;
      const int ent = gent[s * NL + L];
      int eo[8];  // density offsets of the 8 elements (nbf^2 < 2^31), -1: outside the basis
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int v = v0 + j, p = v % nn, q = v / nn;
        const int gp = gfun(A, a, p), gq = gfun(A, a, q);
        eo[j] = (v < n2 && gp >= 0 && gp < A.nrad && gq >= 0 && gq < A.nrad) ? gq * A.nbf + gp : -1;
      }
      // two terms' loads in flight together
      const int u1 = A.kent_ptr[ent + 1];
      for (int uu = A.kent_ptr[ent]; uu < u1; uu += 2) {
        float2 cf[2], pv[2][8];
#pragma unroll
        for (int w = 0; w < 2; ++w) {
          const bool on = uu + w < u1 && act[A.kterm_blk[uu + w]];
          cf[w] = on ? A.kterm_coef2[uu + w] : make_float2(0.f, 0.f);
          const float2* pb = S.p2 + (on ? A.kterm_off[uu + w] : 0);
#pragma unroll
          for (int j = 0; j < 8; ++j) pv[w][j] = (on && eo[j] >= 0) ? pb[eo[j]] : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int w = 0; w < 2; ++w)
#pragma unroll
          for (int j = 0; j < 8; ++j) xs[c][j] = ff_fma(xs[c][j], cf[w], pv[w][j]);
      }
      unsigned eb = 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        xs[c][j] = ff_norm(xs[c][j].hi, xs[c][j].lo);
        eb = max(eb, (__float_as_uint(xs[c][j].hi) >> 23) & 0xFFu);
      }
      atomicMax(&exs[s], (int)eb);
    }
    __syncthreads();
    // ---- digits: B[ks][kx][row slot, k = v mod 16] ----
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int ch = t + c * 256;
      if (ch >= nchunk) continue;
      const int s = ch / (2 * ksteps), kk = ch % (2 * ksteps), ks = kk >> 1, h = kk & 1;
      uint32_t pk[NDX][4];
      digits_of(xs[c], tile_exponent((unsigned)exs[s]), pk);
      const uint32_t off = tc::off_kmajor(s, 8 * h);
#pragma unroll
      for (int k = 0; k < NDX; ++k)
        *reinterpret_cast<uint4*>(Bx + ((size_t)ks * ND + k) * TPLANE + off) =
            make_uint4(pk[k][0], pk[k][1], pk[k][2], pk[k][3]);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();

    // ---- the K loop (one thread): MMAs of step ks from buffer ks & 1; the
    // buffer is refilled with step ks + 2 once those MMAs have finished ----
    if (t == 0) {
      bool ok = true;
      for (int ks = 0; ks < ksteps && ok; ++ks) {
        const int bf = ks & 1;
        ok = tc::mbar_wait(&mb[bf], nfull[bf] & 1u);
        ++nfull[bf];
        if (!ok) break;
        tc::fence_after_sync();
#pragma unroll 1
        for (int kt = 0; kt < ND; ++kt)
          tc::mma_bf16(tD + 16 * kt, dA + (uint64_t)((bf * ND + kt) * APLANE >> 4),
                       dB + (uint64_t)((size_t)ks * ND * TPLANE >> 4), tc::idesc_bf16(128, 16 * (ND - kt), 0, 0),
                       (ks > 0 || kt > 0) ? 1u : 0u);
        tc::mma_commit(&mb[2 + bf]);
        if (ks + 2 < ksteps) {
          ok = tc::mbar_wait(&mb[2 + bf], nempty[bf] & 1u);
          ++nempty[bf];
          if (!ok) break;
          tc::mbar_expect_tx(&mb[bf], ND * APLANE);
          tc::bulk_g2s(Abuf + bf * ND * APLANE, Ag + (size_t)(ks + 2) * ND * APLANE, ND * APLANE, &mb[bf]);
        } else {
          ++nempty[bf];  // that phase completes without a wait
        }
      }
      tc::mma_commit(&mb[4]);
      if (!ok) atomicExch(fail, 1);
    }
    if (!__all_sync(0xffffffffu, tc::mbar_wait(&mb[4], ndone & 1u)) && lane == 0) atomicExch(fail, 1);
    ++ndone;
    tc::fence_after_sync();
    __syncthreads();
    if (fail[0]) break;

    // ---- levels -> float pairs, scaled by 2^(alpha_t + E_slot), accumulated
    // over the multipoles; columns [8 half, 8 half + 8) = slots ----
    {
      float v[ND][8];
      tmem_ld_levels(tD + lane_off + 8 * half, v);
      const int ea = alpha[row];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int s = 8 * half + j;
        if (!sact[L * DSLOT + s]) continue;
        float lv[ND];
#pragma unroll
        for (int d = 0; d < ND; ++d) lv[d] = v[d][j];
        acc[j] = ff_add(acc[j], levels_to_pair(lv, exp2i(ea + tile_exponent((unsigned)exs[s]))));
      }
    }
    tc::fence_before_sync();
    __syncthreads();
  }

  // ---- store K_jk(a,a)[p, q], t = p + q nn; with a symmetric density also
  // the transposed partner K_kj(a,a)[q, p] (j != k) ----
  const bool failed = fail[0] != 0;
  if (trow < n2) {
    const int p = trow % nn, q = trow / nn;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int jk = gjk[8 * half + j];
      if (jk < 0) continue;
      const double y = failed ? __longlong_as_double(0x7ff8000000000000ll) : -pair_to_d(acc[j]);
      k_store_tile(A, S, K, a, a, jk, p, q, y);
      const int j0 = jk % A.nang, k0 = jk / A.nang;
      if (symmetric && j0 != k0) k_store_tile(A, S, K, a, a, k0 + j0 * A.nang, q, p, y);
    }
  }
  if (failed && t == 0) {
    atomicExch(T.err, 1);
    tc::mbar_wait(&mb[4], ndone & 1u);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tD, 128);
}

size_t tc_smem_bytes(int NL, int nang) {
  return (size_t)(NDX + ND) * APLANE + (size_t)2 * NL * ND * TPLANE +
         sizeof(int) * (2 * NL * 16 + 16 + 8 * NL + 8 * NL + 8 + 2) + 16 + (size_t)nang * nang + 64;
}

size_t tc_diag_smem_bytes(int NL, int ksteps, int nang) {
  return (size_t)2 * ND * APLANE + (size_t)ksteps * ND * TPLANE +
         sizeof(int) * (128 + DSLOT + NL * DSLOT * 2 + DSLOT + 2) + 5 * 8 + 8 + (size_t)nang * nang + 64;
}

cudaError_t launch_k_tiles_tc(const DevAtom& A, const DevScratch& S, const DevTC& T, bool symmetric, double* K,
                              cudaStream_t st) {
  const int n = symmetric ? T.n_sym : T.n_all;
  if (n == 0) return cudaSuccess;
  const size_t smem = tc_smem_bytes(A.NL, A.nang);
  const cudaError_t e = smem_limit(k_tiles_tc, smem);
  if (e != cudaSuccess) return e;
  k_tiles_tc<<<n, 256, smem, st>>>(A, S, T, symmetric ? T.units_sym : T.units_all, symmetric ? 1 : 0, K);
  return cudaGetLastError();
}

cudaError_t launch_tk_digits(const DevAtom& A, int mtiles, int ksteps, unsigned char* out, int* rowexp,
                             cudaStream_t st) {
  const int n2 = A.nn * A.nn;
  cudaError_t e = cudaMemsetAsync(out, 0, (size_t)A.NL * A.nel * mtiles * ksteps * ND * APLANE, st);
  if (e != cudaSuccess) return e;
  tc_tk_digits_kernel<<<dim3(mtiles, A.NL * A.nel), 128, 0, st>>>(A.tk, A.NL, A.nel, n2, mtiles, ksteps, out, rowexp);
  return cudaGetLastError();
}

cudaError_t launch_k_diag_tc(const DevAtom& A, const DevScratch& S, const DevTC& T, bool symmetric, double* K,
                             cudaStream_t st) {
  const int n = symmetric ? T.n_dsym : T.n_dall;
  if (n == 0) return cudaSuccess;
  const size_t smem = tc_diag_smem_bytes(A.NL, T.dksteps, A.nang);
  const cudaError_t e = smem_limit(k_diag_tc, smem);
  if (e != cudaSuccess) return e;
  k_diag_tc<<<n, 256, smem, st>>>(A, S, T, symmetric ? 1 : 0, K);
  return cudaGetLastError();
}

}  // namespace hfg

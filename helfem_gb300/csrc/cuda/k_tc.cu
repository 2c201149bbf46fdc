// Split-precision exchange on the tensor cores: the off-diagonal element-pair
// tiles of TwoDBasisT::exchange (src/atomic/TwoDBasis.cpp:879-999) with the
// FE assembly of assemble_K_FE_one_multipole_cached_chol
// (libhelfemqc/include/CoulombExchangeFE.h:484-530),
//     K_jk(a,b) -= sum_L  A_L(a) X_jkL(a,b) B_L(b)^T,
// A/B = r_small/r_big by element order, X the recoupled density tile.
//
// Arithmetic (an Ozaki-style slicing with exact integer sums):
//  * every operand is a fixed-point number below 1 written as balanced
//    base-256 digits: x = sum_k d_k 256^-(k+1), |d_0| <= 256, |d_k| <= 128
//    (k >= 1, the 4th digit of a density tile may reach 256); digits are
//    integers, exact in bf16;
//  * the radial tables are digitised once per atom with one power-of-two
//    scale per row (row sum of |values| <= 1 after scaling); a density tile
//    X (recoupled on the CUDA cores in float pairs) gets one scale per tile;
//  * the tensor core forms the digit products level by level,
//    acc_d = sum_{k+l=d} sum_p a_k b_l (d = 0..6), in FP32 in tensor memory;
//    every acc_d is an integer of magnitude < 2^23, so the FP32 sums are
//    exact;
//  * the levels are carried into balanced digits again on the CUDA cores:
//    the first product (Y = A X, 128 rows = 8 output blocks x 16) becomes the
//    digit operand of the second (Y B^T), whose levels are turned into a
//    float pair, scaled, and accumulated over the multipoles of the output
//    block; one FP64 conversion per output element at the end.
// Truncation (levels above 6 dropped, 48-bit density tiles) leaves ~1e-14 of
// max|K| against the FP64 result.
//
// Work unit = one element pair (a,b) and a group of up to 8 output angular
// blocks; per multipole L the group's entries with that L form one batch of
// M = 128 rows. 256 threads: 8 warps recouple one block each; warps w and
// w+4 read the same tensor-memory lanes and split the columns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>

#include "devatom.cuh"
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

// 8 consecutive tensor-memory columns of this warp's 32 lanes
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
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

struct Smem {
  unsigned char* A1;  // NDX planes: rows (slot, q), K = p (K-major)
  unsigned char* A2;  // ND planes: rows (slot, i), K = q (MN-major)
  unsigned char* T1;  // NL * ND planes of the left tables of element a
  unsigned char* T2;  // NL * ND planes of the right tables of element b
  int* alpha;         // [NL][16] row exponents of the left tables
  int* beta;          // [NL][16] row exponents of the right tables
  int* ex;            // [8] tile exponent of the current batch
  int* sact;          // [8] slot active in the current batch
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
  const int a = u.x, b = u.y, g = u.z;
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
    ip += 8;
    sm.sact = ip;
    ip += 8;
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

  // ---- set-up: tables of this pair, group entries, density-block flags ----
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
    for (int idx = t; idx < 8 * NL; idx += blockDim.x) sm.gent[idx] = T.group_ent[(size_t)g * 8 * NL + idx];
    if (t < 8) sm.gjk[t] = T.group_jk[g * 8 + t];
    for (int idx = t; idx < nang2; idx += blockDim.x) sm.act[idx] = S.act[idx];
    // zero operand planes: rows of an idle slot then hold finite digits
    for (int idx = t; idx < (NDX + ND) * APLANE / 16; idx += blockDim.x)
      reinterpret_cast<uint4*>(sm.A1)[idx] = make_uint4(0, 0, 0, 0);
    if (t == 0) sm.fail[0] = 0;
  }
  tc::fence_async_smem();
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

  // accumulators of this thread's output row (slot, i) and columns r in
  // [8 half, 8 half + 8) of the second product's tensor-memory lanes
  const int m_out = 32 * qw + lane;  // (slot, i)
  const int oslot = m_out >> 4, oi = m_out & 15;
  ffv acc[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) acc[j] = {0.f, 0.f};

  // recoupling thread layout: warp = slot, lane = (q, p-half)
  const int rq = lane & 15, rph = lane >> 4;
  const int gq = gfun(A, b, rq);
  const bool vq = rq < nn && gq >= 0 && gq < A.nrad;
  int gp0 = gfun(A, a, 8 * rph);
  bool vp[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int p = 8 * rph + j, gp = gp0 + j;
    vp[j] = vq && p < nn && gp >= 0 && gp < A.nrad;
  }

  for (int L = 0; L < NL; ++L) {
    // ---- recouple the density tile of (slot = warp, L) and digitise it ----
    const int ent = sm.gent[warp * NL + L];
    const bool active = ent >= 0 && S.ent_act[ent];
    {
      if (active) {
        ffv x[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = {0.f, 0.f};
        const float2* base = S.p2 + (size_t)(vq ? gq : 0) * A.nbf + gp0;
        for (int uu = A.kent_ptr[ent]; uu < A.kent_ptr[ent + 1]; ++uu) {
          if (!sm.act[A.kterm_blk[uu]]) continue;
          const float2 c = A.kterm_coef2[uu];
          const float2* pb = base + A.kterm_off[uu];
#pragma unroll
          for (int j = 0; j < 8; ++j)
            if (vp[j]) x[j] = ff_fma(x[j], c, pb[j]);
        }
        // tile exponent: |X| < 2^E
        unsigned eb = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          x[j] = ff_norm(x[j].hi, x[j].lo);
          eb = max(eb, (__float_as_uint(x[j].hi) >> 23) & 0xFFu);
        }
        eb = __reduce_max_sync(0xffffffffu, eb);
        int E = (int)max(eb, 1u) - 126;
        E = max(E, -100);  // tiles below 2^-100 keep fewer digits (their contribution is negligible)
        const float s = exp2i(24 - E);
        float dg[NDX][8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
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
          const float d5 = rnd_mul(r, 256.0f);
          dg[0][j] = d0;
          dg[1][j] = d1;
          dg[2][j] = d2;
          dg[3][j] = d3;
          dg[4][j] = d4;
          dg[5][j] = d5;
        }
        const uint32_t off = tc::off_kmajor(warp * 16 + rq, 8 * rph);
#pragma unroll
        for (int k = 0; k < NDX; ++k) {
          const uint4 v = make_uint4(pack_bf16(dg[k][0], dg[k][1]), pack_bf16(dg[k][2], dg[k][3]),
                                     pack_bf16(dg[k][4], dg[k][5]), pack_bf16(dg[k][6], dg[k][7]));
          *reinterpret_cast<uint4*>(sm.A1 + k * APLANE + off) = v;
        }
        if (lane == 0) sm.ex[warp] = E;
      }
      if (lane == 0) sm.sact[warp] = active ? 1 : 0;
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    // barrier and block-wide "any slot active" in one (uniform over the CTA)
    const int any = __syncthreads_or(active ? 1 : 0);
    tc::fence_after_sync();
    if (!any) continue;

    // ---- first product: D1[(slot,q), (level, i)] = sum X_k^T A_l ----
    if (t == 0) {
      const uint32_t id1 = tc::idesc_bf16(128, 16, 0, 0);
#pragma unroll 1
      for (int d = 0; d < ND; ++d) {
        bool first = true;
        for (int kx = 0; kx < NDX && kx <= d; ++kx) {
          const int kt = d - kx;
          if (kt >= ND) continue;
          const uint64_t ad = tc::smem_desc(tc::smem_u32(sm.A1 + kx * APLANE));
          const uint64_t bd = tc::smem_desc(tc::smem_u32(sm.T1 + (L * ND + kt) * TPLANE));
          tc::mma_bf16(tD1 + 16 * d, ad, bd, id1, first ? 0u : 1u);
          first = false;
        }
      }
      tc::mma_commit(sm.mbar);
    }
    if (!__all_sync(0xffffffffu, tc::mbar_wait(sm.mbar, phase))) {
      if (lane == 0) atomicExch(sm.fail, 1);
    }
    phase ^= 1u;
    tc::fence_after_sync();
    __syncthreads();
    if (sm.fail[0]) break;

    // ---- levels -> balanced digits of Y, written as the second product's
    // MN-major operand: rows (slot, i), K = q ----
    {
      float v[ND][8];
#pragma unroll
      for (int d = 0; d < ND; ++d) tmem_ld8(tD1 + lane_off + 16 * d + 8 * half, v[d]);
      float y[ND][8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        float lv[ND], yy[ND];
#pragma unroll
        for (int d = 0; d < ND; ++d) lv[d] = v[d][j];
        carry(lv, yy);
#pragma unroll
        for (int k = 0; k < ND; ++k) y[k][j] = yy[k];
      }
      const int slot = m_out >> 4, q = m_out & 15;  // D1 lane = (slot, q)
      const uint32_t off = tc::off_mnmajor(slot * 16 + 8 * half, q);
#pragma unroll
      for (int k = 0; k < ND; ++k) {
        const uint4 w4 = make_uint4(pack_bf16(y[k][0], y[k][1]), pack_bf16(y[k][2], y[k][3]),
                                    pack_bf16(y[k][4], y[k][5]), pack_bf16(y[k][6], y[k][7]));
        *reinterpret_cast<uint4*>(sm.A2 + k * APLANE + off) = w4;
      }
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();

    // ---- second product: D2[(slot,i), (level, r)] = sum Y_k B_l^T ----
    if (t == 0) {
      const uint32_t id2 = tc::idesc_bf16(128, 16, 1, 0);
#pragma unroll 1
      for (int d = 0; d < ND; ++d) {
        bool first = true;
        for (int ky = 0; ky <= d; ++ky) {
          const int kt = d - ky;
          const uint64_t ad = tc::smem_desc(tc::smem_u32(sm.A2 + ky * APLANE));
          const uint64_t bd = tc::smem_desc(tc::smem_u32(sm.T2 + (L * ND + kt) * TPLANE));
          tc::mma_bf16(tD2 + 16 * d, ad, bd, id2, first ? 0u : 1u);
          first = false;
        }
      }
      tc::mma_commit(sm.mbar);
    }
    if (!__all_sync(0xffffffffu, tc::mbar_wait(sm.mbar, phase))) {
      if (lane == 0) atomicExch(sm.fail, 1);
    }
    phase ^= 1u;
    tc::fence_after_sync();
    __syncthreads();
    if (sm.fail[0]) break;

    // ---- levels -> float pairs, scaled, accumulated over the multipoles ----
    {
      float v[ND][8];
#pragma unroll
      for (int d = 0; d < ND; ++d) tmem_ld8(tD2 + lane_off + 16 * d + 8 * half, v[d]);
      if (sm.sact[oslot]) {
        const int ea = sm.alpha[L * 16 + oi] + sm.ex[oslot];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          float lv[ND], z[ND];
#pragma unroll
          for (int d = 0; d < ND; ++d) lv[d] = v[d][j];
          carry(lv, z);
          // value = sum_k z_k 256^-(k+1): exact head, rounded tail
          const float h = __fmaf_rn(z[1], 1.0f / 65536.0f, __fmul_rn(z[0], 1.0f / 256.0f));
          const float m2 = __fmul_rn(z[2], 1.0f / 16777216.0f);
          const float sh = __fadd_rn(h, m2);
          const float bb = __fsub_rn(sh, h);
          const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(sh, bb)), __fsub_rn(m2, bb));
          float tail = 0.f;
#pragma unroll
          for (int k = ND - 1; k >= 3; --k) tail = __fmaf_rn(tail, 1.0f / 256.0f, z[k]);
          tail = __fmul_rn(tail, 1.0f / 4294967296.0f);  // z_3 weight 2^-32
          const float sc = exp2i(ea + sm.beta[L * 16 + 8 * half + j]);
          const ffv val = {__fmul_rn(sh, sc), __fmul_rn(__fadd_rn(e, tail), sc)};
          acc[j] = ff_add(acc[j], val);
        }
      }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
  }

  // ---- store: K_jk(a,b) rows p = oi, columns q = 8 half + j; the transposed
  // partner K_kj(b,a) through shared memory ----
  const bool failed = sm.fail[0] != 0;
  const int jk = sm.gjk[oslot];
  if (jk >= 0) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const double y = failed ? __longlong_as_double(0x7ff8000000000000ll) : -ff_to_d(acc[j]);
      k_store_tile(A, S, K, a, b, jk, oi, 8 * half + j, y);
    }
  }
  if (symmetric) {
    double* stage = reinterpret_cast<double*>(sm.A1);  // 8 x 16 x 16 doubles, the first product is done
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 8; ++j)
      stage[(oslot * 16 + oi) * 16 + 8 * half + j] =
          failed ? __longlong_as_double(0x7ff8000000000000ll) : -ff_to_d(acc[j]);
    __syncthreads();
    if (jk >= 0) {
      const int j0 = jk % A.nang, k0 = jk / A.nang;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int qq = 8 * half + j;  // partner row p' = oi, column q' = qq
        k_store_tile(A, S, K, b, a, k0 + j0 * A.nang, oi, qq, stage[(oslot * 16 + qq) * 16 + oi]);
      }
    }
  }
  if (failed && t == 0) {
    atomicExch(T.err, 1);
    // the MMAs of the abandoned batch may still be running: give them one
    // more bounded wait before the tensor memory is released
    tc::mbar_wait(sm.mbar, phase ^ 1u);
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, 256);
}

size_t tc_smem_bytes(int NL, int nang) {
  return (size_t)(NDX + ND) * APLANE + (size_t)2 * NL * ND * TPLANE +
         sizeof(int) * (2 * NL * 16 + 8 + 8 + 8 * NL + 8 + 2) + 16 + (size_t)nang * nang + 64;
}

cudaError_t launch_k_tiles_tc(const DevAtom& A, const DevScratch& S, const DevTC& T, bool symmetric, double* K,
                              cudaStream_t st) {
  const int n = symmetric ? T.n_sym : T.n_all;
  if (n == 0) return cudaSuccess;
  const size_t smem = tc_smem_bytes(A.NL, A.nang);
  static thread_local size_t configured = 0;  // per-thread: the attribute is per device function
  if (smem > configured) {
    const cudaError_t e = cudaFuncSetAttribute(k_tiles_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = smem;
  }
  k_tiles_tc<<<n, 256, smem, st>>>(A, S, T, symmetric ? T.units_sym : T.units_all, symmetric ? 1 : 0, K);
  return cudaGetLastError();
}

}  // namespace hfg

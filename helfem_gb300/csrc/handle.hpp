// The atom handle behind the C ABI and the helpers every entry point shares
// (status/error plumbing, RAII device buffers). Internal to the library.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <algorithm>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "helfem_gb300.h"
#include "cuda/devatom.cuh"
#include "cuda/tab.cuh"
#include "host/atom.hpp"

namespace hfg_abi {

extern thread_local std::string g_err;

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

inline void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess)
    throw CudaError(std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

inline void need(bool c, const char* msg) {
  if (!c) throw std::invalid_argument(msg);
}

template <class F>
hfg_status guard(F&& f) {
  try {
    f();
    g_err.clear();
    return HFG_OK;
  } catch (const std::invalid_argument& e) {
    g_err = e.what();
    return HFG_ERR_ARG;
  } catch (const CudaError& e) {
    g_err = e.what();
    return HFG_ERR_CUDA;
  } catch (const std::bad_alloc&) {
    g_err = "host allocation failed";
    return HFG_ERR_NOMEM;
  } catch (const std::logic_error& e) {
    g_err = e.what();
    return HFG_ERR_STATE;
  } catch (const std::exception& e) {
    g_err = e.what();
    return HFG_ERR_INTERNAL;
  } catch (...) {
    g_err = "unknown error";
    return HFG_ERR_INTERNAL;
  }
}

// Stream-ordered allocation: while an AllocStream guard is alive on a
// thread, device buffers created on that thread are allocated with
// cudaMallocAsync on its stream and later freed with cudaFreeAsync on the
// same stream, from the device's default pool with its release threshold
// raised so freed memory stays cached. Concurrent solves on different
// streams then never pay the device-wide synchronisation of
// cudaMalloc/cudaFree.
extern thread_local cudaStream_t t_alloc_stream;
void retain_pool_memory();  // once per device

struct AllocStream {
  cudaStream_t prev;
  explicit AllocStream(cudaStream_t s) : prev(t_alloc_stream) {
    retain_pool_memory();
    t_alloc_stream = s;
  }
  ~AllocStream() { t_alloc_stream = prev; }
};

// RAII device allocation
struct DBuf {
  void* p = nullptr;
  size_t n = 0;
  cudaStream_t st = nullptr;  // stream of a stream-ordered allocation
  bool async = false;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), st(o.st), async(o.async) { o.p = nullptr; o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p; n = o.n; st = o.st; async = o.async;
      o.p = nullptr; o.n = 0;
    }
    return *this;
  }
  ~DBuf() { release(); }
  void release() {
    if (!p) return;
    if (async) cudaFreeAsync(p, st); else cudaFree(p);
    p = nullptr;
  }
  void alloc(size_t bytes) {
    release();
    n = bytes;
    if (bytes == 0) return;
    st = t_alloc_stream;
    async = st != nullptr;
    cudaError_t e = async ? cudaMallocAsync(&p, bytes, st) : cudaMalloc(&p, bytes);
    if (e == cudaErrorMemoryAllocation) { p = nullptr; throw std::bad_alloc(); }
    ck(e, "device allocation");
  }
  // copies from pageable host memory: the call returns once the source has
  // been staged, so the host vector may be released right after
  template <class T>
  T* upload(const std::vector<T>& v) {
    alloc(std::max<size_t>(1, v.size()) * sizeof(T));
    if (!v.empty())
      ck(async ? cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st)
               : cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice),
         "upload");
    return static_cast<T*>(p);
  }
  template <class T>
  T* as() const { return static_cast<T*>(p); }
};

// owns a stream; declared first in a struct so it outlives the buffers that
// free on it
struct StreamHolder {
  cudaStream_t s = nullptr;
  ~StreamHolder() { if (s) cudaStreamDestroy(s); }
};

}  // namespace hfg_abi

using hfg_abi::DBuf;
using hfg_abi::ck;
using hfg_abi::need;
using hfg_abi::guard;

struct hfg_atom {
  hfg_abi::StreamHolder stream_holder;  // destroyed last
  hfg::AtomHost host;
  int device = 0;
  bool on_device = false;
  cudaStream_t own_stream = nullptr;
  hfg::DevAtom dev{};
  hfg::DevScratch scr{};
  // device copies of the tables
  DBuf d_rs, d_rb, d_cholp, d_rank, d_tk, d_chanL, d_jket_ptr, d_jket_blk, d_jket_coef, d_jbra_ptr,
      d_jbra_chan, d_jbra_coef, d_kjk_ptr, d_kent_L, d_kent_ptr, d_kterm_blk, d_kterm_off, d_kterm_coef;
  DBuf s_jin, s_jscal, s_khalo, s_bnorm, s_p2, s_act, s_entact;
  DBuf d_rs2, d_rb2, d_tk2, d_kcoef2, d_jkc2, d_jbc2, d_cholp2;
  DBuf d_units_all, d_units_sym, d_diag_all, d_diag_sym;
  hfg::KUnits units;
  // tensor-core split exchange: digit tables of the bare and of the
  // Yukawa-screened radial tables, shared groups and units, error flag
  DBuf t_dig, t_exp, ty_dig, ty_exp, t_gjk, t_gent, t_usym, t_uall, t_err;
  DBuf t_tkd, t_tke, ty_tkd, ty_tke, t_dgjk_s, t_dgent_s, t_dgjk_a, t_dgent_a, t_dus, t_dua;
  hfg::DevTC tc{}, tc_rs{};
  bool tc_ok = false;
  // bf16 MMA FLOPs one tensor-core exchange issues with every entry active
  // (index 0: symmetric mode, 1: general)
  double tc_mma_flops[2] = {0.0, 0.0};
  // the split exchange on the tensor cores (off-diagonal element pairs), or
  // nullptr for the float-pair form everywhere (HFG_SPLIT_FORM=pairs)
  const hfg::DevTC* tc_for(bool screened) const {
    if (!tc_ok) return nullptr;
    static const bool pairs = [] {
      const char* v = std::getenv("HFG_SPLIT_FORM");
      return v && std::string(v) == "pairs";
    }();
    if (pairs) return nullptr;
    return screened ? (tc_rs.digits ? &tc_rs : nullptr) : &tc;
  }
  // digits of the radial tables (kind 0 r_small, 1 r_big; per (L, e) a
  // 16 x 16 plane per digit, element (row n, column k) = table(n, k)) and the
  // row exponents; see k_tc.cu for the arithmetic
  void tc_tables(const std::vector<double>& rs, const std::vector<double>& rb, DBuf& dig, DBuf& rexp,
                 hfg::DevTC& out) {
    const hfg::AtomHost& H = host;
    const int nn = H.rad.nn, nel = H.rad.nel, NL = H.NL, ND = TC_NDIGITS;
    const size_t n2 = (size_t)nn * nn;
    std::vector<uint16_t> d((size_t)2 * NL * nel * ND * (TC_TPLANE / 2), 0);
    std::vector<int> ex((size_t)2 * NL * nel * 16, 0);
    auto off = [](int n, int k) { return ((n >> 3) * 256 + (k >> 3) * 128 + (n & 7) * 16 + (k & 7) * 2) / 2; };
    for (int kind = 0; kind < 2; ++kind)
      for (int L = 0; L < NL; ++L)
        for (int e = 0; e < nel; ++e) {
          const double* M = (kind == 0 ? rs : rb).data() + ((size_t)L * nel + e) * n2;
          const size_t blk = ((size_t)kind * NL + L) * nel + e;
          uint16_t* planes = d.data() + blk * ND * (TC_TPLANE / 2);
          for (int n = 0; n < nn; ++n) {
            double rowsum = 0.0;
            for (int k = 0; k < nn; ++k) rowsum += std::fabs(M[n + (size_t)k * nn]);
            int a = 0;
            if (rowsum > 0.0) std::frexp(rowsum, &a);  // rowsum <= 2^a
            ex[blk * 16 + n] = a;
            for (int k = 0; k < nn; ++k) {
              double r = std::ldexp(M[n + (size_t)k * nn], -a);
              for (int kd = 0; kd < ND; ++kd) {
                r *= 256.0;
                const double dg = std::nearbyint(r);
                r -= dg;
                const float f = (float)dg;  // integer |dg| <= 256: exact in bf16
                uint32_t bits;
                std::memcpy(&bits, &f, 4);
                planes[(size_t)kd * (TC_TPLANE / 2) + off(n, k)] = (uint16_t)(bits >> 16);
              }
            }
          }
        }
    out.digits = reinterpret_cast<const unsigned char*>(dig.upload(d));
    out.rowexp = rexp.upload(ex);
  }
  // digit planes of an exchange-ordered tensor (built on the device)
  void tc_tk_tables(const double* tk_dev, DBuf& dig, DBuf& rexp, hfg::DevTC& out) {
    const hfg::AtomHost& H = host;
    const int n2 = H.rad.nn * H.rad.nn;
    out.dmtiles = (n2 + 127) / 128;
    out.dksteps = (n2 + 15) / 16;
    const size_t nslice = (size_t)H.NL * H.rad.nel * out.dmtiles;
    dig.alloc(nslice * out.dksteps * TC_NDIGITS * 4096);
    rexp.alloc(sizeof(int) * nslice * 128);
    hfg::DevAtom A = dev;
    A.tk = tk_dev;
    ck(hfg::launch_tk_digits(A, out.dmtiles, out.dksteps, dig.as<unsigned char>(), rexp.as<int>(), own_stream),
       "exchange tensor digits");
    out.tk_digits = dig.as<unsigned char>();
    out.tk_rowexp = rexp.as<int>();
  }
  // groups of up to 16 diagonal output blocks (sorted by multipole set) and
  // the diagonal units (element, group, row tile)
  void tc_diag_groups(bool sym, DBuf& djk, DBuf& dent, DBuf& du, const int*& gjk_out, const int*& gent_out,
                      const int4*& u_out, int& n_out, int mtiles) {
    const hfg::AtomHost& H = host;
    const int NL = H.NL, nel = H.rad.nel;
    std::vector<int> blocks;
    for (int k = 0; k < H.nang; ++k)
      for (int j = 0; j < H.nang; ++j)
        if (!sym || j <= k) blocks.push_back(j + k * H.nang);
    std::vector<int> sig(blocks.size(), 0);
    for (size_t i = 0; i < blocks.size(); ++i)
      for (int e = H.kjk_ptr[blocks[i]]; e < H.kjk_ptr[blocks[i] + 1]; ++e) sig[i] |= 1 << H.kent_L[e];
    std::vector<int> order(blocks.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return sig[x] < sig[y]; });
    const int G = ((int)blocks.size() + 15) / 16;
    std::vector<int> gjk((size_t)G * 16, -1), gent((size_t)G * 16 * NL, -1);
    for (size_t i = 0; i < order.size(); ++i) {
      const int jk = blocks[order[i]], g = (int)i / 16, s2 = (int)i % 16;
      gjk[(size_t)g * 16 + s2] = jk;
      for (int e = H.kjk_ptr[jk]; e < H.kjk_ptr[jk + 1]; ++e) gent[((size_t)g * 16 + s2) * NL + H.kent_L[e]] = e;
    }
    std::vector<int4> u;
    for (int a = 0; a < nel; ++a)
      for (int mt = 0; mt < mtiles; ++mt)
        for (int g = 0; g < G; ++g) u.push_back(make_int4(a, g, mt, 0));
    {
      long nb = 0;  // (group, L) batches with at least one entry
      for (int g = 0; g < G; ++g)
        for (int L = 0; L < NL; ++L) {
          bool any = false;
          for (int s2 = 0; s2 < 16; ++s2) any |= gent[((size_t)g * 16 + s2) * NL + L] >= 0;
          nb += any ? 1 : 0;
        }
      // per batch and row tile: K steps x (N = 112 + 96 + ... + 16) x 128 x 16
      const int ksteps = (H.rad.nn * H.rad.nn + 15) / 16;
      tc_mma_flops[sym ? 0 : 1] += 2.0 * 128 * 16 * 448 * ksteps * (double)nb * nel * mtiles;
    }
    gjk_out = djk.upload(gjk);
    gent_out = dent.upload(gent);
    u_out = du.upload(u);
    n_out = (int)u.size();
  }
  // off-diagonal tensor-core units: a unit is a range of groups of one
  // element pair (the pair's tables and the tensor memory are set up once per
  // unit); tc_per_fixed groups per unit, or 0: about eight waves of two CTAs
  // per SM. Any partition gives the same K bit for bit.
  int tc_per_fixed = 0;
  void tc_units() {
    const int nel = host.rad.nel, G = tc.ngroups;
    auto units_of = [&](bool sym) {
      const long npairs = sym ? (long)nel * (nel - 1) / 2 : (long)nel * (nel - 1);
      const long want = 8L * 2 * 152;
      int per = (int)std::max<long>(1, std::min<long>(G, (npairs * G + want - 1) / want));
      if (tc_per_fixed > 0) per = std::min(tc_per_fixed, G);
      std::vector<int4> u;
      for (int a = 0; a < nel; ++a)
        for (int b = 0; b < nel; ++b) {
          if (a == b || (sym && b < a)) continue;
          for (int g = 0; g < G; g += per) u.push_back(make_int4(a, b, g, std::min(G, g + per)));
        }
      return u;
    };
    const std::vector<int4> us = units_of(true), ua = units_of(false);
    tc.units_sym = t_usym.upload(us);
    tc.n_sym = (int)us.size();
    tc.units_all = t_uall.upload(ua);
    tc.n_all = (int)ua.size();
    if (tc_rs.digits) {
      tc_rs.units_sym = tc.units_sym;
      tc_rs.n_sym = tc.n_sym;
      tc_rs.units_all = tc.units_all;
      tc_rs.n_all = tc.n_all;
    }
  }
  // output blocks in groups of 8 with similar multipole sets, and the units
  void tc_setup() {
    const hfg::AtomHost& H = host;
    const int nel = H.rad.nel, NL = H.NL, nang2 = H.nang * H.nang;
    if (H.rad.nn > 16 || NL > 8 || nel < 2) return;
    std::vector<int> sig(nang2, 0), order(nang2);
    for (int jk = 0; jk < nang2; ++jk) {
      order[jk] = jk;
      for (int e = H.kjk_ptr[jk]; e < H.kjk_ptr[jk + 1]; ++e) sig[jk] |= 1 << H.kent_L[e];
    }
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return sig[x] < sig[y]; });
    const int G = (nang2 + 7) / 8;
    std::vector<int> gjk((size_t)G * 8, -1), gent((size_t)G * 8 * NL, -1);
    for (int i = 0; i < nang2; ++i) {
      const int jk = order[i], g = i / 8, s = i % 8;
      gjk[(size_t)g * 8 + s] = jk;
      for (int e = H.kjk_ptr[jk]; e < H.kjk_ptr[jk + 1]; ++e) {
        int& slot = gent[((size_t)g * 8 + s) * NL + H.kent_L[e]];
        if (slot >= 0) return;  // two entries with one multipole: keep the float-pair form
        slot = e;
      }
    }
    tc.ngroups = G;
    {
      long nb = 0;  // (group, L) batches with at least one entry
      for (int g = 0; g < G; ++g)
        for (int L = 0; L < NL; ++L) {
          bool any = false;
          for (int s2 = 0; s2 < 8; ++s2) any |= gent[((size_t)g * 8 + s2) * NL + L] >= 0;
          nb += any ? 1 : 0;
        }
      // per batch: 27 + 28 digit-plane products of 128 x 16 x 16
      const double per = 2.0 * 128 * 16 * 16 * 55;
      tc_mma_flops[0] += per * nb * ((double)nel * (nel - 1) / 2);
      tc_mma_flops[1] += per * nb * ((double)nel * (nel - 1));
    }
    tc_tables(H.rs, H.rb, t_dig, t_exp, tc);
    tc.group_jk = t_gjk.upload(gjk);
    tc.group_ent = t_gent.upload(gent);
    tc_units();
    t_err.alloc(sizeof(int));
    ck(cudaMemsetAsync(t_err.p, 0, sizeof(int), own_stream), "memset");
    tc.err = t_err.as<int>();
    tc_tk_tables(dev.tk, t_tkd, t_tke, tc);
    tc_diag_groups(true, t_dgjk_s, t_dgent_s, t_dus, tc.dgroup_jk_sym, tc.dgroup_ent_sym, tc.dunits_sym, tc.n_dsym,
                   tc.dmtiles);
    tc_diag_groups(false, t_dgjk_a, t_dgent_a, t_dua, tc.dgroup_jk_all, tc.dgroup_ent_all, tc.dunits_all, tc.n_dall,
                   tc.dmtiles);
    tc_ok = true;
  }
  // a completion wait inside the tensor-core kernel ran out (checked by the
  // host-pointer entry points after their synchronisation)
  void tc_check() {
    if (!tc_ok) return;
    int e = 0;
    ck(cudaMemcpy(&e, tc.err, sizeof(int), cudaMemcpyDeviceToHost), "D2H");
    if (e) throw std::runtime_error("tensor-core exchange: an MMA completion wait ran out");
  }
  // staging for the host-pointer entry points (allocated on first use)
  DBuf h_in, h_out, h_in2, h_out2, h_e;
  // bytes the last host-pointer Fock call copied each way
  size_t last_h2d = 0, last_d2h = 0;
  // spherically averaged handles: block-diagonal staging of the l-channel
  // density and result (nbf x nbf each, allocated on first use), and the
  // s-only handle on the same radial grid that evaluates their XC
  DBuf sad_in, sad_out;
  std::unique_ptr<hfg_atom> sad_xc;
  DBuf d_xrad;  // radial orthonormaliser invh(S_rad), built by the first hfg_fock_diag
  // second stream and event of the combined J+K host entry point: J's copy
  // back overlaps the exchange build
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_j = nullptr;
  // stream and events of the device-pointer J+K entry point: the Coulomb
  // build is forked from the caller's stream and joined back into it
  cudaStream_t j_stream = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // side stream of the split exchange (its diagonal stage), made on first use
  hfg::SideStream k_side{};
  const hfg::SideStream* side_stream() {
    if (!k_side.s) {
      ck(cudaStreamCreateWithFlags(&k_side.s, cudaStreamNonBlocking), "cudaStreamCreate");
      ck(cudaEventCreateWithFlags(&k_side.fork, cudaEventDisableTiming), "cudaEventCreate");
      ck(cudaEventCreateWithFlags(&k_side.join, cudaEventDisableTiming), "cudaEventCreate");
    }
    return &k_side;
  }
  // Yukawa-screened exchange: the exchange context with the screened radial
  // tables (built by hfg_atom_compute_yukawa)
  hfg::DevAtom dev_rs{};
  bool rs_ready = false;
  // erfc kernel of the range-separated exchange (the pair tables on the
  // device); rs_erfc selects it in hfg_rs_exchange
  bool rs_erfc = false;
  DBuf d_etk;
  void setup_erfc(double mu, bool exact) {
    check_device();
    host.build_erfc(mu, exact);
    hfg_abi::AllocStream alloc_on(own_stream);
    ck(cudaStreamSynchronize(own_stream), "sync");
    d_etk.upload(host.e_tk);
    ck(cudaStreamSynchronize(own_stream), "sync after upload");
    rs_erfc = true;
    rs_ready = true;
  }
  DBuf y_rs, y_rb, y_tk, y_rs2, y_rb2, y_tk2;
  void setup_yukawa(double lambda) {
    check_device();
    rs_erfc = false;
    host.build_yukawa(lambda);
    hfg_abi::AllocStream alloc_on(own_stream);
    ck(cudaStreamSynchronize(own_stream), "sync");
    auto split = [](const std::vector<double>& v) {
      std::vector<float2> o(v.size());
      for (size_t i = 0; i < v.size(); ++i) {
        const float hi = (float)v[i];
        o[i] = make_float2(hi, (float)(v[i] - (double)hi));
      }
      return o;
    };
    dev_rs = dev;
    dev_rs.rs = y_rs.upload(host.y_rs);
    dev_rs.rb = y_rb.upload(host.y_rb);
    dev_rs.tk = y_tk.upload(host.y_tk);
    dev_rs.rs2 = y_rs2.upload(split(host.y_rs));
    dev_rs.rb2 = y_rb2.upload(split(host.y_rb));
    dev_rs.tk2 = y_tk2.upload(split(host.y_tk));
    if (tc_ok) {
      tc_rs = tc;
      tc_tables(host.y_rs, host.y_rb, ty_dig, ty_exp, tc_rs);
      tc_tk_tables(dev_rs.tk, ty_tkd, ty_tke, tc_rs);
    }
    ck(cudaStreamSynchronize(own_stream), "sync after upload");
    rs_ready = true;
  }
  // DFT grid (built on first use or by hfg_dft_grid)
  hfg::DevXC xc{};
  hfg::XcScratch xs{};
  bool xc_ready = false;
  DBuf x_wang, x_isin, x_W, x_Wt, x_Wp, x_r, x_wr, x_R, x_dR, xs_D, xs_Dr, xs_F, xs_U, xs_ep;
  hfg::Profiler prof;
  std::vector<cudaEvent_t> prof_ev;
  std::vector<int> prof_cls;

  // last use of the handle's buffers on a caller stream; destruction orders
  // the stream-ordered frees after it
  cudaEvent_t last_use = nullptr;
  void mark_use(cudaStream_t st) {
    if (last_use) cudaEventRecord(last_use, st);
  }

  ~hfg_atom() {
    if (ev_j) cudaEventDestroy(ev_j);
    if (k_side.fork) cudaEventDestroy(k_side.fork);
    if (k_side.join) cudaEventDestroy(k_side.join);
    if (k_side.s) {
      cudaStreamSynchronize(k_side.s);
      cudaStreamDestroy(k_side.s);
    }
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (j_stream) {
      cudaStreamSynchronize(j_stream);
      cudaStreamDestroy(j_stream);
    }
    if (copy_stream) {
      cudaStreamSynchronize(copy_stream);
      cudaStreamDestroy(copy_stream);
    }
    free_profiler();
    if (last_use) {
      if (own_stream) cudaStreamWaitEvent(own_stream, last_use, 0);
      cudaEventDestroy(last_use);
    }
  }

  void free_profiler() {
    for (cudaEvent_t e : prof_ev) cudaEventDestroy(e);
    prof_ev.clear();
    prof_cls.clear();
    prof = hfg::Profiler();
  }

  void enable_profiler(int cap) {
    free_profiler();
    if (cap <= 0) return;
    prof_ev.resize(2 * (size_t)cap);
    for (auto& e : prof_ev) ck(cudaEventCreate(&e), "cudaEventCreate");
    prof_cls.assign(cap, 0);
    prof.ev = prof_ev.data();
    prof.cls = prof_cls.data();
    prof.cap = cap;
    prof.n = 0;
    prof.on = true;
  }

  void check_device() const {
    if (!on_device) throw std::logic_error("handle was created host-only; device entry points are unavailable");
    int d = -1;
    ck(cudaGetDevice(&d), "cudaGetDevice");
    if (d != device) throw std::invalid_argument("handle used on a different CUDA device than it was created on");
  }

  void upload() {
    using namespace hfg;
    const AtomHost& H = host;
    ck(cudaGetDevice(&device), "cudaGetDevice");
    if (!own_stream) {
      ck(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking), "cudaStreamCreate");
      stream_holder.s = own_stream;
    }
    hfg_abi::AllocStream alloc_on(own_stream);
    DevAtom& A = dev;
    A.nn = H.rad.nn;
    A.nel = H.rad.nel;
    A.nrad = H.rad.nrad;
    A.nang = H.nang;
    A.nbf = H.nbf;
    A.NL = H.NL;
    A.rs = d_rs.upload(H.rs);
    A.rb = d_rb.upload(H.rb);
    if (H.twoe_on_host) {
      A.cholp = d_cholp.upload(H.cholp);
      A.rank = d_rank.upload(H.chol_rank);
      A.tk = d_tk.upload(H.tk);
    } else {
      tabulate_device();
    }
    A.rmax = H.rmax;
    std::vector<int> chanL;
    for (auto& c : H.chans) chanL.push_back(c.L);
    A.nchan = (int)H.chans.size();
    A.chanL = d_chanL.upload(chanL);
    A.jket_ptr = d_jket_ptr.upload(H.jket_ptr);
    A.jket_blk = d_jket_blk.upload(H.jket_blk);
    A.jket_coef = d_jket_coef.upload(H.jket_coef);
    A.jbra_ptr = d_jbra_ptr.upload(H.jbra_ptr);
    A.jbra_chan = d_jbra_chan.upload(H.jbra_chan);
    A.jbra_coef = d_jbra_coef.upload(H.jbra_coef);
    A.kjk_ptr = d_kjk_ptr.upload(H.kjk_ptr);
    A.kent_L = d_kent_L.upload(H.kent_L);
    A.kent_ptr = d_kent_ptr.upload(H.kent_ptr);
    A.kterm_blk = d_kterm_blk.upload(H.kterm_blk);
    {
      need((double)H.nbf * H.nbf < 2147483647.0, "basis too large for 32-bit density offsets");
      std::vector<int> off(H.kterm_blk.size());
      for (size_t u = 0; u < off.size(); ++u) {
        const int blk = H.kterm_blk[u], i = blk % H.nang, l = blk / H.nang;
        off[u] = l * H.rad.nrad * H.nbf + i * H.rad.nrad;
      }
      A.kterm_off = d_kterm_off.upload(off);
    }
    A.nent = (int)H.kent_L.size();
    A.kterm_coef = d_kterm_coef.upload(H.kterm_coef);
    int mx = 0;
    for (int jk = 0; jk < H.nang * H.nang; ++jk) {
      int n = 0;
      for (int e = H.kjk_ptr[jk]; e < H.kjk_ptr[jk + 1]; ++e) n += H.kent_ptr[e + 1] - H.kent_ptr[e];
      mx = std::max(mx, n);
    }
    A.max_terms_per_jk = mx;
    for (int ij = 0; ij < H.nang * H.nang; ++ij)
      if (H.jbra_ptr[ij + 1] - H.jbra_ptr[ij] > 64) throw std::invalid_argument("too many Coulomb bra terms");
    const size_t n2 = (size_t)A.nn * A.nn;
    s_jin.alloc(sizeof(double) * A.nchan * A.nel * n2);
    s_jscal.alloc(sizeof(double) * A.nchan * A.nel * 2);
    s_khalo.alloc(sizeof(double) * (size_t)A.nel * A.nel * A.nang * A.nang * (2 * A.nn - 1));
    s_bnorm.alloc(sizeof(double) * (size_t)A.nang * A.nang * NORM_SPLIT);
    s_act.alloc((size_t)A.nang * A.nang);
    s_entact.alloc(std::max<size_t>(1, (size_t)A.nent));
    scr.jin = s_jin.as<double>();
    scr.jscal = s_jscal.as<double>();
    scr.khalo = s_khalo.as<double>();
    scr.bnorm = s_bnorm.as<double>();
    scr.act = s_act.as<unsigned char>();
    scr.ent_act = s_entact.as<unsigned char>();
    scr.p2 = nullptr;  // allocated on the first split-precision call
    ck(cudaEventCreateWithFlags(&last_use, cudaEventDisableTiming), "cudaEventCreate");
    auto split = [](const std::vector<double>& v) {
      std::vector<float2> o(v.size());
      for (size_t i = 0; i < v.size(); ++i) {
        const float hi = (float)v[i];
        o[i] = make_float2(hi, (float)(v[i] - (double)hi));
      }
      return o;
    };
    A.rs2 = d_rs2.upload(split(H.rs));
    A.rb2 = d_rb2.upload(split(H.rb));
    {
      const size_t ntk = (size_t)A.NL * A.nel * n2 * n2;
      d_tk2.alloc(sizeof(float2) * std::max<size_t>(1, ntk));
      ck(hfg::launch_split_f2(A.tk, d_tk2.as<float2>(), ntk, own_stream), "split copy of the exchange tensor");
      A.tk2 = d_tk2.as<float2>();
    }
    A.kterm_coef2 = d_kcoef2.upload(split(H.kterm_coef));
    A.jket_coef2 = d_jkc2.upload(split(H.jket_coef));
    A.jbra_coef2 = d_jbc2.upload(split(H.jbra_coef));
    build_units();
    tc_setup();
    ck(cudaStreamSynchronize(own_stream), "sync after upload");
    on_device = true;
  }

  // float-pair copy of the in-element factor for the split Coulomb form,
  // made on its first use (it doubles the factor's footprint)
  void ensure_split_coulomb() {
    if (dev.cholp2) return;
    hfg_abi::AllocStream alloc_on(own_stream);
    const size_t n = (size_t)host.NL * host.rad.nel * host.rad.nn * host.rad.nn * host.rmax;
    d_cholp2.alloc(sizeof(float2) * std::max<size_t>(1, n));
    ck(hfg::launch_split_f2(dev.cholp, d_cholp2.as<float2>(), n, own_stream), "split copy of the in-element factor");
    ck(cudaStreamSynchronize(own_stream), "sync after the split copy");
    dev.cholp2 = d_cholp2.as<float2>();
  }

  // In-element factors and exchange tensor tabulated on the device (FP64,
  // the host tabulation's quadrature and pivoting rule); fills the host's
  // ranks and rmax. Scratch (pair-packed tensor, full-width factor) is
  // released on the handle's stream.
  void tabulate_device() {
    using namespace hfg;
    AtomHost& H = host;
    const int nn = H.rad.nn, nel = H.rad.nel, NL = H.NL;
    const size_t n2 = (size_t)nn * nn, nblk = (size_t)NL * nel;
    std::vector<double> xo, wo, xi, wi, xin;
    twoe_points(xo, wo, xi, wi, xin);
    if (H.rad.tw_Bo.empty() || H.rad.tw_Bin.empty()) H.rad.prepare_twoe();
    std::vector<unsigned char> ok((size_t)nel * nn);
    for (int e = 0; e < nel; ++e)
      for (int k = 0; k < nn; ++k) ok[(size_t)e * nn + k] = H.rad.valid(e, k) ? 1 : 0;
    DBuf b_bval, b_xo, b_wo, b_xi, b_wi, b_Bo, b_Bin, b_ok, b_T1, b_L;
    TabInput in{};
    in.nn = nn;
    in.nel = nel;
    in.NL = NL;
    in.no = TWOE_NO;
    in.ni = TWOE_NI;
    in.bval = b_bval.upload(H.rad.bval);
    in.xo = b_xo.upload(xo);
    in.wo = b_wo.upload(wo);
    in.xi = b_xi.upload(xi);
    in.wi = b_wi.upload(wi);
    in.Bo = b_Bo.upload(H.rad.tw_Bo);
    in.Bin = b_Bin.upload(H.rad.tw_Bin);
    in.ok = b_ok.upload(ok);
    in.tol = H.chol_tol;
    b_T1.alloc(sizeof(double) * tab_t1_doubles(nn, nel, NL));
    b_L.alloc(sizeof(double) * tab_factor_doubles(nn, nel, NL));
    d_rank.alloc(sizeof(int) * nblk);
    ck(launch_tab_factor(in, b_T1.as<double>(), b_L.as<double>(), d_rank.as<int>(), own_stream),
       "in-element tensor and factor");
    H.chol_rank.assign(nblk, 0);
    ck(cudaMemcpyAsync(H.chol_rank.data(), d_rank.p, sizeof(int) * nblk, cudaMemcpyDeviceToHost, own_stream),
       "factor ranks");
    ck(cudaStreamSynchronize(own_stream), "sync after the factorisation");
    H.rmax = 1;
    for (int r : H.chol_rank) H.rmax = std::max(H.rmax, r);
    d_cholp.alloc(sizeof(double) * nblk * n2 * H.rmax);
    d_tk.alloc(sizeof(double) * nblk * n2 * n2);
    ck(launch_tab_finish(in, b_L.as<double>(), d_rank.as<int>(), H.rmax, d_cholp.as<double>(), d_tk.as<double>(),
                         own_stream),
       "padded factor and exchange tensor");
    dev.cholp = d_cholp.as<double>();
    dev.rank = d_rank.as<int>();
    dev.tk = d_tk.as<double>();
  }

  // Host copies of the factors of a device-tabulated handle (compact
  // reference layout and the padded one), fetched on first request.
  std::mutex host_fill_mu;
  void ensure_host_factors() {
    std::lock_guard<std::mutex> g(host_fill_mu);
    hfg::AtomHost& H = host;
    if (H.twoe_on_host || !H.chol.empty()) return;
    check_device();
    const int nn = H.rad.nn, nel = H.rad.nel;
    const size_t n2 = (size_t)nn * nn, nblk = (size_t)H.NL * nel;
    std::vector<double> cp(nblk * n2 * H.rmax);
    ck(cudaMemcpyAsync(cp.data(), dev.cholp, sizeof(double) * cp.size(), cudaMemcpyDeviceToHost, own_stream),
       "factor download");
    ck(cudaStreamSynchronize(own_stream), "sync after the factor download");
    std::vector<std::vector<double>> ch(nblk);
    for (int L = 0; L < H.NL; ++L)
      for (int e = 0; e < nel; ++e) {
        const size_t le = (size_t)L * nel + e;
        const int r = H.chol_rank[le], p0 = H.rad.pfirst(e), ni = H.rad.nfun(e);
        std::vector<double>& c = ch[le];
        c.assign((size_t)ni * ni * r, 0.0);
        for (int p = 0; p < r; ++p)
          for (int b = 0; b < ni; ++b)
            for (int a2 = 0; a2 < ni; ++a2)
              c[(a2 + (size_t)b * ni) + (size_t)p * ni * ni] =
                  cp[le * n2 * H.rmax + (a2 + p0) + (size_t)(b + p0) * nn + (size_t)p * n2];
      }
    H.cholp = std::move(cp);
    H.chol = std::move(ch);
  }

  // Exchange work units: element pairs split into balanced ranges of output
  // angular blocks (enough units to keep every SM busy to the end), then
  // one unit per (diagonal element, output block); off-diagonal units first
  // so the short diagonal ones fill the tail.
  // nsplit_fixed > 0: that many output-block ranges per off-diagonal element
  // pair (set by the autotuner); 0: enough units to fill the GPU
  int nsplit_fixed = 0;
  void build_units() {
    const hfg::AtomHost& H = host;
    const int nel = H.rad.nel, nang2 = H.nang * H.nang;
    std::vector<int> cnt(nang2);
    long tot = 0;
    for (int jk = 0; jk < nang2; ++jk) {
      cnt[jk] = H.kjk_ptr[jk + 1] - H.kjk_ptr[jk];
      tot += cnt[jk];
    }
    auto ranges = [&](int nsplit) {
      std::vector<int> cut(1, 0);
      long acc = 0;
      int s = 1;
      for (int jk = 0; jk < nang2; ++jk) {
        acc += cnt[jk];
        if (s < nsplit && acc * nsplit >= tot * s) { cut.push_back(jk + 1); ++s; }
      }
      if (cut.back() != nang2) cut.push_back(nang2);
      return cut;
    };
    auto make = [&](bool sym, std::vector<int>& dj, int& noff) {
      std::vector<int4> u;
      const long npairs = sym ? (long)nel * (nel - 1) / 2 : (long)nel * (nel - 1);
      int nsplit = (int)std::min<long>(std::max<long>(1, (2432 + npairs - 1) / std::max<long>(npairs, 1)), 8);
      if (nsplit_fixed > 0) nsplit = nsplit_fixed;
      nsplit = std::min(nsplit, nang2);
      const std::vector<int> cut = ranges(nsplit);
      for (int a = 0; a < nel; ++a)
        for (int b = 0; b < nel; ++b) {
          if (a == b || (sym && b < a)) continue;
          for (size_t s = 0; s + 1 < cut.size(); ++s)
            if (cut[s + 1] > cut[s]) u.push_back(make_int4(a, b, cut[s], cut[s + 1]));
        }
      noff = (int)u.size();
      dj.clear();
      for (int k = 0; k < H.nang; ++k)
        for (int j = 0; j < H.nang; ++j)
          if (!sym || j <= k) dj.push_back(j + k * H.nang);
      for (int a = 0; a < nel; ++a)
        for (int w = 0; w < (int)dj.size(); ++w) u.push_back(make_int4(a, a, w, w + 1));
      return u;
    };
    std::vector<int> dja, djs;
    std::vector<int4> ua = make(false, dja, units.n_off_all), us = make(true, djs, units.n_off_sym);
    units.all = d_units_all.upload(ua);
    units.n_all = (int)ua.size();
    units.sym = d_units_sym.upload(us);
    units.n_sym = (int)us.size();
    units.diag_all = d_diag_all.upload(dja);
    units.diag_sym = d_diag_sym.upload(djs);
  }

  void setup_xc(int ldft, int mdft) {
    if (host.spherical)
      throw std::logic_error("a spherically averaged handle has no angular XC grid (its density is radial)");
    hfg_abi::AllocStream alloc_on(own_stream);
    host.build_dft_grid(ldft, mdft);
    const hfg::AtomHost& H = host;
    xc.nquad = H.nquad;
    xc.nap = H.nap;
    xc.wang = x_wang.upload(H.xc_wang);
    xc.isin = x_isin.upload(H.xc_isin);
    xc.W = x_W.upload(H.xc_W);
    xc.Wt = x_Wt.upload(H.xc_Wt);
    xc.Wp = x_Wp.upload(H.xc_Wp);
    xc.r = x_r.upload(H.xc_r);
    xc.wr = x_wr.upload(H.xc_wr);
    xc.R = x_R.upload(H.xc_R);
    xc.dR = x_dR.upload(H.xc_dR);
    const size_t nel = H.rad.nel, nq = H.nquad, nab = (size_t)H.nang * H.nang, nap = H.nap;
    xs_D.alloc(sizeof(double) * 2 * nel * nab * nq);
    xs_Dr.alloc(sizeof(double) * 2 * nel * nab * nq);
    xs_F.alloc(sizeof(double) * 8 * nel * nq * nap);
    xs_U.alloc(sizeof(double) * 8 * nel * nab * nq);
    xs_ep.alloc(sizeof(double) * 2 * nel * nq);
    xs.D = xs_D.as<double>();
    xs.Dr = xs_Dr.as<double>();
    xs.F = xs_F.as<double>();
    xs.U = xs_U.as<double>();
    xs.epart = xs_ep.as<double>();
    ck(cudaStreamSynchronize(own_stream), "sync after grid upload");
    xc_ready = true;
  }

  void staging() {
    hfg_abi::AllocStream alloc_on(own_stream);
    const size_t bytes = sizeof(double) * (size_t)host.nbf * host.nbf;
    if (h_in.n != bytes) h_in.alloc(bytes);
    if (h_out.n != bytes) h_out.alloc(bytes);
  }
};


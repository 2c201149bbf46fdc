// C ABI of the diatomic Fock build (declarations and contract in
// include/helfem_gb300.h). The handle owns the host tabulation, the device
// tables and the per-call scratch; every entry point converts exceptions
// and CUDA errors into status codes.
#include <algorithm>
#include <cstring>

#include "cuda/devdiatomic.cuh"
#include "cuda/dtab.cuh"
#include "handle.hpp"
#include "host/diatomic.hpp"

struct hfg_diatomic {
  hfg_abi::StreamHolder stream_holder;  // destroyed last
  hfg::DiatomicHost host;
  int device = 0;
  bool on_device = false;
  cudaStream_t own_stream = nullptr;
  hfg::DevDiatomic dev{};
  hfg::DevDiatomicScratch scr{};
  DBuf d_p0, d_p2, d_q0, d_q2, d_cdB, d_cds, d_cdrank, d_tx, d_lmfac, d_al_ptr, d_al_b, d_al_c0, d_al_c2, d_chL,
      d_chM, d_chilm, d_chfac, d_jbra_ptr, d_jbra_chan, d_jbra_c0, d_jbra_c2, d_kjk_ptr, d_kentL, d_kentMa,
      d_kentilm, d_kentjk, d_pairs_all, d_pairs_sym, d_pure, d_poff, d_pstart;
  DBuf s_jin, s_jscal, s_khalo, s_bnorm, s_act, s_entact, s_jkact, s_jklist, s_counts, s_Pd, s_Fd;
  DBuf d_p0s, d_p2s, d_q0s, d_q2s, d_txs, d_alc0s, d_alc2s, d_lmfacs, d_kexp, s_pd2;  // split-precision path
  DBuf h_in, h_out;
  cudaEvent_t last_use = nullptr;
  std::vector<double> lmfac_host;
  // pure-m DFT grid (built on first use)
  hfg::DevDiatomicXC xc{};
  hfg::DiatomicXcScratch xs{};
  bool xc_ready = false;
  DBuf x_ps, x_pt, x_mult, x_W, x_Wt, x_R, x_dR, x_w, x_hinv, x_fk, x_fms, x_fmt, xs_D, xs_Dr, xs_F, xs_U, xs_ep,
      h_in2, h_out2, h_e;

  ~hfg_diatomic() {
    if (last_use) {
      if (own_stream) cudaStreamWaitEvent(own_stream, last_use, 0);
      cudaEventDestroy(last_use);
    }
  }
  void mark_use(cudaStream_t st) {
    if (last_use) cudaEventRecord(last_use, st);
  }
  void check_device() const {
    if (!on_device) throw std::logic_error("handle was created host-only; device entry points are unavailable");
    int d = -1;
    ck(cudaGetDevice(&d), "cudaGetDevice");
    if (d != device) throw std::invalid_argument("handle used on a different CUDA device than it was created on");
  }

  void upload() {
    using namespace hfg;
    const DiatomicHost& H = host;
    ck(cudaGetDevice(&device), "cudaGetDevice");
    ck(cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    stream_holder.s = own_stream;
    hfg_abi::AllocStream alloc_on(own_stream);
    DevDiatomic& D = dev;
    D.nn = H.nn;
    D.nel = H.nel;
    D.nrad = H.nrad;
    D.nang = H.nang;
    D.nd = H.ndummy;
    D.nlm = H.nlm;
    D.Lmax = H.Lmax;
    D.mmax = H.mmax;
    D.nM = H.nM;
    D.nbf = H.nbf;
    {
      std::vector<int> off(H.nang), st(H.nang);
      for (int a = 0, o = 0; a < H.nang; ++a) {
        st[a] = H.mval[a] == 0 ? 0 : 1;
        off[a] = o;
        o += H.nrad - st[a];
      }
      D.poff = d_poff.upload(off);
      D.pstart = d_pstart.upload(st);
    }
    if (H.twoe_on_host) {
      D.p0 = d_p0.upload(H.p0);
      D.p2 = d_p2.upload(H.p2);
      D.q0 = d_q0.upload(H.q0);
      D.q2 = d_q2.upload(H.q2);
      D.cdB = d_cdB.upload(H.cd_B);
      D.cds = d_cds.upload(H.cd_s);
      D.cdrank = d_cdrank.upload(H.cd_rank);
    } else {
      tabulate_device();
    }
    D.rmax = H.rmax;
    std::vector<double> lmf(H.nlm);
    for (int i = 0; i < H.nlm; ++i) {
      const int L = H.lm_L[i], Ma = H.lm_M[i];
      double fr = 1.0;
      for (int p = L + Ma; p > L - Ma; --p) fr *= p;
      lmf[i] = 4.0 * M_PI * std::pow(H.Rhalf, 5) / fr;
    }
    D.lmfac = d_lmfac.upload(lmf);
    lmfac_host = lmf;
    D.al_ptr = d_al_ptr.upload(H.al_ptr);
    D.al_b = d_al_b.upload(H.al_b);
    D.al_c0 = d_al_c0.upload(H.al_c0);
    D.al_c2 = d_al_c2.upload(H.al_c2);
    D.nchan = (int)H.ch_L.size();
    D.ch_L = d_chL.upload(H.ch_L);
    D.ch_M = d_chM.upload(H.ch_M);
    D.ch_ilm = d_chilm.upload(H.ch_ilm);
    D.ch_fac = d_chfac.upload(H.ch_fac);
    D.jbra_ptr = d_jbra_ptr.upload(H.jbra_ptr);
    D.jbra_chan = d_jbra_chan.upload(H.jbra_chan);
    D.jbra_c0 = d_jbra_c0.upload(H.jbra_c0);
    D.jbra_c2 = d_jbra_c2.upload(H.jbra_c2);
    D.nent = (int)H.kent_L.size();
    D.kjk_ptr = d_kjk_ptr.upload(H.kjk_ptr);
    D.kent_L = d_kentL.upload(H.kent_L);
    D.kent_Ma = d_kentMa.upload(H.kent_Ma);
    D.kent_ilm = d_kentilm.upload(H.kent_ilm);
    std::vector<int> kjk(D.nent);
    for (int jk = 0; jk < H.nang * H.nang; ++jk)
      for (int e = H.kjk_ptr[jk]; e < H.kjk_ptr[jk + 1]; ++e) kjk[e] = jk;
    D.kent_jk = d_kentjk.upload(kjk);
    std::vector<int2> pa, ps;
    for (int b = 0; b < H.nel; ++b)
      for (int a = 0; a < H.nel; ++a) {
        if (a == b) continue;
        pa.push_back(make_int2(a, b));
        if (a < b) ps.push_back(make_int2(a, b));
      }
    D.pairs_all = d_pairs_all.upload(pa);
    D.npairs_all = (int)pa.size();
    D.pairs_sym = d_pairs_sym.upload(ps);
    D.npairs_sym = (int)ps.size();
    d_pure.upload(H.pure);
    const size_t n2 = (size_t)H.nn * H.nn, nang2 = (size_t)H.nang * H.nang, nd = (size_t)H.ndummy;
    d_tx.alloc(sizeof(double) * (size_t)H.nlm * H.nel * 4 * n2 * n2);
    D.tx = d_tx.as<double>();
    scr.pd2 = nullptr;
    ck(hfg::launch_diatomic_tx(D, d_tx.as<double>(), own_stream), "in-element kernel build");
    s_jin.alloc(sizeof(double) * (size_t)D.nchan * H.nel * 2 * n2);
    s_jscal.alloc(sizeof(double) * (size_t)D.nchan * H.nel * 4);
    s_khalo.alloc(sizeof(double) * (size_t)H.nel * H.nel * nang2 * (2 * H.nn - 1));
    s_bnorm.alloc(sizeof(double) * nang2 * DNORM_SPLIT);
    s_act.alloc(nang2);
    s_entact.alloc(std::max<size_t>(1, D.nent));
    s_jkact.alloc(nang2);
    s_jklist.alloc(sizeof(int) * 2 * nang2);
    s_counts.alloc(sizeof(int) * 2);
    s_Pd.alloc(sizeof(double) * nd * nd);
    s_Fd.alloc(sizeof(double) * nd * nd);
    scr.jin = s_jin.as<double>();
    scr.jscal = s_jscal.as<double>();
    scr.khalo = s_khalo.as<double>();
    scr.bnorm = s_bnorm.as<double>();
    scr.act = s_act.as<unsigned char>();
    scr.ent_act = s_entact.as<unsigned char>();
    scr.jk_act = s_jkact.as<unsigned char>();
    scr.jk_list = s_jklist.as<int>();
    scr.counts = s_counts.as<int>();
    ck(cudaEventCreateWithFlags(&last_use, cudaEventDisableTiming), "cudaEventCreate");
    ck(cudaStreamSynchronize(own_stream), "sync after upload");
    on_device = true;
  }

  // Two-electron primitives tabulated on the device (the host tabulation's
  // rules and pivoting): Legendre functions at the disjoint and outer points,
  // the disjoint tiles, then the in-element kernel and its factor in groups
  // of elements whose scratch stays within a fixed budget. Each group's
  // factor is compacted to the group's largest rank; once every rank is
  // known the groups are packed into the padded layout of the host tables.
  // The disjoint tiles are copied back to the host vectors (the split
  // tables and hfg_diatomic_tables read them there); the factor stays on
  // the device.
  void tabulate_device() {
    using namespace hfg;
    DiatomicHost& H = host;
    const int nn = H.nn, nel = H.nel, nlm = H.nlm, n2 = nn * nn, N = 2 * n2;
    int Mtop = 0;
    for (int m : H.lm_M) Mtop = std::max(Mtop, m);
    DiatomicHost::TwoeRules R;
    H.twoe_rules(R);
    std::vector<unsigned char> ok((size_t)nel * nn);
    for (int e = 0; e < nel; ++e)
      for (int p = 0; p < nn; ++p) ok[(size_t)e * nn + p] = e * (nn - 1) + p < H.nrad ? 1 : 0;
    std::vector<int> lmidx((size_t)(Mtop + 1) * (H.Lmax + 1), -1);
    for (int i = 0; i < nlm; ++i) lmidx[(size_t)H.lm_M[i] * (H.Lmax + 1) + H.lm_L[i]] = i;
    DBuf b_bval, b_xg, b_wg, b_xo, b_wo, b_xi, b_wi, b_Bg, b_B1g, b_B1z, b_B2g, b_B2z, b_ok, b_lmL, b_lmM, b_lmidx,
        b_PQ, b_scr, b_Bsc, b_ssc, b_rank;
    DTabInput in{};
    in.nn = nn;
    in.nel = nel;
    in.nlm = nlm;
    in.Lmax = H.Lmax;
    in.Mtop = Mtop;
    in.n1e = R.n1e;
    in.no = R.no;
    in.ni = R.ni;
    in.bval = b_bval.upload(H.bval);
    in.xg = b_xg.upload(R.xg);
    in.wg = b_wg.upload(R.wg);
    in.xo = b_xo.upload(R.xo);
    in.wo = b_wo.upload(R.wo);
    in.xi = b_xi.upload(R.xi);
    in.wi = b_wi.upload(R.wi);
    in.Bg = b_Bg.upload(R.Bg);
    in.B1g = b_B1g.upload(R.B1g);
    in.B1z = b_B1z.upload(R.B1z);
    in.B2g = b_B2g.upload(R.B2g);
    in.B2z = b_B2z.upload(R.B2z);
    in.ok = b_ok.upload(ok);
    in.lm_L = b_lmL.upload(H.lm_L);
    in.lm_M = b_lmM.upload(H.lm_M);
    in.lmidx = b_lmidx.upload(lmidx);
    in.thresh = H.cd_thresh;
    b_PQ.alloc(sizeof(double) * dtab_pq_doubles(in));
    ck(launch_dtab_pq(in, b_PQ.as<double>(), own_stream), "Legendre functions at the quadrature points");
    const size_t ntab = (size_t)nlm * nel * n2;
    d_p0.alloc(sizeof(double) * ntab);
    d_p2.alloc(sizeof(double) * ntab);
    d_q0.alloc(sizeof(double) * ntab);
    d_q2.alloc(sizeof(double) * ntab);
    ck(launch_dtab_disjoint(in, b_PQ.as<double>(), d_p0.as<double>(), d_p2.as<double>(), d_q0.as<double>(),
                            d_q2.as<double>(), own_stream),
       "disjoint integrals");
    // element groups within about 1 GiB of scratch (in-element products,
    // the kernel before symmetrisation and the factor at capacity capR)
    int capR = std::min(N, 128);
    auto per_element = [&](int cap) {
      return sizeof(double) * (dtab_group_doubles(in, 1, cap) + (size_t)nlm * N * cap + (size_t)nlm * cap);
    };
    const size_t budget = (size_t)1 << 30;
    auto group_size = [&](int cap) {
      return (int)std::max<size_t>(1, std::min<size_t>((size_t)nel, budget / per_element(cap)));
    };
    int ge = group_size(capR);
    auto alloc_group = [&]() {
      const size_t ng = (size_t)ge * nlm;
      b_scr.alloc(sizeof(double) * dtab_group_doubles(in, ge, capR));
      b_Bsc.alloc(sizeof(double) * ng * N * capR);
      b_ssc.alloc(sizeof(double) * ng * capR);
    };
    alloc_group();
    b_rank.alloc(sizeof(int) * (size_t)nel * nlm);
    std::vector<int> rk((size_t)nel * nlm, 0);
    struct Group { int e0, ne, cap; DBuf B, s; };
    std::vector<Group> groups;
    for (int e0 = 0; e0 < nel;) {
      const int ne = std::min(ge, nel - e0), ng = ne * nlm;
      int* rank_g = b_rank.as<int>() + (size_t)e0 * nlm;
      ck(launch_dtab_factor(in, b_PQ.as<double>(), e0, ne, capR, b_scr.as<double>(), b_Bsc.as<double>(),
                            b_ssc.as<double>(), rank_g, own_stream),
         "in-element kernel and factor");
      ck(cudaMemcpyAsync(rk.data() + (size_t)e0 * nlm, rank_g, sizeof(int) * ng, cudaMemcpyDeviceToHost, own_stream),
         "factor ranks");
      ck(cudaStreamSynchronize(own_stream), "sync after a factor group");
      int rg = 1;
      bool over = false;
      for (int g = 0; g < ng; ++g) {
        const int r = rk[(size_t)e0 * nlm + g];
        if (r < 0) over = true;
        rg = std::max(rg, r);
      }
      if (over) {  // a rank above the capacity: redo this group at full capacity
        if (capR == N) throw std::runtime_error("diatomic device tabulation: factor rank out of range");
        capR = N;
        ge = group_size(capR);
        alloc_group();
        continue;
      }
      Group G{e0, ne, rg, DBuf(), DBuf()};
      G.B.alloc(sizeof(double) * (size_t)ng * N * rg);
      G.s.alloc(sizeof(double) * (size_t)ng * rg);
      ck(launch_dtab_pack(N, ng, nlm, nel, e0, 0, capR, rg, b_Bsc.as<double>(), b_ssc.as<double>(), rank_g,
                          G.B.as<double>(), G.s.as<double>(), own_stream),
         "factor compaction");
      groups.push_back(std::move(G));
      e0 += ne;
    }
    b_scr.release();
    b_Bsc.release();
    b_ssc.release();
    H.rmax = 1;
    for (const Group& G : groups) H.rmax = std::max(H.rmax, G.cap);
    d_cdB.alloc(sizeof(double) * (size_t)nlm * nel * N * H.rmax);
    d_cds.alloc(sizeof(double) * (size_t)nlm * nel * H.rmax);
    for (const Group& G : groups)
      ck(launch_dtab_pack(N, G.ne * nlm, nlm, nel, G.e0, 1, G.cap, H.rmax, G.B.as<double>(), G.s.as<double>(),
                          b_rank.as<int>() + (size_t)G.e0 * nlm, d_cdB.as<double>(), d_cds.as<double>(),
                          own_stream),
         "padded factor");
    H.cd_rank.assign((size_t)nlm * nel, 0);
    for (int e = 0; e < nel; ++e)
      for (int i = 0; i < nlm; ++i) H.cd_rank[(size_t)i * nel + e] = rk[(size_t)e * nlm + i];
    dev.cdrank = d_cdrank.upload(H.cd_rank);
    dev.cdB = d_cdB.as<double>();
    dev.cds = d_cds.as<double>();
    dev.p0 = d_p0.as<double>();
    dev.p2 = d_p2.as<double>();
    dev.q0 = d_q0.as<double>();
    dev.q2 = d_q2.as<double>();
    H.p0.resize(ntab);
    H.p2.resize(ntab);
    H.q0.resize(ntab);
    H.q2.resize(ntab);
    const std::pair<std::vector<double>*, const DBuf*> dl[4] = {{&H.p0, &d_p0}, {&H.p2, &d_p2}, {&H.q0, &d_q0},
                                                                 {&H.q2, &d_q2}};
    for (const auto& x : dl)
      ck(cudaMemcpyAsync(x.first->data(), x.second->p, sizeof(double) * ntab, cudaMemcpyDeviceToHost, own_stream),
         "disjoint tiles to the host");
    ck(cudaStreamSynchronize(own_stream), "sync after the device tabulation");
  }

  // split tables and the split density buffer, on the first split-precision call
  void ensure_split() {
    if (dev.txs) return;
    hfg_abi::AllocStream alloc_on(own_stream);
    auto split = [](const std::vector<double>& v) {
      std::vector<float2> o(v.size());
      for (size_t i = 0; i < v.size(); ++i) {
        const float hi = (float)v[i];
        o[i] = make_float2(hi, (float)(v[i] - (double)hi));
      }
      return o;
    };
    const hfg::DiatomicHost& H = host;
    // per-(multipole, element) power-of-two rescaling into the FP32 range
    const size_t n2 = (size_t)H.nn * H.nn, ntile = (size_t)H.nlm * H.nel;
    std::vector<int> kexp(ntile, 0);
    std::vector<double> p0(H.p0), p2(H.p2), q0(H.q0), q2(H.q2);
    for (size_t t = 0; t < ntile; ++t) {
      double mx = 0.0;
      for (size_t i = 0; i < n2; ++i) mx = std::max(mx, std::max(std::fabs(H.p0[t * n2 + i]), std::fabs(H.p2[t * n2 + i])));
      int e = 0;
      if (mx > 0.0) std::frexp(mx, &e);
      kexp[t] = e;
      for (size_t i = 0; i < n2; ++i) {
        p0[t * n2 + i] = std::ldexp(p0[t * n2 + i], -e);
        p2[t * n2 + i] = std::ldexp(p2[t * n2 + i], -e);
        q0[t * n2 + i] = std::ldexp(q0[t * n2 + i], e);
        q2[t * n2 + i] = std::ldexp(q2[t * n2 + i], e);
      }
    }
    dev.kexp = d_kexp.upload(kexp);
    dev.p0s = d_p0s.upload(split(p0));
    dev.p2s = d_p2s.upload(split(p2));
    dev.q0s = d_q0s.upload(split(q0));
    dev.q2s = d_q2s.upload(split(q2));
    dev.al_c0s = d_alc0s.upload(split(H.al_c0));
    dev.al_c2s = d_alc2s.upload(split(H.al_c2));
    dev.lmfacs = d_lmfacs.upload(split(lmfac_host));
    const size_t ntx = d_tx.n / sizeof(double);
    d_txs.alloc(sizeof(float2) * ntx);
    ck(hfg::launch_diatomic_split_tx(d_tx.as<double>(), d_txs.as<float2>(), ntx, own_stream), "split tables");
    s_pd2.alloc(sizeof(float2) * (size_t)H.ndummy * H.ndummy);
    scr.pd2 = s_pd2.as<float2>();
    ck(cudaStreamSynchronize(own_stream), "sync after split tables");
    dev.txs = d_txs.as<float2>();
  }

  // J or K of a pure-basis density (device pointers) on stream st
  void build(const double* P, double* F, bool exchange, bool symmetric, cudaStream_t st, bool split = false,
             bool inline_diag = false) {
    check_device();
    const hfg::DiatomicHost& H = host;
    if (split) ensure_split();
    if (!exchange) {  // J reads the pure density and writes the pure J directly
      ck(hfg::launch_diatomic_coulomb(dev, scr, P, F, st), "coulomb");
      mark_use(st);
      return;
    }
    ck(hfg::launch_diatomic_expand(P, H.nbf, d_pure.as<int>(), s_Pd.as<double>(), H.ndummy, st), "expand");
    if (split)
      ck(hfg::launch_diatomic_exchange_split(dev, scr, s_Pd.as<double>(), s_Fd.as<double>(), symmetric, st,
                                             inline_diag),
         "exchange (split)");
    else
      ck(hfg::launch_diatomic_exchange(dev, scr, s_Pd.as<double>(), s_Fd.as<double>(), symmetric, st), "exchange");
    ck(hfg::launch_diatomic_gather(s_Fd.as<double>(), H.ndummy, d_pure.as<int>(), H.nbf, F, st), "gather");
    mark_use(st);
  }

  void setup_xc(int lang) {
    check_device();
    hfg_abi::AllocStream alloc_on(own_stream);
    host.build_xc_grid(lang);
    const hfg::DiatomicHost& H = host;
    need(H.xc_lang <= 1024, "hfg_diatomic_dft_grid: at most 1024 nu points");
    xc.nq = H.xc_nq;
    xc.na = H.xc_lang;
    xc.npair = H.xc_npair;
    xc.ps = x_ps.upload(H.xc_ps);
    xc.pt = x_pt.upload(H.xc_pt);
    xc.mult = x_mult.upload(H.xc_mult);
    xc.nfock = (int)H.xc_fk.size();
    xc.fk = x_fk.upload(H.xc_fk);
    xc.fms = x_fms.upload(H.xc_fms);
    xc.fmt = x_fmt.upload(H.xc_fmt);
    xc.W = x_W.upload(H.xc_W);
    xc.Wt = x_Wt.upload(H.xc_Wt);
    xc.R = x_R.upload(H.xc_R);
    xc.dR = x_dR.upload(H.xc_dR);
    xc.w = x_w.upload(H.xc_w);
    xc.hinv = x_hinv.upload(H.xc_hinv);
    const size_t nel = H.nel, nq = H.xc_nq, np = H.xc_npair, na = H.xc_lang;
    xs_D.alloc(sizeof(double) * 2 * nel * nq * np);
    xs_Dr.alloc(sizeof(double) * 2 * nel * nq * np);
    xs_F.alloc(sizeof(double) * 6 * nel * nq * na);
    xs_U.alloc(sizeof(double) * 6 * nel * np * nq);
    xs_ep.alloc(sizeof(double) * 2 * nel * nq);
    xs.D = xs_D.as<double>();
    xs.Dr = xs_Dr.as<double>();
    xs.F = xs_F.as<double>();
    xs.U = xs_U.as<double>();
    xs.epart = xs_ep.as<double>();
    ck(cudaStreamSynchronize(own_stream), "sync after grid upload");
    xc_ready = true;
  }

  // XC potential of pure-basis spin densities (device pointers); Pb == null:
  // restricted, Pa the total density
  void xc_build(int xid, int cid, const double* Pa, const double* Pb, double* Ha, double* Hb, double* energies,
                double thr, cudaStream_t st) {
    check_device();
    if (!xc_ready) setup_xc(0);
    ck(hfg::launch_diatomic_xc(dev, xc, xs, xid, cid, Pa, Pb, Ha, Hb, energies, thr, st), "xc kernels");
    mark_use(st);
  }

  void build_host(const double* P, double* F, bool exchange, bool symmetric, bool split = false) {
    check_device();
    hfg_abi::AllocStream alloc_on(own_stream);
    const size_t bytes = sizeof(double) * (size_t)host.nbf * host.nbf;
    if (h_in.n != bytes) h_in.alloc(bytes);
    if (h_out.n != bytes) h_out.alloc(bytes);
    ck(cudaMemcpyAsync(h_in.p, P, bytes, cudaMemcpyHostToDevice, own_stream), "copy in");
    build(h_in.as<double>(), h_out.as<double>(), exchange, symmetric, own_stream, split);
    ck(cudaMemcpyAsync(F, h_out.p, bytes, cudaMemcpyDeviceToHost, own_stream), "copy out");
    ck(cudaStreamSynchronize(own_stream), "sync");
  }
};

namespace {
cudaStream_t to_stream(void* s) { return static_cast<cudaStream_t>(s); }
}  // namespace

extern "C" {

hfg_status hfg_diatomic_create(const hfg_diatomic_desc* desc, hfg_diatomic** out) {
  return guard([&] {
    need(desc != nullptr && out != nullptr, "hfg_diatomic_create: null argument");
    need(desc->bval && desc->lval && desc->mval && desc->nelem >= 2 && desc->nang >= 1,
         "hfg_diatomic_create: bad description");
    need(desc->nang <= 255, "hfg_diatomic_create: at most 255 angular functions");
    std::unique_ptr<hfg_diatomic> d(new hfg_diatomic());
    std::vector<double> bval(desc->bval, desc->bval + desc->nelem + 1);
    std::vector<int> lv(desc->lval, desc->lval + desc->nang), mv(desc->mval, desc->mval + desc->nang);
    need(desc->host_only >= 0 && desc->host_only <= 2, "hfg_diatomic_create: host_only must be 0, 1 or 2");
    d->host.build(desc->Z1, desc->Z2, desc->Rhalf, desc->nnodes, bval, lv, mv, desc->cd_thresh,
                  desc->host_only != 0);
    if (desc->host_only != 1) d->upload();
    *out = d.release();
  });
}

hfg_status hfg_diatomic_destroy(hfg_diatomic* d) {
  return guard([&] { delete d; });
}

hfg_status hfg_diatomic_get_dims(const hfg_diatomic* d, hfg_diatomic_dims_t* dims) {
  return guard([&] {
    need(d && dims, "hfg_diatomic_get_dims: null argument");
    const hfg::DiatomicHost& H = d->host;
    dims->nrad = H.nrad;
    dims->nang = H.nang;
    dims->nel = H.nel;
    dims->nnodes = H.nn;
    dims->ndummy = H.ndummy;
    dims->nbf = H.nbf;
    dims->nlm = H.nlm;
    dims->Lmax = H.Lmax;
    dims->rmax = H.rmax;
    dims->nchan = (int)H.ch_L.size();
    dims->nent = (int)H.kent_L.size();
  });
}

hfg_status hfg_diatomic_pure_indices(const hfg_diatomic* d, int* idx) {
  return guard([&] {
    need(d && idx, "hfg_diatomic_pure_indices: null argument");
    std::copy(d->host.pure.begin(), d->host.pure.end(), idx);
  });
}

static hfg_status one_e(const hfg_diatomic* d, double* out, int which) {
  return guard([&] {
    need(d && out, "hfg_diatomic one-electron: null argument");
    std::vector<double> M;
    if (which == 0) d->host.overlap(M);
    else if (which == 1) d->host.kinetic(M);
    else d->host.nuclear(M);
    std::copy(M.begin(), M.end(), out);
  });
}
hfg_status hfg_diatomic_overlap(const hfg_diatomic* d, double* S) { return one_e(d, S, 0); }
hfg_status hfg_diatomic_kinetic(const hfg_diatomic* d, double* T) { return one_e(d, T, 1); }
hfg_status hfg_diatomic_nuclear(const hfg_diatomic* d, double* V) { return one_e(d, V, 2); }

hfg_status hfg_diatomic_one_electron_block(const hfg_diatomic* d, int which, int mblock, double* out, int* n) {
  return guard([&] {
    need(d && n && which >= 0 && which <= 2, "hfg_diatomic_one_electron_block: bad arguments");
    std::vector<double> M;
    int nb = 0;
    d->host.one_electron_block(which, mblock, M, nb);
    *n = nb;
    if (out) std::copy(M.begin(), M.end(), out);
  });
}

hfg_status hfg_diatomic_tables(const hfg_diatomic* d, int which, int ilm, int iel, int* L, int* M, int* rank,
                               double* out, double* sigma) {
  return guard([&] {
    need(d != nullptr, "hfg_diatomic_tables: null handle");
    const hfg::DiatomicHost& H = d->host;
    need(ilm >= 0 && ilm < H.nlm && iel >= 0 && iel < H.nel && which >= 0 && which <= 4,
         "hfg_diatomic_tables: index out of range");
    if (L) *L = H.lm_L[ilm];
    if (M) *M = H.lm_M[ilm];
    const size_t le = (size_t)ilm * H.nel + iel, n2 = (size_t)H.nn * H.nn;
    if (rank) *rank = H.cd_rank[le];
    if (!out) return;
    if (which < 4) {
      const std::vector<double>* src[4] = {&H.p0, &H.p2, &H.q0, &H.q2};
      std::copy(src[which]->begin() + le * n2, src[which]->begin() + (le + 1) * n2, out);
    } else if (H.twoe_on_host) {
      const size_t N = 2 * n2, r = H.cd_rank[le];
      std::copy(H.cd_B.begin() + le * N * H.rmax, H.cd_B.begin() + le * N * H.rmax + N * r, out);
      if (sigma) std::copy(H.cd_s.begin() + le * H.rmax, H.cd_s.begin() + le * H.rmax + r, sigma);
    } else {  // device-tabulated: the factor lives on the device only
      d->check_device();
      const size_t N = 2 * n2, r = H.cd_rank[le];
      const double* B = static_cast<const double*>(d->d_cdB.p) + le * N * H.rmax;
      const double* sg = static_cast<const double*>(d->d_cds.p) + le * H.rmax;
      if (r) {
        ck(cudaMemcpy(out, B, sizeof(double) * N * r, cudaMemcpyDeviceToHost), "factor download");
        if (sigma) ck(cudaMemcpy(sigma, sg, sizeof(double) * r, cudaMemcpyDeviceToHost), "sign download");
      }
    }
  });
}

hfg_status hfg_legendre_pq(int Lmax, int Mmax, double mu, double* P, double* Q) {
  return guard([&] {
    need(P && Q && Lmax >= 0 && Mmax >= 0 && mu > 0, "hfg_legendre_pq: bad arguments");
    hfg::legendre_pq(Lmax, Mmax, mu, P, Q);
  });
}

hfg_status hfg_gaunt_mod(int lj, int mj, int L, int M, int li, int mi, double* value) {
  return guard([&] {
    need(value != nullptr, "hfg_gaunt_mod: null argument");
    if (mj != M + mi) { *value = 0.0; return; }
    const double c0 = 2.0 / 3.0 * std::sqrt(M_PI), c2 = 4.0 / 15.0 * std::sqrt(5.0 * M_PI);
    double v = c0 * hfg::gaunt_coeff(L, M, 0, 0, L) * hfg::gaunt_coeff(lj, mj, li, mi, L);
    for (int Lp = std::max(std::max(L - 2, 0), std::abs(M)); Lp <= L + 2; ++Lp)
      v += c2 * hfg::gaunt_coeff(Lp, M, 2, 0, L) * hfg::gaunt_coeff(lj, mj, li, mi, Lp);
    *value = v;
  });
}

hfg_status hfg_diatomic_coulomb(hfg_diatomic* d, const double* P, double* J, void* stream) {
  return guard([&] {
    need(d && P && J, "hfg_diatomic_coulomb: null argument");
    d->build(P, J, false, false, to_stream(stream));
  });
}

hfg_status hfg_diatomic_exchange(hfg_diatomic* d, const double* P, double* K, int flags, void* stream) {
  return guard([&] {
    need(d && P && K, "hfg_diatomic_exchange: null argument");
    need((flags & ~(HFG_EXCHANGE_SYMMETRIC | HFG_EXCHANGE_SPLIT | HFG_EXCHANGE_ITEMWISE)) == 0,
         "hfg_diatomic_exchange: unsupported flags");
    d->build(P, K, true, (flags & HFG_EXCHANGE_SYMMETRIC) != 0, to_stream(stream), (flags & HFG_EXCHANGE_SPLIT) != 0,
             (flags & HFG_EXCHANGE_ITEMWISE) != 0);
  });
}

hfg_status hfg_diatomic_coulomb_host(hfg_diatomic* d, const double* P, double* J) {
  return guard([&] {
    need(d && P && J, "hfg_diatomic_coulomb_host: null argument");
    d->build_host(P, J, false, false);
  });
}

hfg_status hfg_diatomic_exchange_host(hfg_diatomic* d, const double* P, double* K, int flags) {
  return guard([&] {
    need(d && P && K, "hfg_diatomic_exchange_host: null argument");
    need((flags & ~(HFG_EXCHANGE_SYMMETRIC | HFG_EXCHANGE_SPLIT)) == 0,
         "hfg_diatomic_exchange_host: unsupported flags");
    d->build_host(P, K, true, (flags & HFG_EXCHANGE_SYMMETRIC) != 0, (flags & HFG_EXCHANGE_SPLIT) != 0);
  });
}

hfg_status hfg_diatomic_dft_grid(hfg_diatomic* d, int lang) {
  return guard([&] {
    need(d != nullptr && lang >= 0, "hfg_diatomic_dft_grid: bad arguments");
    d->setup_xc(lang);
  });
}

static void check_dxc_args(int x_func, int c_func) {
  need(hfg::xc_func_supported(x_func) && hfg::xc_func_supported(c_func),
       "hfg_diatomic_xc: unsupported functional id (supported: 1 lda_x, 7 lda_c_vwn, 12 lda_c_pw, 101 gga_x_pbe, "
       "130 gga_c_pbe)");
}

hfg_status hfg_diatomic_xc(hfg_diatomic* d, int x_func, int c_func, const double* Pa, const double* Pb, double* Ha,
                           double* Hb, double* energies, double thr, void* stream) {
  return guard([&] {
    need(d && Pa && Ha, "hfg_diatomic_xc: null argument");
    need(!Pb || Hb, "hfg_diatomic_xc: an unrestricted call needs Hb");
    check_dxc_args(x_func, c_func);
    d->xc_build(x_func, c_func, Pa, Pb, Ha, Hb, energies, thr, to_stream(stream));
  });
}

hfg_status hfg_diatomic_xc_host(hfg_diatomic* d, int x_func, int c_func, const double* Pa, const double* Pb,
                                double* Ha, double* Hb, double* Exc, double* Nel, double thr) {
  return guard([&] {
    need(d && Pa && Ha, "hfg_diatomic_xc_host: null argument");
    need(!Pb || Hb, "hfg_diatomic_xc_host: an unrestricted call needs Hb");
    check_dxc_args(x_func, c_func);
    d->check_device();
    const size_t bytes = sizeof(double) * (size_t)d->host.nbf * d->host.nbf;
    {
      hfg_abi::AllocStream alloc_on(d->own_stream);
      if (d->h_in.n != bytes) d->h_in.alloc(bytes);
      if (d->h_out.n != bytes) d->h_out.alloc(bytes);
      if (Pb && d->h_in2.n != bytes) d->h_in2.alloc(bytes);
      if (Pb && d->h_out2.n != bytes) d->h_out2.alloc(bytes);
      if (d->h_e.n == 0) d->h_e.alloc(2 * sizeof(double));
    }
    cudaStream_t st = d->own_stream;
    ck(cudaMemcpyAsync(d->h_in.p, Pa, bytes, cudaMemcpyHostToDevice, st), "H2D copy");
    if (Pb) ck(cudaMemcpyAsync(d->h_in2.p, Pb, bytes, cudaMemcpyHostToDevice, st), "H2D copy");
    d->xc_build(x_func, c_func, d->h_in.as<double>(), Pb ? d->h_in2.as<double>() : nullptr, d->h_out.as<double>(),
                Pb ? d->h_out2.as<double>() : nullptr, d->h_e.as<double>(), thr, st);
    double e[2];
    ck(cudaMemcpyAsync(Ha, d->h_out.p, bytes, cudaMemcpyDeviceToHost, st), "D2H copy");
    if (Pb) ck(cudaMemcpyAsync(Hb, d->h_out2.p, bytes, cudaMemcpyDeviceToHost, st), "D2H copy");
    ck(cudaMemcpyAsync(e, d->h_e.p, sizeof(e), cudaMemcpyDeviceToHost, st), "D2H copy");
    ck(cudaStreamSynchronize(st), "stream sync");
    if (Exc) *Exc = e[0];
    if (Nel) *Nel = e[1];
  });
}

hfg_status hfg_diatomic_work(const hfg_diatomic* d, const unsigned char* act, const unsigned char* jk_mask,
                             hfg_diatomic_work_t* w) {
  return guard([&] {
    need(d && w, "hfg_diatomic_work: null argument");
    const hfg::DiatomicHost& H = d->host;
    std::memset(w, 0, sizeof(*w));
    const int nang = H.nang, nel = H.nel;
    // padded tiles, as computed: per (element pair, entry) the two stages of
    // off-diagonal products cost 12 nn^3 flops; per (element, entry) the four
    // exchange-ordered in-element blocks 8 nn^4; the recoupling about 4 flops
    // per (density term, tile element)
    const double n2 = (double)H.nn * H.nn, nn3 = n2 * H.nn, npo = (double)nel * (nel - 1);
    for (int k = 0; k < nang; ++k)
      for (int j = 0; j < nang; ++j) {
        const int jk = j + k * nang;
        if (jk_mask && !jk_mask[jk]) continue;
        for (int ent = H.kjk_ptr[jk]; ent < H.kjk_ptr[jk + 1]; ++ent) {
          const int L = H.kent_L[ent], Ma = H.kent_Ma[ent];
          double terms = 0.0;
          for (int sg = 0; sg < (Ma ? 2 : 1); ++sg) {
            const int M = sg ? -Ma : Ma;
            const int xj = H.al_index(j, L, M), xk = H.al_index(k, L, M);
            for (int uj = H.al_ptr[xj]; uj < H.al_ptr[xj + 1]; ++uj)
              for (int uk = H.al_ptr[xk]; uk < H.al_ptr[xk + 1]; ++uk)
                if (!act || act[H.al_b[uj] + H.al_b[uk] * nang]) terms += 1.0;
          }
          if (terms == 0.0) continue;
          const double off = 12.0 * nn3 * npo, dia = 8.0 * n2 * n2 * nel;
          const double roff = 4.0 * terms * n2 * npo, rdia = 4.0 * terms * n2 * nel;
          w->k_offdiag_flops += off;
          w->k_diag_flops += dia;
          w->k_recouple_flops += roff + rdia;
          w->n_entries += 1.0;
          w->k_offdiag_sym_flops += 0.5 * off;
          w->k_recouple_sym_flops += 0.5 * roff;
          if (j <= k) {
            w->k_diag_sym_flops += dia;
            w->k_recouple_sym_flops += rdia;
            w->n_entries_sym += 1.0;
          }
        }
      }
  });
}

}  // extern "C"

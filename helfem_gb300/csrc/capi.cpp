// C ABI of the engine (declarations and contract in include/helfem_gb300.h).
// Every entry point converts exceptions and CUDA errors into status codes and
// a thread-local message; nothing throws across the boundary.
#include "handle.hpp"
#include "cuda/scf_kernels.cuh"

#include <mutex>

namespace hfg_abi {
thread_local std::string g_err;
thread_local cudaStream_t t_alloc_stream = nullptr;

void retain_pool_memory() {
  static std::mutex mu;
  static std::vector<char> done(64, 0);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
  std::lock_guard<std::mutex> lk(mu);
  if (done[dev]) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
    unsigned long long thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  done[dev] = 1;
}
}
using hfg_abi::g_err;

namespace {

void write_full(const hfg_atom* a, const std::vector<double>& rad, double scale, const std::vector<double>* lrad,
                double* out) {
  const int nr = a->host.rad.nrad, nb = a->host.nbf;
  std::memset(out, 0, sizeof(double) * (size_t)nb * nb);
  for (int ia = 0; ia < a->host.nang; ++ia) {
    const double lf = lrad ? (double)a->host.lval[ia] * (a->host.lval[ia] + 1) : 0.0;
    for (int c = 0; c < nr; ++c)
      for (int r = 0; r < nr; ++r) {
        double v = scale * rad[r + (size_t)c * nr];
        if (lrad) v += lf * (*lrad)[r + (size_t)c * nr];
        out[(size_t)(ia * nr + c) * nb + ia * nr + r] = v;
      }
  }
}

}  // namespace

extern "C" {

const char* hfg_last_error(void) { return g_err.c_str(); }

hfg_status hfg_grid(double rmax, int nelem, int igrid, double zexp, double* bval) {
  return guard([&] {
    need(bval != nullptr && nelem >= 1 && rmax > 0, "hfg_grid: bad arguments");
    std::vector<double> b(nelem + 1);
    switch (igrid) {
      case 1:
        for (int i = 0; i <= nelem; ++i) b[i] = (i == nelem) ? rmax : i * (rmax / nelem);
        break;
      case 2:
        for (int i = 0; i <= nelem; ++i) b[i] = (double)i * i * rmax / ((double)nelem * nelem);
        break;
      case 3:
        for (int i = 0; i <= nelem; ++i) b[i] = rmax * std::pow((double)i / nelem, zexp);
        break;
      case 4: {
        const double up = std::pow(std::log(rmax + 1.0), 1.0 / zexp);
        const double step = up / nelem;
        for (int i = 0; i <= nelem; ++i) {
          const double t = (i == nelem) ? up : i * step;
          b[i] = std::exp(std::pow(t, zexp)) - 1.0;
        }
        break;
      }
      case 5: {
        need(zexp > 0 && zexp < 1, "hfg_grid: geometric grid needs 0 < zexp < 1");
        std::vector<double> hk(nelem);
        hk[nelem - 1] = (1 - zexp) / (1 - std::pow(zexp, nelem)) * rmax;
        for (int i = nelem - 2; i >= 0; --i) hk[i] = zexp * hk[i + 1];
        b[0] = 0;
        for (int i = 0; i < nelem; ++i) b[i + 1] = b[i] + hk[i];
        break;
      }
      default:
        throw std::invalid_argument("hfg_grid: unknown grid type");
    }
    b[0] = 0.0;
    b[nelem] = rmax;
    std::memcpy(bval, b.data(), sizeof(double) * (nelem + 1));
  });
}

hfg_status hfg_angular_basis(int lmax, int mmax, int* nang, int* lval, int* mval) {
  return guard([&] {
    need(nang != nullptr && lmax >= 0 && mmax >= 0, "hfg_angular_basis: bad arguments");
    int n = 0;
    for (int mabs = 0; mabs <= mmax; ++mabs)
      for (int l = mabs; l <= lmax; ++l) {
        if (lval) { lval[n] = l; mval[n] = mabs; }
        ++n;
        if (mabs > 0) {
          if (lval) { lval[n] = l; mval[n] = -mabs; }
          ++n;
        }
      }
    *nang = n;
  });
}

hfg_status hfg_atom_create(const hfg_atom_desc* d, hfg_atom** out) {
  return guard([&] {
    need(d != nullptr && out != nullptr, "hfg_atom_create: null argument");
    need(d->nnodes >= 3 && d->nnodes <= 17, "hfg_atom_create: nnodes must be in 3..17");
    need(d->nelem >= 2, "hfg_atom_create: need at least two elements");
    need(d->bval && d->lval && d->mval && d->nang >= 1, "hfg_atom_create: missing arrays");
    std::vector<double> bval(d->bval, d->bval + d->nelem + 1);
    std::vector<int> lv(d->lval, d->lval + d->nang), mv(d->mval, d->mval + d->nang);
    for (int l : lv) need(l <= 3, "hfg_atom_create: l <= 3 supported");
    std::unique_ptr<hfg_atom> a(new hfg_atom());
    need(d->host_only >= 0 && d->host_only <= 2, "hfg_atom_create: host_only must be 0, 1 or 2");
    // 0: device handle, two-electron tables tabulated on the device;
    // 1: host only; 2: device handle with the host tabulation uploaded
    a->host.build(d->Z, d->nnodes, bval, lv, mv, d->nquad, d->chol_tol, d->host_only != 0);
    if (d->host_only != 1) a->upload();
    *out = a.release();
  });
}

hfg_status hfg_sadatom_create(const hfg_sadatom_desc* d, hfg_atom** out) {
  return guard([&] {
    need(d != nullptr && out != nullptr, "hfg_sadatom_create: null argument");
    need(d->nnodes >= 3 && d->nnodes <= 17, "hfg_sadatom_create: nnodes must be in 3..17");
    need(d->nelem >= 2 && d->bval, "hfg_sadatom_create: need at least two elements");
    need(d->lmax >= 0 && d->lmax <= 3, "hfg_sadatom_create: lmax must be in 0..3");
    need(d->host_only >= 0 && d->host_only <= 2, "hfg_sadatom_create: host_only must be 0, 1 or 2");
    std::vector<double> bval(d->bval, d->bval + d->nelem + 1);
    std::vector<int> lv(d->lmax + 1), mv(d->lmax + 1, 0);
    for (int l = 0; l <= d->lmax; ++l) lv[l] = l;
    std::unique_ptr<hfg_atom> a(new hfg_atom());
    a->host.spherical = true;
    a->host.build(d->Z, d->nnodes, bval, lv, mv, d->nquad, d->chol_tol, d->host_only != 0);
    if (d->host_only != 1) a->upload();
    *out = a.release();
  });
}

// Spherically averaged handles: the l-channel matrices (nblk slices of
// nrad x nrad, column-major, one after the other) <-> the diagonal blocks
// of the (l, 0) basis's nbf x nbf matrix. Host or device pointers.
static void sad_expand(hfg_atom* a, const double* cube, int nblk, cudaStream_t st) {
  const size_t nr = a->host.rad.nrad, nbf = a->host.nbf;
  if (a->sad_in.n != sizeof(double) * nbf * nbf) {
    // allocated stream-ordered on the handle's stream, first used on st
    hfg_abi::AllocStream alloc_on(a->own_stream);
    a->sad_in.alloc(sizeof(double) * nbf * nbf);
    a->sad_out.alloc(sizeof(double) * nbf * nbf);
    ck(cudaStreamSynchronize(a->own_stream), "sync after the staging allocation");
  }
  double* full = a->sad_in.as<double>();
  ck(cudaMemsetAsync(full, 0, sizeof(double) * nbf * nbf, st), "staging clear");
  for (int l = 0; l < nblk; ++l)
    ck(cudaMemcpy2DAsync(full + l * nr + l * nr * nbf, sizeof(double) * nbf, cube + l * nr * nr, sizeof(double) * nr,
                         sizeof(double) * nr, nr, cudaMemcpyDefault, st),
       "channel density in");
}

static void sad_extract(hfg_atom* a, double* cube, int nblk, cudaStream_t st) {
  const size_t nr = a->host.rad.nrad, nbf = a->host.nbf;
  const double* full = a->sad_out.as<double>();
  for (int l = 0; l < nblk; ++l)
    ck(cudaMemcpy2DAsync(cube + l * nr * nr, sizeof(double) * nr, full + l * nr + l * nr * nbf, sizeof(double) * nbf,
                         sizeof(double) * nr, nr, cudaMemcpyDefault, st),
       "channel result out");
}

// kind 0: J of the radial density (one slice in, one out); 1: K of the
// channel densities; 2: the range-separated K
static void sad_call(hfg_atom* a, const double* P, double* out, int kind, int flags, cudaStream_t st) {
  need(a && P && out, "null argument");
  need(a->host.spherical, "not a spherically averaged handle (create it with hfg_sadatom_create)");
  a->check_device();
  const int nblk = kind == 0 ? 1 : a->host.nang;
  sad_expand(a, P, nblk, st);
  double* in = a->sad_in.as<double>();
  double* res = a->sad_out.as<double>();
  hfg_status s = kind == 0   ? hfg_coulomb(a, in, res, st)
                 : kind == 1 ? hfg_exchange_ex(a, in, res, flags, st)
                             : hfg_rs_exchange(a, in, res, flags, st);
  if (s != HFG_OK) throw std::runtime_error(hfg_last_error());
  sad_extract(a, out, nblk, st);
  a->mark_use(st);
}

hfg_status hfg_sadatom_coulomb(hfg_atom* a, const double* P, double* J, void* stream) {
  return guard([&] { sad_call(a, P, J, 0, 0, (cudaStream_t)stream); });
}

hfg_status hfg_sadatom_exchange(hfg_atom* a, const double* P, double* K, int flags, void* stream) {
  return guard([&] { sad_call(a, P, K, 1, flags, (cudaStream_t)stream); });
}

hfg_status hfg_sadatom_rs_exchange(hfg_atom* a, const double* P, double* K, int flags, void* stream) {
  return guard([&] { sad_call(a, P, K, 2, flags, (cudaStream_t)stream); });
}

static void sad_host(hfg_atom* a, const double* P, double* out, int kind, int flags) {
  need(a != nullptr, "null argument");
  sad_call(a, P, out, kind, flags, a->own_stream);
  ck(cudaStreamSynchronize(a->own_stream), "stream sync");
  if (kind != 0 && (flags & HFG_EXCHANGE_SPLIT)) a->tc_check();
}

hfg_status hfg_sadatom_coulomb_host(hfg_atom* a, const double* P, double* J) {
  return guard([&] { sad_host(a, P, J, 0, 0); });
}

hfg_status hfg_sadatom_exchange_host(hfg_atom* a, const double* P, double* K, int flags) {
  return guard([&] { sad_host(a, P, K, 1, flags); });
}

hfg_status hfg_sadatom_rs_exchange_host(hfg_atom* a, const double* P, double* K, int flags) {
  return guard([&] { sad_host(a, P, K, 2, flags); });
}

// XC of the spherically averaged atom: its density is radial, so the XC
// potential block of every channel is that of an s-only basis on the same
// radial grid fed with the radial density (int B_a B_b v_xc dr, the block a
// closed-shell atom's m-resolved solution carries on every (l, m))
static hfg_atom* sad_xc_atom(hfg_atom* a) {
  need(a != nullptr, "null argument");
  need(a->host.spherical, "not a spherically averaged handle (create it with hfg_sadatom_create)");
  a->check_device();
  if (!a->sad_xc) {
    const hfg::AtomHost& H = a->host;
    std::unique_ptr<hfg_atom> s(new hfg_atom());
    s->host.build(H.Z, H.rad.nn, H.rad.bval, std::vector<int>{0}, std::vector<int>{0}, H.nquad, H.chol_tol, true);
    s->upload();
    a->sad_xc = std::move(s);
  }
  return a->sad_xc.get();
}

hfg_status hfg_sadatom_xc(hfg_atom* a, int x_func, int c_func, const double* Pa, const double* Pb, double* Ha,
                          double* Hb, double* energies, double thr, void* stream) {
  return guard([&] {
    hfg_atom* s = sad_xc_atom(a);
    if (hfg_xc(s, x_func, c_func, Pa, Pb, Ha, Hb, energies, thr, stream) != HFG_OK)
      throw std::runtime_error(hfg_last_error());
  });
}

hfg_status hfg_sadatom_xc_host(hfg_atom* a, int x_func, int c_func, const double* Pa, const double* Pb, double* Ha,
                               double* Hb, double* Exc, double* Nel, double thr) {
  return guard([&] {
    hfg_atom* s = sad_xc_atom(a);
    if (hfg_xc_host(s, x_func, c_func, Pa, Pb, Ha, Hb, Exc, Nel, thr) != HFG_OK)
      throw std::runtime_error(hfg_last_error());
  });
}

hfg_status hfg_atom_destroy(hfg_atom* atom) {
  return guard([&] { delete atom; });
}

hfg_status hfg_atom_get_dims(const hfg_atom* a, hfg_atom_dims_t* d) {
  return guard([&] {
    need(a && d, "hfg_atom_get_dims: null argument");
    d->nrad = a->host.rad.nrad;
    d->nang = a->host.nang;
    d->nbf = a->host.nbf;
    d->nelem = a->host.rad.nel;
    d->nnodes = a->host.rad.nn;
    d->NL = a->host.NL;
    d->rmax = a->host.rmax;
  });
}

hfg_status hfg_overlap(const hfg_atom* a, double* S) {
  return guard([&] { need(a && S, "null argument"); write_full(a, a->host.Srad, 1.0, nullptr, S); });
}

hfg_status hfg_kinetic(const hfg_atom* a, double* T) {
  return guard([&] { need(a && T, "null argument"); write_full(a, a->host.Trad, 1.0, &a->host.Tlrad, T); });
}

hfg_status hfg_nuclear(const hfg_atom* a, double* V) {
  return guard([&] { need(a && V, "null argument"); write_full(a, a->host.Vrad, -(double)a->host.Z, nullptr, V); });
}

hfg_status hfg_atom_radial_tables(const hfg_atom* a, int L, int iel, int* ni, double* rsmall, double* rbig,
                                  int* rank, double* chol) {
  return guard([&] {
    need(a != nullptr, "null handle");
    const hfg::AtomHost& H = a->host;
    need(L >= 0 && L < H.NL && iel >= 0 && iel < H.rad.nel, "L or iel out of range");
    const_cast<hfg_atom*>(a)->ensure_host_factors();
    const int nn = H.rad.nn, p0 = H.rad.pfirst(iel), n = H.rad.nfun(iel);
    const size_t le = (size_t)L * H.rad.nel + iel;
    if (ni) *ni = n;
    for (int b = 0; b < n; ++b)
      for (int c = 0; c < n; ++c) {
        if (rsmall) rsmall[c + (size_t)b * n] = H.rs[le * nn * nn + (c + p0) + (size_t)(b + p0) * nn];
        if (rbig) rbig[c + (size_t)b * n] = H.rb[le * nn * nn + (c + p0) + (size_t)(b + p0) * nn];
      }
    if (rank) *rank = H.chol_rank[le];
    if (chol) std::memcpy(chol, H.chol[le].data(), sizeof(double) * H.chol[le].size());
  });
}

hfg_status hfg_gaunt(int L, int M, int l, int m, int lp, double* value) {
  return guard([&] { need(value != nullptr, "null argument"); *value = hfg::gaunt_coeff(L, M, l, m, lp); });
}

hfg_status hfg_coulomb(hfg_atom* a, const double* P, double* J, void* stream) {
  return guard([&] {
    need(a && P && J, "hfg_coulomb: null argument");
    a->check_device();
    ck(hfg::launch_coulomb_fp64(a->dev, a->scr, P, J, true, (cudaStream_t)stream, &a->prof), "coulomb kernels");
    a->mark_use((cudaStream_t)stream);
  });
}

hfg_status hfg_coulomb_ex(hfg_atom* a, const double* P, double* J, int flags, void* stream) {
  return guard([&] {
    need(a && P && J, "hfg_coulomb_ex: null argument");
    need((flags & ~HFG_COULOMB_SPLIT) == 0, "hfg_coulomb_ex: unknown flags");
    a->check_device();
    if (flags & HFG_COULOMB_SPLIT) {
      a->ensure_split_coulomb();
      ck(hfg::launch_coulomb_split(a->dev, a->scr, P, J, true, (cudaStream_t)stream, &a->prof),
         "coulomb kernels (split)");
    } else {
      ck(hfg::launch_coulomb_fp64(a->dev, a->scr, P, J, true, (cudaStream_t)stream, &a->prof), "coulomb kernels");
    }
    a->mark_use((cudaStream_t)stream);
  });
}

hfg_status hfg_coulomb_acc(hfg_atom* a, const double* P, double* F, void* stream) {
  return guard([&] {
    need(a && P && F, "hfg_coulomb_acc: null argument");
    a->check_device();
    ck(hfg::launch_coulomb_fp64(a->dev, a->scr, P, F, false, (cudaStream_t)stream, &a->prof), "coulomb kernels");
    a->mark_use((cudaStream_t)stream);
  });
}

hfg_status hfg_coulomb_noalloc(hfg_atom* a, const double* P, double* J, void* stream) {
  return guard([&] {
    need(a && P && J, "hfg_coulomb_noalloc: null argument");
    a->check_device();
    const size_t n2 = (size_t)a->dev.nn * a->dev.nn;
    const size_t need_jin = (size_t)a->dev.nchan * a->dev.nel * n2;
    const size_t need_all = need_jin + (size_t)a->dev.nchan * a->dev.nel * 2;
    if (need_all > (size_t)HFG_NOALLOC_SCRATCH_DOUBLES)
      throw std::invalid_argument("hfg_coulomb_noalloc: atom needs " + std::to_string(need_all) +
                                  " doubles of Coulomb scratch, the static array holds " +
                                  std::to_string((size_t)HFG_NOALLOC_SCRATCH_DOUBLES));
    double* base = nullptr;
    ck(hfg::noalloc_coulomb_scratch(need_all, &base), "static Coulomb scratch");
    hfg::DevScratch s = a->scr;
    s.jin = base;
    s.jscal = base + need_jin;
    ck(hfg::launch_coulomb_fp64(a->dev, s, P, J, true, (cudaStream_t)stream, nullptr), "coulomb kernels");
    a->mark_use((cudaStream_t)stream);
  });
}

hfg_status hfg_tc_selftest(const float* A, const float* B, float* D, int N, int ksteps, int a_mn_major,
                           int b_mn_major, int swap_offsets) {
  return guard([&] {
    need(A && B && D, "hfg_tc_selftest: null argument");
    need(N >= 16 && N <= 256 && N % 16 == 0 && ksteps >= 1 && ksteps <= 8, "hfg_tc_selftest: bad shape");
    int timed_out = 0;
    ck(hfg::tc_selftest(A, B, D, N, ksteps, a_mn_major ? 1 : 0, b_mn_major ? 1 : 0, swap_offsets ? 1 : 0,
                        &timed_out),
       "tensor-core self-test");
    need(!timed_out, "hfg_tc_selftest: the MMA completion wait ran out");
  });
}

hfg_status hfg_tc_peak(int ctas_per_sm, int iters, double* tflops, double* ms) {
  return guard([&] {
    need(tflops && ms && ctas_per_sm >= 1 && ctas_per_sm <= 2 && iters >= 1, "hfg_tc_peak: bad arguments");
    int timed_out = 0;
    ck(hfg::tc_peak(ctas_per_sm, iters, tflops, ms, &timed_out), "tensor-core peak probe");
    need(!timed_out, "hfg_tc_peak: the MMA completion wait ran out");
  });
}

hfg_status hfg_exchange(hfg_atom* a, const double* P, double* K, void* stream) {
  return hfg_exchange_ex(a, P, K, 0, stream);
}

hfg_status hfg_exchange_ex(hfg_atom* a, const double* P, double* K, int flags, void* stream) {
  return guard([&] {
    need(a && P && K, "hfg_exchange: null argument");
    need((flags & ~(HFG_EXCHANGE_SYMMETRIC | HFG_EXCHANGE_SPLIT)) == 0, "hfg_exchange_ex: unknown flags");
    a->check_device();
    const bool sym = (flags & HFG_EXCHANGE_SYMMETRIC) != 0;
    if (flags & HFG_EXCHANGE_SPLIT) {
      const size_t bytes = sizeof(float2) * (size_t)a->host.nbf * a->host.nbf;
      if (a->s_p2.n != bytes) {
        hfg_abi::AllocStream alloc_on(a->own_stream);
        a->s_p2.alloc(bytes);
        a->scr.p2 = a->s_p2.as<float2>();
        ck(cudaStreamSynchronize(a->own_stream), "sync");
      }
      ck(hfg::launch_exchange_split(a->dev, a->scr, a->units, P, K, sym, (cudaStream_t)stream, &a->prof,
                                    a->tc_for(false), a->side_stream()),
         "exchange kernels (split)");
    } else {
      ck(hfg::launch_exchange_fp64(a->dev, a->scr, a->units, P, K, sym, (cudaStream_t)stream, &a->prof),
         "exchange kernels");
    }
    a->mark_use((cudaStream_t)stream);
  });
}

// Host density -> device. A density the caller declares symmetric
// (HFG_EXCHANGE_SYMMETRIC) crosses the host link as its lower column blocks
// only (16 blocks of columns, each from its first column's row down:
// about 53 % of the bytes), and the device mirrors the rest; otherwise one
// full copy. Returns the bytes copied.
static size_t upload_density(double* dst, const double* src, int n, bool symmetric, cudaStream_t st) {
  const size_t ld = sizeof(double) * (size_t)n;
  if (!symmetric || n < 64) {
    ck(cudaMemcpyAsync(dst, src, ld * n, cudaMemcpyHostToDevice, st), "H2D copy");
    return ld * n;
  }
  const int bw = (n + 15) / 16;
  size_t bytes = 0;
  for (int c0 = 0; c0 < n; c0 += bw) {
    const int w = std::min(bw, n - c0);
    const size_t off = (size_t)c0 + (size_t)c0 * n, rows = (size_t)(n - c0);
    ck(cudaMemcpy2DAsync(dst + off, ld, src + off, ld, sizeof(double) * rows, w, cudaMemcpyHostToDevice, st),
       "H2D copy");
    bytes += sizeof(double) * rows * w;
  }
  ck(hfg::launch_mirror_blocks(dst, n, bw, st), "density mirror");
  return bytes;
}

static void host_call(hfg_atom* a, const double* P, double* out, bool coulomb, int flags, bool screened = false) {
  need(a && P && out, "null argument");
  need((flags & ~(HFG_EXCHANGE_SYMMETRIC | HFG_EXCHANGE_SPLIT)) == 0, "unknown flags");
  a->check_device();
  if (screened && !a->rs_ready)
    throw std::logic_error("Primitive teis have not been computed!\n");
  const hfg::DevAtom& ctx = screened ? a->dev_rs : a->dev;
  a->staging();
  const size_t bytes = sizeof(double) * (size_t)a->host.nbf * a->host.nbf;
  cudaStream_t st = a->own_stream;
  a->last_h2d = upload_density(a->h_in.as<double>(), P, a->host.nbf, !coulomb && (flags & HFG_EXCHANGE_SYMMETRIC), st);
  if (!coulomb && screened && a->rs_erfc) {
    need((flags & HFG_EXCHANGE_SPLIT) == 0, "the erfc kernel has no split form");
    ck(hfg::launch_exchange_erfc(a->dev, a->scr, a->d_etk.as<double>(), a->h_in.as<double>(),
                                 a->h_out.as<double>(), st, &a->prof),
       "erfc exchange");
  } else if (coulomb) {
    ck(hfg::launch_coulomb_fp64(a->dev, a->scr, a->h_in.as<double>(), a->h_out.as<double>(), true, st, &a->prof),
       "coulomb");
  } else if (flags & HFG_EXCHANGE_SPLIT) {
    const size_t b2 = sizeof(float2) * (size_t)a->host.nbf * a->host.nbf;
    if (a->s_p2.n != b2) {
      hfg_abi::AllocStream alloc_on(a->own_stream);
      a->s_p2.alloc(b2);
      a->scr.p2 = a->s_p2.as<float2>();
    }
    ck(hfg::launch_exchange_split(ctx, a->scr, a->units, a->h_in.as<double>(), a->h_out.as<double>(),
                                  (flags & HFG_EXCHANGE_SYMMETRIC) != 0, st, &a->prof, a->tc_for(screened),
                                  a->side_stream()),
       "exchange (split)");
  } else {
    ck(hfg::launch_exchange_fp64(ctx, a->scr, a->units, a->h_in.as<double>(), a->h_out.as<double>(),
                                 (flags & HFG_EXCHANGE_SYMMETRIC) != 0, st, &a->prof),
       "exchange");
  }
  ck(cudaMemcpyAsync(out, a->h_out.p, bytes, cudaMemcpyDeviceToHost, st), "D2H copy");
  a->last_d2h = bytes;
  ck(cudaStreamSynchronize(st), "stream sync");
  if (!coulomb && (flags & HFG_EXCHANGE_SPLIT)) a->tc_check();
}

// J(PJ) and K(PK) with one staging of the density when PK == PJ, the
// exchange build running while J is copied back on a second stream
static void jk_host(hfg_atom* a, const double* PJ, const double* PK, double* J, double* K, int flags) {
  need(a && PJ && PK && J && K, "null argument");
  need((flags & ~(HFG_EXCHANGE_SYMMETRIC | HFG_EXCHANGE_SPLIT | HFG_COULOMB_SPLIT)) == 0, "unknown flags");
  a->check_device();
  a->staging();
  const size_t bytes = sizeof(double) * (size_t)a->host.nbf * a->host.nbf;
  cudaStream_t st = a->own_stream;
  if (!a->copy_stream) ck(cudaStreamCreateWithFlags(&a->copy_stream, cudaStreamNonBlocking), "cudaStreamCreate");
  if (!a->ev_j) ck(cudaEventCreateWithFlags(&a->ev_j, cudaEventDisableTiming), "cudaEventCreate");
  const bool same = (PK == PJ);
  if (!same) {
    hfg_abi::AllocStream alloc_on(st);
    if (a->h_in2.n != bytes) a->h_in2.alloc(bytes);
  }
  {
    hfg_abi::AllocStream alloc_on(st);
    if (a->h_out2.n != bytes) a->h_out2.alloc(bytes);
  }
  // PJ is promised symmetric only when it is PK itself
  const bool sym = (flags & HFG_EXCHANGE_SYMMETRIC) != 0;
  a->last_h2d = upload_density(a->h_in.as<double>(), PJ, a->host.nbf, sym && same, st);
  if (flags & HFG_COULOMB_SPLIT) {
    a->ensure_split_coulomb();
    ck(hfg::launch_coulomb_split(a->dev, a->scr, a->h_in.as<double>(), a->h_out.as<double>(), true, st, &a->prof),
       "coulomb (split)");
  } else {
    ck(hfg::launch_coulomb_fp64(a->dev, a->scr, a->h_in.as<double>(), a->h_out.as<double>(), true, st, &a->prof),
       "coulomb");
  }
  ck(cudaEventRecord(a->ev_j, st), "event");
  ck(cudaStreamWaitEvent(a->copy_stream, a->ev_j, 0), "wait");
  ck(cudaMemcpyAsync(J, a->h_out.p, bytes, cudaMemcpyDeviceToHost, a->copy_stream), "D2H copy");
  const double* Pk = a->h_in.as<double>();
  if (!same) {
    a->last_h2d += upload_density(a->h_in2.as<double>(), PK, a->host.nbf, sym, st);
    Pk = a->h_in2.as<double>();
  }
  if (flags & HFG_EXCHANGE_SPLIT) {
    const size_t b2 = sizeof(float2) * (size_t)a->host.nbf * a->host.nbf;
    if (a->s_p2.n != b2) {
      hfg_abi::AllocStream alloc_on(st);
      a->s_p2.alloc(b2);
      a->scr.p2 = a->s_p2.as<float2>();
    }
    ck(hfg::launch_exchange_split(a->dev, a->scr, a->units, Pk, a->h_out2.as<double>(),
                                  (flags & HFG_EXCHANGE_SYMMETRIC) != 0, st, &a->prof, a->tc_for(false),
                                  a->side_stream()),
       "exchange (split)");
  } else {
    ck(hfg::launch_exchange_fp64(a->dev, a->scr, a->units, Pk, a->h_out2.as<double>(),
                                 (flags & HFG_EXCHANGE_SYMMETRIC) != 0, st, &a->prof),
       "exchange");
  }
  ck(cudaMemcpyAsync(K, a->h_out2.p, bytes, cudaMemcpyDeviceToHost, st), "D2H copy");
  a->last_d2h = 2 * bytes;
  ck(cudaStreamSynchronize(st), "stream sync");
  ck(cudaStreamSynchronize(a->copy_stream), "stream sync");
  if (flags & HFG_EXCHANGE_SPLIT) a->tc_check();
}

hfg_status hfg_jk(hfg_atom* a, const double* PJ, const double* PK, double* J, double* K, int flags, void* stream) {
  return guard([&] {
    need(a && PJ && PK && J && K, "hfg_jk: null argument");
    need((flags & ~(HFG_EXCHANGE_SYMMETRIC | HFG_EXCHANGE_SPLIT | HFG_COULOMB_SPLIT)) == 0, "hfg_jk: unknown flags");
    need(J != K, "hfg_jk: J and K must be different buffers");
    a->check_device();
    cudaStream_t st = (cudaStream_t)stream;
    if (!a->j_stream) ck(cudaStreamCreateWithFlags(&a->j_stream, cudaStreamNonBlocking), "cudaStreamCreate");
    if (!a->ev_fork) ck(cudaEventCreateWithFlags(&a->ev_fork, cudaEventDisableTiming), "cudaEventCreate");
    if (!a->ev_join) ck(cudaEventCreateWithFlags(&a->ev_join, cudaEventDisableTiming), "cudaEventCreate");
    const bool split_k = (flags & HFG_EXCHANGE_SPLIT) != 0, split_j = (flags & HFG_COULOMB_SPLIT) != 0;
    if (split_j) a->ensure_split_coulomb();
    if (split_k) {
      const size_t bytes = sizeof(float2) * (size_t)a->host.nbf * a->host.nbf;
      if (a->s_p2.n != bytes) {
        hfg_abi::AllocStream alloc_on(a->own_stream);
        a->s_p2.alloc(bytes);
        a->scr.p2 = a->s_p2.as<float2>();
        ck(cudaStreamSynchronize(a->own_stream), "sync");
      }
    }
    // J on the handle's second stream, after everything already on `stream`
    ck(cudaEventRecord(a->ev_fork, st), "event");
    ck(cudaStreamWaitEvent(a->j_stream, a->ev_fork, 0), "wait");
    if (split_j)
      ck(hfg::launch_coulomb_split(a->dev, a->scr, PJ, J, true, a->j_stream, &a->prof), "coulomb kernels (split)");
    else
      ck(hfg::launch_coulomb_fp64(a->dev, a->scr, PJ, J, true, a->j_stream, &a->prof), "coulomb kernels");
    ck(cudaEventRecord(a->ev_join, a->j_stream), "event");
    // K on the caller's stream meanwhile
    const bool sym = (flags & HFG_EXCHANGE_SYMMETRIC) != 0;
    if (split_k)
      ck(hfg::launch_exchange_split(a->dev, a->scr, a->units, PK, K, sym, st, &a->prof, a->tc_for(false),
                                    a->side_stream()),
         "exchange kernels (split)");
    else
      ck(hfg::launch_exchange_fp64(a->dev, a->scr, a->units, PK, K, sym, st, &a->prof), "exchange kernels");
    ck(cudaStreamWaitEvent(st, a->ev_join, 0), "join");
    a->mark_use(st);
  });
}

hfg_status hfg_jk_host(hfg_atom* a, const double* PJ, const double* PK, double* J, double* K, int flags) {
  return guard([&] { jk_host(a, PJ, PK, J, K, flags); });
}

hfg_status hfg_host_copy_bytes(const hfg_atom* a, size_t* h2d, size_t* d2h) {
  return guard([&] {
    need(a && h2d && d2h, "hfg_host_copy_bytes: null argument");
    *h2d = a->last_h2d;
    *d2h = a->last_d2h;
  });
}

// Autotuner: times the exchange tile kernel for candidate partitions of the
// work units (output-block ranges per element pair) on a synthetic density
// with every block active, keeps the fastest
hfg_status hfg_atom_autotune(hfg_atom* a, int flags, int* best_nsplit, double* best_ms) {
  return guard([&] {
    need(a != nullptr, "hfg_atom_autotune: null argument");
    need((flags & ~(HFG_EXCHANGE_SYMMETRIC | HFG_EXCHANGE_SPLIT)) == 0, "unknown flags");
    a->check_device();
    cudaStream_t st = a->own_stream;
    hfg_abi::AllocStream alloc_on(st);
    const size_t n = (size_t)a->host.nbf, bytes = sizeof(double) * n * n;
    DBuf P, K;
    P.alloc(bytes);
    K.alloc(bytes);
    hfg::fill_test_density(P.as<double>(), (int)n, st);
    if ((flags & HFG_EXCHANGE_SPLIT) && a->s_p2.n != sizeof(float2) * n * n) {
      a->s_p2.alloc(sizeof(float2) * n * n);
      a->scr.p2 = a->s_p2.as<float2>();
    }
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "event");
    ck(cudaEventCreate(&e1), "event");
    auto run = [&]() {
      const bool sym = (flags & HFG_EXCHANGE_SYMMETRIC) != 0;
      if (flags & HFG_EXCHANGE_SPLIT)
        ck(hfg::launch_exchange_split(a->dev, a->scr, a->units, P.as<double>(), K.as<double>(), sym, st, nullptr,
                                      a->tc_for(false), a->side_stream()),
           "exchange");
      else
        ck(hfg::launch_exchange_fp64(a->dev, a->scr, a->units, P.as<double>(), K.as<double>(), sym, st, nullptr),
           "exchange");
    };
    double best = 1e300;
    int bestn = 0;
    // the tensor-core split form: groups of 8 output blocks per element-pair
    // unit; otherwise output-block ranges per element pair
    const bool tcform = (flags & HFG_EXCHANGE_SPLIT) && a->tc_for(false) != nullptr;
    const std::vector<int> cand = tcform ? std::vector<int>{0, 1, 2, 3, 4, 6, a->tc.ngroups}
                                         : std::vector<int>{0, 1, 2, 4, 8, 16};
    for (int ns : cand) {
      if (tcform) {
        ck(cudaStreamSynchronize(st), "sync");
        a->tc_per_fixed = ns;
        a->tc_units();
      } else {
        a->nsplit_fixed = ns;
        a->build_units();
      }
      run();
      ck(cudaEventRecord(e0, st), "event");
      for (int r = 0; r < 3; ++r) run();
      ck(cudaEventRecord(e1, st), "event");
      ck(cudaEventSynchronize(e1), "sync");
      float ms = 0.f;
      ck(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
      if (ms / 3.0 < best) {
        best = ms / 3.0;
        bestn = ns;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ck(cudaStreamSynchronize(st), "sync");
    if (tcform) {
      a->tc_per_fixed = bestn;
      a->tc_units();
    } else {
      a->nsplit_fixed = bestn;
      a->build_units();
    }
    ck(cudaStreamSynchronize(st), "sync");
    if (best_nsplit) *best_nsplit = bestn;
    if (best_ms) *best_ms = best;
  });
}

hfg_status hfg_atom_set_partition(hfg_atom* a, int nsplit) {
  return guard([&] {
    need(a != nullptr && nsplit >= 0, "hfg_atom_set_partition: bad arguments");
    a->check_device();
    hfg_abi::AllocStream alloc_on(a->own_stream);
    ck(cudaStreamSynchronize(a->own_stream), "sync");
    a->nsplit_fixed = nsplit;
    a->build_units();
    if (a->tc_ok) {
      a->tc_per_fixed = nsplit;
      a->tc_units();
    }
    ck(cudaStreamSynchronize(a->own_stream), "sync");
  });
}

hfg_status hfg_atom_compute_yukawa(hfg_atom* a, double lambda) {
  return guard([&] {
    need(a != nullptr && lambda > 0.0, "hfg_atom_compute_yukawa: bad arguments");
    if (a->on_device)
      a->setup_yukawa(lambda);
    else
      a->host.build_yukawa(lambda);  // host-only handle: tables for checking
  });
}

hfg_status hfg_atom_compute_erfc(hfg_atom* a, double mu, int flags) {
  return guard([&] {
    need(a != nullptr && mu > 0.0, "hfg_atom_compute_erfc: bad arguments");
    need((flags & ~HFG_ERFC_EXACT_BINOMIAL) == 0, "hfg_atom_compute_erfc: unknown flags");
    const bool exact = (flags & HFG_ERFC_EXACT_BINOMIAL) != 0;
    if (a->on_device)
      a->setup_erfc(mu, exact);
    else
      a->host.build_erfc(mu, exact);  // host-only handle: tables for checking
  });
}

hfg_status hfg_atom_erfc_table(const hfg_atom* a, int L, int iel, int kel, double* out) {
  return guard([&] {
    need(a != nullptr && out != nullptr, "hfg_atom_erfc_table: null argument");
    const hfg::AtomHost& H = a->host;
    need(H.e_mu > 0.0, "hfg_atom_erfc_table: hfg_atom_compute_erfc has not been called");
    need(L >= 0 && L < H.NL && iel >= 0 && iel < H.rad.nel && kel >= 0 && kel < H.rad.nel,
         "hfg_atom_erfc_table: L, iel or kel out of range");
    const size_t n2 = (size_t)H.rad.nn * H.rad.nn;
    const size_t o = (((size_t)L * H.rad.nel + iel) * H.rad.nel + kel) * n2 * n2;
    std::copy(H.e_tk.begin() + o, H.e_tk.begin() + o + n2 * n2, out);
  });
}

hfg_status hfg_atom_yukawa_tables(const hfg_atom* a, int L, int iel, double* rsmall, double* rbig, double* tk) {
  return guard([&] {
    need(a != nullptr, "hfg_atom_yukawa_tables: null handle");
    const hfg::AtomHost& H = a->host;
    need(H.y_lambda > 0.0, "hfg_atom_yukawa_tables: hfg_atom_compute_yukawa has not been called");
    need(L >= 0 && L < H.NL && iel >= 0 && iel < H.rad.nel, "hfg_atom_yukawa_tables: L or iel out of range");
    const size_t n2 = (size_t)H.rad.nn * H.rad.nn, le = (size_t)L * H.rad.nel + iel;
    if (rsmall) std::copy(H.y_rs.begin() + le * n2, H.y_rs.begin() + (le + 1) * n2, rsmall);
    if (rbig) std::copy(H.y_rb.begin() + le * n2, H.y_rb.begin() + (le + 1) * n2, rbig);
    if (tk) std::copy(H.y_tk.begin() + le * n2 * n2, H.y_tk.begin() + (le + 1) * n2 * n2, tk);
  });
}

hfg_status hfg_rs_exchange(hfg_atom* a, const double* P, double* K, int flags, void* stream) {
  return guard([&] {
    need(a && P && K, "hfg_rs_exchange: null argument");
    need((flags & ~(HFG_EXCHANGE_SYMMETRIC | HFG_EXCHANGE_SPLIT)) == 0, "hfg_rs_exchange: unknown flags");
    a->check_device();
    if (!a->rs_ready) throw std::logic_error("Primitive teis have not been computed!\n");
    const bool sym = (flags & HFG_EXCHANGE_SYMMETRIC) != 0;
    if (a->rs_erfc) {
      need((flags & HFG_EXCHANGE_SPLIT) == 0, "hfg_rs_exchange: the erfc kernel has no split form");
      ck(hfg::launch_exchange_erfc(a->dev, a->scr, a->d_etk.as<double>(), P, K, (cudaStream_t)stream, &a->prof),
         "erfc exchange");
    } else if (flags & HFG_EXCHANGE_SPLIT) {
      const size_t b2 = sizeof(float2) * (size_t)a->host.nbf * a->host.nbf;
      if (a->s_p2.n != b2) {
        hfg_abi::AllocStream alloc_on(a->own_stream);
        a->s_p2.alloc(b2);
        a->scr.p2 = a->s_p2.as<float2>();
      }
      ck(hfg::launch_exchange_split(a->dev_rs, a->scr, a->units, P, K, sym, (cudaStream_t)stream, &a->prof,
                                    a->tc_for(true), a->side_stream()),
         "screened exchange (split)");
    } else {
      ck(hfg::launch_exchange_fp64(a->dev_rs, a->scr, a->units, P, K, sym, (cudaStream_t)stream, &a->prof),
         "screened exchange");
    }
    a->mark_use((cudaStream_t)stream);
  });
}

hfg_status hfg_rs_exchange_host(hfg_atom* a, const double* P, double* K, int flags) {
  return guard([&] { host_call(a, P, K, false, flags, true); });
}

hfg_status hfg_coulomb_host(hfg_atom* a, const double* P, double* J) {
  return guard([&] { host_call(a, P, J, true, 0); });
}

hfg_status hfg_exchange_host(hfg_atom* a, const double* P, double* K) {
  return guard([&] { host_call(a, P, K, false, 0); });
}

hfg_status hfg_exchange_host_ex(hfg_atom* a, const double* P, double* K, int flags) {
  return guard([&] { host_call(a, P, K, false, flags); });
}

hfg_status hfg_atom_tc_work(const hfg_atom* a, int symmetric, double* mma_flops) {
  return guard([&] {
    need(a != nullptr && mma_flops != nullptr, "hfg_atom_tc_work: null argument");
    a->check_device();
    *mma_flops = a->tc_ok ? a->tc_mma_flops[symmetric ? 0 : 1] : 0.0;
  });
}

hfg_status hfg_atom_work(const hfg_atom* a, hfg_work_t* w) {
  return guard([&] {
    need(a != nullptr && w != nullptr, "hfg_atom_work: null argument");
    const hfg::AtomHost& H = a->host;
    const int nel = H.rad.nel;
    std::vector<double> N(nel);
    double S2 = 0.0;
    for (int e = 0; e < nel; ++e) { N[e] = H.rad.nfun(e); S2 += N[e] * N[e]; }
    double off_pair = 0.0, off_prod = 0.0, diag_pair = 0.0, diag_prod = 0.0;
    for (int x = 0; x < nel; ++x)
      for (int y = 0; y < nel; ++y) {
        if (x == y) {
          diag_pair += N[x] * N[x];
          diag_prod += 2.0 * N[x] * N[x] * N[x] * N[x];
        } else {
          off_pair += N[x] * N[y];
          off_prod += 2.0 * N[x] * N[x] * N[y] + 2.0 * N[x] * N[y] * N[y];
        }
      }
    const double nent = (double)H.kent_L.size(), nterm = (double)H.kterm_blk.size();
    w->n_k_entries = (int)H.kent_L.size();
    w->n_k_terms = (int)H.kterm_blk.size();
    w->k_offdiag_flops = nent * off_prod + 2.0 * nterm * off_pair;
    w->k_diag_flops = nent * diag_prod + 2.0 * nterm * diag_pair;
    // symmetric mode: pairs a < b, diagonal blocks j <= k
    double sent = 0.0, sterm = 0.0;
    for (int k = 0; k < H.nang; ++k)
      for (int j = 0; j <= k; ++j) {
        const int jk = j + k * H.nang;
        for (int e = H.kjk_ptr[jk]; e < H.kjk_ptr[jk + 1]; ++e) {
          sent += 1.0;
          sterm += H.kent_ptr[e + 1] - H.kent_ptr[e];
        }
      }
    w->k_offdiag_sym_flops = 0.5 * w->k_offdiag_flops;
    w->k_diag_sym_flops = sent * diag_prod + 2.0 * sterm * diag_pair;
    w->k_bytes = 16.0 * (double)H.nbf * H.nbf;
    double jf = 0.0;
    for (size_t ch = 0; ch < H.chans.size(); ++ch) {
      const double nket = H.jket_ptr[ch + 1] - H.jket_ptr[ch];
      const int L = H.chans[ch].L;
      for (int e = 0; e < nel; ++e)
        jf += 2.0 * nket * N[e] * N[e] + 4.0 * N[e] * N[e] + 4.0 * N[e] * N[e] * H.chol_rank[(size_t)L * nel + e];
    }
    jf += 6.0 * (double)H.jbra_chan.size() * S2;
    w->j_flops = jf;
    w->j_bytes = 16.0 * (double)H.nang * H.nang * S2;
  });
}

hfg_status hfg_dft_grid(hfg_atom* a, int ldft, int mdft) {
  return guard([&] {
    need(a != nullptr && ldft >= 0 && mdft >= 0, "hfg_dft_grid: bad arguments");
    a->check_device();
    a->setup_xc(ldft, mdft);
  });
}

static void check_xc_args(int x_func, int c_func) {
  need(hfg::xc_func_supported(x_func) && hfg::xc_func_supported(c_func),
       "hfg_xc: unsupported functional id (supported: 1 lda_x, 7 lda_c_vwn, 12 lda_c_pw, 101 gga_x_pbe, "
       "130 gga_c_pbe)");
}

hfg_status hfg_xc(hfg_atom* a, int x_func, int c_func, const double* Pa, const double* Pb, double* Ha, double* Hb,
                  double* energies, double thr, void* stream) {
  return guard([&] {
    need(a && Pa && Ha, "hfg_xc: null argument");
    need(!Pb || Hb, "hfg_xc: an unrestricted call needs Hb");
    check_xc_args(x_func, c_func);
    a->check_device();
    if (!a->xc_ready) a->setup_xc(0, 0);
    ck(hfg::launch_xc_fp64(a->dev, a->xc, a->xs, x_func, c_func, Pa, Pb, Ha, Hb, energies, thr,
                           (cudaStream_t)stream),
       "xc kernels");
    a->mark_use((cudaStream_t)stream);
  });
}

hfg_status hfg_xc_host(hfg_atom* a, int x_func, int c_func, const double* Pa, const double* Pb, double* Ha,
                       double* Hb, double* Exc, double* Nel, double thr) {
  return guard([&] {
    need(a && Pa && Ha, "hfg_xc_host: null argument");
    need(!Pb || Hb, "hfg_xc_host: an unrestricted call needs Hb");
    check_xc_args(x_func, c_func);
    a->check_device();
    if (!a->xc_ready) a->setup_xc(0, 0);
    a->staging();
    const size_t bytes = sizeof(double) * (size_t)a->host.nbf * a->host.nbf;
    {
      hfg_abi::AllocStream alloc_on(a->own_stream);
      if (Pb) {
        if (a->h_in2.n != bytes) a->h_in2.alloc(bytes);
        if (a->h_out2.n != bytes) a->h_out2.alloc(bytes);
      }
      if (a->h_e.n == 0) a->h_e.alloc(2 * sizeof(double));
    }
    cudaStream_t st = a->own_stream;
    ck(cudaMemcpyAsync(a->h_in.p, Pa, bytes, cudaMemcpyHostToDevice, st), "H2D copy");
    if (Pb) ck(cudaMemcpyAsync(a->h_in2.p, Pb, bytes, cudaMemcpyHostToDevice, st), "H2D copy");
    ck(hfg::launch_xc_fp64(a->dev, a->xc, a->xs, x_func, c_func, a->h_in.as<double>(),
                           Pb ? a->h_in2.as<double>() : nullptr, a->h_out.as<double>(),
                           Pb ? a->h_out2.as<double>() : nullptr, a->h_e.as<double>(), thr, st),
       "xc kernels");
    double e[2];
    ck(cudaMemcpyAsync(Ha, a->h_out.p, bytes, cudaMemcpyDeviceToHost, st), "D2H copy");
    if (Pb) ck(cudaMemcpyAsync(Hb, a->h_out2.p, bytes, cudaMemcpyDeviceToHost, st), "D2H copy");
    ck(cudaMemcpyAsync(e, a->h_e.p, sizeof(e), cudaMemcpyDeviceToHost, st), "D2H copy");
    ck(cudaStreamSynchronize(st), "stream sync");
    if (Exc) *Exc = e[0];
    if (Nel) *Nel = e[1];
  });
}

hfg_status hfg_profile_enable(hfg_atom* a, int capacity) {
  return guard([&] {
    need(a != nullptr && capacity >= 0, "hfg_profile_enable: bad arguments");
    a->check_device();
    a->enable_profiler(capacity);
  });
}

hfg_status hfg_profile_classes(hfg_atom* a, unsigned mask) {
  return guard([&] {
    need(a != nullptr, "hfg_profile_classes: null argument");
    a->prof.mask = mask;
  });
}

hfg_status hfg_profile_read(hfg_atom* a, hfg_profile_t* out, int reset) {
  return guard([&] {
    need(a != nullptr && out != nullptr, "hfg_profile_read: null argument");
    std::memset(out, 0, sizeof(*out));
    for (int i = 0; i < a->prof.n; ++i) {
      ck(cudaEventSynchronize(a->prof.ev[2 * i + 1]), "cudaEventSynchronize");
      float ms = 0.f;
      ck(cudaEventElapsedTime(&ms, a->prof.ev[2 * i], a->prof.ev[2 * i + 1]), "cudaEventElapsedTime");
      const int k = a->prof.cls[i];
      out->launches[k] += 1;
      out->ms[k] += ms;
    }
    if (reset) a->prof.n = 0;
  });
}

}  // extern "C"

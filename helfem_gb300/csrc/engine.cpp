// Batched / serving runtime for atomic SCF solves on one GPU.
//
// The reference solves one atom per process (src/atomic/main.cpp); many-atom
// throughput there means many processes (tests/run_tests.py --jobs). Here a
// native engine keeps the GPU busy with many solves at once:
//  * N worker threads, each with its own CUDA stream and cuBLAS/cuSOLVER
//    handles, run whole solves (host tabulation, upload, device SCF);
//  * admission by HBM footprint: a queued job starts only when its estimated
//    device footprint fits in the budget still free (first fitting job in
//    arrival order), so small requests flow past a large one while memory is
//    short and the budget is never oversubscribed;
//  * every device buffer of a job is stream-ordered on its worker's stream,
//    so solves overlap on the device without allocation syncs;
//  * per-job timestamps give queue wait, set-up and SCF time.
// A job's result does not depend on what else runs (each solve owns its
// buffers and runs in a fixed operation order), which the tests check.
#include <cublas_v2.h>
#include <cusolverDn.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>

#include "handle.hpp"

void hfg_scf_impl(hfg_atom* a, const hfg_scf_desc* d, hfg_scf_result* res, double* orbital_energies,
                  cudaStream_t stream, cublasHandle_t bl, cusolverDnHandle_t so);

namespace {

using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t0, Clock::time_point t1) {
  return std::chrono::duration<double, std::milli>(t1 - t0).count();
}

struct Job {
  unsigned long long id = 0;
  // owned copies of the caller's arrays
  std::vector<double> bval;
  std::vector<int> lval, mval, fixed;
  std::vector<double> l_occ;
  hfg_atom_desc atom{};
  hfg_scf_desc scf{};
  size_t footprint = 0;
  int status = 0;  // 0 queued, 1 running, 2 done, 3 failed
  hfg_scf_result res{};
  Clock::time_point t_submit, t_start, t_setup, t_end;
  std::string error;
};

}  // namespace

// Device bytes a solve will hold (tables, Fock-build scratch, SCF buffers,
// DFT grid), from the basis dimensions alone.
size_t hfg_job_footprint(const hfg_atom_desc& a, const hfg_scf_desc& s) {
  const double nn = a.nnodes, nel = a.nelem, n2 = nn * nn;
  int lmax = 0, mmx = 0;
  for (int i = 0; i < a.nang; ++i) {
    lmax = std::max(lmax, a.lval[i]);
    mmx = std::max(mmx, std::abs(a.mval[i]));
  }
  const double NL = 2 * lmax + 1, nang = a.nang, nrad = nel * (nn - 1) - 1, nbf = nang * nrad;
  const double rmax = std::min(n2, 2 * nn - 1);
  double b = 8.0 * NL * nel * (4 * n2 + n2 * rmax + 2 * n2 * n2);  // rs, rb (+split), factor, tensor (+split)
  b += 8.0 * nel * nel * nang * nang * (2 * nn - 1);                // exchange halo
  b += 8.0 * NL * NL * nel * (n2 + 2);                              // Coulomb scratch (channel bound)
  const int nspin = s.restricted ? 1 : 2;
  b += 8.0 * nbf * nbf * 13;                                        // T V H P Ps J K XC F
  b += 8.0 * nbf * nbf * 0.5 * nspin * 20;                          // blocks, eigenvectors, DIIS history
  // device tabulation scratch (pair-packed tensor, full-width factor), freed
  // before the SCF buffers are allocated
  const double tab = 8.0 * NL * nel * (1.5 * n2 * n2);
  b += std::max(0.0, tab - 8.0 * nbf * nbf * (13 + 10 * nspin));
  if (s.x_func || s.c_func) {
    const double nq = a.nquad > 0 ? a.nquad : 5 * nn, nap = (4.0 * lmax + 12) * (4.0 * mmx + 12);
    b += 8.0 * (4 * nel * nang * nang * nq + 8 * nel * nq * nap + 8 * nel * nang * nang * nq + 3 * nang * nang * nap);
  }
  return (size_t)(b * 1.05) + (64u << 20);
}

struct hfg_engine {
  int device = 0;
  size_t budget = 0, in_use = 0;
  int running = 0;
  std::atomic<unsigned long long> next_id{1};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Job*> queue;
  std::map<unsigned long long, std::unique_ptr<Job>> jobs;
  std::vector<std::thread> workers;
  bool stop = false;
  int waiters = 0;  // threads inside hfg_engine_wait (destroy waits for them to leave)
  int omp_threads = 1;

  Job* pick_locked() {
    for (auto it = queue.begin(); it != queue.end(); ++it) {
      Job* j = *it;
      // a job larger than the whole budget runs alone rather than never
      if (j->footprint + in_use <= budget || (running == 0 && j->footprint > budget)) {
        queue.erase(it);
        return j;
      }
    }
    return nullptr;
  }

  void worker_main() {
    cudaSetDevice(device);
#ifdef _OPENMP
    omp_set_num_threads(omp_threads);
#endif
    cudaStream_t st = nullptr;
    cublasHandle_t bl = nullptr;
    cusolverDnHandle_t so = nullptr;
    const bool ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
                    cublasCreate(&bl) == CUBLAS_STATUS_SUCCESS && cublasSetStream(bl, st) == CUBLAS_STATUS_SUCCESS &&
                    cusolverDnCreate(&so) == CUSOLVER_STATUS_SUCCESS &&
                    cusolverDnSetStream(so, st) == CUSOLVER_STATUS_SUCCESS;
    for (;;) {
      Job* job = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || (job = pick_locked()) != nullptr; });
        if (!job) break;  // stopping
        in_use += job->footprint;
        ++running;
        job->status = 1;
        job->t_start = Clock::now();
      }
      std::string err;
      hfg_scf_result res{};
      Clock::time_point t_setup = Clock::now();
      if (!ok) {
        err = "worker could not create its CUDA stream or library handles";
      } else {
        try {
          std::unique_ptr<hfg_atom> atom(new hfg_atom());
          atom->host.build(job->atom.Z, job->atom.nnodes, job->bval, job->lval, job->mval, job->atom.nquad,
                           job->atom.chol_tol, job->atom.host_only == 2);
          atom->own_stream = st;  // the worker's stream; the atom does not own it
          atom->upload();
          t_setup = Clock::now();
          hfg_scf_impl(atom.get(), &job->scf, &res, nullptr, st, bl, so);
          atom.reset();
          if (cudaStreamSynchronize(st) != cudaSuccess) err = "stream error after the solve";
          // an unconverged solve is a failed request, not an energy
          else if (!res.converged)
            err = "SCF did not converge in " + std::to_string(res.iterations) + " iterations";
        } catch (const std::exception& e) {
          err = e.what();
          cudaStreamSynchronize(st);
        }
      }
      {
        std::lock_guard<std::mutex> lk(mu);
        in_use -= job->footprint;
        --running;
        job->res = res;
        job->error = err;
        job->t_setup = t_setup;
        job->t_end = Clock::now();
        job->status = err.empty() ? 2 : 3;
      }
      cv_done.notify_all();
      cv_work.notify_all();  // memory freed: queued jobs may now fit
    }
    if (so) cusolverDnDestroy(so);
    if (bl) cublasDestroy(bl);
    if (st) cudaStreamDestroy(st);
  }
};

extern "C" {

hfg_status hfg_engine_create(int n_workers, double hbm_budget_gb, hfg_engine** out) {
  return guard([&] {
    need(out != nullptr && n_workers >= 1 && n_workers <= 256 && hbm_budget_gb > 0, "hfg_engine_create: bad arguments");
    std::unique_ptr<hfg_engine> e(new hfg_engine());
    ck(cudaGetDevice(&e->device), "cudaGetDevice");
    hfg_abi::retain_pool_memory();
    e->budget = (size_t)(hbm_budget_gb * 1e9);
    const unsigned hc = std::max(1u, std::thread::hardware_concurrency());
    e->omp_threads = std::max(1, (int)(hc / (unsigned)n_workers));
    for (int i = 0; i < n_workers; ++i) e->workers.emplace_back([p = e.get()] { p->worker_main(); });
    *out = e.release();
  });
}

hfg_status hfg_engine_submit(hfg_engine* e, const hfg_atom_desc* atom, const hfg_scf_desc* scf,
                             unsigned long long* job_id) {
  return guard([&] {
    need(e && atom && scf && job_id, "hfg_engine_submit: null argument");
    need(atom->nnodes >= 3 && atom->nnodes <= 17 && atom->nelem >= 2 && atom->nang >= 1 && atom->bval &&
             atom->lval && atom->mval,
         "hfg_engine_submit: bad atom description");
    std::unique_ptr<Job> j(new Job());
    j->bval.assign(atom->bval, atom->bval + atom->nelem + 1);
    j->lval.assign(atom->lval, atom->lval + atom->nang);
    j->mval.assign(atom->mval, atom->mval + atom->nang);
    for (int l : j->lval) need(l >= 0 && l <= 3, "hfg_engine_submit: l <= 3 supported");
    j->atom = *atom;
    j->atom.bval = j->bval.data();
    j->atom.lval = j->lval.data();
    j->atom.mval = j->mval.data();
    j->scf = *scf;
    if (scf->fixed_occ) {
      j->fixed.assign(scf->fixed_occ, scf->fixed_occ + 2 * scf->n_fixed_blocks);
      j->scf.fixed_occ = j->fixed.data();
    }
    if (scf->l_occ) {
      need(scf->n_l_occ >= 1 && scf->n_l_occ <= 64, "hfg_engine_submit: bad l_occ size");
      j->l_occ.assign(scf->l_occ, scf->l_occ + 2 * scf->n_l_occ);
      j->scf.l_occ = j->l_occ.data();
    }
    j->footprint = hfg_job_footprint(j->atom, j->scf);
    j->t_submit = Clock::now();
    j->id = e->next_id++;
    *job_id = j->id;
    {
      std::lock_guard<std::mutex> lk(e->mu);
      need(!e->stop, "hfg_engine_submit: engine is shutting down");
      e->queue.push_back(j.get());
      e->jobs[j->id] = std::move(j);
    }
    e->cv_work.notify_one();
  });
}

hfg_status hfg_engine_wait(hfg_engine* e, unsigned long long job_id, double timeout_s, hfg_job_result* out) {
  return guard([&] {
    need(e && out, "hfg_engine_wait: null argument");
    std::unique_lock<std::mutex> lk(e->mu);
    need(e->jobs.find(job_id) != e->jobs.end(), "hfg_engine_wait: unknown job id");
    // counted while inside, so that destroy does not free the engine under a
    // waiter; the job is looked up again after every wake-up because another
    // waiter on the same id may have taken (and erased) the result
    struct Count {
      hfg_engine* e;
      explicit Count(hfg_engine* e_) : e(e_) { ++e->waiters; }
      ~Count() {
        --e->waiters;
        e->cv_done.notify_all();
      }
    } count(e);
    auto done = [&] {
      auto f = e->jobs.find(job_id);
      return f == e->jobs.end() || f->second->status >= 2;
    };
    if (timeout_s < 0) e->cv_done.wait(lk, done);
    else e->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done);
    auto it = e->jobs.find(job_id);
    need(it != e->jobs.end(), "hfg_engine_wait: the result of this job was taken by another waiter");
    Job* j = it->second.get();
    std::memset(out, 0, sizeof(*out));
    out->status = j->status;
    out->footprint_bytes = (double)j->footprint;
    if (j->status >= 2) {
      out->scf = j->res;
      out->queue_ms = ms_since(j->t_submit, j->t_start);
      out->setup_ms = ms_since(j->t_start, j->t_setup);
      out->scf_ms = ms_since(j->t_setup, j->t_end);
      out->total_ms = ms_since(j->t_submit, j->t_end);
      std::strncpy(out->error, j->error.c_str(), sizeof(out->error) - 1);
      e->jobs.erase(it);  // results are handed out once
    }
  });
}

hfg_status hfg_engine_stats(hfg_engine* e, int* queued, int* running, double* in_use_gb) {
  return guard([&] {
    need(e != nullptr, "hfg_engine_stats: null argument");
    std::lock_guard<std::mutex> lk(e->mu);
    if (queued) *queued = (int)e->queue.size();
    if (running) *running = e->running;
    if (in_use_gb) *in_use_gb = e->in_use / 1e9;
  });
}

hfg_status hfg_engine_destroy(hfg_engine* e) {
  return guard([&] {
    if (!e) return;
    {
      std::lock_guard<std::mutex> lk(e->mu);
      e->stop = true;
      for (Job* j : e->queue) {
        j->status = 3;
        j->error = "cancelled: engine destroyed";
      }
      e->queue.clear();
    }
    e->cv_work.notify_all();
    for (auto& t : e->workers) t.join();
    {
      // every job is now done or cancelled: waiters wake, copy their result
      // and leave before the engine is freed
      std::unique_lock<std::mutex> lk(e->mu);
      e->cv_done.notify_all();
      e->cv_done.wait(lk, [&] { return e->waiters == 0; });
    }
    delete e;
  });
}

}  // extern "C"

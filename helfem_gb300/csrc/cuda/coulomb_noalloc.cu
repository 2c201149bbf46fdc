// Scratch for hfg_coulomb_noalloc: a fixed, statically allocated device array
// instead of the per-handle buffers that hfg_atom_create allocates.
//
// Who needs this: callers whose per-call path may not allocate device memory
// at all - hosts that hand the engine a fixed device budget and own every
// allocation themselves (a framework's caching allocator), and latency-critical loops
// that must not risk the implicit synchronisation or failure of an
// allocation. They create the atom once at set-up, then call the
// allocation-free Coulomb build as often as they like.
//
// Limits and sharing rules:
//  * the array holds HFG_NOALLOC_SCRATCH_DOUBLES doubles (4 MiB); atoms that
//    need more (n_channels * n_elements * (nnodes^2 + 2) doubles) are
//    rejected with HFG_ERR_ARG;
//  * every device that loads the library holds the array until the process
//    exits;
//  * all calls share the one array and it keeps the previous call's
//    contents: the Coulomb kernels overwrite every scratch entry they read,
//    so nothing has to start at zero, but calls that overlap on the GPU
//    (different streams, or different host threads) race on it and must be
//    serialised by the caller;
//  * the first call on each device resolves the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call
//    before any stream capture begins.
#include <cuda_runtime.h>

#include <mutex>

#include "devatom.cuh"

namespace hfg {

static __device__ __align__(256) double g_coulomb_scratch[HFG_NOALLOC_SCRATCH_DOUBLES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_ptr[kMaxDevices] = {};
}  // namespace

cudaError_t noalloc_coulomb_scratch(size_t doubles_needed, double** out) {
  if (doubles_needed > (size_t)HFG_NOALLOC_SCRATCH_DOUBLES) return cudaErrorInvalidValue;
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_ptr[dev]) {
    // the host-side name is only a stand-in; the kernels need the device address
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_coulomb_scratch);
    if (e != cudaSuccess) return e;
    g_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_ptr[dev];
  return cudaSuccess;
}

}  // namespace hfg

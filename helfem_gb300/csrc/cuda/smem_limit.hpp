// Dynamic shared-memory limits of kernels launched from several host threads.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <map>
#include <mutex>
#include <utility>

namespace hfg {

// Make launches of `fn` with up to `bytes` of dynamic shared memory valid.
// The limit (cudaFuncAttributeMaxDynamicSharedMemorySize) belongs to the
// function in the device's context and is shared by every host thread, so it
// is only ever raised, under one lock: a thread preparing a smaller launch
// can never lower it under another thread's larger one (which would then
// fail with cudaErrorInvalidValue).
inline cudaError_t smem_limit(const void* fn, size_t bytes) {
  if (bytes <= 48 * 1024) return cudaSuccess;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> lim;
  std::lock_guard<std::mutex> g(mu);
  size_t& cur = lim[{fn, dev}];
  if (bytes <= cur) return cudaSuccess;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}
template <class F>
inline cudaError_t smem_limit(F* fn, size_t bytes) {
  return smem_limit(reinterpret_cast<const void*>(fn), bytes);
}

}  // namespace hfg

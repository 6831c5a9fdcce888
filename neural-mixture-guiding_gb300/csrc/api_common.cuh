// api_common.cuh -- host-side helpers shared by the C-ABI translation units:
// thread-local error text, argument checks and CUDA error mapping.
#pragma once
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include <map>
#include <mutex>
#include <utility>

#include "../../include/nmg.h"

namespace nmg {

// Records a formatted message as this thread's last error and returns `st`.
nmg_status set_error(nmg_status st, const char* fmt, ...);

inline nmg_status check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(NMG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return NMG_OK;
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Raises a kernel's dynamic shared-memory limit to at least `bytes`, once per
// (kernel, device): launches inside a stream capture then make no attribute
// calls.
inline nmg_status ensure_smem(const void* kern, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  size_t& have = done[{kern, dev}];
  if (have >= bytes) return NMG_OK;
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (optin > 0 && bytes > size_t(optin))
    return set_error(NMG_ERR_UNSUPPORTED, "kernel needs %zu B of shared memory, the device allows %d B", bytes, optin);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
  if (e != cudaSuccess) {
    cudaGetLastError();  // not sticky: keep it from being reported by a later launch check
    return set_error(NMG_ERR_CUDA, "shared memory %zu B: %s", bytes, cudaGetErrorString(e));
  }
  have = bytes;
  return NMG_OK;
}

// Number of SMs of the current device (looked up once per device).
inline int sm_count() {
  static std::mutex mu;
  static std::map<int, int> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(dev);
  if (it != cache.end()) return it->second;
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
  cache[dev] = n;
  return n;
}

}  // namespace nmg

#define NMG_REQUIRE(cond, ...)                                    \
  do {                                                           \
    if (!(cond)) return nmg::set_error(NMG_ERR_INVALID_ARG, __VA_ARGS__); \
  } while (0)

#define NMG_TRY(x)               \
  do {                           \
    nmg_status s_ = (x);         \
    if (s_ != NMG_OK) return s_; \
  } while (0)

#define NMG_CUDA_TRY(call)                                                                 \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return nmg::set_error(e_ == cudaErrorMemoryAllocation ? NMG_ERR_OOM : NMG_ERR_CUDA, \
                            "%s: %s", #call, cudaGetErrorString(e_));                      \
  } while (0)

// api_common.cuh -- host-side helpers shared by the C-ABI translation units:
// thread-local error text, argument checks and CUDA error mapping.
#pragma once
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

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

}  // namespace nmg

#define NMG_REQUIRE(cond, ...)                                    \
  do {                                                           \
    if (!(cond)) return nmg::set_error(NMG_ERR_INVALID_ARG, __VA_ARGS__); \
  } while (0)

#define NMG_CUDA_TRY(call)                                                                 \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return nmg::set_error(e_ == cudaErrorMemoryAllocation ? NMG_ERR_OOM : NMG_ERR_CUDA, \
                            "%s: %s", #call, cudaGetErrorString(e_));                      \
  } while (0)

// common.h -- shared host-side helpers for the gpuh2h library: status codes,
// the thread-local last-error string, CUDA error checks and a wall clock.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "gpuh2h.h"
#include "status.h"

namespace gh {

void set_last_error(const std::string &msg);

#define GH_CUDA(call)                                                                              \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess)                                                                         \
      throw ::gh::Error(H2H_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_) + " (" + \
                                          __FILE__ + ":" + std::to_string(__LINE__) + ")");        \
  } while (0)

struct Clock {
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  void reset() { t0 = std::chrono::steady_clock::now(); }
  // microseconds since reset, matching the reference's time_Mine (Graph_D.cuh:39-55)
  long long us() const {
    return std::chrono::duration_cast<std::chrono::microseconds>(std::chrono::steady_clock::now() - t0).count();
  }
};

// Largest dynamic shared memory a kernel may request: the per-block opt-in
// limit minus the kernel's own static shared memory; also raises the
// kernel's attribute to that value.
template <typename K>
inline int enable_max_dynamic_smem(K kernel) {
  int dev = 0, optin = 0;
  GH_CUDA(cudaGetDevice(&dev));
  GH_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  GH_CUDA(cudaFuncGetAttributes(&fa, kernel));
  int dyn = optin - (int)fa.sharedSizeBytes;
  GH_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn));
  return dyn;
}

// Bound on one spin-wait of a kernel (a dependency or a barrier), in SM clock
// cycles: 2 s at 2 GHz, or GPUH2H_SPIN_LIMIT_MS (profilers replay
// instrumented kernels much slower).
inline long long spin_limit_cycles() {
  long long ms = 2000;
  if (const char *e = std::getenv("GPUH2H_SPIN_LIMIT_MS")) ms = std::max(1LL, std::atoll(e));
  return ms * 2000000LL;
}

inline int ilog2_floor(int64_t x) {  // floor(log2(x)) for x >= 1; equals (int)log2((double)x)
  int k = 0;
  while ((int64_t(2) << k) <= x) k++;
  return k;
}

}  // namespace gh

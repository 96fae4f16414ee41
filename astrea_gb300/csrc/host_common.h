// Host-side helpers shared by the C ABI translation units: error recording
// and the CUDA-call check macro.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/astrea_gb300.h"

extern thread_local std::string g_last_error;

static inline int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
static inline int cuda_fail(cudaError_t e, const char* where) {
  return fail(ASTREA_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define CK(call)                                        \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

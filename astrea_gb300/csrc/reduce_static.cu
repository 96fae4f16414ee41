// Conserved-quantity sums that allocate nothing: the same two-pass Neumaier
// reduction as astrea_reduce_conserved, with its partial sums in a fixed
// file-scope device array instead of buffers owned by an engine handle.
//
// Who needs it: a caller that holds only a state pointer and may not allocate
// device memory at that moment - a grid living in a batched arena (a serving
// process whose HBM is fully budgeted to arenas), or a monitor that reports
// totals while the device is out of memory.  Creating a single-grid handle just
// to get the sums would allocate the full set of stage buffers of that grid.
#include <mutex>

#include "host_common.h"
#include "stage.cuh"

using namespace astrea;

namespace {

constexpr int kBlocks = 152;     // pass-1 blocks, as in astrea_reduce_conserved (same summation order)
constexpr int kMaxVars = 8;      // largest variable count the scratch holds partials for
constexpr int kPartDoubles = kBlocks * kMaxVars * 2;          // (sum, compensation) per block and variable
constexpr int kScratchDoubles = kPartDoubles + kMaxVars;      // + the folded sums: 2440 doubles, 19,520 bytes
constexpr int kMaxDevices = 64;

// One copy per device (per CUDA context).  Pass 1 writes every partial it
// covers before pass 2 reads it, and pass 2 writes every sum before the copy
// to the host, so nothing here has to start at zero.
static __device__ __align__(256) double g_reduce_scratch[kScratchDoubles];

std::mutex g_setup_mutex;
double* g_scratch_of_device[kMaxDevices] = {};

// The device address of the scratch on the current device, looked up once per
// device with that device current.
int scratch_on_current_device(double** out) {
  int dev = -1;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(ASTREA_ERR_ARG, "device ordinal beyond the static scratch table");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_of_device[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_reduce_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static reduction scratch)");
    g_scratch_of_device[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_of_device[dev];
  return ASTREA_OK;
}

template <typename T>
int reduce_with(double* scratch, const void* state, long long cells, int nv, double* host, cudaStream_t st) {
  double* part = scratch;
  double* sums = scratch + kPartDoubles;
  sums_pass1<T><<<kBlocks, 256, 0, st>>>(static_cast<const T*>(state), cells, cells, nv, part);
  CK(cudaGetLastError());
  sums_pass2<<<1, 32, 0, st>>>(part, kBlocks, nv, sums);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(host, sums, sizeof(double) * nv, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return ASTREA_OK;
}

}  // namespace

extern "C" {

int astrea_reduce_conserved_static(const void* state, int precision, long long cells, int nv, double* sums_host,
                                   void* stream) {
  if (!state || !sums_host) return fail(ASTREA_ERR_ARG, "NULL argument");
  if (precision != 32 && precision != 64) return fail(ASTREA_ERR_ARG, "precision must be 32 or 64");
  if (cells < 1) return fail(ASTREA_ERR_ARG, "cells must be at least 1");
  if (nv < 1 || nv > kMaxVars)
    return fail(ASTREA_ERR_ARG, "nv must be 1..8: the static reduction scratch holds partial sums for at most 8 "
                                "variables");
  double* scratch = nullptr;
  const int rc = scratch_on_current_device(&scratch);
  if (rc != ASTREA_OK) return rc;
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  return precision == 64 ? reduce_with<double>(scratch, state, cells, nv, sums_host, st)
                         : reduce_with<float>(scratch, state, cells, nv, sums_host, st);
}

}  // extern "C"

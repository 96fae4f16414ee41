// Launchers of the batched persistent sweep kernel.  Each batch_k_*.cu
// translation unit instantiates the launchers of one (precision, model, axis)
// so that the large kernels compile in parallel; batch_api.cu only takes
// their addresses.
#pragma once
#include "batch.cuh"

namespace astrea {

constexpr int BTS1 = 32, BTS2 = 32, BTT2 = 8;

template <typename T> using BatchFn = cudaError_t (*)(const BatchArgs<T>&, int nctas, cudaStream_t);

template <typename T, int MID, int DIM, int AX>
cudaError_t launch_batched(const BatchArgs<T>& b, int nctas, cudaStream_t st) {
  constexpr int TS = DIM == 1 ? BTS1 : BTS2, TT = DIM == 1 ? 1 : BTT2, NT = DIM == 1 ? 64 : 256;
  constexpr size_t bytes = sizeof(T) * batch_smem_elems<MID, DIM, TS, TT, T>();
  static_assert(bytes <= 220 * 1024, "batched tile exceeds shared memory");
  auto k = batched_sweep_kernel<T, MID, DIM, AX, TS, TT>;
  if (nctas <= 0) return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k<<<nctas, NT, bytes, st>>>(b);
  return cudaGetLastError();
}

template <typename T, int MID, int DIM, int AX> int occupancy() {
  constexpr int TS = DIM == 1 ? BTS1 : BTS2, TT = DIM == 1 ? 1 : BTT2, NT = DIM == 1 ? 64 : 256;
  constexpr size_t bytes = sizeof(T) * batch_smem_elems<MID, DIM, TS, TT, T>();
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batched_sweep_kernel<T, MID, DIM, AX, TS, TT>, NT, bytes);
  return n;
}

template <typename T, int DIM> BatchFn<T> get_batched(int model, int ax) {
  if constexpr (DIM == 1) {
    if (model == 3) return &launch_batched<T, 3, 1, 0>;
    if (model == 8) return &launch_batched<T, 8, 1, 0>;
  } else {
    if (model == 4) return ax == 0 ? &launch_batched<T, 4, 2, 0> : &launch_batched<T, 4, 2, 1>;
    if (model == 8) return ax == 0 ? &launch_batched<T, 8, 2, 0> : &launch_batched<T, 8, 2, 1>;
  }
  return nullptr;
}

template <typename T, int DIM> int get_occupancy(int model, int ax) {
  if constexpr (DIM == 1) return model == 3 ? occupancy<T, 3, 1, 0>() : occupancy<T, 8, 1, 0>();
  else {
    if (model == 4) return ax == 0 ? occupancy<T, 4, 2, 0>() : occupancy<T, 4, 2, 1>();
    return ax == 0 ? occupancy<T, 8, 2, 0>() : occupancy<T, 8, 2, 1>();
  }
}

#define ASTREA_BATCH_INST(T, MID, DIM, AX)                                                   \
  template cudaError_t launch_batched<T, MID, DIM, AX>(const BatchArgs<T>&, int, cudaStream_t); \
  template int occupancy<T, MID, DIM, AX>();

#define ASTREA_BATCH_EXTERN(T, MID, DIM, AX)                                                        \
  extern template cudaError_t launch_batched<T, MID, DIM, AX>(const BatchArgs<T>&, int, cudaStream_t); \
  extern template int occupancy<T, MID, DIM, AX>();

#define ASTREA_EXTERN_BATCH(T)        \
  ASTREA_BATCH_EXTERN(T, 3, 1, 0)     \
  ASTREA_BATCH_EXTERN(T, 8, 1, 0)     \
  ASTREA_BATCH_EXTERN(T, 4, 2, 0)     \
  ASTREA_BATCH_EXTERN(T, 4, 2, 1)     \
  ASTREA_BATCH_EXTERN(T, 8, 2, 0)     \
  ASTREA_BATCH_EXTERN(T, 8, 2, 1)

}  // namespace astrea

// Launchers of the batched persistent sweep kernel.  Each batch_k_*.cu
// translation unit instantiates the launchers of one (precision, model, axis,
// tile) so that the large kernels compile in parallel; batch_api.cu only takes
// their addresses.
#pragma once
#include "batch.cuh"

namespace astrea {

// Tiles: 1D 32 cells x 64 threads.  2D candidates, picked per batch by its
// autotuner: 32 (sweep) x 8 (rows) x 256 threads, and 32 x 15 x 512 threads
// (FP32 2D Euler only, whose shared memory and registers allow it).
constexpr int BTS1 = 32, BNT1 = 64;
constexpr int NBTILES2 = 2;
template <int V> struct BTile2;
template <> struct BTile2<0> { static constexpr int TS = 32, TT = 8, NT = 256; };
template <> struct BTile2<1> { static constexpr int TS = 32, TT = 15, NT = 512; };

template <typename T> using BatchFn = cudaError_t (*)(const BatchArgs<T>&, int nctas, cudaStream_t);

template <int DIM, int V> struct BShape {
  static constexpr int TS = DIM == 1 ? BTS1 : BTile2<V>::TS;
  static constexpr int TT = DIM == 1 ? 1 : BTile2<V>::TT;
  static constexpr int NT = DIM == 1 ? BNT1 : BTile2<V>::NT;
};

// whether tile V is built for (precision, model, dimension)
template <typename T, int MID, int DIM, int V> constexpr bool batch_tile_built() {
  return V == 0 || (DIM == 2 && sizeof(T) == 4 && MID == 4);
}

template <typename T, int MID, int DIM, int AX, int V>
cudaError_t launch_batched(const BatchArgs<T>& b, int nctas, cudaStream_t st) {
  using S = BShape<DIM, V>;
  constexpr size_t bytes = sizeof(T) * batch_smem_elems<MID, DIM, S::TS, S::TT, T>();
  static_assert(bytes <= 220 * 1024, "batched tile exceeds shared memory");
  auto k = batched_sweep_kernel<T, MID, DIM, AX, S::TS, S::TT, S::NT>;
  if (nctas <= 0) return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  k<<<nctas, S::NT, bytes, st>>>(b);
  return cudaGetLastError();
}

template <typename T, int MID, int DIM, int AX, int V> int occupancy() {
  using S = BShape<DIM, V>;
  constexpr size_t bytes = sizeof(T) * batch_smem_elems<MID, DIM, S::TS, S::TT, T>();
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batched_sweep_kernel<T, MID, DIM, AX, S::TS, S::TT, S::NT>, S::NT,
                                                bytes);
  return n;
}

template <typename T, int MID, int DIM, int AX> BatchFn<T> batched_variant(int v) {
  if (v == 0) return &launch_batched<T, MID, DIM, AX, 0>;
  if constexpr (batch_tile_built<T, MID, DIM, 1>()) {
    if (v == 1) return &launch_batched<T, MID, DIM, AX, 1>;
  }
  return nullptr;
}

template <typename T, int MID, int DIM, int AX> int occupancy_variant(int v) {
  if (v == 0) return occupancy<T, MID, DIM, AX, 0>();
  if constexpr (batch_tile_built<T, MID, DIM, 1>()) {
    if (v == 1) return occupancy<T, MID, DIM, AX, 1>();
  }
  return 0;
}

template <typename T, int DIM> BatchFn<T> get_batched(int model, int ax, int v) {
  if constexpr (DIM == 1) {
    if (model == 3) return batched_variant<T, 3, 1, 0>(v);
    if (model == 8) return batched_variant<T, 8, 1, 0>(v);
  } else {
    if (model == 4) return ax == 0 ? batched_variant<T, 4, 2, 0>(v) : batched_variant<T, 4, 2, 1>(v);
    if (model == 8) return ax == 0 ? batched_variant<T, 8, 2, 0>(v) : batched_variant<T, 8, 2, 1>(v);
  }
  return nullptr;
}

template <typename T, int DIM> int get_occupancy(int model, int ax, int v) {
  if constexpr (DIM == 1) return model == 3 ? occupancy_variant<T, 3, 1, 0>(v) : occupancy_variant<T, 8, 1, 0>(v);
  else {
    if (model == 4) return ax == 0 ? occupancy_variant<T, 4, 2, 0>(v) : occupancy_variant<T, 4, 2, 1>(v);
    return ax == 0 ? occupancy_variant<T, 8, 2, 0>(v) : occupancy_variant<T, 8, 2, 1>(v);
  }
}

#define ASTREA_BATCH_INST(T, MID, DIM, AX, V)                                                    \
  template cudaError_t launch_batched<T, MID, DIM, AX, V>(const BatchArgs<T>&, int, cudaStream_t); \
  template int occupancy<T, MID, DIM, AX, V>();

#define ASTREA_BATCH_EXTERN(T, MID, DIM, AX, V)                                                         \
  extern template cudaError_t launch_batched<T, MID, DIM, AX, V>(const BatchArgs<T>&, int, cudaStream_t); \
  extern template int occupancy<T, MID, DIM, AX, V>();

#define ASTREA_EXTERN_BATCH(T)          \
  ASTREA_BATCH_EXTERN(T, 3, 1, 0, 0)    \
  ASTREA_BATCH_EXTERN(T, 8, 1, 0, 0)    \
  ASTREA_BATCH_EXTERN(T, 4, 2, 0, 0)    \
  ASTREA_BATCH_EXTERN(T, 4, 2, 1, 0)    \
  ASTREA_BATCH_EXTERN(T, 8, 2, 0, 0)    \
  ASTREA_BATCH_EXTERN(T, 8, 2, 1, 0)

// the second 2D tile exists for FP32 2D Euler only
#define ASTREA_EXTERN_BATCH_T2         \
  ASTREA_BATCH_EXTERN(float, 4, 2, 0, 1) \
  ASTREA_BATCH_EXTERN(float, 4, 2, 1, 1)

}  // namespace astrea

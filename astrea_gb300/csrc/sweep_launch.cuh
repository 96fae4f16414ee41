// Launchers for the sweep kernel and the (precision, scheme) dispatch tables.
// Each sweep_<prec>_<scheme>.cu translation unit instantiates get_sweep for one
// (precision, scheme) pair so the build compiles them in parallel.
#pragma once
#include "sweep.cuh"

namespace astrea {

template <typename T> using SweepFn = cudaError_t (*)(const SweepArgs<T>&, cudaStream_t);

// Tiles: 1D 32 cells x 64 threads.  2D candidates, picked per grid by the
// engine's autotuner: 32 (sweep) x 8 (rows) x 256 threads, and 32 x 15 x 512
// threads (fewer transverse halo rows per cell, same threads per SM, and the
// 15 x 33 interfaces of the second face level fit one pass of 512 threads;
// Euler tiles only: two CTAs per SM in FP32 at 64 registers, one in FP64 at
// 122 registers and 182 KB of shared memory, where fewer halo cells per cell
// matter because the FP64 pipe bounds the kernel).
constexpr int TS1 = 32, NT1 = 64;
constexpr int NTILES2 = 2;
template <int I> struct Tile2;
template <> struct Tile2<0> { static constexpr int TS = 32, TT = 8, NT = 256; };
template <> struct Tile2<1> { static constexpr int TS = 32, TT = 15, NT = 512; };

template <typename T, int MID, int SCH, int DIM, int TS, int TT> constexpr size_t sweep_smem_bytes() {
  return sizeof(T) * (size_t)Smem<SCH, DIM, TS, TT, Model<MID>::NV, sweep_wsin<SCH, DIM>()>::total;
}

template <typename T, int MID, int SCH, int SOL, int DIM, int AX, int TS, int TT, int NT>
cudaError_t launch_sweep(const SweepArgs<T>& a, cudaStream_t st) {
  constexpr size_t bytes = sweep_smem_bytes<T, MID, SCH, DIM, TS, TT>();
  static_assert(bytes <= 227 * 1024, "sweep tile exceeds the shared memory of one CTA");
  auto k = sweep_kernel<T, MID, SCH, SOL, DIM, AX, TS, TT, NT>;
  int dev = 0;
  cudaGetDevice(&dev);
  static unsigned long long configured = 0ull;  // one bit per device
  const unsigned long long bit = 1ull << (dev & 63);
  if (!(configured & bit)) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e != cudaSuccess) return e;
    configured |= bit;
  }
  if (a.n0 <= 0) return cudaSuccess;  // configure-only call (before any graph capture)
  const int Ns = DIM == 1 ? a.n0 : (AX == 0 ? a.n0 : a.n1);
  const int Nt = DIM == 1 ? 1 : (AX == 0 ? a.n1 : a.n0);
  dim3 grid((Ns + TS - 1) / TS, (Nt + TT - 1) / TT);
  k<<<grid, NT, bytes, st>>>(a);
  return cudaGetLastError();
}

// launcher of one (model, scheme, solver, dimension, axis) for tile candidate ``tile``; nullptr if that
// tile is not built for it
template <typename T, int MID, int SCH, int SOL, int DIM, int AX> SweepFn<T> sweep_for_tile(int tile) {
  if constexpr (DIM == 1) {
    return tile == 0 ? &launch_sweep<T, MID, SCH, SOL, 1, 0, TS1, 1, NT1> : nullptr;
  } else {
    if (tile == 0) return &launch_sweep<T, MID, SCH, SOL, 2, AX, Tile2<0>::TS, Tile2<0>::TT, Tile2<0>::NT>;
    if constexpr (MID != 8) {
      if (tile == 1) return &launch_sweep<T, MID, SCH, SOL, 2, AX, Tile2<1>::TS, Tile2<1>::TT, Tile2<1>::NT>;
    }
    return nullptr;
  }
}

// Supported (model, solver) pairs: Euler models with LLF/HLLC, the 8-variable
// model with LLF/HLLC/HLLD.
template <typename T, int SCH> SweepFn<T> get_sweep(int mid, int sol, int dim, int ax, int tile) {
  if (dim == 1) {
    if (mid == 3) {
      if (sol == LLF) return sweep_for_tile<T, 3, SCH, LLF, 1, 0>(tile);
      if (sol == HLLC) return sweep_for_tile<T, 3, SCH, HLLC, 1, 0>(tile);
    } else if (mid == 8) {
      if (sol == LLF) return sweep_for_tile<T, 8, SCH, LLF, 1, 0>(tile);
      if (sol == HLLC) return sweep_for_tile<T, 8, SCH, HLLC, 1, 0>(tile);
      if (sol == HLLD) return sweep_for_tile<T, 8, SCH, HLLD, 1, 0>(tile);
    }
  } else if (dim == 2) {
    if (mid == 4) {
      if (sol == LLF) return ax == 0 ? sweep_for_tile<T, 4, SCH, LLF, 2, 0>(tile) : sweep_for_tile<T, 4, SCH, LLF, 2, 1>(tile);
      if (sol == HLLC) return ax == 0 ? sweep_for_tile<T, 4, SCH, HLLC, 2, 0>(tile) : sweep_for_tile<T, 4, SCH, HLLC, 2, 1>(tile);
    } else if (mid == 8) {
      if (sol == LLF) return ax == 0 ? sweep_for_tile<T, 8, SCH, LLF, 2, 0>(tile) : sweep_for_tile<T, 8, SCH, LLF, 2, 1>(tile);
      if (sol == HLLC) return ax == 0 ? sweep_for_tile<T, 8, SCH, HLLC, 2, 0>(tile) : sweep_for_tile<T, 8, SCH, HLLC, 2, 1>(tile);
      if (sol == HLLD) return ax == 0 ? sweep_for_tile<T, 8, SCH, HLLD, 2, 0>(tile) : sweep_for_tile<T, 8, SCH, HLLD, 2, 1>(tile);
    }
  }
  return nullptr;
}

#define ASTREA_EXTERN_GET_SWEEP(T)                                               \
  extern template SweepFn<T> get_sweep<T, PCM>(int, int, int, int, int);              \
  extern template SweepFn<T> get_sweep<T, PLM>(int, int, int, int, int);              \
  extern template SweepFn<T> get_sweep<T, PPM>(int, int, int, int, int);              \
  extern template SweepFn<T> get_sweep<T, WENO3>(int, int, int, int, int);            \
  extern template SweepFn<T> get_sweep<T, WENO5>(int, int, int, int, int);            \
  extern template SweepFn<T> get_sweep<T, WENO7>(int, int, int, int, int);

}  // namespace astrea

// Batched execution: many independent grids of uneven sizes advanced together.
//
// Each grid has its own clock (dt, t, t_end) and method (scheme x solver
// "combo"); all grids of a batch share dimension, variable model, precision
// and integrator.  One step of the batch is the same launch sequence as for
// one grid (sweeps, dt, stage-0 combine, fused stage combines, bookkeeping),
// but every sweep launch is one *persistent* kernel whose CTAs pull tiles of
// all grids from a work list (largest grids first) through an atomic counter,
// and dispatch per tile to the grid's (scheme, solver) body.
#pragma once
#include "stage.cuh"

namespace astrea {

// combos of a batch (scheme x solver); the solver column is HLLC for Euler models, HLLD for MHD
enum Combo { C_PLM_LLF = 0, C_PLM_HLL = 1, C_PPM_LLF = 2, C_PPM_HLL = 3, C_WENO5_LLF = 4, C_WENO5_HLL = 5, N_COMBO = 6 };

template <typename T> struct BGrid {
  long long base;   // element offset of the grid's first plane in every arena
  long long cells;  // n0 * n1
  int n0, n1, bc, limiter, combo, physical;
  T gamma, gm1;
  double dx;
};

struct BItem {
  int g, s0, t0;
};

template <typename T> struct BatchArgs {
  const BGrid<T>* grids;
  const BItem* items;
  int nitems;
  int* counter;
  Clock* clocks;
  T* u;      // state arena
  T* k0;     // stage arenas
  T* k1;
  T* d0;     // divergence arenas
  T* d1;
  T* ws0;    // 2D: cell averages of the stage input for the axis-0 and axis-1 sweeps (the same arena in FP32)
  T* ws1;
  int stage, mode, integ, want_emax, last_stage, dout_sel;
};

// 2D high-order combos stage the cell averages of a pre-pass (batched_cell_average_kernel)
template <int MID, int DIM, int TS, int TT, typename T> constexpr size_t batch_smem_elems() {
  constexpr int NV = Model<MID>::NV;
  constexpr int a = Smem<PLM, DIM, TS, TT, NV>::total, b = Smem<PPM, DIM, TS, TT, NV, DIM == 2>::total,
                c = Smem<WENO5, DIM, TS, TT, NV, DIM == 2>::total;
  constexpr int m = a > b ? a : b;
  return (size_t)(m > c ? m : c);
}

// (FP64 keeps one CTA per SM here: the dispatch over six method bodies needs more registers)
template <typename T, int MID, int DIM, int AX, int TS, int TT, int NT>
__global__ void __launch_bounds__((NT > 256 ? NT : 256),
                                  (sizeof(T) == 8 ? 1 : SweepOcc<T, MID, (NT > 256 ? NT : 256)>::value))
    batched_sweep_kernel(const BatchArgs<T> b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_item;
  constexpr int HLL = MID == 8 ? HLLD : HLLC;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(b.counter, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= b.nitems) break;
    const BItem w = b.items[it];
    const BGrid<T> gd = b.grids[w.g];
    Clock* clk = b.clocks + w.g;
    if (clk->done) continue;
    T* cur = b.stage == 0 ? b.u : ((b.stage - 1) % 2 == 0 ? b.k0 : b.k1);
    T* out = b.last_stage ? b.u : (b.stage % 2 == 0 ? b.k0 : b.k1);
    SweepArgs<T> a{};
    a.q = cur + gd.base;
    a.plane = gd.cells;
    a.n0 = gd.n0;
    a.n1 = DIM == 1 ? 1 : gd.n1;
    a.bc = gd.bc;
    a.label = -1;
    a.limiter = gd.limiter;
    a.mode = b.mode;
    a.integ = b.integ;
    a.stage = b.stage;
    a.want_emax = b.want_emax;
    a.physical = gd.physical;
    a.gamma = gd.gamma;
    a.gm1 = gd.gm1;
    a.dx = gd.dx;
    a.dout = (b.dout_sel == 0 ? b.d0 : b.d1) + gd.base;
    a.dother = b.d0 + gd.base;
    a.u0 = b.u + gd.base;
    a.out = out + gd.base;
    a.clock = clk;
    constexpr bool WS = DIM == 2;  // PPM / WENO5 tiles stage the pre-pass's cell averages
    if (WS) a.ws = (AX == 0 ? b.ws0 : b.ws1) + gd.base;
    switch (gd.combo) {
      case C_PLM_LLF: sweep_tile<T, MID, PLM, LLF, DIM, AX, TS, TT, NT>(a, w.s0, w.t0, smem_raw); break;
      case C_PLM_HLL: sweep_tile<T, MID, PLM, HLL, DIM, AX, TS, TT, NT>(a, w.s0, w.t0, smem_raw); break;
      case C_PPM_LLF: sweep_tile<T, MID, PPM, LLF, DIM, AX, TS, TT, NT, false, WS>(a, w.s0, w.t0, smem_raw); break;
      case C_PPM_HLL: sweep_tile<T, MID, PPM, HLL, DIM, AX, TS, TT, NT, false, WS>(a, w.s0, w.t0, smem_raw); break;
      case C_WENO5_LLF: sweep_tile<T, MID, WENO5, LLF, DIM, AX, TS, TT, NT, false, WS>(a, w.s0, w.t0, smem_raw); break;
      default: sweep_tile<T, MID, WENO5, HLL, DIM, AX, TS, TT, NT, false, WS>(a, w.s0, w.t0, smem_raw); break;
    }
  }
}

// stage-0 combine over all grids: one CTA per tile of the axis-0 work list
template <typename T>
__global__ void batched_combine0_kernel(const BatchArgs<T> b, const BItem* __restrict__ items, int nv, int dim2,
                                        int single_stage, int TS, int TT) {
  const BItem w = items[blockIdx.x];
  const Clock& clk = b.clocks[w.g];
  if (clk.done) return;
  const BGrid<T>& gd = b.grids[w.g];
  const T dt = T(clk.dt);
  T* out = single_stage ? b.u : b.k0;
  for (int e = threadIdx.x; e < TS * TT; e += blockDim.x) {
    const int i = w.s0 + e / TT, j = w.t0 + e % TT;  // axis-0 frame: i along n0, j along n1 (contiguous)
    if (i >= gd.n0 || j >= gd.n1) continue;
    const long long cell = (long long)i * gd.n1 + j;
    for (int s = 0; s < nv; ++s) {
      const long long e2 = gd.base + s * gd.cells + cell;
      const T total_ = dim2 ? b.d0[e2] + b.d1[e2] : b.d0[e2];
      const T L = -total_;
      out[e2] = combine<T>(b.integ, 0, b.u[e2], b.u[e2], L, dt);
    }
  }
}

}  // namespace astrea

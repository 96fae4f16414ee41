// Cell-averaged primitives of a 2D state: the first level of the high-order
// sweeps (fv.high_order_convert_conservative, fv.py:126-143), computed once per
// stage for both sweeps instead of once per sweep tile with halos.
//
//   wS = c2p(q - d2q/24) + d2(c2p(q))/24,   d2 = the sweep axis's second
//   difference, then the transverse one's
//
// The two sweeps add the two axes' corrections in opposite orders, which round
// differently, so the kernel writes one copy per sweep: w_ax0 for the axis-0
// sweep (axis 0 first), w_ax1 for the axis-1 sweep (FP64; see below for
// FP32).  Edge cells take their neighbours through the input boundary map
// (clamp for outflow, wrap for periodic), the values a sweep tile's q level
// holds there when the tile forms wS itself (the per-tile path of sweep.cuh,
// which 1D tiles still take).  The arithmetic is that path's, operation for
// operation.
#pragma once
#include "batch.cuh"

namespace astrea {

// One warp per strip of 30 columns x TY rows: its 32 lanes sit on 32
// consecutive columns (lanes 0 and 31 are the strip's halo) and walk down the
// rows, keeping rows i-1, i, i+1 (state and point primitives) in registers and
// taking the axis-1 neighbours from the adjacent lanes; each row's state is
// loaded two rows before it is converted.  No shared memory, no block barriers.
constexpr int CA_W = 30, CA_NT = 256, CA_WARPS = CA_NT / 32;
template <typename T, int MID> struct CellAvgTile {
  static constexpr int TY = 16;  // rows per strip
};

// The FP64 kernels write both sweep orders (bit-level parity); the FP32 ones
// write the axis-0 order only, which both FP32 sweeps read (its rounding differs
// from the other order's in the last FP32 bit).
template <typename T> constexpr bool cell_average_both_orders() { return Prec<T>::EXACT; }

// One strip, rows [i0, i0+TY) and the 30 columns after jb, by one whole warp
// (every lane reaches every shuffle).
template <typename T, int MID>
__device__ __forceinline__ void cell_average_strip(const T* __restrict__ q, T* __restrict__ w_ax0,
                                                   T* __restrict__ w_ax1, int n0, int n1, long long plane, int bc,
                                                   T gm1, int i0, int jb) {
  using M = Model<MID>;
  constexpr int NV = M::NV, TY = CellAvgTile<T, MID>::TY;
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int j = jb + lane;
  const int gj = (j >= 0 && j < n1) ? j : bc_map(j, n1, bc);
  const bool out_lane = lane >= 1 && lane <= CA_W && j < n1;
  auto row_ptr = [&](int i) -> const T* {
    const int gi = (i >= 0 && i < n0) ? i : bc_map(i, n0, bc);
    return q + (long long)gi * n1 + gj;
  };
  auto expand = [&](const T* v, T* x) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = T(0);
#pragma unroll
    for (int s = 0; s < NV; ++s) x[M::var(s)] = v[s];
  };
  T qm[8], q0[8], qp[8], wm[8], w0[8], wp[8], nxt[NV], nxt2[NV];  // nxt: row i+1, nxt2: row i+2
  {
    const T* pm = row_ptr(i0 - 1);
    const T* p0 = row_ptr(i0);
    const T* p1 = row_ptr(i0 + 1);
    const T* p2 = row_ptr(i0 + 2);
    T a[NV], b[NV];
#pragma unroll
    for (int s = 0; s < NV; ++s) {
      a[s] = pm[s * plane];
      b[s] = p0[s * plane];
      nxt[s] = p1[s * plane];
      nxt2[s] = p2[s * plane];
    }
    expand(a, qm);
    expand(b, q0);
    c2p<M>(qm, wm, gm1);
    c2p<M>(q0, w0, gm1);
  }
  for (int r = 0; r < TY; ++r) {
    const int i = i0 + r;
    if (i >= n0) break;  // whole warp
    expand(nxt, qp);
#pragma unroll
    for (int s = 0; s < NV; ++s) nxt[s] = nxt2[s];
    if (r + 2 < TY) {  // row i+3, two rows ahead of its use
      const T* pn = row_ptr(i + 3);
#pragma unroll
      for (int s = 0; s < NV; ++s) nxt2[s] = pn[s * plane];
    }
    c2p<M>(qp, wp, gm1);
    // axis-1 neighbours from the adjacent lanes
    T ql[8], qr[8], wl[8], wr[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) { ql[k] = qr[k] = wl[k] = wr[k] = T(0); }
#pragma unroll
    for (int s = 0; s < NV; ++s) {
      const int v = M::var(s);
      ql[v] = __shfl_up_sync(FULL, q0[v], 1);
      qr[v] = __shfl_down_sync(FULL, q0[v], 1);
      wl[v] = __shfl_up_sync(FULL, w0[v], 1);
      wr[v] = __shfl_down_sync(FULL, w0[v], 1);
    }
    if (out_lane) {
      T dq0[8], dq1[8], dw0[8], dw1[8];  // second differences along axis 0 and axis 1
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        dq0[k] = (qp[k] - q0[k]) - (q0[k] - qm[k]);
        dq1[k] = (qr[k] - q0[k]) - (q0[k] - ql[k]);
        dw0[k] = (wp[k] - w0[k]) - (w0[k] - wm[k]);
        dw1[k] = (wr[k] - w0[k]) - (w0[k] - wl[k]);
      }
      const long long g = (long long)i * n1 + j;
      // axis-0 sweep: axis 0's correction first
      {
        T qq[8], wc[8], w[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          qq[k] = q0[k] - T(C24) * dq0[k];
          wc[k] = T(C24) * dw0[k];
          qq[k] = qq[k] - T(C24) * dq1[k];
          wc[k] = wc[k] + T(C24) * dw1[k];
        }
        c2p<M>(qq, w, gm1);
#pragma unroll
        for (int s = 0; s < NV; ++s) w_ax0[s * plane + g] = w[M::var(s)] + wc[M::var(s)];
      }
      // axis-1 sweep: axis 1's correction first
      if constexpr (cell_average_both_orders<T>()) {
        T qq[8], wc[8], w[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          qq[k] = q0[k] - T(C24) * dq1[k];
          wc[k] = T(C24) * dw1[k];
          qq[k] = qq[k] - T(C24) * dq0[k];
          wc[k] = wc[k] + T(C24) * dw0[k];
        }
        c2p<M>(qq, w, gm1);
#pragma unroll
        for (int s = 0; s < NV; ++s) w_ax1[s * plane + g] = w[M::var(s)] + wc[M::var(s)];
      }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      qm[k] = q0[k]; q0[k] = qp[k];
      wm[k] = w0[k]; w0[k] = wp[k];
    }
  }
}

template <typename T, int MID>
__global__ void __launch_bounds__(CA_NT) cell_average_kernel(const T* __restrict__ q, T* __restrict__ w_ax0,
                                                             T* __restrict__ w_ax1, int n0, int n1, long long plane,
                                                             int bc, T gm1, const Clock* clk) {
  if (clk->done) return;
  const int i0 = (blockIdx.y * CA_WARPS + (threadIdx.x >> 5)) * CellAvgTile<T, MID>::TY;
  if (i0 >= n0) return;  // whole warp
  cell_average_strip<T, MID>(q, w_ax0, w_ax1, n0, n1, plane, bc, gm1, i0, blockIdx.x * CA_W - 1);
}

// Batched form: one warp per strip of a list over the high-order grids of a batch
// (the stage input and the cell averages at each grid's arena offset).
struct BStrip {
  int g, i0, jb;
};
template <typename T, int MID>
__global__ void __launch_bounds__(CA_NT) batched_cell_average_kernel(const BatchArgs<T> b, const BStrip* __restrict__ strips,
                                                                     int nstrips) {
  const int it = blockIdx.x * CA_WARPS + (threadIdx.x >> 5);
  if (it >= nstrips) return;  // whole warp
  const BStrip w = strips[it];
  if (b.clocks[w.g].done) return;
  const BGrid<T>& gd = b.grids[w.g];
  const T* cur = b.stage == 0 ? b.u : ((b.stage - 1) % 2 == 0 ? b.k0 : b.k1);
  cell_average_strip<T, MID>(cur + gd.base, b.ws0 + gd.base, b.ws1 + gd.base, gd.n0, gd.n1, gd.cells, gd.bc, gd.gm1,
                             w.i0, w.jb);
}

template <typename T> using CellAvgFn = cudaError_t (*)(const T* q, T* w_ax0, T* w_ax1, int n0, int n1,
                                                        long long plane, int bc, T gm1, const Clock* clk,
                                                        cudaStream_t st);

template <typename T, int MID>
cudaError_t launch_cell_average(const T* q, T* w_ax0, T* w_ax1, int n0, int n1, long long plane, int bc, T gm1,
                                const Clock* clk, cudaStream_t st) {
  constexpr int TY = CellAvgTile<T, MID>::TY;
  const dim3 grid((n1 + CA_W - 1) / CA_W, (n0 + TY * CA_WARPS - 1) / (TY * CA_WARPS));
  cell_average_kernel<T, MID><<<grid, CA_NT, 0, st>>>(q, w_ax0, w_ax1, n0, n1, plane, bc, gm1, clk);
  return cudaGetLastError();
}

template <typename T> using BatchedCellAvgFn = cudaError_t (*)(const BatchArgs<T>&, const BStrip*, int, cudaStream_t);

template <typename T, int MID>
cudaError_t launch_batched_cell_average(const BatchArgs<T>& b, const BStrip* strips, int nstrips, cudaStream_t st) {
  if (nstrips <= 0) return cudaSuccess;
  batched_cell_average_kernel<T, MID><<<(nstrips + CA_WARPS - 1) / CA_WARPS, CA_NT, 0, st>>>(b, strips, nstrips);
  return cudaGetLastError();
}

// the launcher of a 2D model (4: Euler, 8: MHD / transverse velocities); nullptr otherwise.
// Instantiated in cellavg_f32.cu (FMA, like the FP32 sweeps) and cellavg_f64.cu
// (no FMA, like the FP64 sweeps).
template <typename T> CellAvgFn<T> get_cell_average(int model) {
  if (model == 4) return &launch_cell_average<T, 4>;
  if (model == 8) return &launch_cell_average<T, 8>;
  return nullptr;
}

template <typename T> BatchedCellAvgFn<T> get_batched_cell_average(int model) {
  if (model == 4) return &launch_batched_cell_average<T, 4>;
  if (model == 8) return &launch_batched_cell_average<T, 8>;
  return nullptr;
}

extern template CellAvgFn<float> get_cell_average<float>(int);
extern template CellAvgFn<double> get_cell_average<double>(int);
extern template BatchedCellAvgFn<float> get_batched_cell_average<float>(int);
extern template BatchedCellAvgFn<double> get_batched_cell_average<double>(int);

}  // namespace astrea

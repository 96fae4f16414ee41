// Element-wise and small kernels around the sweeps: stage-0 combine, the CFL
// time step, step bookkeeping, initial-condition conversion, conservative ->
// primitive conversion and compensated conserved sums.
#pragma once
#include "sweep.cuh"

namespace astrea {

// Stage-0 combine (needs this step's dt, which needs both sweeps' wave speeds):
// k1 = combine(u, u, L0), L0 = -(D_a + D_b)  (evolvers.py:41-60, 165-168)
template <typename T>
__global__ void combine0_kernel(const T* __restrict__ u, const T* __restrict__ da, const T* __restrict__ db,
                                T* __restrict__ out, long long plane, long long n, int nv, int integ, const Clock* clk) {
  if (clk->done) return;
  const T dt = T(clk->dt);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    for (int s = 0; s < nv; ++s) {
      const long long g = s * plane + i;
      const T total = db ? da[g] + db[g] : da[g];
      const T L = -total;
      out[g] = combine<T>(integ, 0, u[g], u[g], L, dt);
    }
  }
}

// One stage of the integrators with more than two live registers
// (evolvers.py:79-206, SSP-RK (5,3), (5,4), (10,4) and classic RK4), after both
// sweeps of the stage stored their divergences: L = -(d0 + d1) and the stage
// formula, with the reference's operation order.  Registers:
//   RK4      R0 = stage input k, R1..R3 = L0..L2
//   SSPRK53  R0..R3 = k1..k4, R4 = L0, R5 = L1
//   SSPRK54  R0..R3 = k1..k4, R4 = L3
//   SSPRK104 R0 = k (first five stages), R1 = k5, R2 = the second accumulator
// ``out`` is the stage's destination register (the state itself at the last stage).
template <typename T> struct RkStage {
  const T* u;
  T* r[6];
  const T* d0;
  const T* d1;
  T* out;
  long long n;
  int integ, stage;
  const Clock* clk;
};

template <typename T> __global__ void rk_stage_kernel(const RkStage<T> a) {
  if (a.clk->done) return;
  const T dt = T(a.clk->dt);
  const int st = a.stage;
  T* const* R = a.r;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < a.n; i += (long long)gridDim.x * blockDim.x) {
    const T L = -(a.d1 ? a.d0[i] + a.d1[i] : a.d0[i]);
    const T u = a.u[i];
    T y;
    switch (a.integ) {
      case RK4:
        if (st < 3) {
          R[1 + st][i] = L;
          y = u + (st < 2 ? (T(.5) * dt) * L : dt * L);
        } else {
          y = u + T(1.0 / 6.0) * (dt * (((R[1][i] + T(2) * R[2][i]) + T(2) * R[3][i]) + L));
        }
        break;
      case SSPRK53: {
        const T c1 = T(.3772689151171);
        if (st == 0) { R[4][i] = L; y = u + (c1 * dt) * L; }
        else if (st == 1) { R[5][i] = L; y = R[0][i] + (c1 * dt) * L; }
        else if (st == 2) y = (T(.56656131914033) * u + T(.43343868085967) * R[1][i]) + (T(.16352294089771) * dt) * L;
        else if (st == 3)
          y = (((T(.09299483444413) * u + T(.0000209036962) * R[0][i]) + T(.90698426185967) * R[2][i])
               + (T(.00071997378654) * dt) * R[4][i]) + (T(.34217696850008) * dt) * L;
        else
          y = (((T(.0073613226092) * u + T(.20127980325145) * R[0][i]) + T(.00182955389682) * R[1][i])
               + T(.78952932024253) * R[3][i])
              + (dt * ((T(.0027771981946) * R[4][i] + T(.00001567934613) * R[5][i]) + T(.29786487010104) * L));
        break;
      }
      case SSPRK54:
        if (st == 0) y = u + (T(.39175222657189) * dt) * L;
        else if (st == 1) y = (T(.444370493651235) * u + T(.555629506348765) * R[0][i]) + (T(.368410593050371) * dt) * L;
        else if (st == 2) y = (T(.620101851488403) * u + T(.379898148511597) * R[1][i]) + (T(.251891774271694) * dt) * L;
        else if (st == 3) {
          R[4][i] = L;
          y = (T(.178079954393132) * u + T(.821920045606868) * R[2][i]) + (T(.544974750228521) * dt) * L;
        } else {
          y = (((T(.517231671970585) * R[1][i] + T(.096059710526147) * R[2][i]) + (T(.06369246866629) * dt) * R[4][i])
               + T(.386708617503269) * R[3][i]) + (T(.226007483236906) * dt) * L;
        }
        break;
      default: {  // SSPRK104
        const T c6 = T(1.0 / 6.0);
        if (st == 0) y = u + (c6 * dt) * L;
        else if (st <= 4) y = R[0][i] + (c6 * dt) * L;
        else if (st == 5) y = (T(3.0 / 5.0) * u + T(6.0 / 15.0) * R[0][i]) + (T(1.0 / 15.0) * dt) * L;
        else if (st == 6) y = R[1][i] + (c6 * dt) * L;
        else if (st <= 9) y = R[2][i] + (c6 * dt) * L;
        else y = ((T(-11.0 / 35.0) * u + T(5.0 / 7.0) * R[1][i]) + T(3.0 / 5.0) * R[2][i]) + (T(1.0 / 10.0) * dt) * L;
        break;
      }
    }
    a.out[i] = y;
  }
}

// dt = cfl * min over axes (in iteration order) of dx / eigmax, clipped to the
// next checkpoint (astrea.py:70-78).  Python's min keeps the first of equal or
// unordered values, which decides how a NaN speed propagates.
static __global__ void dt_kernel(Clock* clocks, int ngrids) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngrids) return;
  Clock& c = clocks[g];
  if (c.done) return;
  const int first = (c.naxes == 2 && c.order == 1) ? 1 : 0;
  const double e_first = __longlong_as_double((long long)c.emax[first]);
  double m = c.dx / e_first;
  if (c.naxes == 2) {
    const double e_second = __longlong_as_double((long long)c.emax[1 - first]);
    const double v = c.dx / e_second;
    if (v < m) m = v;
  }
  double dt = c.cfl * m;
  if (c.t + dt >= c.chkpt * c.idx) {
    dt = c.chkpt * c.idx - c.t;
    c.idx += 1;
  }
  c.dt = dt;
  // A NaN speed gives a NaN dt; an infinite speed (vacuum) gives dt = 0, on which
  // the reference's loop would never reach t_end.  Either way the grid is flagged
  // and stopped (the rest of this step runs, then end_step marks it done).
  if (!(dt > 0.0) || isinf(dt)) c.status |= 1;
}

// After the last stage: advance t, count the step, flip the axis order
// (astrea.py:84-85), reset the speed maxima, and mark the run done once
// t reaches t_end (astrea.py:45, 61-63).
static __global__ void end_step_kernel(Clock* clocks, int ngrids) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngrids) return;
  Clock& c = clocks[g];
  if (c.done) return;
  c.t = c.t + c.dt;
  c.steps += 1;
  if (c.naxes == 2) c.order ^= 1;
  c.emax[0] = 0ull;
  c.emax[1] = 0ull;
  // status bit 0: non-finite or zero dt; bit 1: a tile's bulk copy timed out (its copy may still
  // be in flight), fatal for the grid as well
  if (!(c.t < c.t_end) || (c.status & 3)) c.done = 1;
}

// index helpers in the physical frame: axis 0 (x, stride n1), axis 1 (y, contiguous)
__device__ __forceinline__ long long cell(int i0, int i1, int n1) { return (long long)i0 * n1 + i1; }

// Initial condition: point primitives -> cell-averaged conservatives
// (constructor.initialise, :105-109).  Pass A: convert_primitive
// (pointwise or 4th order over axes 0 then 1); pass B: + 1/24 d2 per axis.
template <typename T, int MID>
__global__ void init_pass_a(const T* __restrict__ w, T* __restrict__ qa, int n0, int n1, long long plane, int dim,
                            int bc, int high_order, T gm1) {
  using M = Model<MID>;
  const long long n = (long long)n0 * n1;
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < n; id += (long long)gridDim.x * blockDim.x) {
    const int i0 = (int)(id / n1), i1 = (int)(id % n1);
    T w0[8], out[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) w0[i] = T(0);
#pragma unroll
    for (int s = 0; s < M::NV; ++s) w0[M::var(s)] = w[s * plane + id];
    if (!high_order) {
      p2c<M>(w0, out, gm1);
    } else {
      T ww[8], qc[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) { ww[i] = w0[i]; qc[i] = T(0); }
      T c0[8];
      p2c<M>(w0, c0, gm1);
      for (int ax = 0; ax < dim; ++ax) {
        const int nn = ax == 0 ? n0 : n1;
        const int ii = ax == 0 ? i0 : i1;
        const int im = bc_map(ii - 1, nn, bc), ip = bc_map(ii + 1, nn, bc);
        const long long gm = ax == 0 ? cell(im, i1, n1) : cell(i0, im, n1);
        const long long gp = ax == 0 ? cell(ip, i1, n1) : cell(i0, ip, n1);
        T wm[8], wp[8], cm[8], cp[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) { wm[i] = T(0); wp[i] = T(0); }
#pragma unroll
        for (int s = 0; s < M::NV; ++s) { wm[M::var(s)] = w[s * plane + gm]; wp[M::var(s)] = w[s * plane + gp]; }
        p2c<M>(wm, cm, gm1);
        p2c<M>(wp, cp, gm1);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          ww[i] = ww[i] - T(C24) * ((wp[i] - w0[i]) - (w0[i] - wm[i]));
          qc[i] = (ax == 0 ? T(0) : qc[i]) + T(C24) * ((cp[i] - c0[i]) - (c0[i] - cm[i]));
        }
      }
      p2c<M>(ww, out, gm1);
#pragma unroll
      for (int i = 0; i < 8; ++i) out[i] = out[i] + qc[i];
    }
#pragma unroll
    for (int s = 0; s < M::NV; ++s) qa[s * plane + id] = out[M::var(s)];
  }
}

// X + 1/24 d2_0 X (+ 1/24 d2_1 X): fv.high_order_convert('cntr') (fv.py:67-85)
template <typename T>
__global__ void centre_to_avg_kernel(const T* __restrict__ x, T* __restrict__ y, int n0, int n1, long long plane,
                                     int nv, int dim, int bc) {
  const long long n = (long long)n0 * n1;
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < n; id += (long long)gridDim.x * blockDim.x) {
    const int i0 = (int)(id / n1), i1 = (int)(id % n1);
    for (int s = 0; s < nv; ++s) {
      const T* X = x + s * plane;
      const T c = X[id];
      T r = c;
      for (int ax = 0; ax < dim; ++ax) {
        const int nn = ax == 0 ? n0 : n1;
        const int ii = ax == 0 ? i0 : i1;
        const int im = bc_map(ii - 1, nn, bc), ip = bc_map(ii + 1, nn, bc);
        const T m = ax == 0 ? X[cell(im, i1, n1)] : X[cell(i0, im, n1)];
        const T p = ax == 0 ? X[cell(ip, i1, n1)] : X[cell(i0, ip, n1)];
        r = r + T(C24) * ((p - c) - (c - m));
      }
      y[s * plane + id] = r;
    }
  }
}

// Conservative -> primitive of a whole grid (sim_variables.convert_conservative,
// pointwise or 4th order over axes 0 then 1; fv.py:97-101, 126-143)
template <typename T, int MID>
__global__ void prim_kernel(const T* __restrict__ q, T* __restrict__ w, int n0, int n1, long long plane, int dim,
                            int bc, int high_order, T gm1) {
  using M = Model<MID>;
  const long long n = (long long)n0 * n1;
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < n; id += (long long)gridDim.x * blockDim.x) {
    const int i0 = (int)(id / n1), i1 = (int)(id % n1);
    T q0[8], out[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) q0[i] = T(0);
#pragma unroll
    for (int s = 0; s < M::NV; ++s) q0[M::var(s)] = q[s * plane + id];
    if (!high_order) {
      c2p<M>(q0, out, gm1);
    } else {
      T qq[8], wc[8], w0[8];
      c2p<M>(q0, w0, gm1);
#pragma unroll
      for (int i = 0; i < 8; ++i) { qq[i] = q0[i]; wc[i] = T(0); }
      for (int ax = 0; ax < dim; ++ax) {
        const int nn = ax == 0 ? n0 : n1;
        const int ii = ax == 0 ? i0 : i1;
        const int im = bc_map(ii - 1, nn, bc), ip = bc_map(ii + 1, nn, bc);
        const long long gm = ax == 0 ? cell(im, i1, n1) : cell(i0, im, n1);
        const long long gp = ax == 0 ? cell(ip, i1, n1) : cell(i0, ip, n1);
        T qm[8], qp[8], wm[8], wp[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) { qm[i] = T(0); qp[i] = T(0); }
#pragma unroll
        for (int s = 0; s < M::NV; ++s) { qm[M::var(s)] = q[s * plane + gm]; qp[M::var(s)] = q[s * plane + gp]; }
        c2p<M>(qm, wm, gm1);
        c2p<M>(qp, wp, gm1);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          qq[i] = qq[i] - T(C24) * ((qp[i] - q0[i]) - (q0[i] - qm[i]));
          wc[i] = (ax == 0 ? T(0) : wc[i]) + T(C24) * ((wp[i] - w0[i]) - (w0[i] - wm[i]));
        }
      }
      c2p<M>(qq, out, gm1);
#pragma unroll
      for (int i = 0; i < 8; ++i) out[i] = out[i] + wc[i];
    }
#pragma unroll
    for (int s = 0; s < M::NV; ++s) w[s * plane + id] = out[M::var(s)];
  }
}

// Neumaier-compensated FP64 sums of every stored component (total mass,
// momentum, energy, flux): pass 1 writes one (sum, compensation) pair per
// block and component, pass 2 folds them in block order.
__device__ __forceinline__ void neumaier_add(double& s, double& c, double x) {
  const double t = s + x;
  c += fabs(s) >= fabs(x) ? (s - t) + x : (x - t) + s;
  s = t;
}

template <typename T>
__global__ void sums_pass1(const T* __restrict__ q, long long plane, long long n, int nv, double* __restrict__ part) {
  __shared__ double ss[256], cc[256];
  for (int s = 0; s < nv; ++s) {
    double sum = 0.0, comp = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
      neumaier_add(sum, comp, (double)q[s * plane + i]);
    ss[threadIdx.x] = sum;
    cc[threadIdx.x] = comp;
    __syncthreads();
    if (threadIdx.x == 0) {
      double S = 0.0, Cc = 0.0;
      for (int k = 0; k < (int)blockDim.x; ++k) { neumaier_add(S, Cc, ss[k]); Cc += cc[k]; }
      part[(blockIdx.x * nv + s) * 2 + 0] = S;
      part[(blockIdx.x * nv + s) * 2 + 1] = Cc;
    }
    __syncthreads();
  }
}

static __global__ void sums_pass2(const double* __restrict__ part, int nblocks, int nv, double* __restrict__ out) {
  const int s = threadIdx.x;
  if (s >= nv) return;
  double S = 0.0, Cc = 0.0;
  for (int b = 0; b < nblocks; ++b) {
    neumaier_add(S, Cc, part[(b * nv + s) * 2 + 0]);
    Cc += part[(b * nv + s) * 2 + 1];
  }
  out[s] = S + Cc;
}

}  // namespace astrea

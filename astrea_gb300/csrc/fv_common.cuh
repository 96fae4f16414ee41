// Common device helpers for the astrea finite-volume kernels (sm_103a).
//
// Arithmetic follows NumPy element-wise semantics of the reference
// (mervyzr/astrea functions/fv.py): masked divide (fv.py:19-20), NaN-propagating
// np.minimum / np.maximum, np.sign.  The FP64 translation units are compiled
// without fused multiply-add so every expression rounds like NumPy does.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace astrea {

// ---------------------------------------------------------------- enums (match include/astrea_gb300.h)
enum Scheme { PCM = 0, PLM = 1, PPM = 2, WENO3 = 3, WENO5 = 4, WENO7 = 5 };
// LW runs the LLF kernels with the Lax-Wendroff interface coefficient (SweepArgs::lw)
enum Solver { LLF = 0, HLLC = 1, HLLD = 2, LW = 3 };
enum Boundary { EDGE = 0, WRAP = 1 };
enum Integrator { EULER = 0, SSPRK22 = 1, SSPRK33 = 2, SSPRK43 = 3, SSPRK53 = 4, SSPRK54 = 5, SSPRK104 = 6, RK4 = 7 };

// ---------------------------------------------------------------- precision traits
template <typename T> struct Prec;
template <> struct Prec<double> { static constexpr bool EXACT = true; };
template <> struct Prec<float> { static constexpr bool EXACT = false; };

// ---------------------------------------------------------------- NumPy-semantics scalar ops
template <typename T> __device__ __forceinline__ bool isnan_(T a) { return a != a; }
// np.maximum / np.minimum: NaN in either operand gives NaN
template <typename T> __device__ __forceinline__ T npmax(T a, T b) { return (a > b || isnan_(a)) ? a : b; }
template <typename T> __device__ __forceinline__ T npmin(T a, T b) { return (a < b || isnan_(a)) ? a : b; }
// FP32 path: one min/max instruction; a NaN operand is dropped instead of propagated
// (the FP32 path is checked against FP64 by error norms, not bit for bit)
template <> __device__ __forceinline__ float npmax<float>(float a, float b) { return fmaxf(a, b); }
template <> __device__ __forceinline__ float npmin<float>(float a, float b) { return fminf(a, b); }
// maximum that keeps a NaN operand in every precision: the wave-speed maxima use it, so that a
// non-finite cell reaches the clock (and stops the grid) in FP32 as in FP64
template <typename T> __device__ __forceinline__ T nanmax(T a, T b) { return (a > b || isnan_(a)) ? a : b; }
// np.sign: -1, 0 (keeps the zero's sign), +1, NaN
template <typename T> __device__ __forceinline__ T npsign(T a) { return a > T(0) ? T(1) : (a < T(0) ? T(-1) : a); }
// fv.divide: a/b where b != 0 else 0
template <typename T> __device__ __forceinline__ T dvd(T a, T b) { return b != T(0) ? a / b : T(0); }
template <typename T> __device__ __forceinline__ T sq(T a) { return a * a; }
// FP32 three-input minimum / maximum (one instruction on sm_100 and later); a NaN operand is
// dropped, as in fminf / fmaxf
__device__ __forceinline__ float fmin3_(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float fmax3_(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
template <typename T> __device__ __forceinline__ T sqrt_(T a) { return sqrt(a); }
template <> __device__ __forceinline__ float sqrt_<float>(float a) { return sqrtf(a); }
template <typename T> __device__ __forceinline__ T abs_(T a) { return fabs(a); }
template <> __device__ __forceinline__ float abs_<float>(float a) { return fabsf(a); }

// ---------------------------------------------------------------- boundary maps
// The reference pads every intermediate with np.pad(mode=edge|wrap).  In the
// kernels each level is stored at *virtual* indices; an access at virtual v of
// a level is served by the value at rho(v): clamp into [0, n-1] for outflow,
// identity for periodic (periodicity is applied once, when the input state is
// loaded with a modulo map).
struct Clamp {
  int lo, hi;
  __device__ __forceinline__ int operator()(int v) const { return v < lo ? lo : (v > hi ? hi : v); }
};
// tiles whose every level stays inside the grid (or periodic grids) need no clamping
struct NoClamp {
  __device__ __forceinline__ int operator()(int v) const { return v; }
};
__device__ __forceinline__ Clamp make_rho(int bc, int n) {
  Clamp c;
  if (bc == EDGE) { c.lo = 0; c.hi = n - 1; }
  else { c.lo = -(1 << 29); c.hi = (1 << 29); }
  return c;
}
// full boundary map onto [0, n) for the input state
__device__ __forceinline__ int bc_map(int v, int n, int bc) {
  if (bc == EDGE) return v < 0 ? 0 : (v >= n ? n - 1 : v);
  int r = v % n;
  return r < 0 ? r + n : r;
}

// ---------------------------------------------------------------- per-run clock (device resident)
// One per grid.  emax holds the per-axis maximum wave speed as the IEEE bit
// pattern of a non-negative double (so atomicMax on the integer orders them;
// NaN patterns sort above +inf, which makes a NaN speed propagate like np.max).
struct Clock {
  double t;        // simulated time at the start of the current step
  double dt;       // step size of the current step
  double t_end;    // end time
  double chkpt;    // t_end / checkpoints
  double cfl;
  double dx;
  unsigned long long emax[2];
  int idx;         // next checkpoint index (astrea.py:74-78)
  int done;        // set once t == t_end at the start of a step
  int steps;       // completed steps
  int order;       // 0: even step (x then y), 1: odd step (y then x)
  int naxes;
  int status;      // bit 0: non-finite wave speed seen
};

}  // namespace astrea

// Physics of the ideal-(M)HD finite-volume update: variable models, prim<->cons
// conversions, physical flux, interface averages, wave speeds and the
// interface Riemann fluxes (LLF, HLLC, HLLD).
//
// Every formula keeps the operation order of the reference NumPy expressions
// (cited per function) so that the FP64 kernels reproduce them bit for bit.
#pragma once
#include "fv_common.cuh"

namespace astrea {

// ---------------------------------------------------------------- variable models
// A model lists which of the eight variables [rho, v_x, v_y, v_z, p, B_x, B_y, B_z]
// are carried; the others are identically zero for the whole run and are
// neither stored nor computed.
//   3: 1D Euler (rho, m_x, E)      4: 2D Euler (rho, m_x, m_y, E)
//   8: full ideal MHD (and hydro with transverse velocities)
template <int MID> struct Model;
template <> struct Model<3> {
  static constexpr int NV = 3;
  static constexpr bool VY = false, VZ = false, MHD = false;
  __host__ __device__ static constexpr int var(int s) { return s == 0 ? 0 : (s == 1 ? 1 : 4); }
};
template <> struct Model<4> {
  static constexpr int NV = 4;
  static constexpr bool VY = true, VZ = false, MHD = false;
  __host__ __device__ static constexpr int var(int s) { return s < 3 ? s : 4; }
};
template <> struct Model<8> {
  static constexpr int NV = 8;
  static constexpr bool VY = true, VZ = true, MHD = true;
  __host__ __device__ static constexpr int var(int s) { return s; }
};

template <class M, int V> struct Has {
  static constexpr bool value = (V == 0 || V == 1 || V == 4) || (V == 2 && M::VY) || (V == 3 && M::VZ) || (V >= 5 && M::MHD);
};

template <typename T> struct V8 { T v[8]; };

template <typename T> __device__ __forceinline__ void zero8(T* x) {
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = T(0);
}

// norm(v)**2 as the reference forms it (np.linalg.norm then **2: sqrt of the
// sequential sum, squared again).  For a single non-zero component the
// result is exactly x*x.  The FP32 path, which is not bit-compared with the
// reference, takes the sum of squares itself (one root and one product less).
template <class M, typename T> __device__ __forceinline__ T nsq_vel(const T* w) {
  if constexpr (!M::VY) {
    return w[1] * w[1];
  } else {
    T s = w[1] * w[1] + w[2] * w[2];
    if constexpr (M::VZ) s = s + w[3] * w[3];
    if constexpr (!Prec<T>::EXACT) return s;
    T r = sqrt_(s);
    return r * r;
  }
}
template <class M, typename T> __device__ __forceinline__ T nsq_mag(const T* w) {
  if constexpr (!M::MHD) {
    return T(0);
  } else {
    const T s = (w[5] * w[5] + w[6] * w[6]) + w[7] * w[7];
    if constexpr (!Prec<T>::EXACT) return s;
    T r = sqrt_(s);
    return r * r;
  }
}
template <typename T> __device__ __forceinline__ T nsq3(T a, T b, T c) {
  const T s = (a * a + b * b) + c * c;
  if constexpr (!Prec<T>::EXACT) return s;
  T r = sqrt_(s);
  return r * r;
}
template <typename T> __device__ __forceinline__ T norm3(T a, T b, T c) { return sqrt_((a * a + b * b) + c * c); }

// ---------------------------------------------------------------- prim <-> cons (fv.py:49-53, 89-101)
// x / (gamma - 1): FP64 divides (NumPy's rounding); FP32 multiplies by the reciprocal, which
// the compiler forms once per kernel (gamma - 1 is a launch constant)
template <typename T> __device__ __forceinline__ T over_gm1(T x, T gm1) {
  if constexpr (Prec<T>::EXACT) return x / gm1;
  else return x * (T(1) / gm1);
}

// point_convert_primitive
template <class M, typename T> __device__ __forceinline__ void p2c(const T* w, T* q, T gm1) {
  q[0] = w[0];
  q[1] = w[1] * w[0];
  q[2] = M::VY ? w[2] * w[0] : T(0);
  q[3] = M::VZ ? w[3] * w[0] : T(0);
  T kin = w[0] * nsq_vel<M>(w);
  if constexpr (M::MHD) q[4] = over_gm1(w[4], gm1) + T(.5) * (kin + nsq_mag<M>(w));
  else q[4] = over_gm1(w[4], gm1) + T(.5) * kin;
  q[5] = w[5]; q[6] = w[6]; q[7] = w[7];
}

// FP64 internal energy E - K of an FP32 conservative state.  Kept out of line so
// that none of its FP64 work is hoisted into the common path of the callers.
template <class M> __device__ __noinline__ float internal_energy_fp64(float q0, float q1, float q2, float q3, float q4,
                                                                    float q5, float q6, float q7) {
  const double rd = (double)q0;
  const double vx = rd != 0.0 ? (double)q1 / rd : 0.0;
  const double vy = M::VY ? (rd != 0.0 ? (double)q2 / rd : 0.0) : 0.0;
  const double vz = M::VZ ? (rd != 0.0 ? (double)q3 / rd : 0.0) : 0.0;
  double Kd = rd * ((vx * vx + vy * vy) + vz * vz);
  if constexpr (M::MHD) Kd = Kd + (((double)q5 * q5 + (double)q6 * q6) + (double)q7 * q7);
  return (float)((double)q4 - 0.5 * Kd);
}

// point_convert_conservative; in FP32 the internal energy of near-vacuum or
// kinetic-dominated cells (E - K small against E) is recovered in FP64.
template <class M, typename T> __device__ __forceinline__ void c2p(const T* q, T* w, T gm1) {
  T rho = q[0];
  w[0] = rho;
  if constexpr (Prec<T>::EXACT) {
    w[1] = dvd(q[1], rho);
    w[2] = M::VY ? dvd(q[2], rho) : T(0);
    w[3] = M::VZ ? dvd(q[3], rho) : T(0);
  } else {
    // FP32: one reciprocal for the velocity components
    const T inv = rho != T(0) ? T(1) / rho : T(0);
    w[1] = q[1] * inv;
    w[2] = M::VY ? q[2] * inv : T(0);
    w[3] = M::VZ ? q[3] * inv : T(0);
  }
  T kin = rho * nsq_vel<M>(w);
  T K = M::MHD ? T(.5) * (kin + nsq_mag<M>(q)) : T(.5) * kin;
  T e = q[4] - K;
  if constexpr (!Prec<T>::EXACT) {
    if (__builtin_expect(!(e > T(1e-3) * abs_(q[4])), 0))
      e = internal_energy_fp64<M>(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7]);
  }
  w[4] = gm1 * e;
  w[5] = q[5]; w[6] = q[6]; w[7] = q[7];
}

// ---------------------------------------------------------------- physical flux (constructor.make_flux, :113-125)
template <class M, int AX, typename T> __device__ __forceinline__ void make_flux(const T* w, T* F, T gamma, T gm1) {
  constexpr int a = AX, o = (AX + 1) % 3, p = (AX + 2) % 3;
  const T rho = w[0], va = w[1 + a], P = w[4];
  const T rv = rho * va;
  F[0] = rv;
  T nB = nsq_mag<M>(w);
  if constexpr (M::MHD) {
    F[a + 1] = ((rho * (va * va) + P) + T(.5) * nB) - w[5 + a] * w[5 + a];
    F[o + 1] = rv * w[1 + o] - w[5 + a] * w[5 + o];
    F[p + 1] = rv * w[1 + p] - w[5 + a] * w[5 + p];
    T vB = (w[1] * w[5] + w[2] * w[6]) + w[3] * w[7];
    F[4] = va * ((((T(.5) * rho) * nsq_vel<M>(w)) + over_gm1(gamma * P, gm1)) + nB) - w[5 + a] * vB;
    F[o + 5] = w[5 + o] * va - w[5 + a] * w[1 + o];
    F[p + 5] = w[5 + p] * va - w[5 + a] * w[1 + p];
    F[a + 5] = T(0);
  } else {
    F[a + 1] = rho * (va * va) + P;
    F[o + 1] = (Has<M, 1 + o>::value) ? rv * w[1 + o] : T(0);
    F[p + 1] = (Has<M, 1 + p>::value) ? rv * w[1 + p] : T(0);
    F[4] = va * (((T(.5) * rho) * nsq_vel<M>(w)) + over_gm1(gamma * P, gm1));
    F[5] = F[6] = F[7] = T(0);
  }
}

// ---------------------------------------------------------------- interface averages
// PLM: arithmetic mean (plm.py:45)
template <class M, typename T> __device__ __forceinline__ void arith_avg(const T* wp, const T* wm, T* y) {
#pragma unroll
  for (int i = 0; i < 8; ++i) y[i] = T(.5) * (wp[i] + wm[i]);
}
// sqrt(rho)-weighted average (constructor.make_Roe_average, :167-176); B takes the opposite weights
template <class M, typename T> __device__ __forceinline__ void roe_avg(const T* wp, const T* wm, T* y) {
  const T rm = sqrt_(wm[0]), rp = sqrt_(wp[0]);
  const T den = rm + rp;
  y[0] = rm * rp;
  if constexpr (Prec<T>::EXACT) {
#pragma unroll
    for (int i = 1; i < 4; ++i) y[i] = dvd(wp[i] * rp + wm[i] * rm, den);
    y[4] = dvd(rp * wp[4] + rm * wm[4], den);
#pragma unroll
    for (int i = 5; i < 8; ++i) y[i] = M::MHD ? dvd(wp[i] * rm + wm[i] * rp, den) : T(0);
  } else {
    // FP32: one reciprocal of the weight sum
    const T inv = den != T(0) ? T(1) / den : T(0);
#pragma unroll
    for (int i = 1; i < 4; ++i) y[i] = (wp[i] * rp + wm[i] * rm) * inv;
    y[4] = (rp * wp[4] + rm * wm[4]) * inv;
#pragma unroll
    for (int i = 5; i < 8; ++i) y[i] = M::MHD ? (wp[i] * rm + wm[i] * rp) * inv : T(0);
  }
}

// ---------------------------------------------------------------- wave speed
// Largest |eigenvalue| of the 8x8 primitive Jacobian (constructor.make_Jacobian,
// fv.compute_eigen) in closed form: |v_n| + c_f; for an unphysical state with
// gamma p / rho < 0 the complex sound pair's modulus sqrt(v_n^2 - a2).
template <class M, int AX, typename T> __device__ __forceinline__ T max_speed(const T* w, T gamma) {
  const T rho = w[0], vn = w[1 + AX];
  const T a2 = (gamma * w[4]) / rho;
  T fast;
  if constexpr (M::MHD) {
    const T b2 = nsq_mag<M>(w) / rho;
    const T bn2 = (w[5 + AX] * w[5 + AX]) / rho;
    const T s = a2 + b2;
    const T cf2 = T(.5) * (s + sqrt_(s * s - (T(4) * a2) * bn2));
    fast = abs_(vn) + sqrt_(cf2);
  } else if constexpr (Prec<T>::EXACT) {
    const T cf2 = T(.5) * (a2 + sqrt_(a2 * a2));
    fast = abs_(vn) + sqrt_(cf2);
  } else {
    // FP32: for a2 >= 0, (a2 + sqrt(a2^2)) / 2 is a2 itself (a2 < 0 is handled below)
    fast = abs_(vn) + sqrt_(a2);
  }
  if (a2 < T(0)) {
    T c = sqrt_(vn * vn - a2);
    return npmax(c, abs_(vn));
  }
  return fast;
}

// ---------------------------------------------------------------- Riemann solvers
// Local Lax-Friedrichs (solvers.py:69-75)
template <class M, typename T>
__device__ __forceinline__ void llf(T alpha, const T* qp, const T* qm, const T* fp, const T* fm, T* F) {
#pragma unroll
  for (int s = 0; s < M::NV; ++s) {
    const int i = M::var(s);
    F[i] = T(.5) * (fm[i] + fp[i]) - T(.5) * ((qp[i] - qm[i]) * alpha);
  }
}

// HLLC (solvers.py:92-138).  ``label`` is the sweep's iteration position: the
// normal velocity is component label+1 while the star normal momentum is
// always written to component 1; with no wave condition met the flux is f_plus.
// ``physical`` (not a reference option): star normal momentum in component
// label+1 and f_minus where sL > 0 (the textbook solver).
template <class M, typename T>
__device__ __forceinline__ void hllc(int label, int physical, T gamma, const T* wp, const T* wm, const T* qp,
                                     const T* qm, const T* fp, const T* fm, T* F) {
  const T rL = wm[0], pL = wm[4], rR = wp[0], pR = wp[4];
  T uL, uR;
  if constexpr (M::VY) { uL = label == 0 ? wm[1] : wm[2]; uR = label == 0 ? wp[1] : wp[2]; }
  else { uL = wm[1]; uR = wp[1]; }
  T cL, cR, sqL, sqR, u_hat, c2_hat;
  if constexpr (Prec<T>::EXACT) {
    cL = sqrt_(gamma * dvd(pL, rL));
    cR = sqrt_(gamma * dvd(pR, rR));
    sqL = sqrt_(rL);
    sqR = sqrt_(rR);
    u_hat = dvd(uL * sqL + uR * sqR, sqL + sqR);
    c2_hat = dvd(sqL * (cL * cL) + sqR * (cR * cR), sqL + sqR)
           + (T(.5) * ((uR - uL) * (uR - uL))) * dvd(sqL * sqR, (sqL + sqR) * (sqL + sqR));
  } else {
    // FP32: one reciprocal square root per density gives its square root (the Roe weight)
    // and, times sqrt(gamma p), the sound speed; sqrt(rho) c^2 = gamma p / sqrt(rho).  A zero
    // density has weight and sound speed 0, as sqrt(0) and the masked divide give.  One
    // reciprocal of the weight sum serves the three Roe-weighted terms.
    const T iL = rL == T(0) ? T(0) : rsqrtf(rL), iR = rR == T(0) ? T(0) : rsqrtf(rR);
    sqL = rL * iL;
    sqR = rR * iR;
    cL = sqrt_(gamma * pL) * iL;
    cR = sqrt_(gamma * pR) * iR;
    const T sw = sqL + sqR, inv = sw != T(0) ? T(1) / sw : T(0);
    u_hat = (uL * sqL + uR * sqR) * inv;
    c2_hat = (gamma * (pL * iL + pR * iR)) * inv + (T(.5) * ((uR - uL) * (uR - uL))) * ((sqL * sqR) * (inv * inv));
  }
  const T ch = sqrt_(c2_hat);
  const T sL = npmin(uL - cL, u_hat - ch);
  const T sR = npmax(uR + cR, u_hat + ch);
  const T sM = dvd(((pR - pL) + (rL * uL) * (sL - uL)) - (rR * uR) * (sR - uR), rL * (sL - uL) - rR * (sR - uR));
  const bool m3 = sR < T(0);
  const bool m2 = (sM <= T(0)) && (T(0) <= sR);
  const bool m1 = (sL <= T(0)) && (T(0) < sM);
  if (m3 || !(m1 || m2)) {
    const T* f0 = (!m3 && physical) ? fm : fp;
#pragma unroll
    for (int s = 0; s < M::NV; ++s) F[M::var(s)] = f0[M::var(s)];
    return;
  }
  // star state of the side that is selected (m2 has priority over m1)
  const T* W = m2 ? wp : wm;
  const T* Q = m2 ? qp : qm;
  const T* f = m2 ? fp : fm;
  const T rho = W[0], p = W[4];
  const T u = m2 ? uR : uL;
  const T s = m2 ? sR : sL;
  const T coeff = dvd(s - u, s - sM);
  T Qs[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) Qs[k] = Q[k] * coeff;
  const T mstar = (rho * coeff) * sM;
  if (physical && label == 1) Qs[2] = mstar;
  else Qs[1] = mstar;
  Qs[4] = Qs[4] + (coeff * (sM - u)) * (rho * sM + dvd(p, s - u));
#pragma unroll
  for (int k = 0; k < M::NV; ++k) {
    const int i = M::var(k);
    F[i] = f[i] + (Qs[i] - Q[i]) * s;
  }
}

// HLLD fast speed: the 'normal' field is always B_x (solvers.py:144-153)
template <typename T> __device__ __forceinline__ T hlld_fast(const T* w, T gamma, int nb) {
  const T rho = w[0];
  const T cs = sqrt_(dvd(gamma * w[4], rho));
  const T sr = sqrt_(rho);
  const T ca = dvd(norm3(w[5], w[6], w[7]), sr);
  const T cax = dvd(nb == 0 ? w[5] : (nb == 1 ? w[6] : w[7]), sr);
  const T cs2 = cs * cs, ca2 = ca * ca;
  return sqrt_(T(.5) * ((cs2 + ca2) + sqrt_(((cs2 + ca2) * (cs2 + ca2)) - ((T(4) * cs2) * (cax * cax)))));
}

template <typename T> __device__ __forceinline__ T pick3(T x0, T x1, T x2, int i) { return i == 0 ? x0 : (i == 1 ? x1 : x2); }

// HLLD as published (Miyoshi & Kusano 2005, eqs. 38-51 and 59-67), used in the
// physical mode: the reference's solver departs from the paper (sR from
// min(uL, uR), star momenta without their density factors, the right Alfven
// speed's sign, momenta in the energy's v.B) and blows up on the Orszag-Tang
// vortex.  One normal field for both sides: the mean of the two face states'.
// A star state whose denominator rho (S - u)(S - S_M) - Bn^2 vanishes keeps its
// transverse velocity and field: relative to its terms, below 1e-10 in FP64 and
// below 1e-5 in FP32, whose round-off alone leaves ~1e-7 of them in the
// difference (a smaller FP32 threshold divides by that noise).
template <typename T> struct HlldStar { T rs, vs, ws, bys, bzs, Es, vbs; };

template <typename T>
__device__ void hlld_textbook(int a, T gamma, const T* wp, const T* wm, const T* qp, const T* qm, const T* fp,
                              const T* fm, T* F) {
  const int o = (a + 1) % 3, p = (a + 2) % 3;
  const T Bn = T(.5) * (pick3(wm[5], wm[6], wm[7], a) + pick3(wp[5], wp[6], wp[7], a));
  const T rL = wm[0], PL = wm[4], rR = wp[0], PR = wp[4];
  const T uL = pick3(wm[1], wm[2], wm[3], a), vL = pick3(wm[1], wm[2], wm[3], o), wL = pick3(wm[1], wm[2], wm[3], p);
  const T uR = pick3(wp[1], wp[2], wp[3], a), vR = pick3(wp[1], wp[2], wp[3], o), wR = pick3(wp[1], wp[2], wp[3], p);
  const T byL = pick3(wm[5], wm[6], wm[7], o), bzL = pick3(wm[5], wm[6], wm[7], p);
  const T byR = pick3(wp[5], wp[6], wp[7], o), bzR = pick3(wp[5], wp[6], wp[7], p);
  const T bn2 = Bn * Bn;
  auto fast = [&](T r, T P, T by, T bz) -> T {
    const T cs2 = dvd(gamma * P, r);
    const T ca2 = dvd((bn2 + by * by) + bz * bz, r);
    const T cx2 = dvd(bn2, r);
    const T sm = cs2 + ca2;
    return sqrt_(T(.5) * (sm + sqrt_(npmax(sm * sm - (T(4) * cs2) * cx2, T(0)))));
  };
  const T cf = npmax(fast(rL, PL, byL, bzL), fast(rR, PR, byR, bzR));
  const T sL = npmin(uL, uR) - cf;
  const T sR = npmax(uL, uR) + cf;
  const T ptL = PL + T(.5) * ((bn2 + byL * byL) + bzL * bzL);
  const T ptR = PR + T(.5) * ((bn2 + byR * byR) + bzR * bzR);
  const T dL = sL - uL, dR = sR - uR;
  const T den = dR * rR - dL * rL;
  const T sM = dvd((((dR * rR) * uR - (dL * rL) * uL) - ptR) + ptL, den);
  const T pts = dvd(((dR * rR) * ptL - (dL * rL) * ptR) + ((rL * rR) * (dR * dL)) * (uR - uL), den);
  auto star = [&](T r, T u, T v, T w, T by, T bz, T E, T pt, T s, T d) -> HlldStar<T> {
    HlldStar<T> x;
    x.rs = r * dvd(d, s - sM);
    const T rds = (r * d) * (s - sM);
    const T dn = rds - bn2;
    const bool degen = abs_(dn) <= T(Prec<T>::EXACT ? 1e-10 : 1e-5) * (abs_(rds) + bn2);
    const T g = dvd(sM - u, dn);
    const T fac = dvd((r * d) * d - bn2, dn);
    x.vs = degen ? v : v - (Bn * by) * g;
    x.ws = degen ? w : w - (Bn * bz) * g;
    x.bys = degen ? by : by * fac;
    x.bzs = degen ? bz : bz * fac;
    const T vb = (u * Bn + v * by) + w * bz;
    x.vbs = (sM * Bn + x.vs * x.bys) + x.ws * x.bzs;
    x.Es = dvd(((d * E - pt * u) + pts * sM) + Bn * (vb - x.vbs), s - sM);
    return x;
  };
  const HlldStar<T> L = star(rL, uL, vL, wL, byL, bzL, qm[4], ptL, sL, dL);
  const HlldStar<T> R = star(rR, uR, vR, wR, byR, bzR, qp[4], ptR, sR, dR);
  const T sqL = sqrt_(L.rs), sqR = sqrt_(R.rs);
  const T ssL = sM - dvd(abs_(Bn), sqL);
  const T ssR = sM + dvd(abs_(Bn), sqR);
  const T sg = npsign(Bn);
  const T d2 = sqL + sqR;
  const T vss = dvd((sqL * L.vs + sqR * R.vs) + (R.bys - L.bys) * sg, d2);
  const T wss = dvd((sqL * L.ws + sqR * R.ws) + (R.bzs - L.bzs) * sg, d2);
  const T byss = dvd((sqL * R.bys + sqR * L.bys) + ((sqL * sqR) * (R.vs - L.vs)) * sg, d2);
  const T bzss = dvd((sqL * R.bzs + sqR * L.bzs) + ((sqL * sqR) * (R.ws - L.ws)) * sg, d2);
  const T vbss = (sM * Bn + vss * byss) + wss * bzss;
  const T EssL = L.Es - (sqL * (L.vbs - vbss)) * sg;
  const T EssR = R.Es + (sqR * (R.vbs - vbss)) * sg;
  const bool m1 = (sL <= T(0)) && (T(0) < ssL), m2 = (ssL <= T(0)) && (T(0) < sM);
  const bool m3 = (sM <= T(0)) && (T(0) < ssR), m4 = (ssR <= T(0)) && (T(0) <= sR), m5 = sR < T(0);
  // component k of the conserved vector of a (star or double-star) state
  auto U = [&](int k, T r, T v, T w, T E, T by, T bz) -> T {
    if (k == 0) return r;
    if (k == 4) return E;
    if (k < 4) return k - 1 == a ? r * sM : (k - 1 == o ? r * v : r * w);
    return k - 5 == a ? Bn : (k - 5 == o ? by : bz);
  };
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const T usL = U(k, L.rs, L.vs, L.ws, L.Es, L.bys, L.bzs), usR = U(k, R.rs, R.vs, R.ws, R.Es, R.bys, R.bzs);
    const T ussL = U(k, L.rs, vss, wss, EssL, byss, bzss), ussR = U(k, R.rs, vss, wss, EssR, byss, bzss);
    const T fsL = fm[k] + (usL - qm[k]) * sL, fsR = fp[k] + (usR - qp[k]) * sR;
    const T fssL = fsL + (ussL - usL) * ssL, fssR = fsR + (ussR - usR) * ssR;
    T f = fm[k];
    if (m1) f = fsL;
    if (m2) f = fssL;
    if (m3) f = fssR;
    if (m4) f = fsR;
    if (m5) f = fp[k];
    F[k] = f;
  }
}

// HLLD of Miyoshi & Kusano (solvers.py:142-232), reference quirks kept.  Bn is
// component label+5 of the cell-averaged state right of the interface.
template <typename T>
__device__ void hlld(int label, int physical, T gamma, const T* wSr, const T* wp, const T* wm, const T* qp,
                     const T* qm, const T* fp, const T* fm, T* F) {
  if (physical) {
    hlld_textbook<T>(label, gamma, wp, wm, qp, qm, fp, fm, F);
    return;
  }
  const int a = label, o = label + 1, p = (label + 2) % 3;
  const T rL = wm[0], pL = wm[4], rR = wp[0], pR = wp[4];
  const T uL = pick3(wm[1], wm[2], wm[3], a), uR = pick3(wp[1], wp[2], wp[3], a);
  const T Bn = pick3(wSr[5], wSr[6], wSr[7], a);
  const int nb = physical ? label : 0;
  const T cfL = hlld_fast(wm, gamma, nb), cfR = hlld_fast(wp, gamma, nb);
  const T umin = npmin(uL, uR), cmax = npmax(cfL, cfR);
  const T sL = umin - cmax, sR = umin + cmax;
  const T nBL = nsq3(wm[5], wm[6], wm[7]), nBR = nsq3(wp[5], wp[6], wp[7]);
  const T den0 = rL * (sL - uL) - rR * (sR - uR);
  const T sM = dvd(((((pR - pL) + (rL * uL) * (sL - uL)) - (rR * uR) * (sR - uR)) + T(.5) * nBR) - T(.5) * nBL, den0);
  const T rLs = rL * dvd(sL - uL, sL - sM), rRs = rR * dvd(sR - uR, sR - sM);
  const T sLs = sM - dvd(pick3(wm[5], wm[6], wm[7], a), sqrt_(rLs));
  const T sRs = sM - dvd(pick3(wp[5], wp[6], wp[7], a), sqrt_(rRs));

  const bool c5 = sR < T(0);
  const bool c4 = (sRs <= T(0)) && (T(0) <= sR);
  const bool c3 = (sM <= T(0)) && (T(0) < sRs);
  const bool c2 = (sLs <= T(0)) && (T(0) < sM);
  const bool c1 = (sL <= T(0)) && (T(0) < sLs);
  if (c5) {
#pragma unroll
    for (int i = 0; i < 8; ++i) F[i] = fp[i];
    return;
  }
  if (!(c1 || c2 || c3 || c4)) {
#pragma unroll
    for (int i = 0; i < 8; ++i) F[i] = fm[i];
    return;
  }
  const T p_star = dvd(((rL * (pR + T(.5) * nBR)) * (sL - uL) - (rR * (pL + T(.5) * nBL)) * (sR - uR))
                       + ((rR * rL) * (sL - uL)) * (sR - uR), den0);
  const T Bn2 = Bn * Bn;
  // transverse star states of both sides (needed by the double-star states)
  T vy[2], vz[2], by[2], bz[2];
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const T* w = side == 0 ? wm : wp;
    const T rho = w[0], u = side == 0 ? uL : uR, s = side == 0 ? sL : sR;
    const T den = ((rho * (s - u)) * (s - sM)) - Bn2;
    const T vo = pick3(w[1], w[2], w[3], o), vp = pick3(w[1], w[2], w[3], p);
    const T Bo = pick3(w[5], w[6], w[7], o), Bp = pick3(w[5], w[6], w[7], p);
    vy[side] = vo - (Bn * Bo) * dvd(sM - u, den);
    vz[side] = vp - (Bn * Bp) * dvd(sM - u, den);
    by[side] = Bo * dvd(rho * ((s - u) * (s - u)) - Bn2, den);
    bz[side] = Bp * dvd(rho * ((s - u) * (s - u)) - Bn2, den);
  }
  const bool right = c3 || c4;
  const int side = right ? 1 : 0;
  const T* w = right ? wp : wm;
  const T* Q = right ? qp : qm;
  const T* f = right ? fp : fm;
  const T rho = w[0], u = right ? uR : uL, s = right ? sR : sL, P = w[4], nB = right ? nBR : nBL;
  const T rs = right ? rRs : rLs;
  // star state: velocity/field components in the (a, o, p) frame
  T Qs[8];
  Qs[0] = rs;
  const T mA = rho * sM, mO = rho * vy[side], mP = rho * vz[side];
  const T bA = pick3(Q[5], Q[6], Q[7], a);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    Qs[1 + i] = i == a ? mA : (i == o ? mO : mP);
    Qs[5 + i] = i == a ? bA : (i == o ? by[side] : bz[side]);
  }
  const T vB = (w[1] * w[5] + w[2] * w[6]) + w[3] * w[7];
  const T QsVB = (Qs[1] * Qs[5] + Qs[2] * Qs[6]) + Qs[3] * Qs[7];
  Qs[4] = dvd((((Q[4] * (s - u)) - u * (P + T(.5) * nB)) + p_star * sM) + Bn * (vB - QsVB), s - sM);
  if (right ? c4 : c1) {
#pragma unroll
    for (int i = 0; i < 8; ++i) F[i] = f[i] + (Qs[i] - Q[i]) * s;
    return;
  }
  // double-star state
  const T sqLs = sqrt_(rLs), sqRs = sqrt_(rRs);
  const T sgn = npsign(Bn);
  const T dsum = sqLs + sqRs;
  const T vy2 = dvd((vy[1] * sqRs + vy[0] * sqLs) + sgn * (by[0] - by[1]), dsum);
  const T vz2 = dvd((vz[1] * sqRs + vz[0] * sqLs) + sgn * (bz[0] - bz[1]), dsum);
  const T srr = sqrt_(rRs * rLs);
  const T By2 = dvd((by[0] * sqRs + by[1] * sqLs) + (sgn * (vy[0] - vy[1])) * srr, dsum);
  const T Bz2 = dvd((bz[0] * sqRs + bz[1] * sqLs) + (sgn * (vz[0] - vz[1])) * srr, dsum);
  T Q2[8];
  Q2[0] = rs;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    Q2[1 + i] = i == a ? sM : (i == o ? vy2 : vz2);
    Q2[5 + i] = i == a ? bA : (i == o ? By2 : Bz2);
  }
  const T Q2VB = (Q2[1] * Q2[5] + Q2[2] * Q2[6]) + Q2[3] * Q2[7];
  const T sq = right ? sqRs : sqLs;
  Q2[4] = Qs[4] - (sq * sgn) * (QsVB - Q2VB);
  const T ss = right ? sRs : sLs;
#pragma unroll
  for (int i = 0; i < 8; ++i) F[i] = f[i] + (Q2[i] - Qs[i]) * ss;
}

}  // namespace astrea

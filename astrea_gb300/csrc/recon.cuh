// Reconstruction of face values from cell-averaged primitives along a sweep.
//
// Each function evaluates one component of one cell.  ``at(x)`` returns the
// cell-averaged primitive at virtual index x (already boundary-mapped);
// ``rho`` maps a virtual index of the *same* intermediate onto the index that
// serves it (clamp for outflow, identity for periodic), so that each
// intermediate (face value, second/third differences) is padded on its own,
// like the reference's repeated np.pad calls.
#pragma once
#include "fv_common.cuh"

namespace astrea {

// Reach of each scheme along the sweep (cells left / right of the cell)
template <int SCH> struct Reach;
template <> struct Reach<PCM> { static constexpr int L = 0, R = 0; };
template <> struct Reach<PLM> { static constexpr int L = 1, R = 1; };
// PPM: the faces need 2 cells each side and the limiter 2 more; optional flattening
// reads pressure 3 cells beyond the face range, hence one more on the left.
template <> struct Reach<PPM> { static constexpr int L = 4, R = 4; };
template <> struct Reach<WENO3> { static constexpr int L = 1, R = 1; };
template <> struct Reach<WENO5> { static constexpr int L = 2, R = 2; };
template <> struct Reach<WENO7> { static constexpr int L = 3, R = 3; };

// PLM with minmod (limiters.py:10-19) or superbee (limiters.py:47-49) slopes; plm.py:26-36
template <typename T, class A, class RH>
__device__ __forceinline__ void recon_plm(const A& at, const RH& rho, int r, int limiter, T& wL, T& wR) {
  const T c = at(r), m = at(rho(r - 1)), p = at(rho(r + 1));
  const T a = c - m, b = p - c;
  T s;
  if (limiter == 0) {
    s = (a * b > T(0)) ? (abs_(a) < abs_(b) ? a : b) : T(0);
  } else {
    const T rr = dvd(a, b);
    const T phi = npmax(T(0), npmax(npmin(T(2) * rr, T(1)), npmin(rr, T(2))));
    s = phi * b;
  }
  const T g = T(.5) * s;
  wL = c - g;
  wR = c + g;
}

// 4th-order face value at x+1/2 (ppm.py:38)
template <typename T, class A, class RH> __device__ __forceinline__ T ppm_face(const A& at, const RH& rho, int x) {
  return T(7.0 / 12.0) * (at(x) + at(rho(x + 1))) - T(1.0 / 12.0) * (at(rho(x - 1)) + at(rho(x + 2)));
}
template <typename T, class A, class RH> __device__ __forceinline__ T ppm_d2c(const A& at, const RH& rho, int x) {
  return (at(rho(x - 1)) - T(2) * at(x)) + at(rho(x + 1));
}
template <typename T, class A, class RH> __device__ __forceinline__ T ppm_d3(const A& at, const RH& rho, int x) {
  return ppm_d2c<T>(at, rho, rho(x + 1)) - ppm_d2c<T>(at, rho, x);
}

// PPM faces with the McCorquodale & Colella extremum-preserving limiter
// (ppm.py:30-72 with author 'mc'; limiters.extrapolant_limiter, limiters.py:82-143).
// For finite data the limiter's no-extremum-anywhere branch
// (limiters.py:141-143) gives the same values as the main branch, so the main
// branch is evaluated for every cell.
// The McCorquodale & Colella limiter of one cell from its stencil values:
// w at r-2..r+2, the unlimited faces at r-1/2 and r+1/2, second differences
// d2c at r-1..r+1 and third differences d3 at r-2, r-1, r, r+2.
template <typename T>
__device__ __forceinline__ void ppm_mc_limit(T w0, T wm1, T wp1, T wm2, T wp2, T fL, T fR, T d2c_m, T d2c, T d2c_p,
                                             T d3_m2, T d3_m1, T d3, T d3_p2, T& wL, T& wR) {
  const T C = T(1.25);
  const T dwm = w0 - fL, dwp = fR - w0;
  const T d2w = T(6) * ((fL - T(2) * w0) + fR);
  const bool extremum = (dwm * dwp <= T(0)) || ((w0 - wm2) * (wp2 - w0) <= T(0));
  // min(|d2w|, C|d2c|, C|d2c_p|, C|d2c_m|): C > 0 and rounding is monotone, so the three
  // products' minimum is the product of the minimum (the same value, NaN included)
  T rl, d3min, d3max;
  if constexpr (Prec<T>::EXACT) {
    const T cmin = npmin(abs_(d2w), C * npmin(npmin(abs_(d2c), abs_(d2c_p)), abs_(d2c_m)));
    const T scale = npmax(abs_(w0), npmax(npmax(abs_(wm1), abs_(wp1)), npmax(abs_(wm2), abs_(wp2))));
    const bool sensitive = abs_(d2w) > T(1e-12) * scale;
    const T d2w_lim = extremum ? npsign(d2c) * cmin : T(0);
    rl = sensitive ? dvd(d2w_lim, d2w) : T(0);
    d3min = npmin(npmin(d3_m1, d3), npmin(d3_m2, d3_p2));
    d3max = npmax(npmax(d3_m1, d3), npmax(d3_m2, d3_p2));
  } else {
    // FP32: three-input minima and maxima; sign(d2c) * cmin is cmin with d2c's sign (cmin
    // is 0 where d2c is), and a sensitive d2w is non-zero, so the quotient needs no zero test
    const T cmin = fminf(abs_(d2w), C * fmin3_(abs_(d2c), abs_(d2c_p), abs_(d2c_m)));
    const T scale = fmax3_(fmax3_(abs_(w0), abs_(wm1), abs_(wp1)), abs_(wm2), abs_(wp2));
    const bool sensitive = abs_(d2w) > T(1e-12) * scale;
    const T d2w_lim = extremum ? copysignf(cmin, d2c) : T(0);
    rl = sensitive ? __fdividef(d2w_lim, d2w) : T(0);
    d3min = fmin3_(fminf(d3_m1, d3), d3_m2, d3_p2);
    d3max = fmax3_(fmaxf(d3_m1, d3), d3_m2, d3_p2);
  }
  const bool limit = (rl < T(1.0 - 1e-12)) || (T(.1) * npmax(abs_(d3max), abs_(d3min)) <= (d3max - d3min));
  T L = fL, R = fR;
  if ((dwm * dwp < T(0)) && limit) {
    L = w0 - rl * dwm;
    R = w0 + rl * dwp;
  }
  if (limit && abs_(dwm) >= T(2) * abs_(dwp)) L = (w0 - (T(2) * (T(1) - rl)) * dwp) - rl * dwm;
  if (limit && abs_(dwp) >= T(2) * abs_(dwm)) R = (w0 + (T(2) * (T(1) - rl)) * dwm) + rl * dwp;
  wL = L;
  wR = R;
}

// A face value at x+1/2 blended towards the cell value at x by the flattening
// coefficient eta(x) (ppm.py:67 with apply_flattener): f * eta + w * (1 - eta);
// FP32 as w + eta * (f - w) (one rounding less).
template <typename T> __device__ __forceinline__ T ppm_flatten(T f, T w, T eta) {
  if constexpr (Prec<T>::EXACT) return f * eta + w * (T(1) - eta);
  else return w + eta * (f - w);
}

// ``eta`` (nullptr: no flattening) gives the flattening coefficient at a mapped cell index.
template <typename T, class A, class RH>
__device__ __forceinline__ void recon_ppm(const A& at, const RH& rho, int r, T& wL, T& wR, const T* eta = nullptr) {
  const T w0 = at(r), wm1 = at(rho(r - 1)), wp1 = at(rho(r + 1)), wm2 = at(rho(r - 2)), wp2 = at(rho(r + 2));
  T fL = ppm_face<T>(at, rho, rho(r - 1));
  T fR = ppm_face<T>(at, rho, r);
  if (eta) {
    fL = ppm_flatten<T>(fL, wm1, eta[rho(r - 1)]);
    fR = ppm_flatten<T>(fR, w0, eta[r]);
  }
  const T d2c = (wm1 - T(2) * w0) + wp1;
  const T d2c_m = ppm_d2c<T>(at, rho, rho(r - 1));
  const T d2c_p = ppm_d2c<T>(at, rho, rho(r + 1));
  const T d3 = ppm_d3<T>(at, rho, r);
  const T d3_m1 = ppm_d3<T>(at, rho, rho(r - 1));
  const T d3_m2 = ppm_d3<T>(at, rho, rho(r - 2));
  const T d3_p2 = ppm_d3<T>(at, rho, rho(r + 2));
  ppm_mc_limit<T>(w0, wm1, wp1, wm2, wp2, fL, fR, d2c_m, d2c, d2c_p, d3_m2, d3_m1, d3, d3_p2, wL, wR);
}

// The same reconstruction for K consecutive cells r0 .. r0+K-1 where no index
// needs a boundary map (interior or periodic tiles): the cells' stencils
// overlap, so every face value, second and third difference is computed once
// and shared instead of once per cell that uses it.  Same expressions, same
// results.  ``out(k, wL, wR, fR)`` receives cell r0+k and its unlimited face
// value at r0+k+1/2.
template <typename T, int K, class A, class OUT>
__device__ __forceinline__ void recon_ppm_strip(const A& at, int r0, const OUT& out, const T* eta = nullptr) {
  T w[K + 7];     // x = r0-3 .. r0+K+3
  T d2[K + 5];    // x = r0-2 .. r0+K+2
  T d3[K + 4];    // x = r0-2 .. r0+K+1
  T f[K + 1];     // faces at x+1/2, x = r0-1 .. r0+K-1
#pragma unroll
  for (int i = 0; i < K + 7; ++i) w[i] = at(r0 - 3 + i);
#pragma unroll
  for (int j = 0; j < K + 5; ++j) d2[j] = (w[j] - T(2) * w[j + 1]) + w[j + 2];
#pragma unroll
  for (int j = 0; j < K + 4; ++j) d3[j] = d2[j + 1] - d2[j];
#pragma unroll
  for (int j = 0; j < K + 1; ++j) f[j] = T(7.0 / 12.0) * (w[j + 2] + w[j + 3]) - T(1.0 / 12.0) * (w[j + 1] + w[j + 4]);
  if (eta) {
#pragma unroll
    for (int j = 0; j < K + 1; ++j) f[j] = ppm_flatten<T>(f[j], w[j + 2], eta[r0 - 1 + j]);
  }
#pragma unroll
  for (int k = 0; k < K; ++k) {
    T wl, wr;
    ppm_mc_limit<T>(w[k + 3], w[k + 2], w[k + 4], w[k + 1], w[k + 5], f[k], f[k + 1], d2[k + 1], d2[k + 2],
                    d2[k + 3], d3[k], d3[k + 1], d3[k + 2], d3[k + 4], wl, wr);
    out(k, wl, wr, f[k + 1]);
  }
}

// WENO-JS, eps = 1e-6 (weno.py:22-149)
template <typename T, class A, class RH>
__device__ __forceinline__ void recon_weno3(const A& at, const RH& rho, int r, T& wL, T& wR) {
  const T eps = T(1e-6);
  const T z = at(r), m1 = at(rho(r - 1)), p1 = at(rho(r + 1));
  const T g0 = T(1.0 / 3.0), g1 = T(2.0 / 3.0);
  const T b0 = (z - m1) * (z - m1), b1 = (p1 - z) * (p1 - z);
  const T e0 = (b0 + eps) * (b0 + eps), e1 = (b1 + eps) * (b1 + eps);
  const T a0g0 = g0 / e0, a1g1 = g1 / e1, a1g0 = g0 / e1, a0g1 = g1 / e0;
  wR = (a0g0 / (a0g0 + a1g1)) * (T(1.5) * z - T(.5) * m1) + (a1g1 / (a0g0 + a1g1)) * (T(.5) * z + T(.5) * p1);
  wL = (a1g0 / (a0g1 + a1g0)) * (T(1.5) * z - T(.5) * p1) + (a0g1 / (a0g1 + a1g0)) * (T(.5) * z + T(.5) * m1);
}

template <typename T, class A, class RH>
__device__ __forceinline__ void recon_weno5(const A& at, const RH& rho, int r, T& wL, T& wR) {
  const T eps = T(1e-6);
  const T z = at(r), m1 = at(rho(r - 1)), p1 = at(rho(r + 1)), m2 = at(rho(r - 2)), p2 = at(rho(r + 2));
  const T g0 = T(1.0 / 10.0), g1 = T(3.0 / 5.0), g2 = T(3.0 / 10.0);
  const T c1312 = T(13.0 / 12.0), c14 = T(1.0 / 4.0);
  const T t0 = (m2 - T(2) * m1) + z, u0 = (m2 - T(4) * m1) + T(3) * z;
  const T t1 = (m1 - T(2) * z) + p1, u1 = m1 - p1;
  const T t2 = (z - T(2) * p1) + p2, u2 = (T(3) * z - T(4) * p1) + p2;
  const T b0 = c1312 * (t0 * t0) + c14 * (u0 * u0);
  const T b1 = c1312 * (t1 * t1) + c14 * (u1 * u1);
  const T b2 = c1312 * (t2 * t2) + c14 * (u2 * u2);
  const T e0 = (b0 + eps) * (b0 + eps), e1 = (b1 + eps) * (b1 + eps), e2 = (b2 + eps) * (b2 + eps);
  {
    const T a0 = g0 / e0, a1 = g1 / e1, a2 = g2 / e2;
    const T s = (a0 + a1) + a2;
    wR = ((a0 / s) * ((T(1.0 / 3.0) * m2 - T(7.0 / 6.0) * m1) + T(11.0 / 6.0) * z)
          + (a1 / s) * ((T(-1.0 / 6.0) * m1 + T(5.0 / 6.0) * z) + T(1.0 / 3.0) * p1))
         + (a2 / s) * ((T(1.0 / 3.0) * z + T(5.0 / 6.0) * p1) - T(1.0 / 6.0) * p2);
  }
  {
    const T a0 = g2 / e0, a1 = g1 / e1, a2 = g0 / e2;
    const T s = (a0 + a1) + a2;
    wL = ((a0 / s) * ((T(1.0 / 3.0) * z + T(5.0 / 6.0) * m1) - T(1.0 / 6.0) * m2)
          + (a1 / s) * ((T(-1.0 / 6.0) * p1 + T(5.0 / 6.0) * z) + T(1.0 / 3.0) * m1))
         + (a2 / s) * ((T(1.0 / 3.0) * p2 - T(7.0 / 6.0) * p1) + T(11.0 / 6.0) * z);
  }
}

template <typename T, class A, class RH>
__device__ __forceinline__ void recon_weno7(const A& at, const RH& rho, int r, T& wL, T& wR) {
  const T eps = T(1e-6);
  const T z = at(r), m1 = at(rho(r - 1)), p1 = at(rho(r + 1)), m2 = at(rho(r - 2)), p2 = at(rho(r + 2));
  const T m3 = at(rho(r - 3)), p3 = at(rho(r + 3));
  const T g0 = T(1.0 / 35.0), g1 = T(12.0 / 35.0), g2 = T(18.0 / 35.0), g3 = T(4.0 / 35.0);
  const T b0 = ((m3 * (((T(547) * m3 - T(3882) * m2) + T(4642) * m1) - T(1854) * z)
                 + m2 * ((T(7043) * m2 - T(17246) * m1) + T(7042) * z))
                + m1 * (T(11003) * m1 - T(9402) * z))
               + z * (T(2107) * z);
  const T b1 = ((m2 * (((T(267) * m2 - T(1642) * m1) + T(1602) * z) - T(494) * p1)
                 + m1 * ((T(2843) * m1 - T(5966) * z) + T(1922) * p1))
                + z * (T(3443) * z - T(2522) * p1))
               + p1 * (T(547) * p1);
  const T b2 = ((m1 * (((T(547) * m1 - T(2522) * z) + T(1922) * p1) - T(494) * p2)
                 + z * ((T(3443) * z - T(5966) * p1) + T(1602) * p2))
                + p1 * (T(2843) * p1 - T(1642) * p2))
               + p2 * (T(267) * p2);
  const T b3 = ((z * (((T(2107) * z - T(9402) * p1) + T(7042) * p2) - T(1854) * p3)
                 + p1 * ((T(11003) * p1 - T(17246) * p2) + T(4642) * p3))
                + p2 * (T(7043) * p2 - T(3882) * p3))
               + p3 * (T(547) * p3);
  const T e0 = (b0 + eps) * (b0 + eps), e1 = (b1 + eps) * (b1 + eps), e2 = (b2 + eps) * (b2 + eps), e3 = (b3 + eps) * (b3 + eps);
  {
    const T a0 = g0 / e0, a1 = g1 / e1, a2 = g2 / e2, a3 = g3 / e3;
    const T s = ((a0 + a1) + a2) + a3;
    wR = (((a0 / s) * (((T(-1.0 / 4.0) * m3 + T(13.0 / 12.0) * m2) - T(23.0 / 12.0) * m1) + T(25.0 / 12.0) * z)
           + (a1 / s) * (((T(1.0 / 12.0) * m2 - T(5.0 / 12.0) * m1) + T(13.0 / 12.0) * z) + T(1.0 / 4.0) * p1))
          + (a2 / s) * (((T(-1.0 / 12.0) * m1 + T(7.0 / 12.0) * z) + T(7.0 / 12.0) * p1) - T(1.0 / 12.0) * p2))
         + (a3 / s) * (((T(1.0 / 4.0) * z + T(13.0 / 12.0) * p1) - T(5.0 / 12.0) * p2) + T(1.0 / 12.0) * p3);
  }
  {
    const T a0 = g3 / e0, a1 = g2 / e1, a2 = g1 / e2, a3 = g0 / e3;
    const T s = ((a0 + a1) + a2) + a3;
    wL = (((a0 / s) * (((T(1.0 / 4.0) * z + T(13.0 / 12.0) * m1) - T(5.0 / 12.0) * m2) + T(1.0 / 12.0) * m3)
           + (a1 / s) * (((T(-1.0 / 12.0) * p1 + T(7.0 / 12.0) * z) + T(7.0 / 12.0) * m1) - T(1.0 / 12.0) * m2))
          + (a2 / s) * (((T(1.0 / 12.0) * p2 - T(5.0 / 12.0) * p1) + T(13.0 / 12.0) * z) + T(1.0 / 4.0) * m1))
         + (a3 / s) * (((T(-1.0 / 4.0) * p3 + T(13.0 / 12.0) * p2) - T(23.0 / 12.0) * p1) + T(25.0 / 12.0) * z);
  }
}

template <int SCH, typename T, class A, class RH>
__device__ __forceinline__ void reconstruct(const A& at, const RH& rho, int r, int limiter, T& wL, T& wR,
                                            const T* eta = nullptr) {
  if constexpr (SCH == PCM) { wL = wR = at(r); }
  else if constexpr (SCH == PLM) recon_plm<T>(at, rho, r, limiter, wL, wR);
  else if constexpr (SCH == PPM) recon_ppm<T>(at, rho, r, wL, wR, eta);
  else if constexpr (SCH == WENO3) recon_weno3<T>(at, rho, r, wL, wR);
  else if constexpr (SCH == WENO5) recon_weno5<T>(at, rho, r, wL, wR);
  else recon_weno7<T>(at, rho, r, wL, wR);
}

}  // namespace astrea

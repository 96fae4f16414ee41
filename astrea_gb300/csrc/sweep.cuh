// The sweep kernel: one axis of the spatial operator for one tile of the grid.
//
// A CTA owns TS cells along the sweep axis and TT rows across it.  It stages
// the conservative state of the tile plus halos in shared memory and computes,
// level by level, every intermediate the reference builds with whole-array
// NumPy for that axis (schemes/*.run, solvers.calculate_Riemann_flux):
//
//   q  -> wS (cell-averaged primitives, 2nd or 4th order)      fv.py:89-143
//      -> (wL, wR) face values per cell (PCM/PLM/PPM/WENO)      schemes/*, limiters.py
//      -> interface speeds lambda of the interface averages      fv.compute_eigen
//      -> face-averaged Riemann flux F_avg                         solvers.py:39-42
//      -> [2D] face-centred states, second solve, F_c - d2 F_avg  solvers.py:44-57
//      -> divergence (F[i+1]-F[i])/dx                              evolvers.py:41-49
//
// and then either stores the divergence (first sweep of a stage) or adds the
// other sweep's divergence and applies the Runge-Kutta stage combine
// (last sweep of a stage).  2D high-order tiles of the single-grid and batched
// engines start at wS instead: a per-stage pre-pass (cellavg.cuh) forms it once
// for both sweeps, and the tile stages it (WSIN).  Every level is held at *virtual* indices; an
// access at virtual v of a level is served by the value at rho(v) (clamp for
// outflow), which is the reference's per-intermediate np.pad.
#pragma once
#include <type_traits>

#include "physics.cuh"
#include "recon.cuh"
#include "tma.cuh"

namespace astrea {

constexpr double C24 = 1.0 / 24.0;

// The 4th-order transverse conversion x0 - (1/24) (xp - 2 x0 + xm) of the reference
// (fv.py:105-122, 147-153).  FP64 keeps its operation order (bit parity with NumPy); FP32, which
// is not bit-compared, forms (1 + 1/12) x0 - (1/24)(xp + xm): three instructions instead of four.
template <typename T> __device__ __forceinline__ T conv24(T x0, T xm, T xp) {
  if constexpr (Prec<T>::EXACT) return x0 - T(C24) * ((xp - x0) - (x0 - xm));
  else return T(1.0 + 2.0 * C24) * x0 - T(C24) * (xp + xm);
}
// y - (1/24)(xp - 2 x0 + xm) (the same correction applied to another value)
template <typename T> __device__ __forceinline__ T sub_d2_24(T y, T x0, T xm, T xp) {
  if constexpr (Prec<T>::EXACT) return y - T(C24) * ((xp - x0) - (x0 - xm));
  else return (y + T(2.0 * C24) * x0) - T(C24) * (xp + xm);
}
// y + (1/24)(xp - 2 x0 + xm)
template <typename T> __device__ __forceinline__ T add_d2_24(T y, T x0, T xm, T xp) {
  if constexpr (Prec<T>::EXACT) return y + T(C24) * ((xp - x0) - (x0 - xm));
  else return (y - T(2.0 * C24) * x0) + T(C24) * (xp + xm);
}

// The same three conversions over all variables of a state (8-slot arrays).  For the FP32
// 2D-Euler model the four stored variables (slots 0, 1, 2, 4) go through the packed FP32 pipe
// two at a time (one fma2/add2/mul2 instruction per pair): the same operations as the scalar
// forms, half the instructions.
template <class M, typename T> constexpr bool kPacked4 = std::is_same<T, float>::value && M::NV == 4;
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }
template <class M, typename T> __device__ __forceinline__ void conv24_all(const T* x0, const T* xm, const T* xp, T* out) {
  if constexpr (kPacked4<M, T>) {
    const float2 A = f2(1.0f + float(2.0 * C24), 1.0f + float(2.0 * C24)), nc = f2(-float(C24), -float(C24));
    const float2 a = __ffma2_rn(nc, __fadd2_rn(f2(xp[0], xp[1]), f2(xm[0], xm[1])), __fmul2_rn(A, f2(x0[0], x0[1])));
    const float2 b = __ffma2_rn(nc, __fadd2_rn(f2(xp[2], xp[4]), f2(xm[2], xm[4])), __fmul2_rn(A, f2(x0[2], x0[4])));
    out[0] = a.x; out[1] = a.y; out[2] = b.x; out[4] = b.y;
    out[3] = out[5] = out[6] = out[7] = T(0);
  } else {
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = conv24<T>(x0[i], xm[i], xp[i]);
  }
}
// out = y + sign * (1/24)(xp - 2 x0 + xm), sign = -1 (sub_d2_24) or +1 (add_d2_24)
template <class M, typename T, int SIGN>
__device__ __forceinline__ void d2_24_all(const T* y, const T* x0, const T* xm, const T* xp, T* out) {
  if constexpr (kPacked4<M, T>) {
    const float c = float(C24), c2 = float(2.0 * C24);
    const float2 k1 = f2(SIGN > 0 ? -c2 : c2, SIGN > 0 ? -c2 : c2), k2 = f2(SIGN > 0 ? c : -c, SIGN > 0 ? c : -c);
    const float2 a = __ffma2_rn(k2, __fadd2_rn(f2(xp[0], xp[1]), f2(xm[0], xm[1])), __ffma2_rn(k1, f2(x0[0], x0[1]), f2(y[0], y[1])));
    const float2 b = __ffma2_rn(k2, __fadd2_rn(f2(xp[2], xp[4]), f2(xm[2], xm[4])), __ffma2_rn(k1, f2(x0[2], x0[4]), f2(y[2], y[4])));
    out[0] = a.x; out[1] = a.y; out[2] = b.x; out[4] = b.y;
    out[3] = out[5] = out[6] = out[7] = T(0);
  } else {
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = SIGN > 0 ? add_d2_24<T>(y[i], x0[i], xm[i], xp[i]) : sub_d2_24<T>(y[i], x0[i], xm[i], xp[i]);
  }
}

template <typename T> struct SweepArgs {
  const T* q;         // stage input state, NV planes
  long long plane;    // plane stride (elements)
  int n0, n1;         // grid extents: axis 0 (x), axis 1 (y, contiguous); 1D: n0 = N, n1 = 1
  int bc;
  int label;          // HLLC/HLLD axis label (iteration position); < 0: from the clock's axis order
  int limiter;        // PLM slope limiter: 0 minmod, 1 superbee
  int mode;           // 0: store divergence, 1: add other divergence + combine, 2: combine (sole sweep)
  int integ, stage;   // Runge-Kutta scheme and stage for the combine
  int want_emax;      // accumulate the max wave speed of this axis into the clock
  int physical;       // textbook HLLC/HLLD (label = physical axis) instead of the reference's
  int lw;             // LLF kernels: the Lax-Wendroff coefficient v_n^2 / max|lambda| instead of max|lambda|
  T gamma, gm1;
  double dx;
  T* dout;            // mode 0: divergence output (NV planes)
  const T* dother;    // mode 1: divergence of the other sweep
  const T* u0;        // step-start state
  T* out;             // combine output
  T* out_host;        // optional: the combine output also stored to page-locked host memory (same layout)
  Clock* clock;
  T* flux_out;        // optional: interface fluxes [NV][Ns+1][Nt]
  T* wface_out;       // optional (2D MHD): face value at i+1/2 of every cell, physical layout [8][n0][n1]
  int flatten;        // PPM: Colella (1990) flattening of the face values
  int viscosity;      // PPM: McCorquodale & Colella (2011) artificial viscosity added to the fluxes
  T av_alpha, av_beta;
  const CUtensorMap* tmaps;  // optional (2D): TMA maps of the staged level, indexed [axis][tile]; nullptr: plain loads
  const T* ws;        // 2D high-order single-grid sweeps: the stage input's cell-averaged primitives in this
                      // sweep's axis order (NV planes, from cell_average_kernel); they replace q's levels
  const CUtensorMap* qmaps;  // optional (with ws): TMA maps of q for the viscous strip (StripBox), [axis][tile]
};

// plane index of primitive variable v in model M (-1 if M does not store it)
template <class M> __host__ __device__ constexpr int plane_of(int v) {
  for (int s = 0; s < M::NV; ++s)
    if (M::var(s) == v) return s;
  return -1;
}

// Cells per thread in the shared-stencil PPM level of a 2D tile: a divisor of the
// level width (7 or 5), or 1 (per-cell evaluation).  1D tiles keep one cell per
// thread: they have too few rows to fill a CTA with strips.
template <int RW, int DIM> struct PpmStrip {
  static constexpr int K = DIM != 2 ? 1 : (RW % 7 == 0 ? 7 : (RW % 5 == 0 ? 5 : 1));
};

template <int SCH, int DIM, int TS, int TT> struct Geom {
  static constexpr bool HO = SCH >= PPM;  // 4th-order conversions (generic.py:250-255)
  static constexpr bool ROE = SCH >= PPM; // Roe-type interface average for the wave speed
  // sweep-axis ranges [s0+BEG, s0+TS+END) of each level
  static constexpr int R_BEG = -1, R_END = 2;
  static constexpr int W_BEG = R_BEG - Reach<SCH>::L, W_END = R_END + Reach<SCH>::R;
  static constexpr int Q_BEG = W_BEG - (HO ? 1 : 0), Q_END = W_END + (HO ? 1 : 0);
  static constexpr int QW = TS + Q_END - Q_BEG, WW = TS + W_END - W_BEG, RW = TS + R_END - R_BEG;
  static constexpr int YW = TS + 2;  // lambda of the interface averages right of cells s0-1 .. s0+TS
  static constexpr int KW = TS + 1;  // interfaces s0 .. s0+TS
  // transverse halos (2D): rows [t0-H, t0+TT+H)
  static constexpr int FT = DIM == 2 ? 1 : 0;
  static constexpr int RT = DIM == 2 ? (HO ? 2 : 1) : 0;
  static constexpr int WT = RT;
  static constexpr int QT = DIM == 2 ? (HO ? 3 : 1) : 0;
  static constexpr int QH = TT + 2 * QT, WH = TT + 2 * WT, RH = TT + 2 * RT, FH = TT + 2 * FT;
};

// The TMA box of a tile's staged level: the cell-averaged primitives wS of the
// high-order schemes, the state q of the others (whose q and wS levels have the
// same extent).  Axis 1 sweeps run along the contiguous
// axis (box x = sweep, y = rows), axis 0 sweeps across it (box x = rows, y =
// sweep); the box's x origin is rounded down to 16 bytes and its x extent up to
// 16 bytes, and XOFF is where the staged level starts inside the box's x.
// When TT is not a multiple of 16 bytes' worth of elements (axis 0 sweeps), the
// x origin of a tile's box is rounded down per tile (DYN) and the box is wide
// enough for every remainder.
template <typename T, int SCH, int DIM, int AX, int TS, int TT, int NV> struct TmaBox {
  using G = Geom<SCH, DIM, TS, TT>;
  static constexpr int A = 16 / (int)sizeof(T);
  static constexpr bool DYN = AX == 0 && TT % A != 0;
  static constexpr int XB = AX == 1 ? floor_to(G::W_BEG, A) : floor_to(-G::WT, A);
  static constexpr int BW = AX == 1 ? ceil_to(TS + G::W_END - XB, A)
                                    : (DYN ? ceil_to(G::WH + A - 1, A) : ceil_to(TT + G::WT - XB, A));
  static constexpr int BH = AX == 1 ? G::WH : G::WW;
  static constexpr int XOFF = AX == 1 ? G::W_BEG - XB : -G::WT - XB;
  static constexpr int BYTES = NV * BH * BW * (int)sizeof(T);
  static constexpr int TILE_ID = TT == 8 ? 0 : 1;
  static_assert(BW <= 256 && BH <= 256 && (BW * (int)sizeof(T)) % 16 == 0, "TMA box limits");
  // x origin of the box and the staged level's first column inside it, for the tile at (s0, t0)
  __host__ __device__ static int x0(int s0, int t0) {
    if (AX == 1) return s0 + XB;
    return DYN ? ((t0 - G::WT) / A) * A : t0 + XB;  // t0 - WT >= 0 whenever the box is used
  }
  __host__ __device__ static int xoff(int t0) { return DYN ? (t0 - G::WT) - x0(0, t0) : XOFF; }
  // the box of the tile at (s0, t0) lies inside an n0 x n1 grid
  __host__ __device__ static bool inside(int s0, int t0, int n0, int n1) {
    return AX == 1 ? (s0 + XB >= 0 && s0 + XB + BW <= n1 && t0 - G::WT >= 0 && t0 - G::WT + BH <= n0)
                   : (t0 - G::WT >= 0 && x0(s0, t0) + BW <= n1 && s0 + G::W_BEG >= 0 && s0 + G::W_BEG + BH <= n0);
  }
};

// The TMA box of the viscous strip of a WSIN PPM tile: the state on cells
// [s0-1, s0+TS] along the sweep and rows [t0, t0+TT) across it, with the box's
// x origin rounded down and its x extent up to 16 bytes (as TmaBox).
template <typename T, int AX, int TS, int TT> struct StripBox {
  static constexpr int A = 16 / (int)sizeof(T);
  static constexpr bool DYN = AX == 0 && TT % A != 0;
  static constexpr int BW = AX == 1 ? ceil_to(TS + 1 + A, A) : (DYN ? ceil_to(TT + A - 1, A) : TT);
  static constexpr int BH = AX == 1 ? TT : TS + 2;
  static constexpr int TILE_ID = TT == 8 ? 0 : 1;
  static_assert(BW <= 256 && BH <= 256 && (BW * (int)sizeof(T)) % 16 == 0, "TMA box limits");
  __host__ __device__ static int x0(int s0, int t0) { return AX == 1 ? s0 - A : (DYN ? (t0 / A) * A : t0); }
  __host__ __device__ static int y0(int s0, int t0) { return AX == 1 ? t0 : s0 - 1; }
  // the box lies inside an n0 x n1 grid
  __host__ __device__ static bool inside(int s0, int t0, int n0, int n1) {
    return AX == 1 ? (s0 - A >= 0 && s0 - A + BW <= n1 && t0 + TT <= n0)
                   : (x0(s0, t0) + BW <= n1 && s0 - 1 >= 0 && s0 - 1 + BH <= n0);
  }
  // element of plane v, cell x along the sweep (in [s0-1, s0+TS]), row rt (in [t0, t0+TT))
  __host__ __device__ static int at(int v, int x, int rt, int s0, int t0) {
    return AX == 1 ? (v * BH + (rt - t0)) * BW + (x - (s0 - A)) : (v * BH + (x - (s0 - 1))) * BW + (rt - x0(s0, t0));
  }
};

// Cell-interleaved levels (the face values R, the five face arrays and the final fluxes F)
// hold the variables of one cell side by side, padded to a whole number of 16-byte units, so
// that a cell's variables move with one or two vector loads and stores: the element (li, s)
// of such a level is at li * NVP + s.  The staged levels (q, its primitives, wS) keep one plane
// per variable, which the along-the-sweep stencils read one variable at a time.
template <int NV> struct Interleave {
  static constexpr int NVP = NV == 3 ? 4 : NV;
};

// WSIN: the tile stages the precomputed wS level and has no q level.  Every level starts at a
// multiple of four elements (16 bytes or more) from the 16-byte aligned dynamic shared memory.
template <int SCH, int DIM, int TS, int TT, int NV, bool WSIN = false> struct Smem {
  using G = Geom<SCH, DIM, TS, TT>;
  static constexpr int NVP = Interleave<NV>::NVP;
  static constexpr int n_q = WSIN ? 0 : ceil_to(NV * G::QH * G::QW, 4);
  static constexpr int n_qw = G::HO ? n_q : 0;
  static constexpr int n_face = DIM == 2 ? 5 * NVP * G::FH * G::KW : 0;
  static constexpr int n_F = NVP * TT * G::KW;
  // the face arrays reuse the q level once it is dead; PCM reads raw q on faces, so it keeps q
  static constexpr int FA_OFF = SCH == PCM ? n_q : 0;
  static constexpr int n_region0 = ceil_to((n_q + n_qw) > (FA_OFF + n_face + n_F) ? (n_q + n_qw) : (FA_OFF + n_face + n_F), 4);
  // WSIN tiles of axis-0 sweeps read the w level where its bulk copy lands: room for that box
  // (at most WH + 3 elements across, rounded to 16 bytes) and 128 bytes of alignment
  static constexpr int n_w_box = (WSIN && DIM == 2) ? NV * G::WW * ceil_to(G::WH + 3, 4) + 32 : 0;
  static constexpr int n_w = ceil_to(NV * G::WH * G::WW > n_w_box ? NV * G::WH * G::WW : n_w_box, 4);
  static constexpr int n_R = 2 * NVP * G::RH * G::RW;
  static constexpr int n_lam = G::FH * G::YW;
  static constexpr int base = ceil_to(n_region0 + n_w + n_R + n_lam + 64, 4);
  // PPM extras: flattening coefficients on the rows of the face level and the
  // columns [s0-2, s0+TS+2), and the viscous face fluxes of the tile's interfaces.
  // In 2D the viscous fluxes sit where the final fluxes go (they are added there),
  // and the coefficients in the gap of region 0 between the staged state and the
  // face arrays; otherwise both go past the end.
  // The coefficients need chi_bar one column further on each side (n_cb).
  static constexpr int n_eta = SCH == PPM ? G::RH * (G::RW + 1) : 0;
  static constexpr int n_cb = SCH == PPM ? G::RH * (G::RW + 3) : 0;
  static constexpr int n_mu = SCH == PPM ? NVP * TT * G::KW : 0;  // interleaved like F (it sits where F goes)
  static constexpr bool MU_IN_F = DIM == 2;
  static constexpr bool ETA_IN_GAP = DIM == 2 && (n_q + n_qw + n_eta + n_cb <= FA_OFF + n_face);
  static constexpr int MU_OFF = MU_IN_F ? FA_OFF + n_face : base;
  static constexpr int ETA_OFF = ETA_IN_GAP ? n_q + n_qw : base + (MU_IN_F ? 0 : n_mu);
  static constexpr int CB_OFF = ETA_OFF + n_eta;
  static constexpr int total0 = base + (MU_IN_F ? 0 : n_mu) + (ETA_IN_GAP ? 0 : n_eta + n_cb);
  // WSIN PPM tiles: the state on the viscous faces' cells (columns [s0-1, s0+TS], the
  // tile's rows), staged for the viscous fluxes, after the coefficients when it fits
  // (per-thread layout [NV][TT][TS+2], or a StripBox of either axis plus 128 bytes of alignment)
  static constexpr int QSW = TS + 2;
  static constexpr int n_qs_box = NV * ((TS + 8) * TT > (TT + 6) * (TS + 2) ? (TS + 8) * TT : (TT + 6) * (TS + 2)) + 32;
  static constexpr int n_qs = (WSIN && SCH == PPM) ? (NV * TT * QSW > n_qs_box ? NV * TT * QSW : n_qs_box) : 0;
  static constexpr bool QS_IN_GAP = ETA_IN_GAP && (n_q + n_qw + n_eta + n_cb + n_qs <= FA_OFF + n_face);
  static constexpr int QS_OFF = QS_IN_GAP ? CB_OFF + n_cb : total0;
  static constexpr int total = total0 + (QS_IN_GAP ? 0 : n_qs);
};

// Addressing of the w level: element (plane pl, row r, column c), rows and columns counted
// from the level's first, at pl * PS + r * PR + c * PC.  A plane per variable with rows along
// the sweep, or (IN_BOX) the axis-0 bulk-copy box as it lands: the box's x runs across the
// sweep, so rows are contiguous there.
template <bool IN_BOX, class G, class B> struct WLayout {
  static constexpr int PS = G::WH * G::WW, PR = G::WW, PC = 1;
};
template <class G, class B> struct WLayout<true, G, B> {
  static constexpr int PS = B::BH * B::BW, PR = 1, PC = B::BW;
};

template <class M, typename T> __device__ __forceinline__ void load_sm(const T* base, int stride, int idx, T* x) {
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = T(0);
#pragma unroll
  for (int s = 0; s < M::NV; ++s) x[M::var(s)] = base[s * stride + idx];
}
template <class M, typename T> __device__ __forceinline__ void store_sm(T* base, int stride, int idx, const T* x) {
#pragma unroll
  for (int s = 0; s < M::NV; ++s) base[s * stride + idx] = x[M::var(s)];
}

// Element li of a cell-interleaved level (16-byte vector accesses: the level's base and
// li * NVP * sizeof(T) are multiples of 16 bytes by construction of Smem)
template <class M, typename T> __device__ __forceinline__ void load_aos(const T* base, int li, T* x) {
  constexpr int NVP = Interleave<M::NV>::NVP, PER = 16 / (int)sizeof(T);
  static_assert(NVP % PER == 0, "a cell's interleaved variables fill whole 16-byte units");
  T v[NVP];
  const T* p = base + li * NVP;
#pragma unroll
  for (int c = 0; c < NVP / PER; ++c) {
    if constexpr (sizeof(T) == 4) {
      const float4 u = reinterpret_cast<const float4*>(p)[c];
      v[4 * c] = u.x; v[4 * c + 1] = u.y; v[4 * c + 2] = u.z; v[4 * c + 3] = u.w;
    } else {
      const double2 u = reinterpret_cast<const double2*>(p)[c];
      v[2 * c] = u.x; v[2 * c + 1] = u.y;
    }
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = T(0);
#pragma unroll
  for (int s = 0; s < M::NV; ++s) x[M::var(s)] = v[s];
}
template <class M, typename T> __device__ __forceinline__ void store_aos(T* base, int li, const T* x) {
  constexpr int NVP = Interleave<M::NV>::NVP, PER = 16 / (int)sizeof(T);
  T v[NVP];
#pragma unroll
  for (int s = 0; s < NVP; ++s) v[s] = s < M::NV ? x[M::var(s < M::NV ? s : 0)] : T(0);
  T* p = base + li * NVP;
#pragma unroll
  for (int c = 0; c < NVP / PER; ++c) {
    if constexpr (sizeof(T) == 4) reinterpret_cast<float4*>(p)[c] = make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]);
    else reinterpret_cast<double2*>(p)[c] = make_double2(v[2 * c], v[2 * c + 1]);
  }
}

// Stage combines (evolvers.py:150-185), with the reference's operation order
template <typename T> __device__ __forceinline__ T combine(int integ, int stage, T u, T cur, T L, T dt) {
  switch (integ) {
    case SSPRK33:
      if (stage == 0) return u + dt * L;
      if (stage == 1) return T(.25) * ((T(3) * u + cur) + dt * L);
      return T(1.0 / 3.0) * ((u + T(2) * cur) + (T(2) * dt) * L);
    case SSPRK22:
      if (stage == 0) return u + dt * L;
      return T(.5) * ((u + cur) + dt * L);
    case SSPRK43:
      if (stage == 0) return u + (T(.5) * dt) * L;
      if (stage == 1) return cur + (T(.5) * dt) * L;
      if (stage == 2) return T(1.0 / 6.0) * ((T(4) * u + T(2) * cur) + dt * L);
      return cur + (T(.5) * dt) * L;
    default:  // forward Euler
      return u + dt * L;
  }
}

// Block maximum in T (converting a float to double is exact and monotone, so the
// maximum of the floats is the maximum of their doubles), one atomic per CTA; a NaN
// speed wins (the clock's atomicMax on IEEE bits orders NaN above +inf).
template <typename T> __device__ __forceinline__ void block_max_to_clock(T v, unsigned long long* dst) {
  __shared__ T red[32];
  T x = v;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = nanmax(x, __shfl_xor_sync(0xffffffffu, x, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = x;
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    T y = lane < nw ? red[lane] : T(0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) y = nanmax(y, __shfl_xor_sync(0xffffffffu, y, o));
    if (lane == 0) atomicMax(dst, (unsigned long long)__double_as_longlong((double)y));
  }
}

// One tile: cells [s0, s0+TS) along the sweep and rows [t0, t0+TT) across it.
// Called by the single-grid kernel (one tile per CTA) and by the batched
// persistent kernel (a work list of tiles of many grids).  WSIN: the tile
// stages the precomputed cell-averaged primitives a.ws instead of forming them
// from the state (2D high-order schemes, single-grid kernel).
template <typename T, int MID, int SCH, int SOL, int DIM, int AX, int TS, int TT, bool CL, int NT, bool TMA = false,
          bool WSIN = false>
__device__ __forceinline__ void sweep_tile_body(const SweepArgs<T>& a, const int s0, const int t0,
                                                unsigned char* __restrict__ smem_raw) {
  using M = Model<MID>;
  using G = Geom<SCH, DIM, TS, TT>;
  using S = Smem<SCH, DIM, TS, TT, M::NV, WSIN>;
  static_assert(!WSIN || (DIM == 2 && G::HO), "precomputed wS is for 2D high-order tiles");
  static_assert(!TMA || WSIN || !G::HO, "the TMA box holds the wS level: high-order tiles stage it precomputed");
  static_assert(S::FA_OFF % 4 == 0 && S::n_face % 4 == 0 && S::n_region0 % 4 == 0 && S::n_w % 4 == 0 &&
                    S::n_R % 4 == 0 && S::n_F % 4 == 0 && (SCH != PPM || S::MU_OFF % 4 == 0),
                "cell-interleaved levels start on 16-byte boundaries");
  constexpr int NVP = Interleave<M::NV>::NVP;
  constexpr int NV = M::NV;
  T* sm = reinterpret_cast<T*>(smem_raw);
  T* s_q = sm;                       // region 0 (a): q and its point primitives
  T* s_qw = s_q + S::n_q;
  T* s_fa = sm + S::FA_OFF;          // region 0 (b): face arrays (2D) and F
  T* s_F = s_fa + S::n_face;
  T* s_w = sm + S::n_region0;
  T* s_R = s_w + S::n_w;
  // the w level: planar at s_w, or (axis-0 sweeps staged by bulk copy) the copied box itself
  constexpr bool W_IN_BOX = WSIN && TMA && DIM == 2 && AX == 0;
  using WL = WLayout<W_IN_BOX, G, TmaBox<T, SCH, 2, 0, TS, TT, M::NV>>;
  T* s_wb = s_w;
  // element (plane pl, real row rt, real column x) of the w level
  auto wat = [&](int pl, int rt, int x) -> T {
    return s_wb[pl * WL::PS + (rt - (t0 - G::WT)) * WL::PR + (x - (s0 + G::W_BEG)) * WL::PC];
  };
  T* s_lam = s_R + S::n_R;

  const int Ns = DIM == 1 ? a.n0 : (AX == 0 ? a.n0 : a.n1);
  const int Nt = DIM == 1 ? 1 : (AX == 0 ? a.n1 : a.n0);
  using Rho = typename std::conditional<CL, Clamp, NoClamp>::type;
  Rho rs_, rt_;
  if constexpr (CL) {
    rs_ = make_rho(a.bc, Ns);
    rt_ = make_rho(a.bc, Nt);
  }
  const T gamma = a.gamma, gm1 = a.gm1;
  // the CTA size is a compile-time constant, so the per-level loops have known trip counts
  const int tid = threadIdx.x;
  constexpr int nth = NT;
  // axis label of this sweep: its position in the step's iteration order
  const int label = a.physical ? (DIM == 1 ? 0 : AX)
                  : (a.label >= 0 ? a.label : (DIM == 1 ? 0 : (AX == 0 ? a.clock->order : 1 - a.clock->order)));

  auto gidx = [&](int gs, int gt) -> long long {
    if (DIM == 1) return gs;
    return AX == 0 ? (long long)gs * a.n1 + gt : (long long)gt * a.n1 + gs;
  };

  // element (gs, gt) of a grid-sized input, at a virtual index served by the boundary map
  auto gmap = [&](int v, int n) -> int { return (v >= 0 && v < n) ? v : bc_map(v, n, a.bc); };
  // Stage combine (mode 1): the other divergence, u0 and the stage state of the tile's own
  // cells are read only by the last level; their lines are requested from L2 now.  Each
  // memory row of the tile is one segment of at most 128 bytes in FP32 (two lines at most),
  // 256 bytes in FP64 (two lines, aligned): its first and last elements' lines cover it.
  if constexpr (DIM == 2) {
    if (a.mode == 1) {
      constexpr int MR = AX == 1 ? TT : TS;  // memory rows of the tile (axis-0 indices)
      const int seg = AX == 1 ? (s0 + TS <= Ns ? TS : Ns - s0) : (t0 + TT <= Nt ? TT : Nt - t0);
      for (int e = tid; e < 3 * NV * MR * 2; e += nth) {
        const int end = e & 1, r = (e >> 1) % MR, rest = (e >> 1) / MR, v = rest % NV, arr = rest / NV;
        const int vs = AX == 1 ? s0 + end * (seg - 1) : s0 + r, vt = AX == 1 ? t0 + r : t0 + end * (seg - 1);
        if (vs >= Ns || vt >= Nt) continue;
        const T* base = arr == 0 ? a.dother : (arr == 1 ? a.u0 : a.q);
        prefetch_l2(base + v * a.plane + gidx(vs, vt));
      }
    }
  }
  // WSIN PPM tiles with viscosity: the viscous strip arrives by bulk copy (same for the whole CTA)
  bool strip_tma = false;
  T* qs_box = nullptr;
  if constexpr (WSIN && TMA && SCH == PPM) {
    using SB = StripBox<T, AX, TS, TT>;
    static_assert(NV * SB::BH * SB::BW + 128 / (int)sizeof(T) <= S::n_qs, "viscous strip box exceeds its region");
    strip_tma = a.viscosity && a.qmaps != nullptr && SB::inside(s0, t0, a.n0, a.n1);
    qs_box = align128_shared(sm + S::QS_OFF);
  }

  if constexpr (WSIN) {
    // ---- level wS, staged: the cell-averaged primitives of the stage input, precomputed
    // for this sweep's axis order (the same values levels q and wS form below)
    constexpr int W = G::WW, H = G::WH;
    // PPM with viscosity: the state on the cells either side of the tile's interfaces, for
    // the viscous fluxes: a second bulk copy beside the wS box when both lie inside the grid,
    // else per-thread loads (in the bulk-copy path their loads overlap the copy)
    auto stage_strip = [&]() {
      if constexpr (SCH == PPM) {
        if (a.viscosity) {
          constexpr int QW = S::QSW;
          T* s_qs = sm + S::QS_OFF;
          for (int e = tid; e < QW * TT; e += nth) {
            int row, col;
            if (AX == 0) { row = e % TT; col = e / TT; } else { col = e % QW; row = e / QW; }
            const long long g = gidx(gmap(s0 - 1 + col, Ns), gmap(t0 + row, Nt));
#pragma unroll
            for (int s = 0; s < NV; ++s) s_qs[(s * TT + row) * QW + col] = a.q[s * a.plane + g];
          }
        }
      }
    };
    if constexpr (TMA) {
      using B = TmaBox<T, SCH, DIM, AX, TS, TT, NV>;
      using SB = StripBox<T, AX, TS, TT>;
      __shared__ unsigned long long s_bar;
      // axis 0: the box lands in the w level's region and is read in place; axis 1: it lands
      // in the (still unused) R region and is copied into the planar w level
      T* stage = align128_shared(AX == 0 ? s_w : s_R);
      if (tid == 0) {
        mbar_init(&s_bar, 1);
        mbar_fence_init();
        unsigned bytes = (unsigned)B::BYTES;
        if (strip_tma) bytes += (unsigned)(NV * SB::BH * SB::BW * (int)sizeof(T));
        mbar_arrive_expect_tx(&s_bar, bytes);
        const CUtensorMap* map = a.tmaps + (AX * 2 + B::TILE_ID);
        if (AX == 1) tma_load_3d(stage, map, B::x0(s0, t0), t0 - G::WT, 0, &s_bar);
        else tma_load_3d(stage, map, B::x0(s0, t0), s0 + G::W_BEG, 0, &s_bar);
        if (strip_tma) tma_load_3d(qs_box, a.qmaps + (AX * 2 + SB::TILE_ID), SB::x0(s0, t0), SB::y0(s0, t0), 0, &s_bar);
      }
      // only warp 0 waits on the barrier: its lanes see thread 0's initialisation after a
      // warp barrier; the other warps wait in the block barrier below
      if (tid < 32) __syncwarp();
      if (!strip_tma) stage_strip();
      // one warp polls the barrier; the others sleep in the block barrier, which then
      // orders the copied data (visible to the polling warp) before their reads
      const bool landed = tid < 32 ? mbar_wait_timed(&s_bar, 0, kCopyWaitNs) : true;
      if (!__syncthreads_and(landed)) {
        // the copy did not complete in time: flag the grid, wait (bounded) for the copy, stop this tile
        if (tid == 0) {
          atomicOr(&a.clock->status, 2);
          mbar_wait_timed(&s_bar, 0, kDrainWaitNs);
        }
        return;
      }
      const int xo = B::xoff(t0);
      if constexpr (AX == 0) {
        s_wb = stage + xo;
      } else {
        for (int e = tid; e < W * H; e += nth) {
          const int col = e % W, row = e / W;
#pragma unroll
          for (int s = 0; s < NV; ++s) s_w[(s * H + row) * W + col] = stage[(s * B::BH + row) * B::BW + col + xo];
        }
      }
    } else {
      for (int e = tid; e < W * H; e += nth) {
        int row, col;
        if (AX == 0) { row = e % H; col = e / H; } else { col = e % W; row = e / W; }
        const long long g = gidx(gmap(s0 + G::W_BEG + col, Ns), gmap(t0 - G::WT + row, Nt));
#pragma unroll
        for (int s = 0; s < NV; ++s) s_w[(s * H + row) * W + col] = a.ws[s * a.plane + g];
      }
      stage_strip();
    }
  } else if constexpr (TMA) {
    // ---- level q: conservative state with halos (input boundary map), and its point primitives;
    // one thread issues the bulk copy of the whole box into the (still unused) R region
    using B = TmaBox<T, SCH, DIM, AX, TS, TT, NV>;
    __shared__ unsigned long long s_bar;
    T* stage = align128_shared(s_R);
    if (tid == 0) {
      mbar_init(&s_bar, 1);
      mbar_fence_init();
      mbar_arrive_expect_tx(&s_bar, (unsigned)B::BYTES);
      const CUtensorMap* map = a.tmaps + (AX * 2 + B::TILE_ID);
      if (AX == 1) tma_load_3d(stage, map, B::x0(s0, t0), t0 - G::QT, 0, &s_bar);
      else tma_load_3d(stage, map, B::x0(s0, t0), s0 + G::Q_BEG, 0, &s_bar);
    }
    if (tid < 32) __syncwarp();  // warp 0 polls the barrier after thread 0 initialised it
    const bool landed = tid < 32 ? mbar_wait_timed(&s_bar, 0, kCopyWaitNs) : true;
    if (!__syncthreads_and(landed)) {
      // the copy did not complete in time: flag the grid, wait (bounded) for the copy, stop this tile
      if (tid == 0) {
        atomicOr(&a.clock->status, 2);
        mbar_wait_timed(&s_bar, 0, kDrainWaitNs);
      }
      return;
    }
    constexpr int W = G::QW, H = G::QH;
    const int xo = B::xoff(t0);
    for (int e = tid; e < W * H; e += nth) {
      int row, col;
      if (DIM == 2 && AX == 0) { row = e % H; col = e / H; } else { col = e % W; row = e / W; }
      T q[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) q[i] = T(0);
#pragma unroll
      for (int s = 0; s < NV; ++s)
        q[M::var(s)] = AX == 1 ? stage[(s * B::BH + row) * B::BW + col + xo]
                               : stage[(s * B::BH + col) * B::BW + row + xo];
      const int li = row * W + col;
      store_sm<M>(s_q, H * W, li, q);
      if constexpr (G::HO) {
        T w[8];
        c2p<M>(q, w, gm1);
        store_sm<M>(s_qw, H * W, li, w);
      }
    }
  } else {
    constexpr int W = G::QW, H = G::QH;
    for (int e = tid; e < W * H; e += nth) {
      int row, col;
      if (DIM == 2 && AX == 0) { row = e % H; col = e / H; } else { col = e % W; row = e / W; }
      const int vs = s0 + G::Q_BEG + col, vt = t0 - G::QT + row;
      const int gs = (vs >= 0 && vs < Ns) ? vs : bc_map(vs, Ns, a.bc);
      const int gt = DIM == 2 ? ((vt >= 0 && vt < Nt) ? vt : bc_map(vt, Nt, a.bc)) : 0;
      const long long g = gidx(gs, gt);
      T q[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) q[i] = T(0);
#pragma unroll
      for (int s = 0; s < NV; ++s) q[M::var(s)] = a.q[s * a.plane + g];
      const int li = row * W + col;
      store_sm<M>(s_q, H * W, li, q);
      if constexpr (G::HO) {
        T w[8];
        c2p<M>(q, w, gm1);
        store_sm<M>(s_qw, H * W, li, w);
      }
    }
  }
  // (read in place, the staged level was ordered by the copy's barrier already)
  if constexpr (!W_IN_BOX) __syncthreads();

  // ---- level wS: cell-averaged primitives
  // (items laid out with the staged level's row pitch, so that a warp's loads
  // stay in consecutive banks across a row change; the two extra columns idle)
  if constexpr (!WSIN) {
    constexpr int W = G::WW, H = G::WH, QW = G::QW, QH = G::QH;
    for (int e = tid; e < QW * H; e += nth) {
      const int row = e / QW, col = e % QW;
      if (col >= W) continue;
      const int vs = s0 + G::W_BEG + col, vt = t0 - G::WT + row;
      const int rs = rs_(vs), rt = DIM == 2 ? rt_(vt) : 0;
      const int qc = rs - (s0 + G::Q_BEG), qr = rt - (t0 - G::QT);
      T w[8];
      if constexpr (G::HO) {
        // fv.high_order_convert_conservative: sweep axis first, then transverse (fv.py:126-143)
        const int qcm = rs_(rs - 1) - (s0 + G::Q_BEG), qcp = rs_(rs + 1) - (s0 + G::Q_BEG);
        T qq[8], wc[8];
        T q0[8], qm[8], qp[8], w0[8], wm[8], wp[8];
        load_sm<M>(s_q, QH * QW, qr * QW + qc, q0);
        load_sm<M>(s_q, QH * QW, qr * QW + qcm, qm);
        load_sm<M>(s_q, QH * QW, qr * QW + qcp, qp);
        load_sm<M>(s_qw, QH * QW, qr * QW + qc, w0);
        load_sm<M>(s_qw, QH * QW, qr * QW + qcm, wm);
        load_sm<M>(s_qw, QH * QW, qr * QW + qcp, wp);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          qq[i] = q0[i] - T(C24) * ((qp[i] - q0[i]) - (q0[i] - qm[i]));
          wc[i] = T(C24) * ((wp[i] - w0[i]) - (w0[i] - wm[i]));
        }
        if constexpr (DIM == 2) {
          const int qrm = rt_(rt - 1) - (t0 - G::QT), qrp = rt_(rt + 1) - (t0 - G::QT);
          load_sm<M>(s_q, QH * QW, qrm * QW + qc, qm);
          load_sm<M>(s_q, QH * QW, qrp * QW + qc, qp);
          load_sm<M>(s_qw, QH * QW, qrm * QW + qc, wm);
          load_sm<M>(s_qw, QH * QW, qrp * QW + qc, wp);
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            qq[i] = qq[i] - T(C24) * ((qp[i] - q0[i]) - (q0[i] - qm[i]));
            wc[i] = wc[i] + T(C24) * ((wp[i] - w0[i]) - (w0[i] - wm[i]));
          }
        }
        c2p<M>(qq, w, gm1);
#pragma unroll
        for (int i = 0; i < 8; ++i) w[i] = w[i] + wc[i];
      } else {
        T q0[8];
        load_sm<M>(s_q, QH * QW, qr * QW + qc, q0);
        c2p<M>(q0, w, gm1);
      }
      store_sm<M>(s_w, H * W, row * W + col, w);
    }
    __syncthreads();
  }

  // ---- PPM extras (optional): flattening coefficients (ppm.apply_flattener,
  // ppm.py:111-134) and artificial-viscosity face fluxes (ppm.apply_artificial_viscosity,
  // ppm.py:138-170).  Neither runs in the reference (its code for them fails); the
  // kernels follow those formulas with the two corrections from the cited papers
  // that the oracle makes (strong compressive jumps only; no second factor dx).
  T* s_eta = sm + S::ETA_OFF;
  T* s_mu = sm + S::MU_OFF;
  if constexpr (SCH == PPM) {
    if (a.flatten || a.viscosity) {
      constexpr int PP = plane_of<M>(4), PR = plane_of<M>(0);
      constexpr int PN = plane_of<M>(1 + (DIM == 1 ? 0 : AX));
      constexpr int PT = DIM == 2 ? plane_of<M>(1 + (1 - AX)) : 0;
      // w level at real column x and real row rt
      auto wv = [&](int pl, int x, int rt) -> T { return wat(pl, rt, x); };
      if (a.flatten) {
        // chi_bar on columns [s0-3, s0+TS+3), then eta on [s0-2, s0+TS+2) from it; each
        // intermediate is served at a virtual index by its value at the mapped index
        constexpr int CW = G::RW + 3, EW = G::RW + 1, H = G::RH;
        constexpr int CB_BEG = G::R_BEG - 2, E_BEG = G::R_BEG - 1;
        constexpr double DZ = 0.85 - 0.75;
        // chi_bar of one column from the pressures at y-2..y+2 and the normal velocities
        // at y-1, y+1; dp1 = P(y+1) - P(y-1)
        auto chi_bar = [&](T pm2, T pm1, T pp1, T pp2, T vm1, T vp1, T dp1) -> T {
          // only strong, compressive pressure jumps are flattened (Colella & Woodward 1984, A.1);
          // elsewhere chi_bar = 1 and z is not needed
          const bool not_compressive = (vm1 - vp1) <= T(0);
          const bool weak = dvd(abs_(dp1), npmin(pp1, pm1)) <= T(.33);
          T cb = T(1);
          if (!(not_compressive || weak)) {
            const T dp2 = pp2 - pm2;
            const T z = dvd(abs_(dp1), abs_(dp2));
            cb = T(1) - dvd(z - T(.75), T(DZ));
            if (z > T(.85)) cb = T(0);
            if (z < T(.75)) cb = T(1);
          }
          return cb;
        };
        constexpr int FK = 4;  // eta columns per thread on tiles without a boundary map
        if constexpr (DIM == 2 && !CL && EW % FK == 0) {
          // one thread per strip of FK eta columns of a row: the chi_bar values it needs and
          // the pressure differences eta's sign shares with them stay in registers
          constexpr int NSF = EW / FK;
          for (int e = tid; e < NSF * H; e += nth) {
            const int strip = e / H, row = e % H;
            const int rt = t0 - G::RT + row, x0 = s0 + E_BEG + strip * FK;
            T P[FK + 6], V[FK + 4];  // P at x0-3 .. x0+FK+2, V at x0-2 .. x0+FK+1
#pragma unroll
            for (int i = 0; i < FK + 6; ++i) P[i] = wv(PP, x0 - 3 + i, rt);
#pragma unroll
            for (int i = 0; i < FK + 4; ++i) V[i] = wv(PN, x0 - 2 + i, rt);
            T cb[FK + 2], dp[FK + 2];  // at x0-1 .. x0+FK
#pragma unroll
            for (int i = 0; i < FK + 2; ++i) {
              dp[i] = P[i + 3] - P[i + 1];
              cb[i] = chi_bar(P[i], P[i + 1], P[i + 3], P[i + 4], V[i], V[i + 2], dp[i]);
            }
#pragma unroll
            for (int k = 0; k < FK; ++k) {
              const T sgn = npsign(dp[k + 1]);
              T chi = cb[k + 1];
              if (sgn < T(0)) chi = npmin(cb[k + 1], cb[k + 2]);
              if (sgn > T(0)) chi = npmin(cb[k + 1], cb[k]);
              s_eta[row * EW + strip * FK + k] = chi;
            }
          }
        } else {
          T* s_cb = sm + S::CB_OFF;
          for (int e = tid; e < CW * H; e += nth) {
            const int row = e / CW, col = e % CW;
            const int y = rs_(s0 + CB_BEG + col), rt = DIM == 2 ? rt_(t0 - G::RT + row) : 0;
            auto P = [&](int x) -> T { return wv(PP, x, rt); };
            const T dp1 = P(rs_(y + 1)) - P(rs_(y - 1));
            s_cb[row * CW + col] = chi_bar(P(rs_(y - 2)), P(rs_(y - 1)), P(rs_(y + 1)), P(rs_(y + 2)),
                                           wv(PN, rs_(y - 1), rt), wv(PN, rs_(y + 1), rt), dp1);
          }
          __syncthreads();
          for (int e = tid; e < EW * H; e += nth) {
            const int row = e / EW, col = e % EW;
            const int x = rs_(s0 + E_BEG + col), rt = DIM == 2 ? rt_(t0 - G::RT + row) : 0;
            const T* cbrow = s_cb + row * CW - (s0 + CB_BEG);
            const T cb = cbrow[x];
            const T sgn = npsign(wv(PP, rs_(x + 1), rt) - wv(PP, rs_(x - 1), rt));
            T chi = cb;
            if (sgn < T(0)) chi = npmin(cb, cbrow[rs_(x + 1)]);
            if (sgn > T(0)) chi = npmin(cb, cbrow[rs_(x - 1)]);
            s_eta[row * EW + col] = chi;
          }
        }
      }
      if (a.viscosity) {
        // mu at face x+1/2 for the interface right of cell x = rho(vk-1)
        constexpr int W = G::KW;
        for (int e = tid; e < W * TT; e += nth) {
          // axis 0: consecutive threads on consecutive rows, which are contiguous in the
          // staged levels of that axis (the in-place box and the viscous strip box)
          int row, col;
          if (DIM == 2 && AX == 0) { row = e % TT; col = e / TT; } else { row = e / W; col = e % W; }
          const int vk = s0 + col, vt = t0 + row;
          const int rt = DIM == 2 ? rt_(vt) : 0;
          const int x = rs_(vk - 1), xp = rs_(x + 1);
          T lam = wv(PN, xp, rt) - wv(PN, x, rt);
          if constexpr (DIM == 2) {
            const int rm = rt_(rt - 1), rp = rt_(rt + 1);
            const T dvt_x = wv(PT, x, rp) - wv(PT, x, rm);
            const T dvt_xp = wv(PT, xp, rp) - wv(PT, xp, rm);
            lam = lam + T(.25) * (dvt_xp + dvt_x);
          }
          // only compressive faces are viscous; the coefficient is formed only there
          T nu = T(0);
          if (!(lam >= T(0))) {
            const T cs_x = sqrt_(dvd(gamma * wv(PP, x, rt), wv(PR, x, rt)));
            const T cs_xp = sqrt_(dvd(gamma * wv(PP, xp, rt), wv(PR, xp, rt)));
            const T cmin = npmin(cs_x, cs_xp);
            nu = npmin(T(1), dvd(lam * lam, a.av_beta * (cmin * cmin))) * lam;
          }
          T mu[8];
#pragma unroll
          for (int i = 0; i < 8; ++i) mu[i] = T(0);
          if constexpr (WSIN) {
            // x, xp lie in [s0-1, s0+TS] and rt in [t0, t0+TT) (clamped or not): the staged strip
            if (strip_tma) {
              using SB = StripBox<T, AX, TS, TT>;
#pragma unroll
              for (int v = 0; v < NV; ++v)
                mu[M::var(v)] =
                    a.av_alpha * (nu * (qs_box[SB::at(v, xp, rt, s0, t0)] - qs_box[SB::at(v, x, rt, s0, t0)]));
            } else {
              const T* qrow = sm + S::QS_OFF + (rt - t0) * S::QSW - (s0 - 1);
#pragma unroll
              for (int v = 0; v < NV; ++v) {
                const T* qv = qrow + v * TT * S::QSW;
                mu[M::var(v)] = a.av_alpha * (nu * (qv[xp] - qv[x]));
              }
            }
          } else {
            const T* qrow = s_q + (rt - (t0 - G::QT)) * G::QW - (s0 + G::Q_BEG);
#pragma unroll
            for (int v = 0; v < NV; ++v) {
              const T* qv = qrow + v * G::QH * G::QW;
              mu[M::var(v)] = a.av_alpha * (nu * (qv[xp] - qv[x]));
            }
          }
          store_aos<M>(s_mu, row * W + col, mu);
        }
      }
      __syncthreads();
    }
  }

  // ---- level R: reconstructed face values (wL at i-1/2, wR at i+1/2) of each cell
  if constexpr (SCH == PPM && !CL && PpmStrip<G::RW, DIM>::K > 1) {
    // no boundary map on this tile: one thread per strip of K cells shares the stencil work
    constexpr int K = PpmStrip<G::RW, DIM>::K, NS = G::RW / K;
    constexpr int W = G::RW, H = G::RH;
    for (int e = tid; e < NS * H * NV; e += nth) {
      // strip-major order, the variables of a cell on consecutive threads: a warp's scalar
      // stores into the cell-interleaved level hit distinct banks
      const int strip = e / (NV * H), rem = e % (NV * H);
      const int s = rem % NV, row = rem / NV, col0 = strip * K;
      const int vs0 = s0 + G::R_BEG + col0, vt = t0 - G::RT + row;
      const T* wrow = s_wb + s * WL::PS + (row + (G::WT - G::RT)) * WL::PR - (s0 + G::W_BEG) * WL::PC;
      T* rl = s_R + (row * W + col0) * NVP + s;
      T* rr = rl + NVP * H * W;
      const T* erow = a.flatten ? s_eta + row * (W + 1) - (s0 + G::R_BEG - 1) : nullptr;
      recon_ppm_strip<T, K>([&](int x) -> T { return wrow[x * WL::PC]; }, vs0, [&](int k, T wl, T wr, T fr) {
        rl[k * NVP] = wl;
        rr[k * NVP] = wr;
        const int vs = vs0 + k;
        // face values for the constrained transport (2D MHD grids only)
        if constexpr (M::MHD) {
          if (a.wface_out && vs >= s0 && vs < s0 + TS && vs < Ns && vt >= t0 && vt < t0 + TT && vt < Nt)
            a.wface_out[M::var(s) * a.plane + gidx(vs, vt)] = fr;
        }
      }, erow);
    }
  } else {
    constexpr int W = G::RW, H = G::RH;
    for (int e = tid; e < W * H * NV; e += nth) {
      const int s = e / (W * H), rem = e % (W * H);
      const int row = rem / W, col = rem % W;
      const int vs = s0 + G::R_BEG + col, vt = t0 - G::RT + row;
      const int rs = rs_(vs), rt = DIM == 2 ? rt_(vt) : 0;
      const T* wrow = s_wb + s * WL::PS + (rt - (t0 - G::WT)) * WL::PR - (s0 + G::W_BEG) * WL::PC;
      auto at = [&](int x) -> T { return wrow[x * WL::PC]; };
      const T* erow = (SCH == PPM && a.flatten) ? s_eta + row * (W + 1) - (s0 + G::R_BEG - 1) : nullptr;
      T wl, wr;
      reconstruct<SCH, T>(at, rs_, rs, a.limiter, wl, wr, erow);
      s_R[(row * W + col) * NVP + s] = wl;
      s_R[NVP * H * W + (row * W + col) * NVP + s] = wr;
      if (M::MHD && a.wface_out && vs >= s0 && vs < s0 + TS && vs < Ns && vt >= t0 && vt < t0 + TT && vt < Nt) {
        // the face value the constrained transport uses: PPM's unlimited 4th-order
        // face (ppm.py:38-42), the right face value of the other schemes (weno.py:168, plm.py:39)
        T fv;
        if constexpr (SCH == PPM) fv = erow ? ppm_flatten<T>(ppm_face<T>(at, rs_, rs), at(rs), erow[rs])
                                          : ppm_face<T>(at, rs_, rs);
        else fv = wr;
        a.wface_out[M::var(s) * a.plane + gidx(vs, vt)] = fv;
      }
    }
  }
  __syncthreads();

  // accessors into the R level: virtual cell x (already mapped), real row rt
  auto loadL = [&](int x, int rt, T* out) {
    load_aos<M>(s_R, (rt - (t0 - G::RT)) * G::RW + (x - (s0 + G::R_BEG)), out);
  };
  auto loadR = [&](int x, int rt, T* out) {
    load_aos<M>(s_R + NVP * G::RH * G::RW, (rt - (t0 - G::RT)) * G::RW + (x - (s0 + G::R_BEG)), out);
  };

  // ---- level lambda: wave speed of the interface average right of each cell (fv.compute_eigen)
  // LLF reads the speeds on both sides of every interface of the face levels; the
  // HLL-type solvers use them only for the tile maximum (the time step), so they
  // evaluate the tile's own cells, and only when that maximum is wanted.
  constexpr bool LAM_ALL = SOL == LLF;
  if (LAM_ALL || a.want_emax) {
    constexpr int W = LAM_ALL ? G::YW : TS, H = LAM_ALL ? G::FH : TT;
    constexpr int C_OFF = LAM_ALL ? 0 : 1, R_OFF = LAM_ALL ? 0 : G::FT;
    T lmax = T(0);
    for (int e = tid; e < W * H; e += nth) {
      const int row = e / W + R_OFF, col = e % W + C_OFF;
      const int vj = s0 - 1 + col, vt = t0 - G::FT + row;
      const int rj = rs_(vj), rt = DIM == 2 ? rt_(vt) : 0;
      T y[8];
      if constexpr (SCH == PCM) {
        load_sm<M>(s_w, G::WH * G::WW, (rt - (t0 - G::WT)) * G::WW + (rj - (s0 + G::W_BEG)), y);
      } else {
        T wp[8], wm[8];
        loadL(rs_(rj + 1), rt, wp);
        loadR(rj, rt, wm);
        if constexpr (G::ROE) roe_avg<M>(wp, wm, y);
        else arith_avg<M>(wp, wm, y);
      }
      const T lam = max_speed<M, DIM == 1 ? 0 : AX>(y, gamma);
      if constexpr (LAM_ALL) {
        // Lax-Wendroff (solvers.py:79-88): the squared 'sound speed' over the largest |eigenvalue|,
        // where the sound speed is the entropy-wave eigenvalue v_n of the interface average
        const T vn = y[1 + (DIM == 1 ? 0 : AX)];
        s_lam[row * G::YW + col] = a.lw ? dvd(vn * vn, lam) : lam;
      }
      if (a.want_emax && vj >= s0 && vj < s0 + TS && vj < Ns && vt >= t0 && vt < t0 + TT && vt < Nt) lmax = nanmax(lmax, lam);
    }
    if (a.want_emax) block_max_to_clock(lmax, &a.clock->emax[DIM == 1 ? 0 : AX]);
  }
  // the face levels read the speeds only for LLF; otherwise this level writes no shared
  // memory that they use (its block maximum keeps its own barrier)
  if constexpr (LAM_ALL) __syncthreads();

  // per-interface solve from the six face arrays
  auto solve = [&](int k_local, int lam_row, const T* wSr, const T* wp, const T* wm, const T* qp, const T* qm,
                   const T* fp, const T* fm, T* F) {
    if constexpr (SOL == LLF) {
      const T alpha = npmax(s_lam[lam_row * G::YW + k_local], s_lam[lam_row * G::YW + k_local + 1]);
      llf<M>(alpha, qp, qm, fp, fm, F);
    } else if constexpr (SOL == HLLC) {
      hllc<M>(label, a.physical, gamma, wp, wm, qp, qm, fp, fm, F);
    } else {
      hlld<T>(label, a.physical, gamma, wSr, wp, wm, qp, qm, fp, fm, F);
    }
  };
  auto load_wS = [&](int x, int rt, T* out) {
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i] = T(0);
#pragma unroll
    for (int v = 0; v < NV; ++v) out[M::var(v)] = wat(v, rt, x);
  };
  // face states of interface vk at real row rt
  auto face_states = [&](int vk, int rt, T* wp, T* wm) {
    loadL(rs_(vk), rt, wp);
    loadR(rs_(vk - 1), rt, wm);
  };
  // conservative face state (plus side: cells' left faces; minus side: right faces)
  auto face_cons = [&](int vk, int rt, const T* w, bool plus, T* q) {
    if constexpr (SCH == PCM) {
      // pcm.py:85-99: raw cell averages
      const int x = plus ? rs_(vk) : rs_(vk - 1);
      load_sm<M>(s_q, G::QH * G::QW, (rt - (t0 - G::QT)) * G::QW + (x - (s0 + G::Q_BEG)), q);
    } else if constexpr (G::HO && DIM == 2) {
      // fv.high_order_convert_primitive on a face array: transverse axis only (fv.py:105-122)
      const int rm = rt_(rt - 1), rp = rt_(rt + 1);
      T wm_[8], wp_[8], tmp[8];
      if (plus) { loadL(rs_(vk), rm, wm_); loadL(rs_(vk), rp, wp_); }
      else { loadR(rs_(vk - 1), rm, wm_); loadR(rs_(vk - 1), rp, wp_); }
      if constexpr (kPacked4<M, T>) {
        // FP32 2D Euler: density and the pressure part of the energy are linear in w, so
        // their conversion, p2c(w - d2w/24) + d2(p2c w)/24, is w itself; the momenta and the
        // kinetic energy are the products of the converted w plus the second differences of
        // the point products (the same value, other roundings)
        const float c = float(C24), kc = 1.0f + float(2.0 * C24);
        const float2 nc = f2(-c, -c), K = f2(kc, kc);
        const float2 ra = __ffma2_rn(nc, __fadd2_rn(f2(wp_[0], wp_[1]), f2(wm_[0], wm_[1])), __fmul2_rn(K, f2(w[0], w[1])));
        const float vb = kc * w[2] - c * (wp_[2] + wm_[2]);
        // rho v and rho |v|^2 / 2 of a point state
        auto prod = [&](const float* x, float2& m, float& e) {
          m = __fmul2_rn(f2(x[0], x[0]), f2(x[1], x[2]));
          e = (0.5f * x[0]) * (x[1] * x[1] + x[2] * x[2]);
        };
        float2 m0, mm, mp;
        float e0, em, ep;
        prod(w, m0, e0);
        prod(wm_, mm, em);
        prod(wp_, mp, ep);
        const float2 mc = __fmul2_rn(f2(ra.x, ra.x), f2(ra.y, vb));
        const float ec = (0.5f * ra.x) * (ra.y * ra.y + vb * vb);
        // y + (1/24)(xp - 2 x0 + xm)
        const float2 mq = __ffma2_rn(f2(c, c), __fadd2_rn(mp, mm), __ffma2_rn(f2(-2.0f * c, -2.0f * c), m0, mc));
        const float eq = (ec - (2.0f * c) * e0) + c * (ep + em);
#pragma unroll
        for (int i = 0; i < 8; ++i) q[i] = T(0);
        q[0] = w[0];
        q[1] = mq.x;
        q[2] = mq.y;
        q[4] = over_gm1(w[4], gm1) + eq;
        return;
      }
      T ww[8], qc[8], qm_[8], qp_[8], q0[8];
      conv24_all<M, T>(w, wm_, wp_, ww);
      p2c<M>(w, q0, gm1);
      p2c<M>(wm_, qm_, gm1);
      p2c<M>(wp_, qp_, gm1);
      p2c<M>(ww, tmp, gm1);
      if constexpr (Prec<T>::EXACT) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          qc[i] = T(C24) * ((qp_[i] - q0[i]) - (q0[i] - qm_[i]));
          q[i] = tmp[i] + qc[i];
        }
      } else {
        d2_24_all<M, T, 1>(tmp, q0, qm_, qp_, q);
      }
    } else {
      p2c<M>(w, q, gm1);
    }
  };

  if constexpr (DIM == 1) {
    // ---- 1D: single solve per interface
    constexpr int W = G::KW;
    for (int e = tid; e < W; e += nth) {
      const int vk = s0 + e;
      if (vk > Ns) continue;
      T wp[8], wm[8], qp[8], qm[8], fp[8], fm[8], F[8], wSr[8];
      face_states(vk, 0, wp, wm);
      face_cons(vk, 0, wp, true, qp);
      face_cons(vk, 0, wm, false, qm);
      make_flux<M, 0>(wp, fp, gamma, gm1);
      make_flux<M, 0>(wm, fm, gamma, gm1);
      if constexpr (SOL == HLLD) load_wS(rs_(vk), 0, wSr);
      solve(e, 0, wSr, wp, wm, qp, qm, fp, fm, F);
      if constexpr (SCH == PPM) {
        if (a.viscosity) {
          T mu[8];
          load_aos<M>(s_mu, e, mu);
#pragma unroll
          for (int v = 0; v < NV; ++v) F[M::var(v)] = F[M::var(v)] + mu[M::var(v)];
        }
      }
      store_aos<M>(s_F, e, F);
    }
  } else {
    // ---- 2D level A: face-averaged solve on rows t0-1 .. t0+TT
    constexpr int W = G::KW, H = G::FH;
    T* s_qp = s_fa;
    T* s_qm = s_fa + NVP * H * W;
    T* s_fp = s_fa + 2 * NVP * H * W;
    T* s_fm = s_fa + 3 * NVP * H * W;
    T* s_Fa = s_fa + 4 * NVP * H * W;
    // items with the R level's row pitch (conflict-free loads across a row change)
    for (int e = tid; e < G::RW * H; e += nth) {
      const int row = e / G::RW, col = e % G::RW;
      if (col >= W) continue;
      const int vk = s0 + col, vt = t0 - G::FT + row;
      if (vk > Ns) continue;
      const int rt = rt_(vt);
      T wp[8], wm[8], qp[8], qm[8], fp[8], fm[8], F[8], wSr[8];
      face_states(vk, rt, wp, wm);
      face_cons(vk, rt, wp, true, qp);
      face_cons(vk, rt, wm, false, qm);
      make_flux<M, AX>(wp, fp, gamma, gm1);
      make_flux<M, AX>(wm, fm, gamma, gm1);
      if constexpr (SOL == HLLD) load_wS(rs_(vk), rt, wSr);
      solve(col, row, wSr, wp, wm, qp, qm, fp, fm, F);
      const int li = row * W + col;
      store_aos<M>(s_qp, li, qp);
      store_aos<M>(s_qm, li, qm);
      store_aos<M>(s_fp, li, fp);
      store_aos<M>(s_fm, li, fm);
      store_aos<M>(s_Fa, li, F);
    }
    __syncthreads();
    // ---- 2D level B: face-centred states (fv.high_order_convert 'avg'/'face'), second solve, F_c - d2 F_avg
    for (int e = tid; e < W * TT; e += nth) {
      const int row = e / W, col = e % W;
      const int vk = s0 + col, vt = t0 + row;
      if (vk > Ns) continue;
      const int rt = rt_(vt), rm = rt_(rt - 1), rp = rt_(rt + 1);
      const int fr = rt - (t0 - G::FT), frm = rm - (t0 - G::FT), frp = rp - (t0 - G::FT);
      T x0[8], xm[8], xp[8];
      T cwp[8], cwm[8], cqp[8], cqm[8], cfp[8], cfm[8], Fc[8], wSr[8];
      auto conv = [&](T* out) { conv24_all<M, T>(x0, xm, xp, out); };
      loadL(rs_(vk), rt, x0); loadL(rs_(vk), rm, xm); loadL(rs_(vk), rp, xp);
      conv(cwp);
      loadR(rs_(vk - 1), rt, x0); loadR(rs_(vk - 1), rm, xm); loadR(rs_(vk - 1), rp, xp);
      conv(cwm);
      load_aos<M>(s_qp, fr * W + col, x0); load_aos<M>(s_qp, frm * W + col, xm); load_aos<M>(s_qp, frp * W + col, xp);
      conv(cqp);
      load_aos<M>(s_qm, fr * W + col, x0); load_aos<M>(s_qm, frm * W + col, xm); load_aos<M>(s_qm, frp * W + col, xp);
      conv(cqm);
      load_aos<M>(s_fp, fr * W + col, x0); load_aos<M>(s_fp, frm * W + col, xm); load_aos<M>(s_fp, frp * W + col, xp);
      conv(cfp);
      load_aos<M>(s_fm, fr * W + col, x0); load_aos<M>(s_fm, frm * W + col, xm); load_aos<M>(s_fm, frp * W + col, xp);
      conv(cfm);
      if constexpr (SOL == HLLD) load_wS(rs_(vk), rt, wSr);
      solve(col, fr, wSr, cwp, cwm, cqp, cqm, cfp, cfm, Fc);
      load_aos<M>(s_Fa, fr * W + col, x0); load_aos<M>(s_Fa, frm * W + col, xm); load_aos<M>(s_Fa, frp * W + col, xp);
      T F[8];
      d2_24_all<M, T, -1>(Fc, x0, xm, xp, F);
      if constexpr (SCH == PPM) {
        // the viscous flux of this interface sits where F goes: read it, then overwrite
        if (a.viscosity) {
          T mu[8];
          load_aos<M>(s_mu, row * W + col, mu);
#pragma unroll
          for (int v = 0; v < NV; ++v) F[M::var(v)] = F[M::var(v)] + mu[M::var(v)];
        }
      }
      store_aos<M>(s_F, row * W + col, F);
    }
  }
  __syncthreads();

  // ---- optional: interface fluxes for the evolve_space interface
  if (a.flux_out) {
    constexpr int W = G::KW;
    for (int e = tid; e < W * TT; e += nth) {
      const int row = e / W, col = e % W;
      const int vk = s0 + col, vt = t0 + row;
      if (vk > Ns || vt >= Nt) continue;
      if (col == TS && vk != Ns) continue;  // interface s0+TS belongs to the next tile
      const long long fidx = (long long)vk * Nt + vt;
      const long long fplane = (long long)(Ns + 1) * Nt;
#pragma unroll
      for (int s = 0; s < NV; ++s) a.flux_out[s * fplane + fidx] = s_F[(row * W + col) * NVP + s];
    }
  }

  // ---- divergence and stage combine on the tile's own cells
  {
    constexpr int W = G::KW;
    const T dxT = T(a.dx);
    // FP32 multiplies by the reciprocal of dx, formed in FP32 (FP64 divides, as the reference does)
    T rdx = T(0);
    if constexpr (!Prec<T>::EXACT) rdx = __frcp_rn(dxT);
    const T dtT = T(a.clock->dt);
    for (int e = tid; e < TS * TT; e += nth) {
      int row, col;
      if (DIM == 2 && AX == 0) { row = e % TT; col = e / TT; } else { col = e % TS; row = e / TS; }
      const int vs = s0 + col, vt = t0 + row;
      if (vs >= Ns || vt >= Nt) continue;
      const long long g = gidx(vs, vt);
      T Fr[8], Fl[8];
      load_aos<M>(s_F, row * W + col + 1, Fr);
      load_aos<M>(s_F, row * W + col, Fl);
#pragma unroll
      for (int s = 0; s < NV; ++s) {
        const T D = Prec<T>::EXACT ? (Fr[M::var(s)] - Fl[M::var(s)]) / dxT : (Fr[M::var(s)] - Fl[M::var(s)]) * rdx;
        if (a.mode == 0) {
          a.dout[s * a.plane + g] = D;
        } else {
          const T total = a.mode == 1 ? a.dother[s * a.plane + g] + D : D;
          const T L = -total;
          const T u = a.u0[s * a.plane + g];
          const T cur = a.q[s * a.plane + g];
          const T v = combine<T>(a.integ, a.stage, u, cur, L, dtT);
          a.out[s * a.plane + g] = v;
          if (a.out_host) a.out_host[s * a.plane + g] = v;  // the step's result straight to the host
        }
      }
    }
  }
}

// Clamping is only needed on outflow grids, for tiles whose widest level
// (the staged state, or the staged wS under WSIN) reaches past the grid edge.
// With TMA (single-grid 2D kernels), tiles whose whole TMA box lies inside the
// grid are staged by the bulk copy; the others load per thread as without it.
template <typename T, int MID, int SCH, int SOL, int DIM, int AX, int TS, int TT, int NT = (DIM == 1 ? 64 : 256),
          bool TMA_OK = false, bool WSIN = false>
__device__ __forceinline__ void sweep_tile(const SweepArgs<T>& a, const int s0, const int t0,
                                           unsigned char* __restrict__ smem_raw) {
  using G = Geom<SCH, DIM, TS, TT>;
  using S = Smem<SCH, DIM, TS, TT, Model<MID>::NV, WSIN>;
  const int Ns = DIM == 1 ? a.n0 : (AX == 0 ? a.n0 : a.n1);
  const int Nt = DIM == 1 ? 1 : (AX == 0 ? a.n1 : a.n0);
  if constexpr (TMA_OK && DIM == 2 && (WSIN || !G::HO)) {
    using B = TmaBox<T, SCH, DIM, AX, TS, TT, Model<MID>::NV>;
    if constexpr ((size_t)(AX == 0 ? S::n_w : S::n_R) * sizeof(T) >= (size_t)B::BYTES + 128) {
      const bool box_in = a.tmaps != nullptr && B::inside(s0, t0, a.n0, a.n1);
      if (box_in) {
        sweep_tile_body<T, MID, SCH, SOL, DIM, AX, TS, TT, false, NT, true, WSIN>(a, s0, t0, smem_raw);
        return;
      }
    }
  }
  constexpr int BEG = WSIN ? G::W_BEG : G::Q_BEG, END = WSIN ? G::W_END : G::Q_END, HT = WSIN ? G::WT : G::QT;
  const bool inside = s0 + BEG >= 0 && s0 + TS + END <= Ns && (DIM == 1 || (t0 - HT >= 0 && t0 + TT + HT <= Nt));
  if (a.bc == EDGE && !inside)
    sweep_tile_body<T, MID, SCH, SOL, DIM, AX, TS, TT, true, NT, false, WSIN>(a, s0, t0, smem_raw);
  else sweep_tile_body<T, MID, SCH, SOL, DIM, AX, TS, TT, false, NT, false, WSIN>(a, s0, t0, smem_raw);
}

// The single-grid kernels of 2D high-order schemes stage the precomputed wS.
template <int SCH, int DIM> constexpr bool sweep_wsin() { return DIM == 2 && SCH >= PPM; }

// FP32 Euler tiles fit 1024 threads per SM (<= 64 registers); FP64 Euler tiles of 256
// threads fit two CTAs per SM (<= 128 registers); MHD tiles are larger
template <typename T, int MID, int NT> struct SweepOcc {
  static constexpr int value = (sizeof(T) == 4 && MID != 8) ? (1024 / NT > 0 ? 1024 / NT : 1)
                             : ((sizeof(T) == 8 && MID != 8 && NT == 256) ? 2 : 1);
};

template <typename T, int MID, int SCH, int SOL, int DIM, int AX, int TS, int TT, int NT>
__global__ void __launch_bounds__(NT, (SweepOcc<T, MID, NT>::value)) sweep_kernel(const SweepArgs<T> a) {
  if (a.clock->done) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  sweep_tile<T, MID, SCH, SOL, DIM, AX, TS, TT, NT, true, sweep_wsin<SCH, DIM>()>(a, blockIdx.x * TS, blockIdx.y * TT,
                                                                               smem_raw);
}

}  // namespace astrea

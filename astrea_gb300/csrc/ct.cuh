// Constrained transport for 2D MHD (num_methods/mag_field.py and the magnetic
// parts of num_methods/evolvers.py).
//
//   corner_kernel   transverse PPM of each sweep's face values, upwind corner
//                   speeds and the corner electric field E_z   (mag_field.py:11-187)
//   ct_combine      stage combine with the induction rows replacing the B_x/B_y
//                   divergences, and (stage 0) the face-B re-assignment of the
//                   step-start state                          (evolvers.py:41-76)
//   refine_kernel   face-averaged B back to cell averages     (mag_field.py:191-210)
//
// Layout: all arrays are physical-frame planes [var][ix][iy] (iy contiguous).
#pragma once
#include "sweep.cuh"

namespace astrea {

// corner upwind speeds of an interface-averaged state along normal ``ax``
// (mag_field.compute_corner.get_wavespeeds, :125-152)
template <typename T>
__device__ __forceinline__ void corner_speeds(const T* y, int ax, int hll, T gamma, T& ap, T& am) {
  const T rho = y[0], vn = y[1 + ax], Bn = y[5 + ax], P = y[4];
  if (hll) {
    const T sr = sqrt_(rho);
    const T cs = sqrt_(gamma * dvd(P, rho));
    const T ca = dvd(norm3(y[5], y[6], y[7]), sr);
    const T cax = dvd(Bn, sr);
    const T cs2 = cs * cs, ca2 = ca * ca;
    const T cf = sqrt_(T(.5) * ((cs2 + ca2) + sqrt_(((cs2 + ca2) * (cs2 + ca2)) - ((T(4) * cs2) * (cax * cax)))));
    ap = npmax(T(0), vn + cf);
    am = -npmin(T(0), vn - cf);
  } else {
    // Lax-type solvers: extreme signed eigenvalues of the primitive Jacobian, closed form
    const T a2 = (gamma * P) / rho;
    const T b2 = nsq3(y[5], y[6], y[7]) / rho;
    const T bn2 = (Bn * Bn) / rho;
    const T s = a2 + b2;
    const T cf = sqrt_(T(.5) * (s + sqrt_(s * s - (T(4) * a2) * bn2)));
    ap = npmax(vn + cf, T(0));
    am = -npmin(vn - cf, T(0));
  }
}

constexpr int CTX = 16, CTY = 16;  // corner tile
template <typename T> constexpr size_t corner_smem_bytes() {
  return sizeof(T) * 8 * ((size_t)CTY * (CTX + 8) + (size_t)CTX * (CTY + 8) + 2 * (size_t)CTY * (CTX + 1) + 2 * (size_t)CTX * (CTY + 1));
}

// E_z at corner (ix+1/2, iy+1/2) for every cell (ix, iy).  wfx / wfy are the
// face values of the x and y sweeps (8 planes each).  ``order`` (the step's
// axis order) decides which reconstruction is called north/south and which
// speeds are called 'x' (mag_field.py:163-178 walks a swapped permutation map).
template <typename T>
__global__ void __launch_bounds__(256) corner_kernel(const T* __restrict__ wfx, const T* __restrict__ wfy,
                                                     T* __restrict__ E, int n0, int n1, long long plane, int bc,
                                                     T gamma, int hll, const Clock* clk) {
  if (clk->done) return;
  constexpr int HL = 3, HR = 5;            // PPM reach (3 left, 4 right) + the neighbour cell for the Roe average
  constexpr int AW = CTX + HL + HR;        // wF_y window along x
  constexpr int BW = CTY + HL + HR;        // wF_x window along y
  extern __shared__ __align__(16) unsigned char ct_smem[];
  // wF_y rows (PPM along x), wF_x columns (PPM along y), and their reconstructions
  auto sA = reinterpret_cast<T(*)[CTY][AW]>(ct_smem);
  auto sB = reinterpret_cast<T(*)[CTX][BW]>(ct_smem + sizeof(T) * 8 * CTY * AW);
  auto sDA = reinterpret_cast<T(*)[CTY][CTX + 1]>(ct_smem + sizeof(T) * 8 * (CTY * AW + CTX * BW));
  auto sUA = sDA + 8;
  auto sDB = reinterpret_cast<T(*)[CTX][CTY + 1]>(ct_smem + sizeof(T) * 8 * (CTY * AW + CTX * BW + 2 * CTY * (CTX + 1)));
  auto sUB = sDB + 8;
  const int x0 = blockIdx.x * CTX, y0 = blockIdx.y * CTY;
  const int order = clk->order;
  const Clamp rx = make_rho(bc, n0), ry = make_rho(bc, n1);
  const int tid = threadIdx.y * blockDim.x + threadIdx.x, nth = blockDim.x * blockDim.y;

  for (int e = tid; e < 8 * CTY * AW; e += nth) {
    const int c = e / (CTY * AW), r = (e / AW) % CTY, k = e % AW;
    const int gx = bc_map(x0 - HL + k, n0, bc), gy = bc_map(y0 + r, n1, bc);
    sA[c][r][k] = wfy[c * plane + (long long)gx * n1 + gy];
  }
  for (int e = tid; e < 8 * CTX * BW; e += nth) {
    const int c = e / (CTX * BW), r = (e / BW) % CTX, k = e % BW;
    const int gx = bc_map(x0 + r, n0, bc), gy = bc_map(y0 - HL + k, n1, bc);
    sB[c][r][k] = wfx[c * plane + (long long)gx * n1 + gy];
  }
  __syncthreads();
  // transverse PPM-mc (mag_field.reconstruct_transverse 'ppm'/'mc', :11-65)
  for (int e = tid; e < 8 * CTY * (CTX + 1); e += nth) {
    const int c = e / (CTY * (CTX + 1)), r = (e / (CTX + 1)) % CTY, k = e % (CTX + 1);
    const int v = x0 + k;
    const T* row = &sA[c][r][0] - (x0 - HL);
    auto at = [&](int x) -> T { return row[x]; };
    T d, u;
    recon_ppm<T>(at, rx, rx(v), d, u);
    sDA[c][r][k] = d;
    sUA[c][r][k] = u;
  }
  for (int e = tid; e < 8 * CTX * (CTY + 1); e += nth) {
    const int c = e / (CTX * (CTY + 1)), r = (e / (CTY + 1)) % CTX, k = e % (CTY + 1);
    const int v = y0 + k;
    const T* col = &sB[c][r][0] - (y0 - HL);
    auto at = [&](int x) -> T { return col[x]; };
    T d, u;
    recon_ppm<T>(at, ry, ry(v), d, u);
    sDB[c][r][k] = d;
    sUB[c][r][k] = u;
  }
  __syncthreads();
  for (int e = tid; e < CTX * CTY; e += nth) {
    const int i = e / CTY, j = e % CTY;  // j fastest: iy contiguous in memory
    const int ix = x0 + i, iy = y0 + j;
    if (ix >= n0 || iy >= n1) continue;
    // y-sweep reconstruction (along x): Roe average of wD_y[x+1] and wU_y[x], speeds along x
    T yA[8], yB[8], pl[8], mi[8];
    const int ia = rx(ix + 1) - x0;
    for (int c = 0; c < 8; ++c) { pl[c] = sDA[c][j][ia]; mi[c] = sUA[c][j][i]; }
    roe_avg<Model<8>>(pl, mi, yA);
    const int jb = ry(iy + 1) - y0;
    for (int c = 0; c < 8; ++c) { pl[c] = sDB[c][i][jb]; mi[c] = sUB[c][i][j]; }
    roe_avg<Model<8>>(pl, mi, yB);
    T apA, amA, apB, amB;
    corner_speeds<T>(yA, 0, hll, gamma, apA, amA);
    corner_speeds<T>(yB, 1, hll, gamma, apB, amB);
    // even steps: north/south from the y sweep; odd steps: from the x sweep
    const bool odd = order == 1;
    T n1_, n2_, n5_, s1_, s2_, s5_, e1_, e2_, e6_, w1_, w2_, w6_, apy, amy, apx, amx;
    auto pickA = [&](int c) { return sDA[c][j][i]; };
    auto pickAU = [&](int c) { return sUA[c][j][i]; };
    auto pickB = [&](int c) { return sDB[c][i][j]; };
    auto pickBU = [&](int c) { return sUB[c][i][j]; };
    if (!odd) {
      n1_ = pickA(1); n2_ = pickA(2); n5_ = pickA(5);
      s1_ = pickAU(1); s2_ = pickAU(2); s5_ = pickAU(5);
      e1_ = pickB(1); e2_ = pickB(2); e6_ = pickB(6);
      w1_ = pickBU(1); w2_ = pickBU(2); w6_ = pickBU(6);
      apy = apA; amy = amA; apx = apB; amx = amB;
    } else {
      n1_ = pickB(1); n2_ = pickB(2); n5_ = pickB(5);
      s1_ = pickBU(1); s2_ = pickBU(2); s5_ = pickBU(5);
      e1_ = pickA(1); e2_ = pickA(2); e6_ = pickA(6);
      w1_ = pickAU(1); w2_ = pickAU(2); w6_ = pickAU(6);
      apy = apB; amy = amB; apx = apA; amx = amA;
    }
    const T NE = (T(.5) * (w2_ + s2_)) * s5_ - (T(.5) * (w1_ + s1_)) * w6_;
    const T NW = (T(.5) * (e2_ + s2_)) * s5_ - (T(.5) * (e1_ + s1_)) * e6_;
    const T SE = (T(.5) * (w2_ + n2_)) * n5_ - (T(.5) * (w1_ + n1_)) * w6_;
    const T SW = (T(.5) * (e2_ + n2_)) * n5_ - (T(.5) * (e1_ + n1_)) * e6_;
    const T num = (((apx * apy) * SW + (amx * apy) * SE) + (apx * amy) * NW) + (amx * amy) * NE;
    const T Ez = (dvd(num, (apx + amx) * (apy + amy)) - dvd(apy * amy, apy + amy) * (n5_ - s5_))
                 + dvd(apx * amx, apx + amx) * (e6_ - w6_);
    E[(long long)ix * n1 + iy] = Ez;
  }
}

// Stage combine for 2D MHD.  L = -(D_x + D_y) except the B_x / B_y rows,
// which are the induction differences of E_z (evolvers.py:52-58):
//   total_5 = (E[ix, iy+1] - E[ix, iy]) / dx,  total_6 = -(E[ix+1, iy] - E[ix, iy]) / dx.
// At stage 0 the step-start state first takes the face-averaged B of the two
// sweeps (evolvers.py:73-76); that modified state is the 'grid' of every stage.
template <typename T>
__global__ void ct_combine_kernel(T* __restrict__ u, const T* __restrict__ cur, const T* __restrict__ dx_,
                                  const T* __restrict__ dy_, const T* __restrict__ E, const T* __restrict__ wfx,
                                  const T* __restrict__ wfy, T* __restrict__ out, int n0, int n1, long long plane,
                                  int bc, double dx, int integ, int stage, const Clock* clk) {
  if (clk->done) return;
  const T dt = T(clk->dt), dxT = T(dx);
  const long long n = (long long)n0 * n1;
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < n; id += (long long)gridDim.x * blockDim.x) {
    const int ix = (int)(id / n1), iy = (int)(id % n1);
    if (stage == 0) {
      u[5 * plane + id] = wfx[5 * plane + id];
      u[6 * plane + id] = wfy[6 * plane + id];
    }
    const T e0 = E[id];
    const T eyp = E[(long long)ix * n1 + bc_map(iy + 1, n1, bc)];
    const T exp_ = E[(long long)bc_map(ix + 1, n0, bc) * n1 + iy];
    for (int s = 0; s < 8; ++s) {
      const long long g = s * plane + id;
      T total;
      if (s == 5) total = (eyp - e0) / dxT;
      else if (s == 6) total = (-(exp_ - e0)) / dxT;
      else total = dx_[g] + dy_[g];
      const T L = -total;
      const T uu = u[g];
      const T cc = stage == 0 ? uu : cur[g];
      out[g] = combine<T>(integ, stage, uu, cc, L, dt);
    }
  }
}

// Inverse reconstruction of the face-averaged B (mag_field.inverse_reconstruct,
// :191-210) for component 5+A along axis A; the other variables are copied.
constexpr int RTX = 16, RTY = 16;
template <typename T, int A>
__global__ void __launch_bounds__(256) refine_kernel(const T* __restrict__ in, T* __restrict__ out, int n0, int n1,
                                                     long long plane, int bc, const Clock* clk) {
  if (clk->done) return;
  // frame: axis a (index i) = physical A, transverse (index j) = the other axis
  constexpr int HA_L = 2, HA_R = 3, HT = 2;
  constexpr int WA = (A == 0 ? RTX : RTY) + HA_L + HA_R + 1;
  constexpr int WT = (A == 0 ? RTY : RTX) + 2 * HT;
  __shared__ T sX[WA][WT], sF[WA][WT], sC[WA][WT];
  const int TA = A == 0 ? RTX : RTY, TT_ = A == 0 ? RTY : RTX;
  const int a0 = (A == 0 ? blockIdx.x * RTX : blockIdx.y * RTY);
  const int b0 = (A == 0 ? blockIdx.y * RTY : blockIdx.x * RTX);
  const int na = A == 0 ? n0 : n1, nt = A == 0 ? n1 : n0;
  const Clamp ra = make_rho(bc, na), rt = make_rho(bc, nt);
  const int tid = threadIdx.x, nth = blockDim.x;
  const int comp = 5 + A;
  const T* X = in + comp * plane;
  auto gidx = [&](int ia, int it) -> long long {
    return A == 0 ? (long long)ia * n1 + it : (long long)it * n1 + ia;
  };
  const int abase = a0 - HA_L - 1, tbase = b0 - HT;  // virtual index of local 0
  for (int e = tid; e < WA * WT; e += nth) {
    const int la = e / WT, lt = e % WT;
    sX[la][lt] = X[gidx(bc_map(abase + la, na, bc), bc_map(tbase + lt, nt, bc))];
  }
  __syncthreads();
  constexpr double c24 = 1.0 / 24.0;
  // face-averaged -> face-centred along the transverse axis (fv.high_order_convert 'avg'/'face')
  for (int e = tid; e < WA * WT; e += nth) {
    const int la = e / WT, lt = e % WT;
    const int va = abase + la, vt = tbase + lt;
    if (lt == 0 || lt == WT - 1) continue;
    const int ia = ra(va) - abase, it = rt(vt) - tbase;
    if (ia < 0 || ia >= WA) continue;
    const int itm = rt(rt(vt) - 1) - tbase, itp = rt(rt(vt) + 1) - tbase;
    const T x0 = sX[ia][it];
    sF[la][lt] = x0 - T(c24) * ((sX[ia][itp] - x0) - (x0 - sX[ia][itm]));
  }
  __syncthreads();
  // face-centred -> cell-centred, 4-point along axis A (the stencil centred on cell i+1 is the reference's)
  for (int e = tid; e < WA * WT; e += nth) {
    const int la = e / WT, lt = e % WT;
    const int va = abase + la, vt = tbase + lt;
    if (la < 1 || la > WA - 3 || lt == 0 || lt == WT - 1) continue;
    const int r = ra(va);
    const int it = rt(vt) - tbase;
    const T fm = sF[ra(r - 1) - abase][it], f0 = sF[r - abase][it], fp = sF[ra(r + 1) - abase][it], fp2 = sF[ra(r + 2) - abase][it];
    sC[la][lt] = T(-1.0 / 16.0) * (fm + fp2) + T(9.0 / 16.0) * (f0 + fp);
  }
  __syncthreads();
  // cell-centred -> cell-averaged: + 1/24 d2 along A, then along the transverse axis
  for (int e = tid; e < TA * TT_; e += nth) {
    const int i = e / TT_, j = e % TT_;
    const int va = a0 + i, vt = b0 + j;
    if (va >= na || vt >= nt) continue;
    const int la = va - abase, lt = vt - tbase;
    const T c0 = sC[la][lt];
    const T cam = sC[ra(va - 1) - abase][lt], cap = sC[ra(va + 1) - abase][lt];
    const T ctm = sC[la][rt(vt - 1) - tbase], ctp = sC[la][rt(vt + 1) - tbase];
    const T r = (c0 + T(c24) * ((cap - c0) - (c0 - cam))) + T(c24) * ((ctp - c0) - (c0 - ctm));
    out[comp * plane + gidx(va, vt)] = r;
  }
}

// copy of every variable except B_x and B_y (the refined ones)
template <typename T>
__global__ void copy_nonB_kernel(const T* __restrict__ in, T* __restrict__ out, long long plane, long long n, const Clock* clk) {
  if (clk->done) return;
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < n; id += (long long)gridDim.x * blockDim.x) {
#pragma unroll
    for (int s = 0; s < 8; ++s)
      if (s != 5 && s != 6) out[s * plane + id] = in[s * plane + id];
  }
}

}  // namespace astrea

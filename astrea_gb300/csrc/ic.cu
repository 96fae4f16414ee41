// Initial conditions on the device: the point primitives of the reference's
// test problems (functions/constructor.py:11-103), evaluated per cell from a
// handful of parameters instead of being built on the host and uploaded.
//
// The kinds follow constructor.initialise's dispatch on the config name (the
// name -> kind mapping lives in astrea_gb300/initial.py).  Cell centres are the
// reference's np.linspace(start - dx/2, end + dx/2, N + 2)[1:-1], formed the
// way NumPy forms a linspace (k * step + first), in FP64.
#include <cstring>

#include "host_common.h"
#include "physics.cuh"

using namespace astrea;

namespace {

__device__ __forceinline__ double cell_centre(const astrea_ic& c, int i) {
  const double dx = fabs(c.end - c.start) / c.n;
  const double half = dx / 2;
  const double lo = c.start - half, hi = c.end + half;
  const double step = (hi - lo) / (double)(c.n + 1);
  return (double)(i + 1) * step + lo;
}

__device__ __forceinline__ void set8(double* w, const double* v) {
#pragma unroll
  for (int k = 0; k < 8; ++k) w[k] = v[k];
}

__device__ void point_state_1d(const astrea_ic& c, int i, double* w) {
  const double x = cell_centre(c, i);
  set8(w, c.right);
  const bool in = c.abs_mask ? (fabs(x) <= c.shock) : (x <= c.shock);
  if (in) set8(w, c.left);
  switch (c.kind) {
    case ASTREA_IC_SHU:
      if (x > c.shock) w[0] = c.y_offset + c.ampl * sin((c.freq * M_PI) * x);
      break;
    case ASTREA_IC_SINE:
      w[0] = c.y_offset + c.ampl * sin((c.freq * M_PI) * x);
      break;
    case ASTREA_IC_GAUSS: {
      const double d = x - c.peak_pos;
      w[0] = c.y_offset + c.ampl * exp(-(d * d) / c.fwhm);
      break;
    }
    case ASTREA_IC_LINEAR:
    case ASTREA_IC_LINEAR_MHD: {
      // hydro: (1, -1, 1, 1, 1.5) sound wave; MHD: the Alfven-wave eigenvector
      const double hyd[8] = {1, -1, 1, 1, 1.5, 0, 0, 0};
      const double alf[8] = {0, 0, -.3333333333333333, .9428090415820634, 0, -.3333333333333333, .9428090415820634, 0};
      const double* v = c.kind == ASTREA_IC_LINEAR ? hyd : alf;
      const double s = sin((c.freq * M_PI) * x);
#pragma unroll
      for (int k = 0; k < 8; ++k) w[k] = w[k] + (v[k] * c.ampl) * s;
      break;
    }
    default:
      break;
  }
}

__device__ void point_state_2d(const astrea_ic& c, int i, int j, double* w) {
  const double x = cell_centre(c, i), y = cell_centre(c, j);
  const double centre = (c.end + c.start) / 2;
  set8(w, c.right);
  switch (c.kind) {
    case ASTREA_IC_RADIAL: {  // sedov / blast / rotor (the reference's rotor sets no velocity)
      const double dxc = x - centre, dyc = y - centre, r0 = c.shock - centre;
      if (dxc * dxc + dyc * dyc <= r0 * r0) set8(w, c.left);
      break;
    }
    case ASTREA_IC_GAUSS: {
      const double dxc = x - centre, dyc = y - centre;
      const double r = sqrt(dxc * dxc + dyc * dyc);
      const double d = r - centre;
      w[0] = c.y_offset + c.ampl * exp(-(d * d) / c.fwhm);
      break;
    }
    case ASTREA_IC_KHI:
      if (y <= c.shock) set8(w, c.left);
      w[2] = c.perturb_ampl * sin(((c.freq * M_PI) * x) / (c.end - c.start));
      break;
    case ASTREA_IC_VORTEX: {
      const double xc = (cell_centre(c, 0) + cell_centre(c, c.n - 1)) / 2;
      const double dxc = x - xc, dyc = y - xc;
      const double r = sqrt(dxc * dxc + dyc * dyc);
      const double r2 = r * r;  // the reference squares the radius it took the root of
      const double fp = c.freq * M_PI;
      const double g = c.gamma;
      const double T = 1 - (((g - 1) * (c.vortex_str * c.vortex_str)) / ((2 * g) * (fp * fp))) * exp(1 - r2);
      const double v = (c.vortex_str / fp) * exp((1 - r2) / 2);
      w[0] = pow(T, 1 / (g - 1));
      w[1] = v;
      w[2] = v;
      w[4] = pow(T, g / (g - 1));
      break;
    }
    case ASTREA_IC_QUADRANT:
      if (x <= c.shock) set8(w, c.left);
      if (x <= c.shock && y >= c.shock) set8(w, c.bottom_left);
      if (x > c.shock && y >= c.shock) set8(w, c.bottom_right);
      break;
    case ASTREA_IC_OT:
      if (y <= c.shock) set8(w, c.left);
      w[1] = -sin((2 * M_PI) * y);
      w[2] = sin((2 * M_PI) * x);
      w[5] = -c.ampl * sin((2 * M_PI) * y);
      w[6] = c.ampl * sin((4 * M_PI) * x);
      break;
    default:  // a single jump across x
      if (x < c.shock) set8(w, c.left);
      break;
  }
}

template <typename T, int MID> __global__ void point_state_kernel(const astrea_ic c, T* __restrict__ out) {
  using Mo = Model<MID>;
  const long long n1 = c.dim == 2 ? c.n : 1;
  const long long cells = (long long)c.n * n1;
  for (long long id = blockIdx.x * (long long)blockDim.x + threadIdx.x; id < cells; id += (long long)gridDim.x * blockDim.x) {
    double w[8];
    if (c.dim == 1) point_state_1d(c, (int)id, w);
    else point_state_2d(c, (int)(id / n1), (int)(id % n1), w);
#pragma unroll
    for (int s = 0; s < Mo::NV; ++s) out[s * cells + id] = T(w[Mo::var(s)]);
  }
}

}  // namespace

extern "C" {

int astrea_point_state(const astrea_ic* ic, int precision, int model, void* prim_out, void* stream) {
  if (!ic || !prim_out) return fail(ASTREA_ERR_ARG, "NULL argument");
  if (ic->dim != 1 && ic->dim != 2) return fail(ASTREA_ERR_CONFIG, "dim must be 1 or 2");
  if (ic->n < 1) return fail(ASTREA_ERR_CONFIG, "n must be positive");
  if (precision != 32 && precision != 64) return fail(ASTREA_ERR_CONFIG, "precision must be 32 or 64");
  if (!((ic->dim == 1 && (model == 3 || model == 8)) || (ic->dim == 2 && (model == 4 || model == 8))))
    return fail(ASTREA_ERR_CONFIG, "model must be 3|8 in 1D, 4|8 in 2D");
  const long long cells = (long long)ic->n * (ic->dim == 2 ? ic->n : 1);
  const int threads = 256;
  const int blocks = (int)std::min<long long>((cells + threads - 1) / threads, 152LL * 16);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (precision == 64) {
    double* o = static_cast<double*>(prim_out);
    if (model == 3) point_state_kernel<double, 3><<<blocks, threads, 0, st>>>(*ic, o);
    else if (model == 4) point_state_kernel<double, 4><<<blocks, threads, 0, st>>>(*ic, o);
    else point_state_kernel<double, 8><<<blocks, threads, 0, st>>>(*ic, o);
  } else {
    float* o = static_cast<float*>(prim_out);
    if (model == 3) point_state_kernel<float, 3><<<blocks, threads, 0, st>>>(*ic, o);
    else if (model == 4) point_state_kernel<float, 4><<<blocks, threads, 0, st>>>(*ic, o);
    else point_state_kernel<float, 8><<<blocks, threads, 0, st>>>(*ic, o);
  }
  CK(cudaGetLastError());
  return ASTREA_OK;
}

}  // extern "C"

// Device diagnostics of a primitive snapshot (functions/analytic.py):
// total variation (calculate_TV, :48-63) and solution-error norms
// (calculate_solution_error, :24-45), over the eight primitives plus the
// specific total and internal energies.  Sums are FP64 and compensated; the
// per-block partials live in a fixed device array (no allocation), so calls on
// one device must not overlap.
#include <cmath>
#include <mutex>

#include "host_common.h"
#include "physics.cuh"
#include "stage.cuh"

using namespace astrea;

namespace {

constexpr int kQ = 10;  // 8 primitives, E_tot, E_int
constexpr int kBlocks = 152;
constexpr int kScratch = kBlocks * kQ * 2 + kQ;
static __device__ __align__(256) double g_diag_scratch[kScratch];

std::mutex g_diag_mutex;
double* g_diag_ptr[64] = {};

int diag_scratch(double** out) {
  int dev = -1;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(ASTREA_ERR_ARG, "device ordinal beyond the diagnostics table");
  std::lock_guard<std::mutex> lock(g_diag_mutex);
  if (!g_diag_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_diag_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(diagnostics scratch)");
    g_diag_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_diag_ptr[dev];
  return ASTREA_OK;
}

// the ten quantities of one cell: primitives, E_tot = e_tot / rho, E_int = P / (rho (gamma - 1))
template <typename T, int MID>
__device__ void quantities(const T* __restrict__ w, long long plane, long long id, double gamma, double* x) {
  using Mo = Model<MID>;
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = 0.0;
#pragma unroll
  for (int s = 0; s < Mo::NV; ++s) x[Mo::var(s)] = (double)w[s * plane + id];
  // fv.convert_variable('pressure'): P/(gamma-1) + .5 (rho |v|^2 + |B|^2), norms squared after the root
  const double nv = sqrt((x[1] * x[1] + x[2] * x[2]) + x[3] * x[3]);
  const double nb = sqrt((x[5] * x[5] + x[6] * x[6]) + x[7] * x[7]);
  const double etot = x[4] / (gamma - 1) + .5 * (x[0] * (nv * nv) + nb * nb);
  x[8] = x[0] != 0.0 ? etot / x[0] : 0.0;
  const double den = x[0] * (gamma - 1);
  x[9] = den != 0.0 ? x[4] / den : 0.0;
}

// mode 0: |first differences| along every axis in turn (np.diff over axis 0, then axis 1)
// mode 1: |w - ref|^p (p <= 0: p = 1; p > 10: max)
template <typename T, int MID>
__global__ void diag_pass1(const T* __restrict__ w, const T* __restrict__ ref, int dim, int n0, int n1, double gamma,
                           int mode, double p, double* __restrict__ part) {
  const long long plane = (long long)n0 * n1;
  const int m0 = mode == 0 ? n0 - 1 : n0;
  const int m1 = mode == 0 && dim == 2 ? n1 - 1 : n1;
  const long long count = (long long)m0 * m1;
  const bool maxnorm = mode == 1 && p > 10;
  double sum[kQ], comp[kQ];
#pragma unroll
  for (int q = 0; q < kQ; ++q) { sum[q] = 0.0; comp[q] = 0.0; }
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < count; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e / m1), j = (int)(e % m1);
    double d[kQ];
    if (mode == 0) {
      double a[kQ], b[kQ];
      quantities<T, MID>(w, plane, (long long)i * n1 + j, gamma, a);
      quantities<T, MID>(w, plane, (long long)(i + 1) * n1 + j, gamma, b);
      if (dim == 2) {
        double c[kQ], f[kQ];
        quantities<T, MID>(w, plane, (long long)i * n1 + j + 1, gamma, c);
        quantities<T, MID>(w, plane, (long long)(i + 1) * n1 + j + 1, gamma, f);
#pragma unroll
        for (int q = 0; q < kQ; ++q) d[q] = fabs((f[q] - c[q]) - (b[q] - a[q]));
      } else {
#pragma unroll
        for (int q = 0; q < kQ; ++q) d[q] = fabs(b[q] - a[q]);
      }
    } else {
      double a[kQ], b[kQ];
      quantities<T, MID>(w, plane, (long long)i * n1 + j, gamma, a);
      quantities<T, MID>(ref, plane, (long long)i * n1 + j, gamma, b);
#pragma unroll
      for (int q = 0; q < kQ; ++q) {
        const double x = fabs(a[q] - b[q]);
        d[q] = (maxnorm || p <= 0) ? x : pow(x, p);
      }
    }
#pragma unroll
    for (int q = 0; q < kQ; ++q) {
      if (maxnorm) sum[q] = fmax(sum[q], d[q]);
      else neumaier_add(sum[q], comp[q], d[q]);
    }
  }
  __shared__ double ss[256], cc[256];
  for (int q = 0; q < kQ; ++q) {
    ss[threadIdx.x] = sum[q];
    cc[threadIdx.x] = comp[q];
    __syncthreads();
    if (threadIdx.x == 0) {
      double S = 0.0, Cc = 0.0;
      for (int k = 0; k < (int)blockDim.x; ++k) {
        if (maxnorm) S = fmax(S, ss[k]);
        else { neumaier_add(S, Cc, ss[k]); Cc += cc[k]; }
      }
      part[(blockIdx.x * kQ + q) * 2 + 0] = S;
      part[(blockIdx.x * kQ + q) * 2 + 1] = Cc;
    }
    __syncthreads();
  }
}

__global__ void diag_pass2(const double* __restrict__ part, int nblocks, int maxnorm, double* __restrict__ out) {
  const int q = threadIdx.x;
  if (q >= kQ) return;
  double S = 0.0, Cc = 0.0;
  for (int b = 0; b < nblocks; ++b) {
    if (maxnorm) S = fmax(S, part[(b * kQ + q) * 2]);
    else { neumaier_add(S, Cc, part[(b * kQ + q) * 2]); Cc += part[(b * kQ + q) * 2 + 1]; }
  }
  out[q] = S + Cc;
}

template <typename T>
int run(const void* w, const void* ref, int model, int dim, int n0, int n1, double gamma, int mode, double p,
        double* host, cudaStream_t st) {
  double* scratch = nullptr;
  int rc = diag_scratch(&scratch);
  if (rc) return rc;
  const T* pw = static_cast<const T*>(w);
  const T* pr = static_cast<const T*>(ref);
  switch (model) {
    case 3: diag_pass1<T, 3><<<kBlocks, 256, 0, st>>>(pw, pr, dim, n0, n1, gamma, mode, p, scratch); break;
    case 4: diag_pass1<T, 4><<<kBlocks, 256, 0, st>>>(pw, pr, dim, n0, n1, gamma, mode, p, scratch); break;
    default: diag_pass1<T, 8><<<kBlocks, 256, 0, st>>>(pw, pr, dim, n0, n1, gamma, mode, p, scratch); break;
  }
  CK(cudaGetLastError());
  diag_pass2<<<1, 32, 0, st>>>(scratch, kBlocks, mode == 1 && p > 10, scratch + kBlocks * kQ * 2);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(host, scratch + kBlocks * kQ * 2, sizeof(double) * kQ, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  return ASTREA_OK;
}

int check(const void* w, int precision, int model, int dim, int n0, int n1, double* host) {
  if (!w || !host) return fail(ASTREA_ERR_ARG, "NULL argument");
  if (precision != 32 && precision != 64) return fail(ASTREA_ERR_ARG, "precision must be 32 or 64");
  if (dim != 1 && dim != 2) return fail(ASTREA_ERR_ARG, "dim must be 1 or 2");
  if (n0 < 2 || (dim == 2 && n1 < 2) || (dim == 1 && n1 != 1)) return fail(ASTREA_ERR_ARG, "bad grid size");
  if (!((dim == 1 && (model == 3 || model == 8)) || (dim == 2 && (model == 4 || model == 8))))
    return fail(ASTREA_ERR_ARG, "model must be 3|8 in 1D, 4|8 in 2D");
  return ASTREA_OK;
}

}  // namespace

extern "C" {

int astrea_total_variation(const void* prim, int precision, int model, int dim, int n0, int n1, double gamma,
                           double* tv_host, void* stream) {
  int rc = check(prim, precision, model, dim, n0, n1, tv_host);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return precision == 64 ? run<double>(prim, nullptr, model, dim, n0, n1, gamma, 0, 0.0, tv_host, st)
                         : run<float>(prim, nullptr, model, dim, n0, n1, gamma, 0, 0.0, tv_host, st);
}

int astrea_solution_error(const void* prim, const void* ref, int precision, int model, int dim, int n0, int n1,
                          double gamma, double norm, double* err_host, void* stream) {
  int rc = check(prim, precision, model, dim, n0, n1, err_host);
  if (rc) return rc;
  if (!ref) return fail(ASTREA_ERR_ARG, "NULL argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  rc = precision == 64 ? run<double>(prim, ref, model, dim, n0, n1, gamma, 1, norm, err_host, st)
                       : run<float>(prim, ref, model, dim, n0, n1, gamma, 1, norm, err_host, st);
  if (rc) return rc;
  if (!(norm > 10)) {
    const double nf = 1.0 / std::pow((double)n0, (double)dim);
    for (int q = 0; q < kQ; ++q) err_host[q] = norm <= 0 ? nf * err_host[q] : std::pow(nf * err_host[q], 1.0 / norm);
  }
  return ASTREA_OK;
}

}  // extern "C"

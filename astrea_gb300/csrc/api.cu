// C ABI (include/astrea_gb300.h): handle management and the step sequence.
//
// One step of the core_run loop (astrea.py:66-85) with an s-stage Runge-Kutta
// scheme is enqueued as:
//   stage 0:  sweep x -> D_a, sweep y -> D_b (both accumulate eigmax),
//             dt kernel, combine0 (u, D_a, D_b) -> k1
//   stage s:  sweep x (state k_s) -> D_a, sweep y (state k_s) fused with the
//             stage combine -> k_{s+1} (or u after the last stage)
//   end_step: t += dt, flip the axis order, reset the speed maxima
// In 1D the single sweep fuses the combine directly.  The HLLC/HLLD axis label
// of each sweep is read from the device clock's axis order, so one captured
// graph serves even and odd steps.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/astrea_gb300.h"
#include "cellavg.cuh"
#include "ct.cuh"
#include "stage.cuh"
#include "sweep_launch.cuh"

namespace astrea {
ASTREA_EXTERN_GET_SWEEP(double)
ASTREA_EXTERN_GET_SWEEP(float)
}  // namespace astrea

using namespace astrea;

#include "host_common.h"

thread_local std::string g_last_error;

static int stages_of(int integ) {
  switch (integ) {
    case EULER: return 1;
    case SSPRK22: return 2;
    case SSPRK33: return 3;
    case SSPRK43: return 4;
    case SSPRK53: return 5;
    case SSPRK54: return 5;
    case SSPRK104: return 11;  // the reference's (10,4) evaluates the operator 11 times
    case RK4: return 4;
    default: return -1;
  }
}

// Event pairs around kernel launches, by kernel kind (astrea_step_timed)
struct KTimer {
  std::vector<cudaEvent_t> ev[4][2];
  int open_kind = -1;
  cudaError_t start(int kind, cudaStream_t st) {
    cudaEvent_t e;
    cudaError_t r = cudaEventCreate(&e);
    if (r != cudaSuccess) return r;
    ev[kind][0].push_back(e);
    open_kind = kind;
    return cudaEventRecord(e, st);
  }
  cudaError_t stop(cudaStream_t st) {
    cudaEvent_t e;
    cudaError_t r = cudaEventCreate(&e);
    if (r != cudaSuccess) return r;
    ev[open_kind][1].push_back(e);
    return cudaEventRecord(e, st);
  }
  ~KTimer() {
    for (auto& k : ev)
      for (auto& v : k)
        for (auto e : v) cudaEventDestroy(e);
  }
};
#define TSTART(kind) \
  if (tm) CK(tm->start(kind, st))
#define TSTOP() \
  if (tm) CK(tm->stop(st))

struct IEngine {
  astrea_cfg cfg{};
  int nv = 0;
  long long cells = 0;
  Clock* clk = nullptr;   // [0]: device-time stepping, [1]: explicit-dt (evolve_time / evolve_space)
  double* part = nullptr; // compensated-sum partials
  double* sums = nullptr;
  cudaGraphExec_t graph = nullptr;
  void* graph_state = nullptr;
  // astrea_step_host: a captured step with host input and output, and its buffers
  cudaGraphExec_t graph_host = nullptr;
  const void* graph_host_key[3] = {nullptr, nullptr, nullptr};
  // device-accessible address of page-locked host memory for the final stage's combine to write
  // the state into while it computes (nullptr: the result is copied after the step)
  void* host_out = nullptr;
  cudaStream_t graph_stream = nullptr;
  // whether enqueue_step stores the final state to host_out itself (the SSP-RK paths whose last
  // stage ends in a combining sweep); otherwise the caller copies it after the step
  virtual bool fuses_host_out() const = 0;
  virtual ~IEngine() {
    if (graph) cudaGraphExecDestroy(graph);
    if (graph_host) cudaGraphExecDestroy(graph_host);
    cudaFree(clk);
    cudaFree(part);
    cudaFree(sums);
  }
  virtual int alloc() = 0;
  virtual int enqueue_step(void* state, Clock* c, bool device_dt, cudaStream_t st, KTimer* tm = nullptr) = 0;
  virtual int space(const void* state, int order, void* f0, void* f1, double* eigmax, cudaStream_t st,
                    void* face0 = nullptr, void* face1 = nullptr, void* corner = nullptr) = 0;
  virtual int initialise(const void* prim, void* out, cudaStream_t st) = 0;
  virtual int to_primitive(const void* state, void* out, cudaStream_t st) = 0;
  virtual int reduce(const void* state, double* host, cudaStream_t st) = 0;
  // pick the sweep tile of each axis (once, before the first step; not during a capture)
  virtual int tune(const void* state, cudaStream_t st) = 0;
  // before the first launch on a state pointer (outside a capture): its TMA maps, then tune
  virtual int prepare(const void* state, cudaStream_t st) = 0;
  virtual void tile_of(int ax, int* ts, int* tt) const = 0;
};

// Sweep-tile autotuner: per (precision, model, scheme, solver, flags, grid size,
// device, axis) the fastest candidate tile, timed once on the grid itself and
// shared by every handle with the same key.  ASTREA_SWEEP_TILE=<index> forces a
// candidate on both axes, ASTREA_SWEEP_TILE=<index>,<index> one per axis (where it
// is built).
static std::mutex g_tune_mutex;
static std::map<std::string, int> g_tune_cache;

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to libcuda)
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// TMA box (x, y) of scheme ``scheme`` for (axis, tile): the kernels' TmaBox
template <typename T, int SCH> static void box_of(int ax, int tile, cuuint32_t* bw, cuuint32_t* bh) {
  if (ax == 0) {
    using B0 = TmaBox<T, SCH, 2, 0, Tile2<0>::TS, Tile2<0>::TT, 1>;
    using B1 = TmaBox<T, SCH, 2, 0, Tile2<1>::TS, Tile2<1>::TT, 1>;
    if (tile == 0) { *bw = B0::BW; *bh = B0::BH; }
    else { *bw = B1::BW; *bh = B1::BH; }
  } else {
    using B0 = TmaBox<T, SCH, 2, 1, Tile2<0>::TS, Tile2<0>::TT, 1>;
    using B1 = TmaBox<T, SCH, 2, 1, Tile2<1>::TS, Tile2<1>::TT, 1>;
    if (tile == 0) { *bw = B0::BW; *bh = B0::BH; }
    else { *bw = B1::BW; *bh = B1::BH; }
  }
}
// the viscous strip box (StripBox) of (axis, tile)
template <typename T> static void strip_box(int ax, int tile, cuuint32_t* bw, cuuint32_t* bh) {
  if (ax == 0) {
    using B0 = StripBox<T, 0, Tile2<0>::TS, Tile2<0>::TT>;
    using B1 = StripBox<T, 0, Tile2<1>::TS, Tile2<1>::TT>;
    if (tile == 0) { *bw = B0::BW; *bh = B0::BH; }
    else { *bw = B1::BW; *bh = B1::BH; }
  } else {
    using B0 = StripBox<T, 1, Tile2<0>::TS, Tile2<0>::TT>;
    using B1 = StripBox<T, 1, Tile2<1>::TS, Tile2<1>::TT>;
    if (tile == 0) { *bw = B0::BW; *bh = B0::BH; }
    else { *bw = B1::BW; *bh = B1::BH; }
  }
}
// kind 0: the staged level's box of ``scheme``; kind 1: the viscous strip's box
template <typename T> static void box_for(int scheme, int kind, int ax, int tile, cuuint32_t* bw, cuuint32_t* bh) {
  if (kind == 1) return strip_box<T>(ax, tile, bw, bh);
  switch (scheme) {
    case PCM: box_of<T, PCM>(ax, tile, bw, bh); break;
    case PLM: box_of<T, PLM>(ax, tile, bw, bh); break;
    case PPM: box_of<T, PPM>(ax, tile, bw, bh); break;
    case WENO3: box_of<T, WENO3>(ax, tile, bw, bh); break;
    case WENO5: box_of<T, WENO5>(ax, tile, bw, bh); break;
    default: box_of<T, WENO7>(ax, tile, bw, bh); break;
  }
}

struct astrea_handle {
  IEngine* eng;
};

template <typename T> struct Engine final : IEngine {
  T* k[2] = {nullptr, nullptr};
  T* d[2] = {nullptr, nullptr};
  T* tmp = nullptr;
  T* wf[2] = {nullptr, nullptr};  // 2D MHD: face values of each sweep
  T* ez = nullptr;                // 2D MHD: corner electric field
  SweepFn<T> sweep[2] = {nullptr, nullptr};
  T* reg[6] = {};                    // registers of the integrators with more live stages (rk_stage_kernel)
  T* wsb[2] = {nullptr, nullptr};    // 2D high-order schemes: the stage input's cell averages, one per sweep order
  CellAvgFn<T> cavg = nullptr;
  // TMA maps of every buffer a sweep reads (state, stage buffers, registers): 4 per buffer ([axis][tile])
  // (kind 0: the staged level's box; kind 1: the viscous strip's box, for the stage inputs of PPM with viscosity)
  static constexpr int kMapSlots = 16;
  CUtensorMap* d_maps = nullptr;
  std::vector<std::pair<const void*, int>> map_ptr;
  SweepFn<T> cand[2][NTILES2] = {};  // tile candidates per axis (nullptr: not built for this configuration)
  int tile[2] = {0, 0};
  bool tuned = false;

  ~Engine() override {
    for (int i = 0; i < 2; ++i) { cudaFree(k[i]); cudaFree(d[i]); cudaFree(wf[i]); cudaFree(wsb[i]); }
    for (T* r : reg) cudaFree(r);
    cudaFree(d_maps);
    cudaFree(tmp);
    cudaFree(ez);
  }

  bool ct() const { return (cfg.flags & ASTREA_FLAG_CT) != 0; }
  // 2D high-order sweeps stage the cell averages of a pre-pass (cell_average_kernel)
  bool use_ws() const { return cfg.dim == 2 && cfg.scheme >= PPM; }
  // FP64: one copy per sweep order; FP32: the axis-0 order serves both sweeps
  static constexpr int n_ws() { return cell_average_both_orders<T>() ? 2 : 1; }

  long long plane() const { return cells; }

  int alloc() override {
    const size_t bytes = sizeof(T) * (size_t)nv * (size_t)cells;
    for (int i = 0; i < 2; ++i) {
      if (cudaMalloc(&k[i], bytes) != cudaSuccess) return fail(ASTREA_ERR_OOM, "stage buffer allocation failed");
      if (cudaMalloc(&d[i], bytes) != cudaSuccess) return fail(ASTREA_ERR_OOM, "divergence buffer allocation failed");
    }
    if (cudaMalloc(&tmp, bytes) != cudaSuccess) return fail(ASTREA_ERR_OOM, "scratch allocation failed");
    if (use_ws()) {
      for (int i = 0; i < n_ws(); ++i)
        if (cudaMalloc(&wsb[i], bytes) != cudaSuccess) return fail(ASTREA_ERR_OOM, "cell-average buffer allocation failed");
      cavg = get_cell_average<T>(cfg.model);
      if (!cavg) return fail(ASTREA_ERR_CONFIG, "no cell-average kernel for this model");
    }
    if (cfg.integrator >= SSPRK53) {
      const int nreg = cfg.integrator == SSPRK53 ? 6 : (cfg.integrator == SSPRK104 ? 3 : (cfg.integrator == RK4 ? 4 : 5));
      for (int i = 0; i < nreg; ++i)
        if (cudaMalloc(&reg[i], bytes) != cudaSuccess) return fail(ASTREA_ERR_OOM, "register allocation failed");
    }
    if (ct()) {
      const size_t b8 = sizeof(T) * 8 * (size_t)cells;
      if (cudaMalloc(&wf[0], b8) != cudaSuccess || cudaMalloc(&wf[1], b8) != cudaSuccess ||
          cudaMalloc(&ez, sizeof(T) * (size_t)cells) != cudaSuccess)
        return fail(ASTREA_ERR_OOM, "constrained-transport buffer allocation failed");
      CK(cudaFuncSetAttribute(corner_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)corner_smem_bytes<T>()));
    }
    SweepFn<T> (*getter)(int, int, int, int, int) = nullptr;
    switch (cfg.scheme) {
      case PCM: getter = &get_sweep<T, PCM>; break;
      case PLM: getter = &get_sweep<T, PLM>; break;
      case PPM: getter = &get_sweep<T, PPM>; break;
      case WENO3: getter = &get_sweep<T, WENO3>; break;
      case WENO5: getter = &get_sweep<T, WENO5>; break;
      case WENO7: getter = &get_sweep<T, WENO7>; break;
      default: return fail(ASTREA_ERR_CONFIG, "unknown scheme");
    }
    for (int ax = 0; ax < cfg.dim; ++ax)
      for (int t = 0; t < NTILES2; ++t) cand[ax][t] = getter(cfg.model, cfg.solver == LW ? LLF : cfg.solver, cfg.dim, ax, t);
    sweep[0] = cand[0][0];
    sweep[1] = cfg.dim == 2 ? cand[1][0] : nullptr;
    if (!sweep[0] || (cfg.dim == 2 && !sweep[1]))
      return fail(ASTREA_ERR_CONFIG, "no kernel for this (model, solver, dimension); use model 8 for HLLD or transverse velocities");
    // TMA maps for the engine's own buffers (2D grids whose rows are whole 16-byte units)
    const char* tma_env = std::getenv("ASTREA_TMA");
    if (cfg.dim == 2 && ((size_t)cfg.n1 * sizeof(T)) % 16 == 0 && encode_tiled() && !(tma_env && tma_env[0] == '0')) {
      CK(cudaMalloc(&d_maps, sizeof(CUtensorMap) * 4 * kMapSlots));
      if (use_ws()) {
        for (int i = 0; i < n_ws(); ++i) CK(add_map(wsb[i]));
        if (strip_maps()) {
          for (int i = 0; i < 2; ++i) CK(add_map(k[i], 1));
          for (T* r : reg)
            if (r) CK(add_map(r, 1));
        }
      } else {
        for (int i = 0; i < 2; ++i) CK(add_map(k[i]));
        for (T* r : reg)
          if (r) CK(add_map(r));
      }
    }
    // set the kernels' shared-memory attribute now, outside any stream capture
    SweepArgs<T> probe{};
    probe.n0 = 0;
    for (int ax = 0; ax < cfg.dim; ++ax)
      for (int t = 0; t < NTILES2; ++t)
        if (cand[ax][t]) CK(cand[ax][t](probe, nullptr));
    return ASTREA_OK;
  }

  // the stage inputs of PPM with viscosity get strip maps
  bool strip_maps() const { return use_ws() && cfg.scheme == PPM && (cfg.flags & ASTREA_FLAG_VISCOSITY) != 0; }

  // encode the four TMA maps of a buffer (synchronous; outside any capture)
  cudaError_t add_map(const void* p, int kind = 0) {
    if (!d_maps || !p || find_map(p, kind) || (int)map_ptr.size() >= kMapSlots) return cudaSuccess;
    if ((reinterpret_cast<uintptr_t>(p) & 15) != 0) return cudaSuccess;
    CUtensorMap m[4];
    const cuuint64_t dims[3] = {(cuuint64_t)cfg.n1, (cuuint64_t)cfg.n0, (cuuint64_t)nv};
    const cuuint64_t strides[2] = {(cuuint64_t)cfg.n1 * sizeof(T), (cuuint64_t)cells * sizeof(T)};
    const cuuint32_t estr[3] = {1, 1, 1};
    for (int ax = 0; ax < 2; ++ax)
      for (int tile = 0; tile < 2; ++tile) {
        cuuint32_t box[3] = {0, 0, (cuuint32_t)nv};
        box_for<T>(cfg.scheme, kind, ax, tile, &box[0], &box[1]);
        const CUresult r = encode_tiled()(&m[ax * 2 + tile], sizeof(T) == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64
                                                                             : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
                                          3, const_cast<void*>(p), dims, strides, box, estr,
                                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return cudaSuccess;  // no map: this buffer is staged with plain loads
      }
    cudaError_t e = cudaMemcpy(d_maps + 4 * map_ptr.size(), m, sizeof(m), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    map_ptr.push_back({p, kind});
    return cudaSuccess;
  }
  const CUtensorMap* find_map(const void* p, int kind = 0) const {
    for (size_t i = 0; i < map_ptr.size(); ++i)
      if (map_ptr[i].first == p && map_ptr[i].second == kind) return d_maps + 4 * i;
    return nullptr;
  }

  int prepare(const void* state, cudaStream_t st) override {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(st, &cs));
    if (cs == cudaStreamCaptureStatusNone) {
      if (!use_ws()) CK(add_map(state));
      else if (strip_maps()) CK(add_map(state, 1));
    }
    return tune(state, st);
  }

  void tile_of(int ax, int* ts, int* tt) const override {
    const int t = tile[ax & 1];
    if (cfg.dim == 1) { *ts = TS1; *tt = 1; }
    else if (t == 0) { *ts = Tile2<0>::TS; *tt = Tile2<0>::TT; }
    else { *ts = Tile2<1>::TS; *tt = Tile2<1>::TT; }
  }

  int tune(const void* state, cudaStream_t st) override {
    if (tuned) return ASTREA_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone) return ASTREA_OK;  // keep the default tile inside a capture
    tuned = true;
    const char* env = std::getenv("ASTREA_SWEEP_TILE");
    int forced_ax[2] = {-1, -1};
    if (env && env[0] >= '0' && env[0] <= '9') {
      forced_ax[0] = forced_ax[1] = std::atoi(env);
      const char* comma = std::strchr(env, ',');
      if (comma && comma[1] >= '0' && comma[1] <= '9') forced_ax[1] = std::atoi(comma + 1);
    }
    int dev = 0;
    CK(cudaGetDevice(&dev));
    for (int ax = 0; ax < cfg.dim; ++ax) {
      int n_cand = 0;
      for (int t = 0; t < NTILES2; ++t) n_cand += cand[ax][t] != nullptr;
      const int forced = forced_ax[ax];
      if (forced >= 0 && forced < NTILES2 && cand[ax][forced]) { tile[ax] = forced; sweep[ax] = cand[ax][forced]; continue; }
      if (n_cand < 2) continue;
      char key[160];
      std::snprintf(key, sizeof(key), "%d/%d/%d/%d/%d/%d/%d/%d/%d/%d", (int)sizeof(T), cfg.model, cfg.scheme, cfg.solver,
                    cfg.flags, cfg.n0, cfg.n1, cfg.boundary, dev, ax);
      {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) { tile[ax] = it->second; sweep[ax] = cand[ax][it->second]; continue; }
      }
      // time each candidate: the axis's first sweep (store the divergence) on this grid's state
      Clock* c = clk + 1;
      CK(cudaMemsetAsync(&c->done, 0, sizeof(int), st));
      SweepArgs<T> a = base_args(static_cast<const T*>(state), c);
      a.mode = 0;
      a.want_emax = 0;
      a.dout = d[ax];
      int prc = prep(static_cast<const T*>(state), c, st, nullptr);
      if (prc) return prc;
      cudaEvent_t e0, e1;
      CK(cudaEventCreate(&e0));
      CK(cudaEventCreate(&e1));
      float best = 0.f;
      int best_t = 0;
      for (int t = 0; t < NTILES2; ++t) {
        if (!cand[ax][t]) continue;
        CK(run_sweep(cand[ax][t], ax, a, st));
        CK(cudaEventRecord(e0, st));
        for (int r = 0; r < 3; ++r) CK(run_sweep(cand[ax][t], ax, a, st));
        CK(cudaEventRecord(e1, st));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (t == 0 || ms < best) { best = ms; best_t = t; }
      }
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      tile[ax] = best_t;
      sweep[ax] = cand[ax][best_t];
      std::lock_guard<std::mutex> lock(g_tune_mutex);
      g_tune_cache[key] = best_t;
    }
    return ASTREA_OK;
  }

  SweepArgs<T> base_args(const T* q, Clock* c) const {
    SweepArgs<T> a{};
    a.q = q;
    a.plane = plane();
    a.n0 = cfg.n0;
    a.n1 = cfg.dim == 1 ? 1 : cfg.n1;
    a.bc = cfg.boundary;
    a.label = -1;
    a.limiter = cfg.limiter;
    a.integ = cfg.integrator;
    a.gamma = T(cfg.gamma);
    a.gm1 = T(cfg.gamma - 1.0);
    a.dx = cfg.dx;
    a.clock = c;
    a.physical = (cfg.flags & ASTREA_FLAG_PHYSICAL) ? 1 : 0;
    a.lw = cfg.solver == LW ? 1 : 0;
    a.flatten = (cfg.flags & ASTREA_FLAG_FLATTEN) ? 1 : 0;
    a.viscosity = (cfg.flags & ASTREA_FLAG_VISCOSITY) ? 1 : 0;
    a.av_alpha = T(0.3);
    a.av_beta = T(0.3);
    a.tmaps = use_ws() ? nullptr : find_map(q);
    a.qmaps = strip_maps() ? find_map(q, 1) : nullptr;
    return a;
  }

  // the cell-average pre-pass of a stage input (2D high-order schemes)
  int prep(const T* q, Clock* c, cudaStream_t st, KTimer* tm) {
    if (!use_ws()) return ASTREA_OK;
    TSTART(3);
    CK(cavg(q, wsb[0], wsb[1], cfg.n0, cfg.n1, plane(), cfg.boundary, T(cfg.gamma - 1.0), c, st));
    TSTOP();
    return ASTREA_OK;
  }
  // one sweep along ``ax``, pointed at that axis's cell averages when the scheme uses them
  cudaError_t run_sweep(SweepFn<T> fn, int ax, SweepArgs<T> a, cudaStream_t st) const {
    if (use_ws()) {
      a.ws = wsb[n_ws() == 2 ? ax : 0];
      a.tmaps = find_map(a.ws);
    }
    return fn(a, st);
  }

  // 2D MHD step: per stage both sweeps (storing face values), the corner
  // field, the combine with induction rows, and the inverse reconstruction of B
  int enqueue_step_ct(T* u, Clock* c, bool device_dt, cudaStream_t st, KTimer* tm) {
    const int ns = stages_of(cfg.integrator);
    const int threads = 256;
    const int blocks = (int)std::min<long long>((cells + threads - 1) / threads, 152LL * 16);
    const dim3 cgrid((cfg.n0 + CTX - 1) / CTX, (cfg.n1 + CTY - 1) / CTY);
    const dim3 rgrid((cfg.n0 + RTX - 1) / RTX, (cfg.n1 + RTY - 1) / RTY);
    const int hll = cfg.solver == HLLC || cfg.solver == HLLD;
    for (int s = 0; s < ns; ++s) {
      T* cur = s == 0 ? u : k[(s - 1) % 2];
      T* out = s == ns - 1 ? u : k[s % 2];
      SweepArgs<T> a = base_args(cur, c);
      a.mode = 0;
      a.want_emax = s == 0;
      int prc = prep(cur, c, st, tm);
      if (prc) return prc;
      for (int ax = 0; ax < 2; ++ax) {
        a.dout = d[ax];
        a.wface_out = wf[ax];
        TSTART(0);
        CK(run_sweep(sweep[ax], ax, a, st));
        TSTOP();
      }
      if (s == 0 && device_dt) {
        TSTART(2);
        dt_kernel<<<1, 32, 0, st>>>(c, 1);
        CK(cudaGetLastError());
        TSTOP();
      }
      TSTART(1);
      corner_kernel<T><<<cgrid, 256, corner_smem_bytes<T>(), st>>>(wf[0], wf[1], ez, cfg.n0, cfg.n1, plane(),
                                                                   cfg.boundary, T(cfg.gamma), hll, c);
      CK(cudaGetLastError());
      ct_combine_kernel<T><<<blocks, threads, 0, st>>>(u, cur, d[0], d[1], ez, wf[0], wf[1], tmp, cfg.n0, cfg.n1,
                                                       plane(), cfg.boundary, cfg.dx, cfg.integrator, s, c);
      CK(cudaGetLastError());
      refine_kernel<T, 0><<<rgrid, 256, 0, st>>>(tmp, out, cfg.n0, cfg.n1, plane(), cfg.boundary, c);
      CK(cudaGetLastError());
      refine_kernel<T, 1><<<rgrid, 256, 0, st>>>(tmp, out, cfg.n0, cfg.n1, plane(), cfg.boundary, c);
      CK(cudaGetLastError());
      copy_nonB_kernel<T><<<blocks, threads, 0, st>>>(tmp, out, plane(), cells, c);
      CK(cudaGetLastError());
      TSTOP();
    }
    if (device_dt) {
      TSTART(2);
      end_step_kernel<<<1, 32, 0, st>>>(c, 1);
      CK(cudaGetLastError());
      TSTOP();
    }
    return ASTREA_OK;
  }

  // input state of stage s of the register integrators
  const T* rk_input(int s, const T* u) const {
    if (s == 0) return u;
    switch (cfg.integrator) {
      case RK4: return reg[0];
      case SSPRK53:
      case SSPRK54: return reg[s - 1];
      default: return s <= 5 ? reg[0] : (s == 6 ? reg[1] : reg[2]);  // SSPRK104
    }
  }
  // destination register of stage s (the state at the last stage)
  T* rk_output(int s, T* u) const {
    if (s == stages_of(cfg.integrator) - 1) return u;
    switch (cfg.integrator) {
      case RK4: return reg[0];
      case SSPRK53:
      case SSPRK54: return reg[s];
      default: return s <= 4 ? reg[0] : (s == 5 ? reg[1] : reg[2]);  // SSPRK104
    }
  }

  // SSP-RK (5,3), (5,4), (10,4), RK4: both sweeps of a stage store their divergences,
  // then one element-wise kernel forms L and the stage's register.
  int enqueue_step_rk(T* u, Clock* c, bool device_dt, cudaStream_t st, KTimer* tm) {
    const int ns = stages_of(cfg.integrator);
    const int threads = 256;
    const int blocks = (int)std::min<long long>((cells + threads - 1) / threads, 152LL * 16);
    for (int s = 0; s < ns; ++s) {
      SweepArgs<T> a = base_args(rk_input(s, u), c);
      a.mode = 0;
      a.want_emax = s == 0;
      int prc = prep(rk_input(s, u), c, st, tm);
      if (prc) return prc;
      for (int ax = 0; ax < cfg.dim; ++ax) {
        a.dout = d[ax];
        TSTART(0);
        CK(run_sweep(sweep[ax], ax, a, st));
        TSTOP();
      }
      if (s == 0 && device_dt) {
        TSTART(2);
        dt_kernel<<<1, 32, 0, st>>>(c, 1);
        CK(cudaGetLastError());
        TSTOP();
      }
      RkStage<T> r{};
      r.u = u;
      for (int i = 0; i < 6; ++i) r.r[i] = reg[i];
      r.d0 = d[0];
      r.d1 = cfg.dim == 2 ? d[1] : nullptr;
      r.out = rk_output(s, u);
      r.n = (long long)nv * plane();
      r.integ = cfg.integrator;
      r.stage = s;
      r.clk = c;
      TSTART(1);
      rk_stage_kernel<T><<<blocks, threads, 0, st>>>(r);
      CK(cudaGetLastError());
      TSTOP();
    }
    if (device_dt) {
      TSTART(2);
      end_step_kernel<<<1, 32, 0, st>>>(c, 1);
      CK(cudaGetLastError());
      TSTOP();
    }
    return ASTREA_OK;
  }

  bool fuses_host_out() const override {
    return !ct() && cfg.integrator < SSPRK53 && stages_of(cfg.integrator) >= 2;
  }

  int enqueue_step(void* state, Clock* c, bool device_dt, cudaStream_t st, KTimer* tm = nullptr) override {
    T* u = static_cast<T*>(state);
    if (cfg.integrator >= SSPRK53) return enqueue_step_rk(u, c, device_dt, st, tm);
    const int ns = stages_of(cfg.integrator);
    if (ns < 0) return fail(ASTREA_ERR_CONFIG, "integrator not supported by this library");
    if (ct()) return enqueue_step_ct(u, c, device_dt, st, tm);
    const long long n = cells;
    const int threads = 256;
    const int blocks = (int)std::min<long long>((n + threads - 1) / threads, 152LL * 16);
    // stage 0
    {
      SweepArgs<T> a = base_args(u, c);
      a.mode = 0;
      a.want_emax = 1;
      a.dout = d[0];
      int prc = prep(u, c, st, tm);
      if (prc) return prc;
      TSTART(0);
      CK(run_sweep(sweep[0], 0, a, st));
      TSTOP();
      if (cfg.dim == 2) {
        a.dout = d[1];
        TSTART(0);
        CK(run_sweep(sweep[1], 1, a, st));
        TSTOP();
      }
      if (device_dt) {
        TSTART(2);
        dt_kernel<<<1, 32, 0, st>>>(c, 1);
        CK(cudaGetLastError());
        TSTOP();
      }
      T* out0 = ns == 1 ? u : k[0];
      TSTART(1);
      combine0_kernel<T><<<blocks, threads, 0, st>>>(u, d[0], cfg.dim == 2 ? d[1] : nullptr, out0, plane(), n, nv,
                                                     cfg.integrator, c);
      CK(cudaGetLastError());
      TSTOP();
    }
    for (int s = 1; s < ns; ++s) {
      T* cur = k[(s - 1) % 2];
      T* out = s == ns - 1 ? u : k[s % 2];
      SweepArgs<T> a = base_args(cur, c);
      a.stage = s;
      a.u0 = u;
      a.out = out;
      if (s == ns - 1) a.out_host = static_cast<T*>(host_out);
      int prc = prep(cur, c, st, tm);
      if (prc) return prc;
      if (cfg.dim == 2) {
        a.mode = 0;
        a.dout = d[0];
        TSTART(0);
        CK(run_sweep(sweep[0], 0, a, st));
        TSTOP();
        a.mode = 1;
        a.dother = d[0];
        a.dout = nullptr;
        TSTART(0);
        CK(run_sweep(sweep[1], 1, a, st));
        TSTOP();
      } else {
        a.mode = 2;
        TSTART(0);
        CK(run_sweep(sweep[0], 0, a, st));
        TSTOP();
      }
    }
    if (device_dt) {
      TSTART(2);
      end_step_kernel<<<1, 32, 0, st>>>(c, 1);
      CK(cudaGetLastError());
      TSTOP();
    }
    return ASTREA_OK;
  }

  // face0/face1/corner (constrained transport only): each sweep's face values and the corner field
  int space(const void* state, int order, void* f0, void* f1, double* eigmax, cudaStream_t st, void* face0,
            void* face1, void* corner) override {
    Clock* c = clk + 1;
    CK(cudaMemsetAsync(&c->emax[0], 0, 2 * sizeof(unsigned long long), st));
    CK(cudaMemcpyAsync(&c->order, &order, sizeof(int), cudaMemcpyHostToDevice, st));
    SweepArgs<T> a = base_args(static_cast<const T*>(state), c);
    a.mode = 0;
    a.want_emax = 1;
    a.dout = d[0];
    a.flux_out = static_cast<T*>(f0);
    T* faces[2] = {ct() ? (face0 ? static_cast<T*>(face0) : wf[0]) : nullptr,
                   ct() ? (face1 ? static_cast<T*>(face1) : wf[1]) : nullptr};
    a.wface_out = faces[0];
    int prc = prep(static_cast<const T*>(state), c, st, nullptr);
    if (prc) return prc;
    CK(run_sweep(sweep[0], 0, a, st));
    if (cfg.dim == 2) {
      a.dout = d[1];
      a.flux_out = static_cast<T*>(f1);
      a.wface_out = faces[1];
      CK(run_sweep(sweep[1], 1, a, st));
    }
    if (ct() && corner) {
      const dim3 cgrid((cfg.n0 + CTX - 1) / CTX, (cfg.n1 + CTY - 1) / CTY);
      corner_kernel<T><<<cgrid, 256, corner_smem_bytes<T>(), st>>>(faces[0], faces[1], static_cast<T*>(corner),
                                                                   cfg.n0, cfg.n1, plane(), cfg.boundary,
                                                                   T(cfg.gamma), cfg.solver == HLLC || cfg.solver == HLLD, c);
      CK(cudaGetLastError());
    }
    unsigned long long e[2];
    CK(cudaMemcpyAsync(e, &c->emax[0], sizeof(e), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    double v[2];
    std::memcpy(&v[0], &e[0], sizeof(double));
    std::memcpy(&v[1], &e[1], sizeof(double));
    if (eigmax) { eigmax[0] = v[0]; eigmax[1] = cfg.dim == 2 ? v[1] : 0.0; }
    return ASTREA_OK;
  }

  int initialise(const void* prim, void* out, cudaStream_t st) override {
    const int threads = 256;
    const int blocks = (int)std::min<long long>((cells + threads - 1) / threads, 152LL * 16);
    const int ho = cfg.scheme >= PPM;
    const T gm1 = T(cfg.gamma - 1.0);
    const int n1 = cfg.dim == 1 ? 1 : cfg.n1;
    switch (cfg.model) {
      case 3: init_pass_a<T, 3><<<blocks, threads, 0, st>>>(static_cast<const T*>(prim), tmp, cfg.n0, n1, plane(), cfg.dim, cfg.boundary, ho, gm1); break;
      case 4: init_pass_a<T, 4><<<blocks, threads, 0, st>>>(static_cast<const T*>(prim), tmp, cfg.n0, n1, plane(), cfg.dim, cfg.boundary, ho, gm1); break;
      default: init_pass_a<T, 8><<<blocks, threads, 0, st>>>(static_cast<const T*>(prim), tmp, cfg.n0, n1, plane(), cfg.dim, cfg.boundary, ho, gm1); break;
    }
    CK(cudaGetLastError());
    centre_to_avg_kernel<T><<<blocks, threads, 0, st>>>(tmp, static_cast<T*>(out), cfg.n0, n1, plane(), nv, cfg.dim, cfg.boundary);
    CK(cudaGetLastError());
    return ASTREA_OK;
  }

  int to_primitive(const void* state, void* out, cudaStream_t st) override {
    const int threads = 256;
    const int blocks = (int)std::min<long long>((cells + threads - 1) / threads, 152LL * 16);
    const int ho = cfg.scheme >= PPM;
    const T gm1 = T(cfg.gamma - 1.0);
    const int n1 = cfg.dim == 1 ? 1 : cfg.n1;
    const T* q = static_cast<const T*>(state);
    T* w = static_cast<T*>(out);
    switch (cfg.model) {
      case 3: prim_kernel<T, 3><<<blocks, threads, 0, st>>>(q, w, cfg.n0, n1, plane(), cfg.dim, cfg.boundary, ho, gm1); break;
      case 4: prim_kernel<T, 4><<<blocks, threads, 0, st>>>(q, w, cfg.n0, n1, plane(), cfg.dim, cfg.boundary, ho, gm1); break;
      default: prim_kernel<T, 8><<<blocks, threads, 0, st>>>(q, w, cfg.n0, n1, plane(), cfg.dim, cfg.boundary, ho, gm1); break;
    }
    CK(cudaGetLastError());
    return ASTREA_OK;
  }

  int reduce(const void* state, double* host, cudaStream_t st) override {
    const int nb = 152;
    sums_pass1<T><<<nb, 256, 0, st>>>(static_cast<const T*>(state), plane(), cells, nv, part);
    CK(cudaGetLastError());
    sums_pass2<<<1, 32, 0, st>>>(part, nb, nv, sums);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(host, sums, sizeof(double) * nv, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return ASTREA_OK;
  }
};

static int validate(const astrea_cfg* c) {
  if (!c) return fail(ASTREA_ERR_ARG, "cfg is NULL");
  if (c->dim != 1 && c->dim != 2) return fail(ASTREA_ERR_CONFIG, "dim must be 1 or 2");
  if (c->n0 < 4 || (c->dim == 2 && c->n1 < 4)) return fail(ASTREA_ERR_CONFIG, "at least 4 cells per axis are required");
  if (c->dim == 1 && c->n1 != 1) return fail(ASTREA_ERR_CONFIG, "1D grids have n1 == 1");
  if (c->model != 3 && c->model != 4 && c->model != 8) return fail(ASTREA_ERR_CONFIG, "model must be 3, 4 or 8");
  if (c->model == 3 && c->dim != 1) return fail(ASTREA_ERR_CONFIG, "model 3 is 1D only");
  if (c->model == 4 && c->dim != 2) return fail(ASTREA_ERR_CONFIG, "model 4 is 2D only");
  if (c->precision != 32 && c->precision != 64) return fail(ASTREA_ERR_CONFIG, "precision must be 32 or 64");
  if (c->scheme < 0 || c->scheme > WENO7) return fail(ASTREA_ERR_CONFIG, "unknown scheme");
  if (c->solver < 0 || c->solver > LW) return fail(ASTREA_ERR_CONFIG, "unknown solver");
  if (stages_of(c->integrator) < 0) return fail(ASTREA_ERR_CONFIG, "integrator not supported by this library");
  if (c->boundary != EDGE && c->boundary != WRAP) return fail(ASTREA_ERR_CONFIG, "boundary must be edge(0) or wrap(1)");
  if ((c->flags & ASTREA_FLAG_CT) && (c->dim != 2 || c->model != 8))
    return fail(ASTREA_ERR_CONFIG, "constrained transport needs dim 2 and model 8");
  if ((c->flags & ASTREA_FLAG_CT) && c->integrator >= SSPRK53)
    return fail(ASTREA_ERR_CONFIG, "constrained transport runs with Euler and SSP-RK (2,2), (3,3), (4,3)");
  if ((c->flags & ASTREA_FLAG_CT) && (c->flags & ASTREA_FLAG_FLATTEN) && c->scheme == PPM)
    return fail(ASTREA_ERR_CONFIG, "PPM flattening is not available with constrained transport");
  if (!(c->dx > 0) || !(c->cfl > 0) || !(c->gamma > 1) || c->checkpoints < 1)
    return fail(ASTREA_ERR_CONFIG, "dx, cfl > 0, gamma > 1, checkpoints >= 1 required");
  if ((long long)c->n0 * (long long)(c->dim == 2 ? c->n1 : 1) > (1LL << 31))
    return fail(ASTREA_ERR_CONFIG, "grid larger than 2^31 cells");
  return ASTREA_OK;
}

extern "C" {

int astrea_version(void) { return 100; }

const char* astrea_last_error(void) { return g_last_error.c_str(); }

int astrea_create(const astrea_cfg* cfg, astrea_handle** out) {
  if (!out) return fail(ASTREA_ERR_ARG, "out is NULL");
  *out = nullptr;
  int rc = validate(cfg);
  if (rc) return rc;
  IEngine* e = cfg->precision == 64 ? static_cast<IEngine*>(new Engine<double>()) : static_cast<IEngine*>(new Engine<float>());
  e->cfg = *cfg;
  if (cfg->dim == 1) e->cfg.n1 = 1;
  e->nv = cfg->model;
  e->cells = (long long)cfg->n0 * (cfg->dim == 2 ? cfg->n1 : 1);
  if (cudaMalloc(&e->clk, 2 * sizeof(Clock)) != cudaSuccess || cudaMalloc(&e->part, 152 * 8 * 2 * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&e->sums, 8 * sizeof(double)) != cudaSuccess) {
    delete e;
    return fail(ASTREA_ERR_OOM, "clock allocation failed");
  }
  rc = e->alloc();
  if (rc) {
    delete e;
    return rc;
  }
  astrea_handle* h = new astrea_handle{e};
  rc = astrea_reset_clock(h, 0.0, 1, 0, nullptr);
  if (rc) {
    delete e;
    delete h;
    return rc;
  }
  CK(cudaDeviceSynchronize());
  *out = h;
  return ASTREA_OK;
}

void astrea_destroy(astrea_handle* h) {
  if (!h) return;
  delete h->eng;
  delete h;
}

int astrea_layout(const astrea_handle* h, int* nv, long long* cells) {
  if (!h) return fail(ASTREA_ERR_ARG, "handle is NULL");
  if (nv) *nv = h->eng->nv;
  if (cells) *cells = h->eng->cells;
  return ASTREA_OK;
}

int astrea_initialise(astrea_handle* h, const void* prim, void* state_out, void* stream) {
  if (!h || !prim || !state_out) return fail(ASTREA_ERR_ARG, "NULL argument");
  return h->eng->initialise(prim, state_out, static_cast<cudaStream_t>(stream));
}

int astrea_reset_clock(astrea_handle* h, double t, int idx, int order, void* stream) {
  if (!h) return fail(ASTREA_ERR_ARG, "handle is NULL");
  IEngine* e = h->eng;
  Clock c[2];
  std::memset(c, 0, sizeof(c));
  for (int i = 0; i < 2; ++i) {
    c[i].t = t;
    c[i].dt = 0.0;
    c[i].t_end = e->cfg.t_end;
    c[i].chkpt = e->cfg.t_end / e->cfg.checkpoints;
    c[i].cfl = e->cfg.cfl;
    c[i].dx = e->cfg.dx;
    c[i].idx = idx;
    c[i].order = e->cfg.dim == 2 ? (order & 1) : 0;
    c[i].naxes = e->cfg.dim;
    c[i].done = 0;
  }
  c[0].done = !(t < e->cfg.t_end);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CK(cudaMemcpyAsync(e->clk, c, sizeof(c), cudaMemcpyHostToDevice, st));
  CK(cudaStreamSynchronize(st));
  return ASTREA_OK;
}

int astrea_step(astrea_handle* h, void* state, int nsteps, void* stream) {
  if (!h || !state) return fail(ASTREA_ERR_ARG, "NULL argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int trc = h->eng->prepare(state, st);
  if (trc) return trc;
  for (int i = 0; i < nsteps; ++i) {
    int rc = h->eng->enqueue_step(state, h->eng->clk, true, st);
    if (rc) return rc;
  }
  return ASTREA_OK;
}

int astrea_step_timed(astrea_handle* h, void* state, int nsteps, double* kernel_ms, int* launches, void* stream) {
  if (!h || !state || !kernel_ms || !launches) return fail(ASTREA_ERR_ARG, "NULL argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int trc = h->eng->prepare(state, st);
  if (trc) return trc;
  KTimer tm;
  for (int i = 0; i < nsteps; ++i) {
    int rc = h->eng->enqueue_step(state, h->eng->clk, true, st, &tm);
    if (rc) return rc;
  }
  CK(cudaStreamSynchronize(st));
  for (int k = 0; k < 4; ++k) {
    double ms = 0.0;
    for (size_t i = 0; i < tm.ev[k][0].size(); ++i) {
      float x = 0.f;
      CK(cudaEventElapsedTime(&x, tm.ev[k][0][i], tm.ev[k][1][i]));
      ms += x;
    }
    kernel_ms[k] = ms;
    launches[k] = (int)tm.ev[k][0].size();
  }
  return ASTREA_OK;
}

int astrea_graph_step(astrea_handle* h, void* state, int nsteps, void* stream) {
  if (!h || !state) return fail(ASTREA_ERR_ARG, "NULL argument");
  IEngine* e = h->eng;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int trc = e->prepare(state, st);
  if (trc) return trc;
  if (!e->graph || e->graph_state != state) {
    if (e->graph) {
      cudaGraphExecDestroy(e->graph);
      e->graph = nullptr;
    }
    cudaStream_t cap;
    CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed));
    int rc = e->enqueue_step(state, e->clk, true, cap);
    cudaError_t ce = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (rc) return rc;
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
    ce = cudaGraphInstantiate(&e->graph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaGraphInstantiate");
    e->graph_state = state;
  }
  for (int i = 0; i < nsteps; ++i) CK(cudaGraphLaunch(e->graph, st));
  return ASTREA_OK;
}

int astrea_step_host(astrea_handle* h, void* state, const void* host_in, void* host_out, void* stream) {
  if (!h || !state) return fail(ASTREA_ERR_ARG, "NULL argument");
  IEngine* e = h->eng;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int trc = e->prepare(state, st);
  if (trc) return trc;
  const size_t bytes = (size_t)e->nv * (size_t)e->cells * (e->cfg.precision == 64 ? 8 : 4);
  // host_out is written by the kernels only where it is page-locked memory the device can address
  void* out_dev = nullptr;
  if (host_out) {
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, host_out) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer)
      out_dev = pa.devicePointer;
    cudaGetLastError();  // a pageable pointer is not an error here
  }
  const bool fused = out_dev != nullptr && e->fuses_host_out();
  if (!e->graph_host || e->graph_host_key[0] != state || e->graph_host_key[1] != host_in ||
      e->graph_host_key[2] != host_out) {
    if (e->graph_host) {
      cudaGraphExecDestroy(e->graph_host);
      e->graph_host = nullptr;
    }
    cudaStream_t cap;
    CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed));
    cudaError_t me = cudaSuccess;
    if (host_in) me = cudaMemcpyAsync(state, host_in, bytes, cudaMemcpyHostToDevice, cap);
    e->host_out = fused ? out_dev : nullptr;
    int rc = me == cudaSuccess ? e->enqueue_step(state, e->clk, true, cap) : ASTREA_OK;
    e->host_out = nullptr;
    if (rc == ASTREA_OK && me == cudaSuccess && host_out && !fused)
      me = cudaMemcpyAsync(host_out, state, bytes, cudaMemcpyDeviceToHost, cap);
    cudaError_t ce = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (rc) return rc;
    if (me != cudaSuccess) return cuda_fail(me, "cudaMemcpyAsync (host state)");
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
    ce = cudaGraphInstantiate(&e->graph_host, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaGraphInstantiate");
    e->graph_host_key[0] = state;
    e->graph_host_key[1] = host_in;
    e->graph_host_key[2] = host_out;
  }
  CK(cudaGraphLaunch(e->graph_host, st));
  return ASTREA_OK;
}

int astrea_get_clock(astrea_handle* h, double* t, double* dt, int* steps, int* done, int* status, void* stream) {
  if (!h) return fail(ASTREA_ERR_ARG, "handle is NULL");
  Clock c;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  CK(cudaMemcpyAsync(&c, h->eng->clk, sizeof(Clock), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (t) *t = c.t;
  if (dt) *dt = c.dt;
  if (steps) *steps = c.steps;
  if (done) *done = c.done;
  if (status) *status = c.status;
  return ASTREA_OK;
}

int astrea_clock_async(astrea_handle* h, double* t, int* steps, int* done, void* stream) {
  if (!h || !t || !steps || !done) return fail(ASTREA_ERR_ARG, "NULL argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const Clock* c = h->eng->clk;
  CK(cudaMemcpyAsync(t, &c->t, sizeof(double), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(steps, &c->steps, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(done, &c->done, sizeof(int), cudaMemcpyDeviceToHost, st));
  return ASTREA_OK;
}

int astrea_space(astrea_handle* h, const void* state, int order, void* flux_ax0, void* flux_ax1, double* eigmax,
                 void* stream) {
  if (!h || !state) return fail(ASTREA_ERR_ARG, "NULL argument");
  int trc = h->eng->prepare(state, static_cast<cudaStream_t>(stream));
  if (trc) return trc;
  return h->eng->space(state, order & 1, flux_ax0, flux_ax1, eigmax, static_cast<cudaStream_t>(stream));
}

int astrea_space_ct(astrea_handle* h, const void* state, int order, void* flux_ax0, void* flux_ax1, double* eigmax,
                    void* face_ax0, void* face_ax1, void* corner, void* stream) {
  if (!h || !state) return fail(ASTREA_ERR_ARG, "NULL argument");
  if (!(h->eng->cfg.flags & ASTREA_FLAG_CT)) return fail(ASTREA_ERR_CONFIG, "astrea_space_ct needs ASTREA_FLAG_CT");
  int trc = h->eng->prepare(state, static_cast<cudaStream_t>(stream));
  if (trc) return trc;
  return h->eng->space(state, order & 1, flux_ax0, flux_ax1, eigmax, static_cast<cudaStream_t>(stream), face_ax0,
                       face_ax1, corner);
}

int astrea_time(astrea_handle* h, void* state, double dt, int order, void* stream) {
  if (!h || !state) return fail(ASTREA_ERR_ARG, "NULL argument");
  IEngine* e = h->eng;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int trc = e->prepare(state, st);
  if (trc) return trc;
  Clock c;
  std::memset(&c, 0, sizeof(c));
  c.t = 0.0;
  c.dt = dt;
  c.t_end = 1e300;
  c.chkpt = 1e300;
  c.cfl = e->cfg.cfl;
  c.dx = e->cfg.dx;
  c.idx = 1;
  c.order = e->cfg.dim == 2 ? (order & 1) : 0;
  c.naxes = e->cfg.dim;
  CK(cudaMemcpyAsync(e->clk + 1, &c, sizeof(c), cudaMemcpyHostToDevice, st));
  int rc = e->enqueue_step(state, e->clk + 1, false, st);
  if (rc) return rc;
  CK(cudaStreamSynchronize(st));
  return ASTREA_OK;
}

int astrea_to_primitive(astrea_handle* h, const void* state, void* prim_out, void* stream) {
  if (!h || !state || !prim_out) return fail(ASTREA_ERR_ARG, "NULL argument");
  return h->eng->to_primitive(state, prim_out, static_cast<cudaStream_t>(stream));
}

int astrea_sweep_tile(const astrea_handle* h, int axis, int* ts, int* tt) {
  if (!h || !ts || !tt || axis < 0 || axis > 1) return fail(ASTREA_ERR_ARG, "bad argument");
  h->eng->tile_of(axis, ts, tt);
  return ASTREA_OK;
}

int astrea_reduce_conserved(astrea_handle* h, const void* state, double* sums_host, void* stream) {
  if (!h || !state || !sums_host) return fail(ASTREA_ERR_ARG, "NULL argument");
  return h->eng->reduce(state, sums_host, static_cast<cudaStream_t>(stream));
}

}  // extern "C"

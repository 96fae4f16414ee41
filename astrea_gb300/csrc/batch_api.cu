// C ABI of the batched engine (astrea_batch_*).
//
// A batch owns a fixed number of *slots* and stage buffers for a fixed arena
// capacity.  A slot holds one grid at a caller-chosen element offset of the
// caller's state arena; slots are occupied and released at any time between
// steps (continuous batching).  Each step advances every occupied, unfinished
// slot by one of its own time steps: one persistent kernel per sweep walks a
// work list of tiles of all occupied slots (largest grids first).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "batch_launch.cuh"
#include "cellavg.cuh"
#include "host_common.h"

using namespace astrea;

namespace astrea {
ASTREA_EXTERN_BATCH(float)
ASTREA_EXTERN_BATCH(double)
ASTREA_EXTERN_BATCH_T2
}  // namespace astrea

template <typename T> static BatchFn<T> batched_for(int model, int dim, int ax, int v) {
  return dim == 1 ? get_batched<T, 1>(model, ax, v) : get_batched<T, 2>(model, ax, v);
}
template <typename T> static int occupancy_for(int model, int dim, int ax, int v) {
  return dim == 1 ? get_occupancy<T, 1>(model, ax, v) : get_occupancy<T, 2>(model, ax, v);
}
static int tile_ts(int dim, int v) { return dim == 1 ? BTS1 : (v == 0 ? BTile2<0>::TS : BTile2<1>::TS); }
static int tile_tt(int dim, int v) { return dim == 1 ? 1 : (v == 0 ? BTile2<0>::TT : BTile2<1>::TT); }

namespace {

int combo_of(int scheme, int solver, int model, int* out) {
  const bool hll = solver != LLF;
  if (hll && solver != (model == 8 ? HLLD : HLLC)) return -1;
  switch (scheme) {
    case PLM: *out = hll ? C_PLM_HLL : C_PLM_LLF; return 0;
    case PPM: *out = hll ? C_PPM_HLL : C_PPM_LLF; return 0;
    case WENO5: *out = hll ? C_WENO5_HLL : C_WENO5_LLF; return 0;
    default: return -1;
  }
}

int stages_count(int integ) {
  switch (integ) {
    case EULER: return 1;
    case SSPRK22: return 2;
    case SSPRK33: return 3;
    case SSPRK43: return 4;
    default: return -1;
  }
}

}  // namespace

// Slot changes (occupy, release) are queued on the host and applied on the
// device by the next step, stream-ordered, so that admitting or retiring a grid
// never synchronises the device.  The changes travel as kernel parameters.
template <typename T> struct SlotUpdate {
  int slot, has_grid;
  BGrid<T> grid;
  Clock clock;
};
constexpr int kUpdatesPerLaunch = 16;
template <typename T> struct SlotUpdates {
  SlotUpdate<T> u[kUpdatesPerLaunch];
  int n;
};
static_assert(sizeof(SlotUpdates<double>) <= 4000, "slot updates exceed the kernel parameter space");
template <typename T> __global__ void apply_slot_updates(const SlotUpdates<T> up, BGrid<T>* grids, Clock* clocks) {
  const int i = threadIdx.x;
  if (i >= up.n) return;
  if (up.u[i].has_grid) grids[up.u[i].slot] = up.u[i].grid;
  clocks[up.u[i].slot] = up.u[i].clock;
}

struct IBatch {
  int dim = 2, model = 4, precision = 32, integrator = SSPRK33, max_slots = 0, nv = 0;
  long long capacity = 0;  // elements per arena
  std::vector<astrea_grid> host_grids;
  std::vector<long long> offsets;
  std::vector<char> active;
  bool dirty = true;
  Clock* clocks = nullptr;
  int* counters = nullptr;
  BItem* items[2] = {nullptr, nullptr};
  size_t items_cap[2] = {0, 0};
  int nitems[2] = {0, 0};
  cudaGraphExec_t graph = nullptr;
  void* graph_arena = nullptr;
  virtual ~IBatch() {
    if (graph) cudaGraphExecDestroy(graph);
    cudaFree(clocks);
    cudaFree(counters);
    cudaFree(items[0]);
    cudaFree(items[1]);
  }
  virtual int alloc() = 0;
  // queue the grid of a slot and its initial clock (applied by the next step)
  virtual int set_slot(int slot, const astrea_grid& g, long long offset, const Clock& c) = 0;
  // queue a slot's release: its clock reads done, so every kernel skips it
  virtual void clear_slot(int slot) = 0;
  // apply the queued slot changes on ``st``
  virtual int flush(cudaStream_t st) = 0;
  virtual int rebuild(cudaStream_t st) = 0;
  virtual int enqueue_step(void* arena, cudaStream_t st) = 0;
  virtual int initialise(int slot, const void* prim, void* arena, cudaStream_t st) = 0;
  // pick each axis's tile (once, at the first step with occupied slots; not during a capture)
  virtual int tune(void* arena, cudaStream_t st) = 0;
  int var[2] = {0, 0};
  bool tuned = false;
};

struct astrea_batch {
  IBatch* b;
};

template <typename T> struct Batch final : IBatch {
  T *k0 = nullptr, *k1 = nullptr, *d0 = nullptr, *d1 = nullptr, *tmp = nullptr;
  // 2D: cell averages of each stage input for the high-order grids (FP64: one arena per sweep order)
  T *ws0 = nullptr, *ws1 = nullptr;
  BatchedCellAvgFn<T> cavg = nullptr;
  BStrip* strips = nullptr;
  size_t strips_cap = 0;
  int nstrips = 0;
  BGrid<T>* d_grids = nullptr;
  std::vector<SlotUpdate<T>> pending;  // at most one per slot, in queue order
  // pinned staging of the work lists, two used in turn; each is rewritten only after
  // the copies that read it last have run (its event)
  char* stage_h[2] = {nullptr, nullptr};
  size_t stage_cap[2] = {0, 0};
  cudaEvent_t stage_ev[2] = {nullptr, nullptr};
  int stage_i = 0;
  BatchFn<T> cand[2][NBTILES2] = {};  // tile candidates per axis (nullptr: not built)
  int occ_c[2][NBTILES2] = {};
  int nctas[2] = {0, 0};
  int sms = 152;

  ~Batch() override {
    cudaFree(k0); cudaFree(k1); cudaFree(d0); cudaFree(d1); cudaFree(tmp); cudaFree(d_grids);
    cudaFree(ws0);
    if (ws1 != ws0) cudaFree(ws1);
    cudaFree(strips);
    for (int i = 0; i < 2; ++i) {
      if (stage_ev[i]) cudaEventDestroy(stage_ev[i]);
      cudaFreeHost(stage_h[i]);
    }
  }

  int alloc() override {
    const size_t bytes = sizeof(T) * (size_t)capacity;
    if (cudaMalloc(&k0, bytes) != cudaSuccess || cudaMalloc(&k1, bytes) != cudaSuccess ||
        cudaMalloc(&d0, bytes) != cudaSuccess || cudaMalloc(&d1, bytes) != cudaSuccess ||
        cudaMalloc(&tmp, bytes) != cudaSuccess)
      return fail(ASTREA_ERR_OOM, "batch stage buffers allocation failed");
    if (dim == 2) {
      if (cudaMalloc(&ws0, bytes) != cudaSuccess) return fail(ASTREA_ERR_OOM, "batch cell-average arena allocation failed");
      ws1 = ws0;
      if (cell_average_both_orders<T>() && cudaMalloc(&ws1, bytes) != cudaSuccess) {
        ws1 = nullptr;
        return fail(ASTREA_ERR_OOM, "batch cell-average arena allocation failed");
      }
      cavg = get_batched_cell_average<T>(model);
      if (!cavg) return fail(ASTREA_ERR_CONFIG, "no batched cell-average kernel for this model");
    }
    CK(cudaMalloc(&d_grids, sizeof(BGrid<T>) * max_slots));
    CK(cudaMalloc(&counters, sizeof(int) * 16));
    int dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    for (int ax = 0; ax < dim; ++ax) {
      for (int v = 0; v < NBTILES2; ++v) {
        cand[ax][v] = batched_for<T>(model, dim, ax, v);
        if (!cand[ax][v]) continue;
        BatchArgs<T> probe{};
        CK(cand[ax][v](probe, 0, nullptr));
        occ_c[ax][v] = std::max(1, occupancy_for<T>(model, dim, ax, v));
      }
      if (!cand[ax][0]) return fail(ASTREA_ERR_CONFIG, "no batched kernel for this model/dimension");
    }
    return ASTREA_OK;
  }

  // Batch tile autotuner: time the first sweep of each axis (store the divergence;
  // no clock update) over the current work list for every built tile and keep the
  // fastest.  ASTREA_BATCH_TILE=<index> forces a tile (where it is built).
  int tune(void* arena, cudaStream_t st) override {
    if (tuned) return ASTREA_OK;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(st, &cs));
    if (cs != cudaStreamCaptureStatusNone) return ASTREA_OK;
    if (std::find(active.begin(), active.end(), 1) == active.end()) return ASTREA_OK;
    tuned = true;
    const char* env = std::getenv("ASTREA_BATCH_TILE");
    const int forced = (env && env[0] >= '0' && env[0] <= '9') ? std::atoi(env) : -1;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    for (int ax = 0; ax < dim; ++ax) {
      if (forced >= 0 && forced < NBTILES2 && cand[ax][forced]) { var[ax] = forced; continue; }
      float best = 0.f;
      int best_v = 0;
      for (int v = 0; v < NBTILES2; ++v) {
        if (!cand[ax][v]) continue;
        var[ax] = v;
        int rc = rebuild(st);
        if (rc) return rc;
        BatchArgs<T> b = args(static_cast<T*>(arena));
        b.stage = 0;
        b.mode = 0;
        b.want_emax = 0;
        b.dout_sel = ax;
        rc = launch_cell_average(b, st);
        if (rc) return rc;
        rc = launch_sweep(b, ax, 15, st);
        if (rc) return rc;
        CK(cudaEventRecord(e0, st));
        for (int r = 0; r < 2; ++r) {
          rc = launch_sweep(b, ax, 15, st);
          if (rc) return rc;
        }
        CK(cudaEventRecord(e1, st));
        CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (v == 0 || ms < best) { best = ms; best_v = v; }
      }
      var[ax] = best_v;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    dirty = true;
    return ASTREA_OK;
  }

  int set_slot(int slot, const astrea_grid& a, long long offset, const Clock& c) override {
    BGrid<T> d{};
    d.base = offset;
    d.cells = (long long)a.n0 * (dim == 2 ? a.n1 : 1);
    d.n0 = a.n0;
    d.n1 = dim == 1 ? 1 : a.n1;
    d.bc = a.boundary;
    d.limiter = a.limiter;
    d.physical = (a.flags & ASTREA_FLAG_PHYSICAL) ? 1 : 0;
    if (combo_of(a.scheme, a.solver, model, &d.combo)) return fail(ASTREA_ERR_CONFIG, "unsupported scheme/solver for a batch");
    d.gamma = T(a.gamma);
    d.gm1 = T(a.gamma - 1.0);
    d.dx = a.dx;
    queue(SlotUpdate<T>{slot, 1, d, c});
    return ASTREA_OK;
  }

  void queue(const SlotUpdate<T>& u) {
    for (auto& p : pending)
      if (p.slot == u.slot) {
        if (u.has_grid) { p.has_grid = 1; p.grid = u.grid; }
        p.clock = u.clock;
        return;
      }
    pending.push_back(u);
  }

  void clear_slot(int slot) override {
    SlotUpdate<T> u{};
    u.slot = slot;
    u.has_grid = 0;
    u.clock.done = 1;
    queue(u);
  }

  int flush(cudaStream_t st) override {
    for (size_t i = 0; i < pending.size(); i += kUpdatesPerLaunch) {
      SlotUpdates<T> up{};
      up.n = (int)std::min<size_t>(kUpdatesPerLaunch, pending.size() - i);
      for (int k = 0; k < up.n; ++k) up.u[k] = pending[i + k];
      apply_slot_updates<T><<<1, kUpdatesPerLaunch, 0, st>>>(up, d_grids, clocks);
      CK(cudaGetLastError());
    }
    pending.clear();
    return ASTREA_OK;
  }

  int rebuild(cudaStream_t st) override {
    std::vector<int> order;
    for (int s = 0; s < max_slots; ++s)
      if (active[s]) order.push_back(s);
    auto cells = [&](int s) { return (long long)host_grids[s].n0 * (dim == 2 ? host_grids[s].n1 : 1); };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cells(x) > cells(y); });
    std::vector<BItem> it[2];
    for (int ax = 0; ax < dim; ++ax) {
      const int TS = tile_ts(dim, var[ax]), TT = tile_tt(dim, var[ax]);
      for (int g : order) {
        const astrea_grid& a = host_grids[g];
        const int Ns = dim == 1 ? a.n0 : (ax == 0 ? a.n0 : a.n1);
        const int Nt = dim == 1 ? 1 : (ax == 0 ? a.n1 : a.n0);
        for (int s0 = 0; s0 < Ns; s0 += TS)
          for (int t0 = 0; t0 < Nt; t0 += TT) it[ax].push_back(BItem{g, s0, t0});
      }
      nitems[ax] = (int)it[ax].size();
      if (it[ax].size() > items_cap[ax]) {
        cudaFree(items[ax]);  // (synchronises the device; the lists only grow geometrically)
        items[ax] = nullptr;
        items_cap[ax] = std::max<size_t>(it[ax].size(), 2 * items_cap[ax]);
        CK(cudaMalloc(&items[ax], sizeof(BItem) * items_cap[ax]));
      }
      nctas[ax] = std::max(1, std::min(nitems[ax], occ_c[ax][var[ax]] * sms));
    }
    // cell-average strips of the 2D high-order grids: 30 columns x TY rows each
    nstrips = 0;
    if (dim == 2) {
      constexpr int TY = CellAvgTile<T, 4>::TY;
      static_assert(CellAvgTile<T, 4>::TY == CellAvgTile<T, 8>::TY, "one strip height per precision");
      std::vector<BStrip> sl;
      for (int g : order) {
        const astrea_grid& a = host_grids[g];
        if (a.scheme < PPM) continue;
        for (int i0 = 0; i0 < a.n0; i0 += TY)
          for (int j0 = 0; j0 < a.n1; j0 += CA_W) sl.push_back(BStrip{g, i0, j0 - 1});
      }
      nstrips = (int)sl.size();
      if (sl.size() > strips_cap) {
        cudaFree(strips);
        strips = nullptr;
        strips_cap = std::max<size_t>(sl.size(), 2 * strips_cap);
        CK(cudaMalloc(&strips, sizeof(BStrip) * strips_cap));
      }
      stage_lists(it, sl, st);
    } else {
      stage_lists(it, std::vector<BStrip>(), st);
    }
    dirty = false;
    return ASTREA_OK;
  }

  // upload the work lists on ``st`` through a pinned staging buffer (no device synchronisation)
  int stage_lists(const std::vector<BItem>* it, const std::vector<BStrip>& sl, cudaStream_t st) {
    const size_t b0 = sizeof(BItem) * it[0].size(), b1 = sizeof(BItem) * it[1].size(), b2 = sizeof(BStrip) * sl.size();
    const size_t need = b0 + b1 + b2;
    if (need == 0) return ASTREA_OK;
    const int k = stage_i;
    stage_i ^= 1;
    if (!stage_ev[k]) CK(cudaEventCreateWithFlags(&stage_ev[k], cudaEventDisableTiming));
    else CK(cudaEventSynchronize(stage_ev[k]));  // the copies that last read this buffer have run
    if (need > stage_cap[k]) {
      cudaFreeHost(stage_h[k]);
      stage_h[k] = nullptr;
      stage_cap[k] = std::max(need, 2 * stage_cap[k]);
      CK(cudaMallocHost(reinterpret_cast<void**>(&stage_h[k]), stage_cap[k]));
    }
    char* h = stage_h[k];
    if (b0) std::memcpy(h, it[0].data(), b0);
    if (b1) std::memcpy(h + b0, it[1].data(), b1);
    if (b2) std::memcpy(h + b0 + b1, sl.data(), b2);
    if (b0) CK(cudaMemcpyAsync(items[0], h, b0, cudaMemcpyHostToDevice, st));
    if (b1) CK(cudaMemcpyAsync(items[1], h + b0, b1, cudaMemcpyHostToDevice, st));
    if (b2) CK(cudaMemcpyAsync(strips, h + b0 + b1, b2, cudaMemcpyHostToDevice, st));
    CK(cudaEventRecord(stage_ev[k], st));
    return ASTREA_OK;
  }

  // the cell averages of this stage's input for every 2D high-order grid
  int launch_cell_average(const BatchArgs<T>& b, cudaStream_t st) {
    if (!cavg || nstrips == 0) return ASTREA_OK;
    CK(cavg(b, strips, nstrips, st));
    return ASTREA_OK;
  }

  BatchArgs<T> args(T* u) const {
    BatchArgs<T> b{};
    b.grids = d_grids;
    b.clocks = clocks;
    b.u = u;
    b.k0 = k0;
    b.k1 = k1;
    b.d0 = d0;
    b.d1 = d1;
    b.ws0 = ws0;
    b.ws1 = ws1;
    b.integ = integrator;
    return b;
  }

  int launch_sweep(BatchArgs<T> b, int ax, int slot, cudaStream_t st) {
    if (nitems[ax] == 0) return ASTREA_OK;
    b.items = items[ax];
    b.nitems = nitems[ax];
    b.counter = counters + slot;
    CK(cudaMemsetAsync(counters + slot, 0, sizeof(int), st));
    CK(cand[ax][var[ax]](b, nctas[ax], st));
    return ASTREA_OK;
  }

  int enqueue_step(void* arena, cudaStream_t st) override {
    int frc = flush(st);  // (nothing is queued inside a graph capture: the caller flushed before it)
    if (frc) return frc;
    if (dirty) {
      int rc = rebuild(st);
      if (rc) return rc;
    }
    T* u = static_cast<T*>(arena);
    const int ns = stages_count(integrator);
    int slot = 0;
    BatchArgs<T> b = args(u);
    b.stage = 0;
    b.mode = 0;
    b.want_emax = 1;
    int prc = launch_cell_average(b, st);
    if (prc) return prc;
    for (int ax = 0; ax < dim; ++ax) {
      b.dout_sel = ax;
      int rc = launch_sweep(b, ax, slot++, st);
      if (rc) return rc;
    }
    dt_kernel<<<(max_slots + 127) / 128, 128, 0, st>>>(clocks, max_slots);
    CK(cudaGetLastError());
    if (nitems[0] > 0) {
      const int TS = tile_ts(dim, var[0]), TT = tile_tt(dim, var[0]);
      batched_combine0_kernel<T><<<nitems[0], 256, 0, st>>>(b, items[0], nv, dim == 2, ns == 1, TS, TT);
      CK(cudaGetLastError());
    }
    for (int s = 1; s < ns; ++s) {
      BatchArgs<T> c = args(u);
      c.stage = s;
      c.last_stage = s == ns - 1;
      if (dim == 2) {
        int rc = launch_cell_average(c, st);
        if (rc) return rc;
        c.mode = 0;
        c.dout_sel = 0;
        rc = launch_sweep(c, 0, slot++, st);
        if (rc) return rc;
        c.mode = 1;
        rc = launch_sweep(c, 1, slot++, st);
        if (rc) return rc;
      } else {
        c.mode = 2;
        int rc = launch_sweep(c, 0, slot++, st);
        if (rc) return rc;
      }
    }
    end_step_kernel<<<(max_slots + 127) / 128, 128, 0, st>>>(clocks, max_slots);
    CK(cudaGetLastError());
    return ASTREA_OK;
  }

  int initialise(int slot, const void* prim, void* arena, cudaStream_t st) override {
    const T* w = static_cast<const T*>(prim);
    T* q = static_cast<T*>(arena);
    const astrea_grid& a = host_grids[slot];
    const long long base = offsets[slot], cells = (long long)a.n0 * (dim == 2 ? a.n1 : 1);
    const int n1 = dim == 1 ? 1 : a.n1;
    const int ho = a.scheme >= PPM;
    const int threads = 256;
    const int blocks = (int)std::min<long long>((cells + threads - 1) / threads, 152LL * 8);
    const T gm1 = T(a.gamma - 1.0);
    if (model == 3) init_pass_a<T, 3><<<blocks, threads, 0, st>>>(w + base, tmp + base, a.n0, n1, cells, dim, a.boundary, ho, gm1);
    else if (model == 4) init_pass_a<T, 4><<<blocks, threads, 0, st>>>(w + base, tmp + base, a.n0, n1, cells, dim, a.boundary, ho, gm1);
    else init_pass_a<T, 8><<<blocks, threads, 0, st>>>(w + base, tmp + base, a.n0, n1, cells, dim, a.boundary, ho, gm1);
    CK(cudaGetLastError());
    centre_to_avg_kernel<T><<<blocks, threads, 0, st>>>(tmp + base, q + base, a.n0, n1, cells, nv, dim, a.boundary);
    CK(cudaGetLastError());
    return ASTREA_OK;
  }
};

static int check_grid(int dim, const astrea_grid& a) {
  if (a.n0 < 4 || (dim == 2 && a.n1 < 4) || (dim == 1 && a.n1 != 1) || !(a.dx > 0) || !(a.cfl > 0) || !(a.gamma > 1) ||
      a.checkpoints < 1 || (a.flags & ASTREA_FLAG_CT))
    return fail(ASTREA_ERR_CONFIG, "invalid grid (sizes >= 4, n1 == 1 in 1D, dx, cfl > 0, gamma > 1; no constrained transport)");
  return ASTREA_OK;
}

extern "C" {

int astrea_batch_create(int dim, int model, int precision, int integrator, int max_slots, long long capacity_elems,
                        astrea_batch** out) {
  if (!out || max_slots <= 0 || capacity_elems <= 0) return fail(ASTREA_ERR_ARG, "bad batch arguments");
  *out = nullptr;
  if (dim != 1 && dim != 2) return fail(ASTREA_ERR_CONFIG, "dim must be 1 or 2");
  if (!((dim == 1 && (model == 3 || model == 8)) || (dim == 2 && (model == 4 || model == 8))))
    return fail(ASTREA_ERR_CONFIG, "batch model must be 3|8 in 1D, 4|8 in 2D");
  if (precision != 32 && precision != 64) return fail(ASTREA_ERR_CONFIG, "precision must be 32 or 64");
  if (stages_count(integrator) < 0) return fail(ASTREA_ERR_CONFIG, "integrator not supported");
  IBatch* b = precision == 64 ? static_cast<IBatch*>(new Batch<double>()) : static_cast<IBatch*>(new Batch<float>());
  b->dim = dim;
  b->model = model;
  b->precision = precision;
  b->integrator = integrator;
  b->max_slots = max_slots;
  b->nv = model;
  b->capacity = capacity_elems;
  b->host_grids.assign(max_slots, astrea_grid{});
  b->offsets.assign(max_slots, 0);
  b->active.assign(max_slots, 0);
  std::vector<Clock> clk(max_slots);
  std::memset(clk.data(), 0, sizeof(Clock) * max_slots);
  for (auto& c : clk) c.done = 1;  // empty slots are skipped by every kernel
  if (cudaMalloc(&b->clocks, sizeof(Clock) * max_slots) != cudaSuccess) {
    delete b;
    return fail(ASTREA_ERR_OOM, "batch clock allocation failed");
  }
  cudaMemcpy(b->clocks, clk.data(), sizeof(Clock) * max_slots, cudaMemcpyHostToDevice);
  int rc = b->alloc();
  if (rc) {
    delete b;
    return rc;
  }
  *out = new astrea_batch{b};
  return ASTREA_OK;
}

void astrea_batch_destroy(astrea_batch* h) {
  if (!h) return;
  delete h->b;
  delete h;
}

int astrea_batch_set(astrea_batch* h, int slot, const astrea_grid* grid, long long offset) {
  if (!h || !grid) return fail(ASTREA_ERR_ARG, "NULL argument");
  IBatch* b = h->b;
  if (slot < 0 || slot >= b->max_slots) return fail(ASTREA_ERR_ARG, "slot out of range");
  int rc = check_grid(b->dim, *grid);
  if (rc) return rc;
  const long long need = (long long)b->nv * grid->n0 * (b->dim == 2 ? grid->n1 : 1);
  if (offset < 0 || offset + need > b->capacity) return fail(ASTREA_ERR_OOM, "grid does not fit in the batch arena");
  Clock c;
  std::memset(&c, 0, sizeof(c));
  c.t_end = grid->t_end;
  c.chkpt = grid->t_end / grid->checkpoints;
  c.cfl = grid->cfl;
  c.dx = grid->dx;
  c.idx = 1;
  c.naxes = b->dim;
  c.done = !(0.0 < grid->t_end);
  rc = b->set_slot(slot, *grid, offset, c);  // applied on the device by the next step (or clock read)
  if (rc) return rc;
  b->host_grids[slot] = *grid;
  b->offsets[slot] = offset;
  b->active[slot] = 1;
  b->dirty = true;
  return ASTREA_OK;
}

int astrea_batch_clear(astrea_batch* h, int slot) {
  if (!h) return fail(ASTREA_ERR_ARG, "NULL argument");
  IBatch* b = h->b;
  if (slot < 0 || slot >= b->max_slots) return fail(ASTREA_ERR_ARG, "slot out of range");
  b->clear_slot(slot);  // applied on the device by the next step (or clock read)
  b->active[slot] = 0;
  b->dirty = true;
  return ASTREA_OK;
}

int astrea_batch_initialise(astrea_batch* h, int slot, const void* prim_arena, void* arena, void* stream) {
  if (!h || !prim_arena || !arena) return fail(ASTREA_ERR_ARG, "NULL argument");
  if (slot < 0 || slot >= h->b->max_slots || !h->b->active[slot]) return fail(ASTREA_ERR_ARG, "slot not occupied");
  return h->b->initialise(slot, prim_arena, arena, static_cast<cudaStream_t>(stream));
}

int astrea_batch_tile(const astrea_batch* h, int axis, int* ts, int* tt) {
  if (!h || !ts || !tt || axis < 0 || axis > 1) return fail(ASTREA_ERR_ARG, "bad argument");
  *ts = tile_ts(h->b->dim, h->b->var[axis]);
  *tt = tile_tt(h->b->dim, h->b->var[axis]);
  return ASTREA_OK;
}

int astrea_batch_step(astrea_batch* h, void* arena, int nsteps, void* stream) {
  if (!h || !arena) return fail(ASTREA_ERR_ARG, "NULL argument");
  int frc = h->b->flush(static_cast<cudaStream_t>(stream));
  if (frc) return frc;
  int trc = h->b->tune(arena, static_cast<cudaStream_t>(stream));
  if (trc) return trc;
  for (int i = 0; i < nsteps; ++i) {
    int rc = h->b->enqueue_step(arena, static_cast<cudaStream_t>(stream));
    if (rc) return rc;
  }
  return ASTREA_OK;
}

int astrea_batch_graph_step(astrea_batch* h, void* arena, int nsteps, void* stream) {
  if (!h || !arena) return fail(ASTREA_ERR_ARG, "NULL argument");
  IBatch* b = h->b;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int frc = b->flush(st);  // before any capture: the captured step has nothing queued
  if (frc) return frc;
  int trc = b->tune(arena, st);
  if (trc) return trc;
  if (b->dirty || !b->graph || b->graph_arena != arena) {
    if (b->graph) {
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    if (b->dirty) {
      int rc = b->rebuild(st);
      if (rc) return rc;
    }
    cudaStream_t cap;
    CK(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(cap, cudaStreamCaptureModeRelaxed));
    int rc = b->enqueue_step(arena, cap);
    cudaError_t ce = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (rc) return rc;
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaStreamEndCapture");
    ce = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) return cuda_fail(ce, "cudaGraphInstantiate");
    b->graph_arena = arena;
  }
  for (int i = 0; i < nsteps; ++i) CK(cudaGraphLaunch(b->graph, st));
  return ASTREA_OK;
}

int astrea_batch_clocks(astrea_batch* h, double* t, double* dt, int* steps, int* done, int* status, void* stream) {
  if (!h) return fail(ASTREA_ERR_ARG, "batch is NULL");
  IBatch* b = h->b;
  std::vector<Clock> c(b->max_slots);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int frc = b->flush(st);  // queued slot changes first
  if (frc) return frc;
  CK(cudaMemcpyAsync(c.data(), b->clocks, sizeof(Clock) * b->max_slots, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  for (int g = 0; g < b->max_slots; ++g) {
    if (t) t[g] = c[g].t;
    if (dt) dt[g] = c[g].dt;
    if (steps) steps[g] = c[g].steps;
    if (done) done[g] = c[g].done;
    if (status) status[g] = c[g].status;
  }
  return ASTREA_OK;
}

}  // extern "C"

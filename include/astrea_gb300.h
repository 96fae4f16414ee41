/*
 * astrea_gb300.h -- C ABI of the GB300 (sm_103a) implementation of astrea's
 * per-step finite-volume update.
 *
 * The reference (mervyzr/astrea) is pure Python: its "plugin API" for this
 * path is a pair of functions selected by strings in the ``sim_variables``
 * namedtuple,
 *     num_methods/evolvers.py:12  evolve_space(grid, sim_variables) -> fluxes
 *     num_methods/evolvers.py:38  evolve_time(grid, fluxes, dt, sim_variables) -> grid
 * driven by the step loop astrea.py:31-85 (core_run).  This library is what a
 * foreign-function binding of that path binds: plain pointers and sizes, no
 * Python or torch types.  The Python module ``astrea_gb300.evolvers`` keeps the
 * reference signatures on top of it (ctypes).
 *
 * Memory: every ``state`` argument is a caller-owned *device* buffer holding
 * the cell-averaged conservative variables as ``nv`` component planes
 * (structure of arrays), each plane ``n0*n1`` elements with axis 1 contiguous
 * -- i.e. the reference's (n0, n1, 8) array with the variable axis moved first
 * and the identically-zero variables of the chosen model left out.  Element
 * type is double (precision 64) or float (precision 32).  ``stream`` is a
 * cudaStream_t (NULL = legacy default stream).
 *
 * Errors: every int-returning function returns ASTREA_OK (0) or a negative
 * ASTREA_ERR_* code; nothing throws across the ABI; astrea_last_error() gives
 * a message for the calling thread.  One handle per host thread.
 */
#ifndef ASTREA_GB300_H
#define ASTREA_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define ASTREA_OK 0
#define ASTREA_ERR_CONFIG (-1)    /* unsupported or inconsistent configuration */
#define ASTREA_ERR_CUDA (-2)      /* a CUDA call failed */
#define ASTREA_ERR_OOM (-3)       /* device allocation failed / over budget */
#define ASTREA_ERR_NONFINITE (-4) /* a non-finite wave speed or dt was produced */
#define ASTREA_ERR_TIMEOUT (-5)   /* a bounded device wait gave up */
#define ASTREA_ERR_ARG (-6)       /* bad pointer or size */

/* enums: the reference's strings are mapped onto these by the caller
 * (see astrea_gb300/config.py, mirroring functions/generic.py:159-286) */
enum astrea_scheme { ASTREA_PCM = 0, ASTREA_PLM = 1, ASTREA_PPM = 2, ASTREA_WENO3 = 3, ASTREA_WENO5 = 4, ASTREA_WENO7 = 5 };
/* ASTREA_LW: Lax-Wendroff (num_methods/solvers.py:79-88), the LLF form with the
 * interface coefficient v_n^2 / max|lambda|.  The reference takes its 'sound
 * speed' as the second unique column of the LAPACK eigenvalue array, which is
 * the entropy-wave eigenvalue v_n where LAPACK lists it there (e.g. every
 * interface of a 1D hydro Sod problem) and another eigenvalue elsewhere; this
 * library always uses v_n. */
enum astrea_solver { ASTREA_LLF = 0, ASTREA_HLLC = 1, ASTREA_HLLD = 2, ASTREA_LW = 3 };
enum astrea_integrator { ASTREA_EULER = 0, ASTREA_SSPRK22 = 1, ASTREA_SSPRK33 = 2, ASTREA_SSPRK43 = 3,
                         ASTREA_SSPRK53 = 4, ASTREA_SSPRK54 = 5, ASTREA_SSPRK104 = 6, ASTREA_RK4 = 7 };
enum astrea_boundary { ASTREA_EDGE = 0, ASTREA_WRAP = 1 };
enum astrea_limiter { ASTREA_MINMOD = 0, ASTREA_SUPERBEE = 1 };
/* stored variables: 3 = 1D Euler (rho, m_x, E); 4 = 2D Euler (rho, m_x, m_y, E);
 * 8 = ideal MHD (rho, m_x, m_y, m_z, E, B_x, B_y, B_z) */

typedef struct astrea_cfg {
  int dim;          /* 1 or 2 (sim_variables.dimension) */
  int n0, n1;       /* cells along axis 0 and axis 1 (n1 = 1 in 1D) */
  int model;        /* 3, 4 or 8 */
  int precision;    /* 64 (plain FP64) or 32 (FP32 with FP64 pressure recovery) */
  int scheme;       /* enum astrea_scheme (sim_variables.subgrid) */
  int solver;       /* enum astrea_solver (sim_variables.solver) */
  int integrator;   /* enum astrea_integrator (sim_variables.timestep) */
  int boundary;     /* enum astrea_boundary (sim_variables.boundary) */
  int limiter;      /* PLM slope limiter, enum astrea_limiter */
  double gamma;     /* sim_variables.gamma */
  double dx;        /* sim_variables.dx */
  double cfl;       /* sim_variables.cfl */
  double t_end;     /* sim_variables.t_end */
  int checkpoints;  /* sim_variables.checkpoints */
  int flags;        /* ASTREA_FLAG_* */
} astrea_cfg;

/* flags: ASTREA_FLAG_PHYSICAL selects textbook HLLC/HLLD in place of the
 * reference's (whose 2D sweeps pick the normal velocity by iteration position,
 * write the star normal momentum to component 1 and take f_plus when sL > 0,
 * num_methods/solvers.py:34-36,104-137).  Not a reference option. */
#define ASTREA_FLAG_PHYSICAL 1
/* ASTREA_FLAG_CT: 2D MHD with the reference's fourth-order upwind constrained
 * transport (sim_variables.magnetic_2d; num_methods/mag_field.py).  Requires
 * dim 2 and model 8. */
#define ASTREA_FLAG_CT 2
/* ASTREA_FLAG_FLATTEN / ASTREA_FLAG_VISCOSITY (PPM only; other schemes ignore
 * them): Colella (1990) flattening of the face values and McCorquodale &
 * Colella (2011) artificial viscosity (alpha = beta = 0.3) added to the
 * fluxes, after schemes/ppm.py:111-170 (apply_flattener,
 * apply_artificial_viscosity).  The reference never runs that code (it fails
 * when called).  These follow its formulas with two corrections from the
 * papers it cites: flattening acts only on strong, compressive pressure jumps
 * (Colella & Woodward 1984, A.1), and the viscosity coefficient uses the face
 * velocity difference without a second factor dx.  Flattening is not
 * available with constrained transport. */
#define ASTREA_FLAG_FLATTEN 4
#define ASTREA_FLAG_VISCOSITY 8

typedef struct astrea_handle astrea_handle;

/* Library version (major*10000 + minor*100 + patch). */
int astrea_version(void);
/* Message of the last error on this thread ("" if none). */
const char* astrea_last_error(void);

/* Create a solver for one grid (allocates its stage buffers on the current
 * device).  Replaces building ``sim_variables`` (functions/generic.py:159-286,
 * astrea.py:132-133). */
int astrea_create(const astrea_cfg* cfg, astrea_handle** out);
void astrea_destroy(astrea_handle* h);
/* Number of stored variables (planes) and cells per plane. */
int astrea_layout(const astrea_handle* h, int* nv, long long* cells);

/* Point primitives -> cell-averaged conservatives, like
 * constructor.initialise (functions/constructor.py:105-109).  ``prim`` and
 * ``state_out`` use the state layout (primitive variables in ``prim``). */
int astrea_initialise(astrea_handle* h, const void* prim, void* state_out, void* stream);

/* Reset the device clock (t, next checkpoint index, axis order 0|1). */
int astrea_reset_clock(astrea_handle* h, double t, int idx, int order, void* stream);

/* Advance ``nsteps`` steps of the core_run loop body (astrea.py:66-85): the
 * space operator, dt = cfl*min(dx/eigmax) clipped to the checkpoint, the time
 * integrator, the axis-order flip.  dt and t stay on the device; once t
 * reaches t_end further steps do nothing.  Asynchronous on ``stream``. */
int astrea_step(astrea_handle* h, void* state, int nsteps, void* stream);

/* Same as astrea_step, replaying one captured CUDA graph per step. */
int astrea_graph_step(astrea_handle* h, void* state, int nsteps, void* stream);

/* Same as astrea_step, with a CUDA event pair recorded on ``stream`` around
 * every kernel launch.  kernel_ms[k] / launches[k] (4 entries each) receive
 * the summed device time and the launch count per kernel kind k: 0 sweep,
 * 1 stage combine (stage 0; the register integrators' stage kernel; the
 * constrained-transport kernels), 2 dt and step bookkeeping, 3 the
 * cell-average pre-pass of 2D high-order schemes.  Synchronises ``stream``.
 * (Instrumentation for measurement; no counterpart in the reference.) */
int astrea_step_timed(astrea_handle* h, void* state, int nsteps, double* kernel_ms, int* launches, void* stream);

/* The sweep tile in use along ``axis`` (cells along the sweep x rows across it).
 * 2D grids pick theirs among the built candidates by timing them on the grid
 * at the first step (the environment variable ASTREA_SWEEP_TILE=<index> forces
 * one).  No counterpart in the reference. */
int astrea_sweep_tile(const astrea_handle* h, int axis, int* ts, int* tt);

/* Enqueue on ``stream`` copies of the device clock's time, completed step
 * count and done flag into caller memory (page-locked memory keeps them
 * asynchronous), so that a snapshot can be labelled with its t without
 * waiting for the stream; the values are valid once the stream has passed
 * this point.  No counterpart in the reference (its t is a host variable,
 * astrea.py:44-84). */
int astrea_clock_async(astrea_handle* h, double* t, int* steps, int* done, void* stream);

/* One step of the core_run loop (astrea.py:66-85) for a caller that keeps the
 * grid in host memory between steps: ``host_in`` (nv planes of n0*n1
 * elements, may be NULL) is copied into the device ``state`` first, the step
 * runs with the device dt, and the stepped state is written to ``host_out``
 * (may be NULL; may equal host_in).  Where host_out is page-locked memory the
 * device can address (cudaHostAlloc / torch pin_memory) and the integrator's
 * last stage ends in a combining sweep (SSP-RK (2,2), (3,3), (4,3) without
 * constrained transport), that sweep stores the result to host_out while it
 * computes, so no separate device-to-host copy follows the step; otherwise
 * the state is copied after the step.  The sequence is captured once per
 * (state, host_in, host_out) and replayed; asynchronous on ``stream``.  No
 * counterpart in the reference (its grid always lives in host memory). */
int astrea_step_host(astrea_handle* h, void* state, const void* host_in, void* host_out, void* stream);

/* Read the device clock (synchronises ``stream``).  status bit 0: a
 * non-finite wave speed or dt was seen. */
int astrea_get_clock(astrea_handle* h, double* t, double* dt, int* steps, int* done, int* status, void* stream);

/* evolve_space (num_methods/evolvers.py:12-34): interface fluxes of every
 * axis and the per-axis maximum wave speed.  ``order`` = 0 sweeps axis 0
 * first (even step), 1 sweeps axis 1 first (odd step).  flux_ax0 receives
 * (n0+1)*n1 elements per plane, flux_ax1 (n1+1)*n0 elements per plane (sweep
 * index major, as the reference's transposed arrays); either may be NULL.
 * eigmax (host, 2 doubles) receives eigmax of axis 0 and axis 1.
 * Synchronises ``stream``. */
int astrea_space(astrea_handle* h, const void* state, int order, void* flux_ax0, void* flux_ax1, double* eigmax,
                 void* stream);

/* evolve_space for 2D MHD with constrained transport (ASTREA_FLAG_CT;
 * num_methods/evolvers.py:12-34 with its magnetic block :26-32): everything
 * astrea_space returns, plus what the reference adds to ``fluxes`` for the
 * magnetic update.  face_ax0 / face_ax1 receive each sweep's face values
 * (``data[axes]['wF']``: the value at the face i+1/2 along that sweep of
 * every cell, 8 primitive planes of n0*n1 elements in the physical layout);
 * corner receives the corner electric field E_z of mag_field.compute_corner
 * (mag_field.py:125-187), one n0*n1 plane in the physical layout, whose
 * transposes the reference stores as ``fluxes[axes]['mag_corner']``.  Any
 * output may be NULL (a NULL face output leaves that sweep's face values in
 * the handle's own buffer, from which the corner is still formed).
 * Synchronises ``stream``. */
int astrea_space_ct(astrea_handle* h, const void* state, int order, void* flux_ax0, void* flux_ax1, double* eigmax,
                    void* face_ax0, void* face_ax1, void* corner, void* stream);

/* evolve_time (num_methods/evolvers.py:38-206) with a caller-given dt: the
 * full Runge-Kutta step, in place on ``state``.  The stage-0 fluxes are
 * recomputed on the device from ``state`` (they are a pure function of it). */
int astrea_time(astrea_handle* h, void* state, double dt, int order, void* stream);

/* Conservative -> primitive of the whole grid (sim_variables.convert_conservative),
 * e.g. for the per-step snapshot of astrea.py:47. */
int astrea_to_primitive(astrea_handle* h, const void* state, void* prim_out, void* stream);

/* Compensated (Neumaier, FP64) sums of every stored variable over the grid:
 * total mass, momentum, energy (functions/analytic.py:66-79 sums them on
 * the host).  sums_host receives nv doubles.  Synchronises ``stream``. */
int astrea_reduce_conserved(astrea_handle* h, const void* state, double* sums_host, void* stream);

/* The same sums without a handle and without allocating anything.  This entry
 * point has no counterpart in the reference (which sums with NumPy on the
 * host).  It is for callers that hold only a state pointer and must not
 * allocate device memory at that moment: a grid inside a batched arena in a
 * process whose HBM is fully budgeted to its arenas, or a monitor reporting
 * totals while the device is out of memory.  A handle would allocate the full
 * set of stage buffers of the grid just to sum it.
 *
 * state: nv planes of ``cells`` elements each (float if precision == 32, double
 * if 64), on the current device.  The partial sums live in a fixed device array
 * of 2440 doubles (19,520 bytes) per device: 152 blocks x up to 8 variables x
 * (sum, compensation), plus the 8 folded sums.  nv above 8 (or below 1) is
 * rejected with ASTREA_ERR_ARG.  Nothing in that array needs to start at zero:
 * every partial is written before it is read.  The results equal
 * astrea_reduce_conserved's on the same state (same blocks, same order).
 *
 * The first call on each device, made with that device current, looks up the
 * array's address (cudaGetSymbolAddress); make that first call before any
 * stream capture begins.  CUDA loads a library's kernels and device arrays
 * into a context lazily, so that first call is also when the array (and the
 * two kernels) take their place on the device: make it before the device's
 * memory is exhausted, e.g. at start-up.  The looked-up address is kept for
 * the life of the process; after cudaDeviceReset (or anything else that
 * replaces the device's primary context) it is stale, and this entry point
 * must not be called again in that process.  There is one array per device, so calls that overlap
 * on the same device (from other threads or on other streams) race on it and
 * give wrong sums: serialise them.  Synchronises ``stream``. */
int astrea_reduce_conserved_static(const void* state, int precision, long long cells, int nv, double* sums_host,
                                   void* stream);

/* ------------------------------------------------------------------------
 * Initial conditions on the device (functions/constructor.py:11-103).
 * Point primitives of a test problem, evaluated per cell from the values the
 * reference's test table puts into ``sim_variables`` (initial_left/right,
 * start/end/shock positions, misc parameters), so that nothing grid-sized is
 * uploaded.  ``kind`` follows constructor.initialise's dispatch on the config
 * name; astrea_gb300/initial.py maps names and ``sim_variables`` onto this. */
enum astrea_ic_kind {
  ASTREA_IC_SPLIT = 0,     /* one jump: 2D x < shock, 1D x <= shock (1D |x| <= shock with abs_mask) */
  ASTREA_IC_RADIAL = 1,    /* 2D sedov / blast / rotor: disc of radius shock - centre */
  ASTREA_IC_GAUSS = 2,     /* gaussian density bump (1D or 2D) */
  ASTREA_IC_KHI = 3,       /* 2D Kelvin-Helmholtz: jump across y, sine v_y perturbation */
  ASTREA_IC_VORTEX = 4,    /* 2D isentropic vortex */
  ASTREA_IC_QUADRANT = 5,  /* 2D Lax-Liu four quadrants */
  ASTREA_IC_OT = 6,        /* 2D Orszag-Tang */
  ASTREA_IC_SHU = 7,       /* 1D Shu-Osher: sine density right of the jump */
  ASTREA_IC_SINE = 8,      /* 1D sine density */
  ASTREA_IC_LINEAR = 9,    /* 1D linear sound wave */
  ASTREA_IC_LINEAR_MHD = 10 /* 1D linear Alfven wave */
};
typedef struct astrea_ic {
  int kind, abs_mask;
  int dim, n;              /* n cells per axis */
  double start, end, shock;
  double left[8], right[8], bottom_left[8], bottom_right[8];
  double ampl, freq, y_offset, fwhm, peak_pos, perturb_ampl, vortex_str, omega;
  double gamma;
} astrea_ic;
/* Write the point primitives of ``ic`` into ``prim_out`` (device, the model's
 * planes, float or double by ``precision``); astrea_initialise then forms the
 * cell averages.  Asynchronous on ``stream``. */
int astrea_point_state(const astrea_ic* ic, int precision, int model, void* prim_out, void* stream);

/* ------------------------------------------------------------------------
 * Diagnostics of a primitive snapshot (functions/analytic.py).  ``prim`` (and
 * ``ref``) hold the model's primitive planes on the device (n1 = 1 in 1D).
 * Ten quantities per result: the eight primitives (rho, v_x, v_y, v_z, P, B_x,
 * B_y, B_z; absent ones are zero), the specific total energy E_tot = e_tot/rho
 * and the specific internal energy E_int = P/(rho (gamma - 1)).  Sums are FP64
 * and compensated; the partials live in a fixed device array (no allocation),
 * so calls on one device must not overlap.  Both synchronise ``stream``. */
/* calculate_TV (analytic.py:48-63): sum of |differences| after differencing
 * along axis 0 and then axis 1 (in 2D the mixed difference). */
int astrea_total_variation(const void* prim, int precision, int model, int dim, int n0, int n1, double gamma,
                           double* tv_host, void* stream);
/* calculate_solution_error (analytic.py:24-45) against ``ref`` (e.g. the initial
 * state of a periodic test after whole periods): norm <= 0 gives the L1 norm,
 * norm > 10 the maximum, otherwise the L_norm norm, each normalised by n0^dim. */
int astrea_solution_error(const void* prim, const void* ref, int precision, int model, int dim, int n0, int n1,
                          double gamma, double norm, double* err_host, void* stream);

/* ------------------------------------------------------------------------
 * Batched engine: many independent grids of uneven sizes in one state arena.
 * The reference runs one grid per process (astrea.py:155-190 loops over
 * resolutions one after another); a batch advances every occupied slot per
 * call, each grid with its own dt/t/t_end, with one persistent kernel per
 * sweep whose CTAs pull tiles of all grids from a work list.  Slots can be
 * occupied and released between steps (continuous batching).  No
 * counterpart in the reference.
 * ------------------------------------------------------------------------ */
typedef struct astrea_grid {
  int n0, n1;          /* cells (n1 = 1 in 1D) */
  int scheme;          /* ASTREA_PLM, ASTREA_PPM or ASTREA_WENO5 */
  int solver;          /* ASTREA_LLF, or ASTREA_HLLC (Euler models) / ASTREA_HLLD (model 8) */
  int boundary, limiter, flags;
  double gamma, dx, cfl, t_end;
  int checkpoints;
} astrea_grid;

typedef struct astrea_batch astrea_batch;

/* A batch of up to max_slots grids sharing dim, model (3|8 in 1D, 4|8 in 2D),
 * precision and integrator, with stage buffers for capacity_elems elements
 * of state (the caller's arena has the same size); 2D batches also hold the
 * cell averages of their high-order grids (one arena in FP32, two in FP64). */
int astrea_batch_create(int dim, int model, int precision, int integrator, int max_slots, long long capacity_elems,
                        astrea_batch** out);
void astrea_batch_destroy(astrea_batch* b);
/* Occupy ``slot`` with a grid whose nv planes start at element ``offset`` of
 * the arena; resets the slot's clock to t = 0.  ASTREA_ERR_OOM if it does not fit.
 * Does not touch the device: the slot's descriptor and clock are written by the
 * next astrea_batch_step / astrea_batch_graph_step / astrea_batch_clocks, on
 * that call's stream. */
int astrea_batch_set(astrea_batch* b, int slot, const astrea_grid* grid, long long offset);
/* Release ``slot`` (its grid is no longer advanced; applied like astrea_batch_set). */
int astrea_batch_clear(astrea_batch* b, int slot);
/* The tile in use along ``axis`` (cells along the sweep x rows across it).  A
 * batch picks it among the built candidates by timing them on its work list at
 * its first step (ASTREA_BATCH_TILE=<index> forces one).  No counterpart in the
 * reference. */
int astrea_batch_tile(const astrea_batch* h, int axis, int* ts, int* tt);

/* Point primitives -> cell-averaged conservatives for one slot; ``prim_arena``
 * holds the primitives at the slot's offset. */
int astrea_batch_initialise(astrea_batch* b, int slot, const void* prim_arena, void* arena, void* stream);
int astrea_batch_step(astrea_batch* b, void* arena, int nsteps, void* stream);
/* As astrea_batch_step with one CUDA graph per step (recaptured after set/clear). */
int astrea_batch_graph_step(astrea_batch* b, void* arena, int nsteps, void* stream);
/* Per-slot clocks (arrays of max_slots; any may be NULL); synchronises ``stream``. */
int astrea_batch_clocks(astrea_batch* b, double* t, double* dt, int* steps, int* done, int* status, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* ASTREA_GB300_H */

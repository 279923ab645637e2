/*
 * tfv.h — C ABI of the GB300 structured-grid finite-volume library
 * (libtfv.so, built from torch_gb300/csrc).
 *
 * The library advances Cartesian 1D/2D/3D Euler / reactive Euler grids with
 * TORCH's MUSCL-Hancock + HLLC scheme on one GPU.  It replaces the CPU flux
 * workers behind TORCH's session step:
 *   python/cfdSolver/torchSession.py:374-522      Simulation.step
 *   python/cfdSolver/torchExecution.py:17-68      Execution.map (CPU workers)
 *   python/cfdSolver/torchFlux.py:6-77,125-248    hllc_flux_grid / hllc_flux
 *   python/cfdSolver/torchSolver2D.py:274-466     muscl_hancock_step_2d
 *   python/cfdSolver/torchSolver3D.py:122-203     _hydro
 *
 * Conventions
 *  - Every array pointer is a DEVICE pointer owned by the caller (PyTorch
 *    tensors in the Python host layer).  The library never allocates or frees
 *    device memory; the caller provides a workspace of the size the library
 *    asks for.
 *  - States are (dim+2, nz, ny, nx), x fastest, components
 *    rho, rho*u, [rho*v], [rho*w], E — the reference layout
 *    (python/cfdSolver/torchSession.py:146-150, torchIO.py:5-10).
 *  - Status codes: TFV_OK, TFV_EINVAL (the reference raises ValueError),
 *    TFV_ENUMERIC (RuntimeError: stall / nonphysical / max steps / no stable
 *    reactive step; the session state is unchanged), TFV_ECUDA.
 *  - A batch handle is single-owner and not thread-safe.  Work is enqueued on
 *    the stream given at bind time; only the report calls synchronise.
 */
#ifndef TFV_H
#define TFV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  TFV_OK = 0,
  TFV_EINVAL = 1,
  TFV_ENUMERIC = 2,
  TFV_ECUDA = 3
};

enum { TFV_FP64 = 0, TFV_FP32 = 1 };

/* boundary kinds (python/cfdSolver/torchSession.py:237-241) */
enum { TFV_BC_OPEN = 0, TFV_BC_REFLECTIVE = 1, TFV_BC_PERIODIC = 2, TFV_BC_INFLOW = 3 };

/* limiters (python/cfdSolver/torchSolver3D.py:24) */
enum { TFV_VANLEER = 0, TFV_ALBADA = 1, TFV_MINBEE = 2, TFV_SUPERBEE = 3, TFV_UNOS = 4 };

enum { TFV_ARRHENIUS = 0, TFV_ZND = 1 };
/* chemistry closure: TORCH's SI H2/O2 closure (gamma(lambda), T = p M/(rho R))
 * or the nondimensional one (constant gamma, T = p/rho) */
enum { TFV_CLOSURE_SI = 0, TFV_CLOSURE_NONDIM = 1 };

/* 1D options (python/cfdSolver/torchSolver.py:1108-1118) */
enum { TFV_W_SOUND_SPEED = 0, TFV_W_ZERO = 1 };
enum { TFV_HLLC_VARIANT1 = 0, TFV_HLLC_VARIANT2 = 1 };
enum { TFV_WAVES_PRESSURE = 0, TFV_WAVES_ENTHALPY = 1 };

/* instance status (tfv_report.status) */
enum {
  TFV_READY = 0,          /* next step can run */
  TFV_DONE = 1,           /* time == t_end: further steps are no-ops */
  TFV_ERR_MAXSTEPS = 2,   /* steps >= max_steps before t_end */
  TFV_ERR_STALL = 3,      /* dt not finite, <= 0, or time + dt == time */
  TFV_ERR_NONPHYSICAL = 4,/* nonphysical even after the first-order fallback */
  TFV_ERR_REACTIVE = 5,   /* no CFL-stable reactive step in 60 halvings */
  TFV_ERR_SPECIES = 6,    /* 3D species transport left [-1e-10, 1+1e-10] */
  TFV_ERR_CHEMISTRY = 7,  /* reaction input invalid (reference ValueError) */
  TFV_RETRY = 8           /* reactive dt must be halved (host completes the step) */
};

/* Mirrors Simulation.config for one Cartesian grid
 * (python/cfdSolver/torchSession.py:66-92). */
typedef struct tfv_config {
  int32_t dim;               /* 1, 2 or 3 */
  int32_t counts[3];         /* cells along x, y, z (unused axes = 1) */
  double lengths[3];         /* domain lengths along x, y, z */
  int32_t bc[3];             /* TFV_BC_* per axis x, y, z */
  int32_t limiter;           /* TFV_VANLEER ... */
  double gamma;              /* ratio of specific heats (non-reactive / nondim) */
  double cfl;
  double t_end;
  int64_t max_steps;
  int32_t reactive;          /* 0/1 */
  int32_t kinetic_model;     /* TFV_ARRHENIUS / TFV_ZND */
  int32_t closure;           /* TFV_CLOSURE_SI / TFV_CLOSURE_NONDIM */
  double q_heat;             /* heat release per unit mass and unit lambda */
  double activation;         /* SI: Ea [J/mol]; nondim: Ea/R */
  double pre_exponential;
  double inlet_primitive[4]; /* 2D y-Inflow: rho, u, v, p */
  int32_t controller;        /* 1D only */
  int32_t variant;           /* 1D only */
  int32_t wavespeed;         /* 1D only */
  double spacing[3];         /* cell sizes; 0 means lengths[k] / counts[k] */
} tfv_config;

/* Tile shape of the fused step kernel (chosen by the autotuner). */
typedef struct tfv_tile {
  int32_t tx;      /* cells along x per tile (threads along x) */
  int32_t ty;      /* cells along y per tile (3D only; 1 otherwise) */
  int32_t chunk;   /* planes marched per tile (z in 3D, y in 2D) */
  int32_t persistent_ctas; /* 0 = one CTA per tile, else grid size of a persistent launch */
  int32_t tma;     /* 1: stage planes with tensor copies (cp.async.bulk.tensor) where the
                      grid allows it (x extent a multiple of 16 bytes); 0: plain loads */
} tfv_tile;

/* Per-instance scalars read back after steps. */
typedef struct tfv_report {
  double time;
  double dt;                 /* dt of the next step (or of the last one if not READY) */
  double initial_integral[5];
  double boundary_integral[5];
  double source_integral[5];
  int64_t steps;
  int32_t status;            /* TFV_READY ... */
  int32_t current;           /* index of the current state buffer in the ring */
  int32_t fallback_steps;    /* steps that used the first-order fallback */
  int32_t last_fallback;     /* 1 if the last committed step used it */
} tfv_report;

typedef struct tfv_batch tfv_batch;

/* Library version string. */
const char* tfv_version(void);

/* Text of the last error on this thread (static storage). */
const char* tfv_last_error(void);

/* Create a batch of n instances of one dimension and precision.  Replaces
 * the construction-time validation of Simulation.__init__
 * (python/cfdSolver/torchSession.py:24-158, :190-254). */
int tfv_batch_create(int32_t dim, int32_t precision, int32_t n, const tfv_config* cfgs,
                     const tfv_tile* tile, tfv_batch** out);

/* Device workspace bytes needed by the batch (tile table, descriptors,
 * per-tile partials, scalars, 1D scratch). */
int tfv_batch_workspace_size(const tfv_batch* b, size_t* bytes);

/* Number of state buffers each instance needs in its ring (2, or 3 when
 * reactive). */
int tfv_batch_ring_size(const tfv_batch* b, int32_t* nring);

/* Bind device memory.  states[i*nring + k] is ring buffer k of instance i
 * (each (dim+2)*cells elements of the batch precision); lams / betas likewise
 * (cells elements each, NULL when unused).  Buffer 0 of each ring holds the
 * initial state.  Computes the initial integrals and the first dt
 * (python/cfdSolver/torchSession.py:153-157, :392-396). */
int tfv_batch_bind(tfv_batch* b, void* workspace, void* const* states, void* const* lams,
                   void* const* betas, void* stream);

/* Enqueue up to nsteps complete split steps for every READY instance
 * (python/cfdSolver/torchSession.py:374-522).  Instances that finish or fail
 * stop in place; the others continue.  Asynchronous. */
int tfv_batch_advance(tfv_batch* b, int32_t nsteps);

/* Capture `steps_per_graph` steps into a CUDA graph and use it for
 * subsequent tfv_batch_advance calls (0 disables graphs). */
int tfv_batch_use_graph(tfv_batch* b, int32_t steps_per_graph);

/* Synchronise and copy every instance's scalars into out[0..n).  Completes a
 * pending reactive dt halving (TFV_RETRY) on the host side before
 * returning (python/cfdSolver/torchSession.py:401-411). */
int tfv_batch_report(tfv_batch* b, tfv_report* out);

/* Recompute integrals of the current states into out[n*5] (FP64)
 * (python/cfdSolver/torchSession.py:285-295). */
int tfv_batch_integrals(tfv_batch* b, double* out);

/* Carry instances that already advanced into this (freshly bound) batch:
 * for each i whose report is not all-zero (steps > 0, time > 0 or a nonzero
 * initial mass integral), restore time, steps, integrals, fallback counters
 * and a terminal status, then re-plan dt from the current states; zero
 * reports leave their instance as bound.  The caller passes each instance's
 * current state as ring buffer 0 at bind.  Used to re-batch grids when
 * requests join or leave and to resume a checkpointed session with its exact
 * counters and balances (python/cfdSolver/torchIO.py:233-391 restores the
 * same attributes on the reference's session). */
int tfv_batch_restore(tfv_batch* b, const tfv_report* reports);

/* Re-plan after the caller wrote new values into the current buffers
 * (recomputes dt and status; keeps time, steps and integrals). */
int tfv_batch_replan(tfv_batch* b);

/* Optional per-instance face-flux outputs for the next steps (tests and the
 * reference's return_fluxes=True): flux_x (dim+2, nz, ny, nx+1), flux_y
 * (dim+2, nz, ny+1, nx), flux_z (dim+2, nz+1, ny, nx), device pointers of the
 * batch precision, NULL to disable (python/cfdSolver/torchSolver2D.py:466). */
int tfv_batch_set_flux_outputs(tfv_batch* b, int32_t inst, void* fx, void* fy, void* fz);

/* Run `nsteps` steps with CUDA events around each kernel on the bound stream
 * and return the summed milliseconds of the fused step kernel, of the
 * fallback kernel and of the finalize kernel (measurement support for the
 * roofline figures; results are the same as tfv_batch_advance). */
int tfv_batch_profile(tfv_batch* b, int32_t nsteps, float* ms_step, float* ms_fallback,
                      float* ms_finalize);

int tfv_batch_destroy(tfv_batch* b);

/* Stateless HLLC on n faces in the normal basis (rows rho, m_n, m_t...,
 * E; nv = 4 or 5), per-face gamma_l / gamma_r; fp64 or fp32
 * (python/cfdSolver/torchFlux.py:125-248). */
int tfv_hllc_flux(int32_t precision, int32_t nv, int64_t n, const void* ul, const void* ur,
                  const void* gl, const void* gr, void* out, void* stream);

/* One hydrodynamic step without session bookkeeping, for the reference's
 * step functions (python/cfdSolver/torchSolver2D.py:274-466,
 * torchSolver3D.py:122-203): state_in -> state_out with the given dt and
 * per-cell gamma (NULL: cfg->gamma).  Writes face fluxes when fx/fy/fz are
 * non-NULL and *used_fallback.  Synchronous; needs a workspace of
 * tfv_step_workspace_size bytes. */
int tfv_step_workspace_size(const tfv_config* cfg, int32_t precision, size_t* bytes);
int tfv_hydro_step(const tfv_config* cfg, int32_t precision, const void* state_in,
                   void* state_out, const void* gamma_cells, double dt, void* fx, void* fy,
                   void* fz, void* workspace, int32_t* used_fallback, void* stream);

/* tfv_hydro_step without a workspace and without any device allocation.
 * No counterpart in the reference (TORCH runs on the CPU and never touches
 * device memory).  It is for callers that cannot call cudaMalloc: a host
 * application that owns all GPU memory in a pool of its own and hands this
 * library only the state and flux arrays, or a time-critical loop where the
 * device-wide synchronisation an allocation implies is not acceptable.
 * The step's scratch (descriptors, tile table, per-tile partial sums, and
 * per-cell interface data of 1D tubes) lives in a 1 MiB array inside the
 * library's device image; every GPU that loads the library holds it until the
 * process exits.  Grids whose scratch would not fit are rejected with
 * TFV_EINVAL; tfv_step_workspace_size gives a grid's need (with the default
 * tiles a 3D 256^3 grid needs about 376 KiB in fp32 and 856 KiB in fp64, so
 * fp64 3D grids much larger than 256^3 are rejected; a 2D 4096^2 grid needs
 * 456 KiB in fp32 and 856 KiB in fp64; 1D tubes need about 49 B per cell in
 * fp32 and 97 B in fp64, so tubes beyond about 21,000 / 10,800 cells are
 * rejected).  The array's device
 * address is looked up (cudaGetSymbolAddress) on every call with the calling
 * thread's device current.  The call blocks until the step has finished (it
 * reads the step's status back to the host), so it cannot be used on a
 * capturing stream.  Every call reuses the same array: a call rewrites the
 * descriptors, tile table and scalars (the fallback flag starts at zero) and
 * every partial sum before reading them, but calls that overlap on the GPU
 * (other streams, other host threads) race on the array and must be
 * serialised by the caller. */
int tfv_hydro_step_static(const tfv_config* cfg, int32_t precision, const void* state_in,
                          void* state_out, const void* gamma_cells, double dt, void* fx,
                          void* fy, void* fz, int32_t* used_fallback, void* stream);

/* ---------------------------------------------------------------------------
 * Metric / face-boundary sessions: TORCH's second finite-volume scheme
 * (python/cfdSolver/torchFiniteVolume.py:1-276), used by the reference session
 * for cylindrical, annular and spherical grids and for any grid with per-face
 * boundaries (torchSession.py:303-308, 523-576): MUSCL reconstruction of
 * primitives, area-weighted Rusanov fluxes, geometric source terms, SSPRK2
 * with a first-order retry, up to 20 dt halvings, Strang-split chemistry.
 * ------------------------------------------------------------------------- */

/* geometries (python/cfdSolver/torchGeometry.py:9) */
enum { TFV_GEO_CARTESIAN = 0, TFV_GEO_CYLINDRICAL = 1, TFV_GEO_ANNULAR = 2, TFV_GEO_SPHERICAL = 3 };

/* face boundary kinds (python/cfdSolver/torchBoundaries.py:8-15) */
enum {
  TFV_FACE_OUTFLOW = 0,
  TFV_FACE_WALL = 1,
  TFV_FACE_PERIODIC = 2,
  TFV_FACE_INFLOW = 3,
  TFV_FACE_PRESSURE_OUTLET = 4,
  TFV_FACE_STAGNATION_INLET = 5
};

/* one face (torchBoundaries.py:18-171, normalised): faces are ordered
 * x_min, x_max, y_min, y_max, z_min, z_max */
typedef struct tfv_metric_face {
  int32_t type;              /* TFV_FACE_* */
  int32_t has_backflow;      /* pressure outlet: primitive[] holds the backflow state */
  double primitive[5];       /* inflow state, or the pressure outlet's backflow state */
  double lambda_, beta;      /* fractions carried in (default 1) */
  double pressure;           /* pressure outlet */
  double total_pressure, total_temperature, gas_constant;  /* stagnation inlet */
} tfv_metric_face;

typedef struct tfv_metric_config {
  int32_t dim;
  int32_t n[3];              /* cells along x, y, z */
  double lengths[3];
  int32_t geometry;          /* TFV_GEO_* */
  int32_t limiter;           /* TFV_VANLEER ... */
  int32_t reactive;
  int32_t model;             /* TFV_ARRHENIUS / TFV_ZND (SI closure) */
  double cfl, gamma, t_end;
  int64_t max_steps;
  double q, ea, a;           /* chemistry constants */
  tfv_metric_face faces[6];
} tfv_metric_config;

typedef struct tfv_metric tfv_metric;

/* Number of geometry factors tfv_metric_create expects: the volume factors
 * of each axis (n[a] values, x first), then for each direction d the face
 * factors of each axis a (n[a] + 1 values when a == d, else n[a]).  Volumes
 * and face areas are their outer products, multiplied x, then y, then z
 * (torchGeometry.py:95-170). */
int64_t tfv_metric_factor_count(const tfv_metric_config* cfg);

/* Validate the configuration and lay out the workspace
 * (Simulation.__init__ metric branch, torchSession.py:24-158). */
int tfv_metric_create(int32_t precision, const tfv_metric_config* cfg, const double* factors,
                      tfv_metric** out);
int tfv_metric_workspace_size(tfv_metric* m, size_t* bytes);

/* Attach the workspace (256-byte aligned) and the two state slots (and
 * lambda / beta slots of reactive sessions); slot 0 holds the initial state.
 * Computes the initial integral. */
int tfv_metric_bind(tfv_metric* m, void* workspace, void* const* states, void* const* lams,
                    void* const* betas, void* stream);

/* Up to nsteps transactional steps (torchSession.py:523-576); stops at t_end.
 * A failed step leaves the current state, time and balances unchanged:
 * TFV_EINVAL for boundary or chemistry input the reference rejects with
 * ValueError, TFV_ENUMERIC for stall / maximum steps / positivity. */
int tfv_metric_advance(tfv_metric* m, int32_t nsteps);
int tfv_metric_report(tfv_metric* m, tfv_report* out);

/* Integral of the current state (torchSession.py:284-294) into out[dim+2]. */
int tfv_metric_integrals(tfv_metric* m, double* out);

/* Carry time, steps and balances of an earlier run (checkpoint resume). */
int tfv_metric_restore(tfv_metric* m, const tfv_report* r);

/* Make slot 0 or 1 the current one (after the caller rewrote a state). */
int tfv_metric_set_current(tfv_metric* m, int32_t slot);
int tfv_metric_destroy(tfv_metric* m);

/* Rusanov fluxes of n independent faces (python/cfdSolver/torchFlux.py:80-122,
 * rusanov_flux / rusanov_flux_grid; the adaptive solver's leaf-face batches,
 * torchAdaptive.py:115-135).  left, right: [nv][n] primitive face states
 * (rho, velocities, p) with nv = dim + 2 in 3..5; gl, gr: [n]; out: [nv][n]
 * fluxes; direction: the normal velocity row minus one. */
int tfv_rusanov_flux(int32_t precision, int32_t nv, int64_t n, int32_t direction,
                     const void* left, const void* right, const void* gl, const void* gr,
                     void* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TFV_H */

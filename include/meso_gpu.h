/*
 * meso_gpu.h -- C ABI of the GB300 DUGKS / CDUGKS / Shakhov step library.
 *
 * A drop-in for the step loop of meso-lts (src/meso/exec.cpp:81-165): the
 * host keeps the case file, the Gambit meshes and the output formats, and
 * every call below replaces one member of the reference solver classes
 * (include/solver/boltzmann/{dugks,cdugks,cdugks_shakhov}.h).  Plain C types
 * only: pointers, sizes and the descriptor structs declared here.
 *
 * Conventions
 *   - Every function returns MESO_OK (0) or one MESO_ERR_* code; the message
 *     of the last failure on the calling thread is meso_last_error().
 *     No C++ exception crosses this boundary.
 *   - All arrays are caller-owned host memory, indexed in the ORIGINAL order
 *     of the .neu file (cells and faces as the reference numbers them); the
 *     library renumbers internally (FP64: reverse Cuthill-McKee cells; FP32:
 *     bisection tiles with a local RCM order; faces sorted by owner) and maps
 *     back on every read.
 *   - One context per host thread at a time (contexts are not internally
 *     locked); each context owns one CUDA stream on the current device.
 *   - Vectors are xyz triples, 3 doubles per entry, also in 2D (z = 0).
 */
#ifndef MESO_GPU_H
#define MESO_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MESO_OK 0
#define MESO_ERR_INVALID 1     /* bad argument or descriptor (std::invalid_argument in the reference) */
#define MESO_ERR_CUDA 2        /* CUDA runtime failure, or no usable GPU */
#define MESO_ERR_OOM 3         /* device allocation failed */
#define MESO_ERR_NAN 4         /* a cell produced rho = NaN or T < 0 with no mask (run_state = false) */
#define MESO_ERR_TIMEOUT 5     /* a bounded device wait gave up */
#define MESO_ERR_IO 6          /* case, mesh or DVS file missing or malformed */
#define MESO_ERR_UNSUPPORTED 7 /* valid input that this build does not implement */
#define MESO_ERR_CAPACITY 8    /* request larger than a fixed capacity */

/* ---- solver kinds: the dispatch strings of src/meso/main.cpp:49-54 ------- */
#define MESO_SOLVER_DUGKS 0          /* "dugks@incompressible"  (class DUGKS)          */
#define MESO_SOLVER_CDUGKS 1         /* "cdugks@incompressible" (class CDUGKS)         */
#define MESO_SOLVER_CDUGKS_SHAKHOV 2 /* "cdugks@shakhov"        (class CDUGKS_SHAKHOV) */

/* ---- storage precision of the distribution functions -------------------- */
#define MESO_FP64 0 /* plain form: f, face values and fluxes in FP64 (parity form)            */
#define MESO_FP32 1 /* f stored and streamed in FP32 as the deviation from a reference Maxwellian;
                       face / cell macros, the reference Maxwellian's moments and the wall
                       balance in FP64 (2-D Shakhov without the limiter) */

/* ---- boundary types: BoundaryType of include/solver/config.h:13-23 ------- */
#define MESO_BC_FLUID_INTERIOR 0
#define MESO_BC_FARFIELD_INLET 1
#define MESO_BC_PRESSURE_INLET 2
#define MESO_BC_FREESTREAM_INLET 3
#define MESO_BC_FARFIELD_OUTLET 4
#define MESO_BC_PRESSURE_OUTLET 5
#define MESO_BC_WALL 6
#define MESO_BC_SLIP_WALL 7
#define MESO_BC_SYMMETRY 8

/* ---- patch value types: PatchType of include/solver/config.h:25-36 ------ */
#define MESO_PATCH_ZERO_GRADIENT 0
#define MESO_PATCH_FIXED_VALUE 1
#define MESO_PATCH_CALCULATED 2
#define MESO_PATCH_FROM_FILE 3
#define MESO_PATCH_SWITCH 4

/*
 * Physical mesh, flattened from fvmMesh::Mesh (include/mesh/object.h:93-179)
 * after Mesh::build_geom (src/mesh/object.cpp:94-172).  CSR lists keep the
 * reference's per-cell order: Cell::face_id (local face order) and
 * Cell::neighbors (first-seen order over the cell's faces).
 */
typedef struct meso_mesh_desc {
    int32_t dim;                 /* 2 or 3 (Mesh::NDFVL) */
    int32_t ncell, nface;
    const double *cell_pos;      /* [ncell*3] Cell::position              */
    const double *cell_vol;      /* [ncell]   Cell::volume                */
    const int32_t *cell_group;   /* [ncell]   Cell::group_id (index into groups) */
    const int32_t *cell_face_ptr;/* [ncell+1] CSR into cell_face          */
    const int32_t *cell_face;    /* Cell::face_id                         */
    const int32_t *cell_nbr_ptr; /* [ncell+1] CSR into cell_nbr, lsq_w, lsq_dr */
    const int32_t *cell_nbr;     /* Cell::neighbors                       */
    const double *lsq_w;         /* LeastSquare::weight                   */
    const double *lsq_dr;        /* LeastSquare::dr, 3 per entry          */
    const double *lsq_c;         /* [ncell*9] LeastSquare::Cx, Cy, Cz     */
    const int32_t *face_cell;    /* [nface*2] Face::cell_id {own, nei}; boundary faces {c, c} */
    const double *face_pos;      /* [nface*3] Face::position              */
    const double *face_area;     /* [nface]   Face::area                  */
    const double *face_normal;   /* [nface*3] Face::normal_vector[0] (outward from own; [1] = -[0]) */
    const int32_t *face_mark;    /* [nface]   index into the mark table (0 = fluid-interior) */
    double min_cell_size;        /* Mesh::min_cell_size */
    double total_volume;         /* Mesh::total_volume  */
} meso_mesh_desc;

/*
 * Discrete velocity set, flattened from the DVS Mesh of
 * src/solver/dvs/dvs_generator.cpp (position = xi, volume = weight,
 * symmetry.id = mirror indices).  tensor_n > 0 declares a tensor-product set
 * (Gauss-Hermite, half-range GH, Newton-Cotes) with index i + j*n (+ k*n*n)
 * over the 1-D abscissae `axis`; 0 for Sparse or Gambit velocity meshes.
 */
typedef struct meso_dvs_desc {
    int32_t nv;
    const double *xi;            /* [nv*3] */
    const double *w;             /* [nv]   */
    const int32_t *sym;          /* [nv*3] Symmetry::id, may be NULL (all 0) */
    int32_t tensor_n;
    const double *axis;          /* [tensor_n] or NULL */
    double max_magnitude;        /* Mesh::max_cell_magnitude of the DVS */
} meso_dvs_desc;

/*
 * One face group ([mark] block of the case file, Mark/Patch of
 * include/solver/config.h:38-114).  Missing patch keys take the reference's
 * defaults (src/solver/boundary/patch.cpp:55-85): type 0, scalars 0,
 * vectors 0.
 */
typedef struct meso_mark_desc {
    int32_t type;                /* MESO_BC_* */
    int32_t temperature_type;    /* PatchType of "temperature" (wall balance, cdugks_shakhov.cpp:473-479) */
    int32_t direction;           /* "direction" objectType (symmetry, slip-wall) */
    int32_t pad_;
    double density;              /* "density"     */
    double temperature;          /* "temperature" */
    double pressure;             /* "pressure"    */
    double velocity[3];          /* "velocity"    */
    double alpha_u, alpha_T;     /* "slip-wall-alpha-u", "slip-wall-alpha-T" */
} meso_mark_desc;

/*
 * Solver settings ([settings] of the case file).  The fields each solver
 * reads are the ones its constructor / update_config reads:
 *   CDUGKS  cdugks.cpp:7-15, 41-47;  DUGKS dugks.cpp:7-15, 41-48;
 *   CDUGKS_SHAKHOV cdugks_shakhov.cpp:7-33.
 */
typedef struct meso_params {
    int32_t solver;              /* MESO_SOLVER_* */
    int32_t precision;           /* MESO_FP64 or MESO_FP32 */
    int32_t gradient_switch;     /* "gradient-switch" */
    int32_t limiter_switch;      /* "limiter-switch" (Shakhov) */
    int32_t K;                   /* "gas-k" (Shakhov, integer as in the reference) */
    int32_t residual_interval;   /* 100 in the reference (solver.h:49); 0 disables the check */
    double dt;                   /* "timeStep" (DUGKS: derived from CFL in initial) */
    double R;                    /* "gas-constant" */
    double T0;                   /* "ref-temperature" */
    double rho0, L0;             /* "ref-density", "ref-length" */
    double mu0;                  /* "ref-viscosity" (Shakhov) */
    double vhs_index;            /* "vhs-index" (Shakhov) */
    double Pr;                   /* "Pr" (Shakhov) */
    double Ma, Re;               /* "Ma", "Re" (BGK) */
    double CFL;                  /* "CFL" (DUGKS) */
    double venkata_k;            /* "venkata-limiter-k" */
    double residual_limit;       /* "residual-limit" */
    int32_t residual_fields;     /* fields the convergence test watches: 0 = all the reference watches
                                    (cdugks_shakhov.cpp:747-756), else MESO_RES_* bits; no counterpart
                                    in the reference (served solves converge on U) */
    /* FP32 kernel shape (0 = the library's choice or the autotuner's cached pick); no counterpart in
       the reference: cells per tile (8..48), velocities per lane (1 or 2), velocity groups per tile
       (ngroup 0: the tiles' velocity chunks, tile after tile, cut into one equal run per SM) */
    int32_t tile_cells;
    int32_t vpl;
    int32_t ngroup;
    int32_t pad_;
} meso_params;

#define MESO_RES_RHO 1
#define MESO_RES_T 2
#define MESO_RES_U 4 /* every velocity component */
#define MESO_RES_Q 8
#define MESO_RES_L2 16 /* measure volume-weighted L2-relative change ||new - old|| / ||old|| per component
                          instead of the reference's mean of |new - old| / |old| (field.cpp:223-249),
                          which divides by values near zero (velocity at a vortex centre) */

/* Step state, the reference's run_state / step / solution_time plus the monitor of cdugks_shakhov.cpp:697-719. */
typedef struct meso_status {
    int32_t step;
    int32_t run_state;           /* 1 while running; 0 after convergence or an unmasked NaN/T<0 */
    int32_t converged;           /* 1 if run_state turned 0 by convergence */
    int32_t bad_cells;           /* cells flagged by the last step's monitor */
    int32_t first_bad_cell;      /* original-order id of the first flagged cell, -1 if none */
    int32_t masked_repairs;      /* cumulative mask repairs (cell_value_interp) */
    double solution_time;
    double residual[8];          /* last residuals, in the reference's print order */
    int32_t nresidual;
    int32_t pad_;
} meso_status;

typedef struct meso_ctx meso_ctx;
typedef struct meso_case meso_case;
typedef struct meso_batch meso_batch;

/* Message of the last failure on this thread ("" if none). */
const char *meso_last_error(void);

/* Library build information: "<version> sm_103a <build flags>". */
const char *meso_version(void);

/* ---- host-only case loading (no GPU needed) ----------------------------- */

/*
 * Parse a case file and build everything the reference constructor builds:
 * Config (src/solver/config.cpp:18-108), the Gambit mesh and its geometry
 * (src/mesh/mesh.cpp:4-11, object.cpp:38-172, geom.cpp), the DVS
 * (dvs_generator.cpp), the solver settings (ctor / update_config) and the
 * initial macroscopic fields from the [group] patches (initial(), e.g.
 * cdugks_shakhov.cpp:103-132).  Relative paths resolve against the case
 * file's directory.
 */
int meso_case_load(const char *case_file, meso_case **out);
void meso_case_free(meso_case *c);
/* Views into the loaded case; valid until meso_case_free. */
int meso_case_mesh(const meso_case *c, meso_mesh_desc *mesh);
int meso_case_dvs(const meso_case *c, meso_dvs_desc *dvs);
int meso_case_marks(const meso_case *c, const meso_mark_desc **marks, int32_t *nmarks);
int meso_case_params(const meso_case *c, meso_params *params);
/* Patch values per cell from the [group] blocks (density/velocity/temperature, fixedValue or fromFile).
 * mask[c] = the group's "mask" switch.  Any pointer may be NULL. */
int meso_case_initial_fields(const meso_case *c, double *rho, double *u, double *T, uint8_t *mask);
/* Settings that drive the step loop: max-step, write-interval, read-np-data, output-latest, output-np. */
int meso_case_loop_settings(const meso_case *c, int32_t *max_step, int32_t *write_interval,
                            int32_t *read_np_data, int32_t *output_latest, int32_t *output_np);

/* Mesh::output_grid (src/mesh/mesh_output.cpp:182-215): the case mesh's Tecplot grid file (the
 * grid.plt output() writes at step 0), on the host; the zone header carries the node and cell counts. */
int meso_case_output_grid(const meso_case *c, const char *path);

/* ---- single solve ------------------------------------------------------- */

/*
 * Create a solver context on the current CUDA device from flat descriptors.
 * Replaces the reference constructors (cdugks.cpp:7-39, dugks.cpp:7-39,
 * cdugks_shakhov.cpp:35-60) after the mesh and DVS are built.  mask may be
 * NULL (no cell is masked, cdugks_shakhov.cpp:701-707).
 */
int meso_ctx_create(const meso_mesh_desc *mesh, const meso_dvs_desc *dvs, const meso_mark_desc *marks,
                    int32_t nmarks, const meso_params *params, const uint8_t *mask, meso_ctx **out);

/* Same from a case file: meso_case_load + meso_ctx_create, precision overriding the file's. */
int meso_ctx_create_from_case(const char *case_file, int32_t precision, meso_ctx **out);

void meso_ctx_destroy(meso_ctx *ctx);

/*
 * initial(): equilibrium state from macroscopic fields.
 *   mode 0 -- group-patch path (cdugks.cpp:66-105, cdugks_shakhov.cpp:102-169):
 *             f = equilibrium(rho, u, T); the stored macros are then the
 *             discrete moments of f.  q is ignored.
 *   mode 1 -- read-np-data path (cdugks.cpp:56-65, cdugks_shakhov.cpp:81-101):
 *             f = Maxwell / Shakhov(rho, u, T, q); the macros are kept as given.
 * T and q are ignored by the BGK solvers and may be NULL there.
 */
int meso_init_macros(meso_ctx *ctx, const double *rho, const double *u, const double *T, const double *q,
                     int32_t mode);

/* initial() for a context made by meso_ctx_create_from_case: the case's own groups / read-np-data files. */
int meso_initial(meso_ctx *ctx);

/*
 * nsteps x do_step() (cdugks_shakhov.cpp:724-764, cdugks.cpp:337-371,
 * dugks.cpp:346-383), including the residual check every residual_interval
 * steps and the convergence counter.  Returns early with MESO_OK when
 * run_state turns 0 by convergence, and with MESO_ERR_NAN when it turns 0 by
 * an unmasked NaN / T < 0 cell.  steps_done (may be NULL) receives the count.
 */
int meso_step(meso_ctx *ctx, int32_t nsteps, int32_t *steps_done);

/*
 * Defect correction of the FP32 form (2-D Shakhov FP32 contexts; no counterpart in the reference,
 * whose step is FP64).  With interval > 0, every interval-th step of meso_step runs the plain
 * FP64 step (the reference's arithmetic) and the FP32 step from the same state, keeps their
 * difference as a correction that every following FP32 step adds to its results (state, the
 * conservative update, the heat flux; the state rounded stochastically), and continues from the
 * FP64 step's result.  The FP32 form's fields then settle to the FP64 step's steady state instead
 * of one displaced by the FP32 arithmetic's rounding.  Costs the FP64 step's buffers on the device
 * (about 64 bytes per cell-velocity) and one FP64 + one FP32 step per interval; the corrections
 * start from zero when switched on and are not part of meso_snapshot.  interval = 0 switches it
 * off.  MESO_ERR_UNSUPPORTED for other contexts, MESO_ERR_INVALID for batch members.
 */
int meso_fp32_refine(meso_ctx *ctx, int32_t interval);

/* Macroscopic cell fields rho_cell, vel_cell, T_cell, q_cell (any pointer may be NULL). */
int meso_get_macros(meso_ctx *ctx, double *rho, double *u, double *T, double *q);

/* Shakhov flux moments of the last step (flux_m0, flux_m1, flux_m2; cdugks_shakhov.cpp:636-641). */
int meso_get_flux_moments(meso_ctx *ctx, double *m0, double *m1, double *m2);

int meso_get_status(meso_ctx *ctx, meso_status *st);

/* update_config() (cdugks_shakhov.cpp:7-33): new settings take effect from the next step.
 * solver, precision and K may not change. */
int meso_set_params(meso_ctx *ctx, const meso_params *params);
int meso_get_params(meso_ctx *ctx, meso_params *params);

/* output() of the reference (Tecplot data.plt / grid.plt and the np text files), for case contexts. */
int meso_output(meso_ctx *ctx);

/* Exact device-state snapshot (distribution functions + macros + step counters). */
size_t meso_snapshot_size(meso_ctx *ctx);
int meso_snapshot(meso_ctx *ctx, void *host, size_t bytes);
int meso_restore(meso_ctx *ctx, const void *host, size_t bytes);

/* Device bytes this context holds. */
size_t meso_ctx_device_bytes(meso_ctx *ctx);

/* Time of the last meso_step call on the device, in ms (CUDA events around the launches). */
double meso_last_step_ms(meso_ctx *ctx);

/* Number of kernel launches the last meso_step call issued. */
int64_t meso_last_step_launches(meso_ctx *ctx);

/*
 * Profiling: nsteps real steps (the solution advances) with CUDA events
 * recorded on the context's stream between the step's kernels; ms[k]
 * receives the mean device time of phase k per step, *nphases the phase
 * count.  No counterpart in the reference (which has no timers).
 */
int meso_phase_times(meso_ctx *ctx, int32_t nsteps, double *ms, int32_t max_phases, int32_t *nphases);
/* Kernel name(s) of phase i of this context's step. */
const char *meso_phase_name(meso_ctx *ctx, int32_t i);

/* ---- FP32 kernel-shape autotuner ---------------------------------------- */

/*
 * Measures the FP32 step of this solve for each candidate kernel shape (cells
 * per tile, velocities per lane, velocity groups per tile: meso_params
 * tile_cells / vpl / ngroup), `steps` timed steps each from a uniform
 * equilibrium, and returns in *best the params with the fastest shape (and its
 * time per step in *best_ms, may be NULL).  The shape is remembered for solves
 * with the same cell, face and velocity counts: contexts created afterwards
 * with tile_cells = vpl = ngroup = 0 use it.  No counterpart in the reference.
 */
int meso_autotune(const meso_mesh_desc *mesh, const meso_dvs_desc *dvs, const meso_mark_desc *marks, int32_t nmarks,
                  const meso_params *params, int32_t steps, meso_params *best, double *best_ms);
/* The same for a case file (its mesh, velocity set, marks and settings). */
int meso_autotune_case(const char *case_file, int32_t steps, meso_params *best, double *best_ms);
/* Forget every remembered shape. */
void meso_autotune_forget(void);

/* ---- batched solves ----------------------------------------------------- */

/*
 * A batch steps many FP32 contexts (different meshes, velocity sets and
 * parameters) with one set of launches per step, replayed as a CUDA graph.
 * No counterpart in the reference, which runs one solve per process: each
 * member keeps the reference's per-solve do_step bookkeeping (step,
 * solution_time, residual every residual_interval of its own steps and the
 * 10-check convergence counter, cdugks_shakhov.cpp:724-764); a member that
 * converges or hits an unmasked NaN / T < 0 stops taking steps.  Members must be
 * FP32 contexts on one device, initialised, and in no other batch; while in a
 * batch they are stepped only by meso_batch_step (meso_step refuses them) and
 * do not re-read their case files.  Results, status, output and snapshots are
 * read per member with the meso_ctx functions.  Destroying a member removes it
 * from its batch; destroying the batch leaves the members intact.
 */
int meso_batch_create(meso_ctx *const *ctxs, int32_t n, meso_batch **out);
void meso_batch_destroy(meso_batch *batch);
/* nsteps steps of every running member; *nrunning (may be NULL) receives the members still running. */
int meso_batch_step(meso_batch *batch, int32_t nsteps, int32_t *nrunning);
int32_t meso_batch_size(meso_batch *batch);
/* Device time of the last meso_batch_step call (ms) and the kernel launches it issued. */
double meso_batch_last_step_ms(meso_batch *batch);
int64_t meso_batch_last_step_launches(meso_batch *batch);
/* nsteps steps of the batch with the kernels launched one by one and timed per phase (names as
 * meso_phase_name of a member): ms[k] receives the mean device time of phase k per step.  No
 * counterpart in the reference. */
int meso_batch_phase_times(meso_batch *batch, int32_t nsteps, double *ms, int32_t max_phases, int32_t *nphases);

/* ---- served solves (continuous batching) -------------------------------- */

/*
 * A request server over one device.  Each request is a case file (FP32
 * Shakhov); it is admitted when a member slot is free and the solve fits in
 * the HBM budget and in the device's free memory, then stepped with every
 * other admitted solve by one batch, with its state resident on the device.
 * A solve finishes when it converges (residual settings from the case or the
 * params given at submit), fails (unmasked NaN / T < 0) or reaches the case's
 * max-step, as the reference's handle_solver loop ends a solve
 * (src/meso/exec.cpp:141-165); its memory is then freed for pending requests.
 * No counterpart in the reference, which runs one solve per process.
 * One host thread drives a server.
 */
typedef struct meso_server meso_server;
int meso_server_create(int64_t hbm_budget_bytes, int32_t max_members, meso_server **out);
void meso_server_destroy(meso_server *server);
/* Queue a solve; params (may be NULL) replaces the case file's settings.  *tag identifies it. */
int meso_server_submit(meso_server *server, const char *case_file, const meso_params *params, int64_t *tag);
/* Admit what fits, step the admitted solves nsteps together, retire the finished ones: their
 * tags go to done_tags (capacity max_done), their count to *ndone. */
int meso_server_poll(meso_server *server, int32_t nsteps, int64_t *done_tags, int32_t max_done, int32_t *ndone);
int meso_server_counts(meso_server *server, int32_t *npending, int32_t *nrunning, int32_t *ndone);
/* Result of a finished solve (original cell order; any pointer may be NULL); seconds[0] = submit to
 * finish, seconds[1] = submit to admission (seconds may be NULL). */
int meso_server_result(meso_server *server, int64_t tag, double *rho, double *u, double *T, double *q,
                       meso_status *status, double *seconds);
/* Drop a finished solve's stored result. */
int meso_server_release(meso_server *server, int64_t tag);
/* Device bytes held by the admitted solves. */
int64_t meso_server_device_bytes(meso_server *server);
/* Totals since creation: device time of the batch steps (ms), wall time spent inside
 * meso_server_poll (ms; the rest of it is admission, retirement and batch rebuilds on the host),
 * and batch steps issued.  No counterpart in the reference. */
int meso_server_stats(meso_server *server, double *gpu_ms, double *poll_ms, int64_t *batch_steps);

/* ---- allocation-free entry point --------------------------------------- */

/* Largest ncell meso_shakhov_moments_noalloc accepts. */
#define MESO_NOALLOC_MAX_CELLS 131072

/*
 * Macroscopic moments of a Shakhov state, for callers that cannot call
 * cudaMalloc: a host framework that owns all device memory in its own pool
 * and gives an operator only its input and output buffers, or a serving /
 * real-time loop with a fixed memory budget that must not call cudaMalloc or
 * cudaFree (both synchronize the device) between steps.  No counterpart in
 * the reference; it evaluates the moment sums of initial() (cdugks_shakhov.cpp:
 * 102-169) on the caller's buffers.
 *
 *   g, h   [ncell*nv] state, cell-major (velocity fastest), FP64
 *   xi     [nv*3], w [nv]: discrete velocities and weights
 *   u0     [ncell*3] velocity the heat flux is taken about (c = xi - u0)
 *   R, K   gas constant and gas-k (Cv = (K + 3) R / 2)
 *   rho [ncell], u [ncell*3], T [ncell], q [ncell*3]: outputs
 *   stream a cudaStream_t (NULL: the default stream); the outputs are ready
 *          when the stream reaches the call
 * Every array is device (or managed) memory of the current device; a host
 * pointer or another GPU's buffer fails with MESO_ERR_INVALID.  A CUDA error
 * left pending by the caller's earlier work fails the call with
 * MESO_ERR_CUDA and stays pending for the caller to read.
 *
 * Allocates nothing: no cudaMalloc, cudaFree or allocating library call.
 * Its scratch is one fixed device array of 8 MiB + 64 KiB in this library,
 * present on every GPU that loads the library until the process exits; hence
 * ncell <= MESO_NOALLOC_MAX_CELLS, larger requests fail with
 * MESO_ERR_CAPACITY.  The first call on a device looks up that array's
 * device address (and loads the library's device code there if it is not
 * loaded yet); make that first call before any stream capture.  Every call
 * on a device shares the array: calls that may overlap on the GPU (other
 * streams without ordering, other host threads) race and give wrong results;
 * order them on one stream or synchronize between them.
 */
int meso_shakhov_moments_noalloc(const double *g, const double *h, int32_t ncell, int32_t nv, int32_t dim,
                                 const double *xi, const double *w, const double *u0, double R, double K,
                                 double *rho, double *u, double *T, double *q, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MESO_GPU_H */

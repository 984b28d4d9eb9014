/*
 * sflow.h -- C ABI of the GB300 time-stepping path of IMEX_SfloW2D.
 *
 * The reference solver (Fortran) has no library interface: its driver
 * (src/IMEX_SfloW2D.f90) calls argument-less module procedures that act on
 * module globals.  Each entry point below replaces one of those call sites;
 * the citation next to it names the reference routine it stands in for.
 * A Fortran host binds them with ISO_C_BINDING interfaces, a C, C++ or
 * Python host binds them directly.
 *
 * Conventions
 *  - All entry points return 0 on success, a negative SFLOW_E* code on a
 *    usage / CUDA error (message in sflow_last_error()), or, for the step
 *    routines, a positive bit mask of SFLOW_S* solver status flags (the
 *    reference prints and pauses on READ(*,*) in these situations).
 *  - Host arrays are borrowed for the duration of the call only.
 *  - Host state arrays use the reference layout: q(1:n_vars, 1:nx, 1:ny),
 *    REAL(8), Fortran column-major, variable index fastest
 *    (src/solver_2d.f90:277); the handle keeps a structure-of-arrays copy in
 *    GPU memory and transposes on upload/download.
 *  - A handle is not thread safe; all its device work runs on its own stream.
 */
#ifndef SFLOW_H
#define SFLOW_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SFLOW_ABI_VERSION 2

#define SFLOW_MAX_SOLID 4
/* n_vars = 4 + n_solid (src/inpout_2d.f90:2045-2046 with n_add_gas = 0,
 * no stochastic, no pore pressure, no gas+liquid mixture). */
#define SFLOW_MAX_VARS (4 + SFLOW_MAX_SOLID)
/* vulnerability-table levels of each kind (thickness_levels0 and
 * dyn_pres_levels0 of the reference, inpout_2d.f90:293-294) */
#define SFLOW_MAX_LEVELS 10
/* velocity intervals of a bottom radial source (inpout_2d.f90:900-902) */
#define SFLOW_MAX_INTERVALS 100

/* ---- error codes (negative) ---------------------------------------------- */
#define SFLOW_OK 0
#define SFLOW_EINVAL (-1)     /* bad argument or unsupported parameter set   */
#define SFLOW_ENOMEM (-2)     /* device or host allocation failed            */
#define SFLOW_ECUDA (-3)      /* CUDA runtime error                          */
#define SFLOW_ESTATE (-4)     /* call out of order (e.g. step before upload) */
#define SFLOW_ERANGE (-5)     /* size beyond a fixed capacity                */
#define SFLOW_EBUSY (-6)      /* batch: no free slot, tile-list capacity or
                                 device memory for this run now; retry after
                                 other runs are collected                    */

/* ---- solver status bits (positive), sticky until sflow_clear_status ------ */
#define SFLOW_S_NAN 0x1u          /* NaN after assembly (solver_2d.f90:1381)  */
#define SFLOW_S_NEG_H 0x2u        /* q1 < -1e-7 (solver_2d.f90:1400-1436)     */
#define SFLOW_S_NEG_ALPHA 0x4u    /* solid mass <= -1e-7 (solver_2d.f90:1440) */
#define SFLOW_S_LOW_T 0x8u        /* T < 273 K (solver_2d.f90:1541)           */
#define SFLOW_S_SOLID_GT_MASS 0x10u /* sum solids > q1 (solver_2d.f90:1562)   */
#define SFLOW_S_NEWTON_MAXIT 0x20u  /* Newton hit max_nl_iter                 */
#define SFLOW_S_EROSION 0x40u     /* erosion-step consistency check tripped   */
/* A run stops at the end of the step that raised one of these (where the
 * reference pauses on READ(*,*)); sflow_clear_status lets it continue.
 * The other bits are reported and the run goes on. */
#define SFLOW_S_FATAL (SFLOW_S_NAN | SFLOW_S_NEG_H | SFLOW_S_NEG_ALPHA | SFLOW_S_EROSION)

/* ---- precision of the state and of the explicit (bulk) arithmetic -------- */
#define SFLOW_PREC_FP64 0   /* plain form: everything FP64                      */
#define SFLOW_PREC_FP32 1   /* FP32 state/fluxes; Newton, mass sums, wet/dry
                               thresholds in FP64                              */

/* ---- solver scheme (src/parameters_2d.f90 solver_scheme) ----------------- */
#define SFLOW_SCHEME_KT 0
#define SFLOW_SCHEME_UP 1

typedef struct {
  int32_t flag;   /* 0 Dirichlet value, 1 Neumann slope, 2 one-sided gradient */
  int32_t pad;
  double value;
} SflowBC;     /* TYPE bc (src/parameters_2d.f90:393-396) */

/* Boundary sides, index of SflowParams.bc */
#define SFLOW_W 0
#define SFLOW_E 1
#define SFLOW_S 2
#define SFLOW_N 3

/*
 * Parameters: the subset of the IMEX_SfloW2D.inp namelists that the time
 * step reads.  Names follow the namelist keys (src/inpout_2d.f90:326-391,
 * 1017-1039).  Derived constants (rho_a_amb, eps_sing, h_source from
 * MFR_SOURCE, ...) are computed by sflow_create the way read_param does.
 */
typedef struct {
  int32_t abi_version;          /* = SFLOW_ABI_VERSION */
  int32_t precision;            /* SFLOW_PREC_* */

  /* NEWRUN_PARAMETERS */
  int32_t comp_cells_x, comp_cells_y;
  double x0, y0, cell_size;
  int32_t n_solid;
  int32_t gas_flag, liquid_flag, energy_flag, alpha_flag;
  int32_t rheology_flag;
  int32_t slope_correction_flag, curvature_term_flag;
  int32_t radial_source_flag;

  /* NUMERIC_PARAMETERS */
  int32_t solver_scheme;        /* SFLOW_SCHEME_* */
  int32_t n_rk;                 /* 1..4 */
  double dt0, max_dt, cfl, theta, reconstr_coeff;
  int32_t limiter[SFLOW_MAX_VARS]; /* per conservative variable; u,v copy hu,hv */

  /* *_BOUNDARY_CONDITIONS, per side, per variable (h, hu, hv, T, solids) */
  SflowBC bc[4][SFLOW_MAX_VARS];

  /* EXPL_TERMS_PARAMETERS */
  double grav;

  /* RHEOLOGY_PARAMETERS */
  int32_t rheology_model;       /* 1 Voellmy-Salm, 6 quadratic friction */
  int32_t pad0;
  double mu, xi, friction_factor;

  /* GAS_TRANSPORT_PARAMETERS */
  double pres, sp_heat_a, sp_gas_const_a, kin_visc_a, T_ambient;
  int32_t entrainment_flag;
  int32_t pad1;

  /* LIQUID_TRANSPORT_PARAMETERS */
  double rho_l, sp_heat_l, kin_visc_l, loss_rate;

  /* SOLID_TRANSPORT_PARAMETERS */
  double rho_s[SFLOW_MAX_SOLID], diam_s[SFLOW_MAX_SOLID], sp_heat_s[SFLOW_MAX_SOLID];
  int32_t settling_flag, collective_settling_flag;
  double alphastot_min, maximum_solid_packing, A_drag, B_drag;
  double erosion_coeff;         /* erosion rate coefficient (constitutive_2d.f90:4732) */

  /* RADIAL_SOURCE_PARAMETERS (lateral ring inlet; also the bottom source) */
  double x_source, y_source, r_source, r2_source;
  double vel_source, T_source, h_source, mfr_source;
  double alphas_source[SFLOW_MAX_SOLID];
  double time_param[4];
  double azimuth_source, arc_width_source;

  /* RUN_PARAMETERS */
  double t_start, t_end, dt_output;

  /* ---- fields of ABI version 2 ---- */
  /* VULNERABILITY_TABLE_PARAMETERS (inpout_2d.f90:3792-3870): the levels
   * >= 0 are used, in order (default -1: no table); when only one kind is
   * given the other is a single level 0.  Cell (j,k) sets table entry
   * (i_thk-1)*n_dyn + i_dyn once h >= thickness_levels[i_thk] and
   * p_dyn >= dyn_pres_levels[i_dyn] (IMEX_SfloW2D.f90:351, 489) */
  double thickness_levels[SFLOW_MAX_LEVELS], dyn_pres_levels[SFLOW_MAX_LEVELS];
  /* SOLID_TRANSPORT_PARAMETERS: erosion of an erodible layer
   * (constitutive_2d.f90:4732-4760; inpout_2d.f90:1818-1990).  With
   * erosion_coeff = 0 the reference sets porosity 0, fractions 1/n_solid
   * and T_erodible 300 K; -1 means "not given". */
  double erodible_porosity, T_erodible, initial_erodible_thickness;
  double erodible_fract[SFLOW_MAX_SOLID];
  int32_t erodible_deposit_flag;
  /* NEWRUN_PARAMETERS: the topography follows erosion and deposition,
   * with the topography terms recomputed every step (IMEX_SfloW2D.f90:445) */
  int32_t topo_change_flag;
  /* bottom radial source (NEWRUN bottom_radial_source_flag; cell fractions
   * of the source ellipse, geometry_2d.f90:1899-1994; inflow rate
   * constitutive_2d.f90:3149-3307): vertical inflow velocity vel_source,
   * ellipse semi-axes r_source / r2_source rotated by angle_source
   * (degrees), and optionally n_intervals piecewise-constant velocities
   * vel_intervals from the times t_intervals (else the time_param ramp) */
  int32_t bottom_radial_source_flag, n_intervals;
  double angle_source;
  double t_intervals[SFLOW_MAX_INTERVALS], vel_intervals[SFLOW_MAX_INTERVALS];
  /* SFLOW_PREC_FP32 only: 1 forms the implicit friction step's
   * coefficients and iterates its Newton solve in FP64 (from the FP32
   * state, to a 4-ulp step); 0 (default) iterates in FP32 and finishes with
   * one FP64 Newton step */
  int32_t fp32_newton_fp64;
  int32_t pad2;
  /* RHEOLOGY_PARAMETERS of the mu(I) rheology (rheology_model = 11,
   * constitutive_2d.f90:4384-4458): static and high-I friction, reference
   * inertial number, high-I regularisation; -1 = not given */
  double mu_s, mu_2, I_0, muI_inf;
} SflowParams;

/* Fill p with the defaults of init_param (src/inpout_2d.f90:408-985). */
void sflow_default_params(SflowParams* p);

/* Per-step scalars of the driver log line (src/IMEX_SfloW2D.f90:535-542),
 * accumulated in FP64 with compensated summation. */
typedef struct {
  double t, dt;
  double mass;        /* dx*dy*SUM(q(1,:,:))         */
  double volume;      /* dx*dy*SUM(qp(1,:,:))        */
  double area;        /* dx*dy*COUNT(q(1,:,:)>1e-7)  */
  double solid_mass;  /* dx*dy*SUM(q(5:4+n_solid,:,:)) */
  int64_t solve_cells;   /* active cells of this step (solver_2d.f90:788-811) */
  int64_t steps;         /* steps taken so far */
  uint32_t status;       /* SFLOW_S_* bits seen so far */
  uint32_t pad;
} SflowStepStats;

typedef struct sflow_handle sflow_handle;

/* Last error message of the calling thread ("" if none). */
const char* sflow_last_error(void);

/*
 * Create a solver for one domain.  B_cent: cell-centred topography, nx*ny
 * doubles, column-major (geometry_2d.f90 B_cent(nx,ny)); the topography
 * derivatives (topography_reconstruction, geometry_2d.f90:555-895) and the
 * ring-source geometry (init_source, geometry_2d.f90:907-1323) are derived
 * from it.  Replaces init_grid + init_problem_param +
 * allocate_solver_variables + init_source (IMEX_SfloW2D.f90:186-263).
 */
int sflow_create(const SflowParams* p, const double* B_cent, sflow_handle** out);
void sflow_destroy(sflow_handle* h);

/* State transfer (reference layout, see header comment).  upload also sets
 * t = t_start, dt = dt_old = dt_old_old = dt0 (IMEX_SfloW2D.f90:300-304). */
int sflow_upload_q(sflow_handle* h, const double* q_aos);
int sflow_download_q(sflow_handle* h, double* q_aos);
/* Replace the state only (time, dt history, maxima and counters kept): for
 * a host that owns q between steps and hands it over at every call. */
int sflow_put_q(sflow_handle* h, const double* q_aos);
/* Set the driver clock: t, dt_old, dt_old_old (IMEX_SfloW2D.f90:417-439). */
int sflow_set_clock(sflow_handle* h, double t, double dt_old, double dt_old_old);
/* qp(1:n_vars+2,nx,ny) of the last post-step pass. */
int sflow_download_qp(sflow_handle* h, double* qp_aos);
/* hmax, pdynmax, mod_vel_max, each nx*ny column-major (IMEX_SfloW2D.f90:449-505) */
int sflow_download_maps(sflow_handle* h, double* hmax, double* pdynmax, double* mod_vel_max);

/* check_solve (solver_2d.f90:667-858): active-cell mask of this step. */
int sflow_check_solve(sflow_handle* h, int32_t solve_all);
/* timestep (solver_2d.f90:873-1006): CFL time step over the active cells. */
int sflow_timestep(sflow_handle* h, double* dt_cfl_out);
/* imex_RK_solver (solver_2d.f90:1022-1634) with the given t and dt. */
int sflow_imex_rk(sflow_handle* h, double t, double dt);
/* update_erosion_deposition_cell (solver_2d.f90:2382-2597). */
int sflow_erosion_deposition(sflow_handle* h, double dt);
/* Post-step qc_to_qp + maxima + log sums (IMEX_SfloW2D.f90:449-543);
 * advances t by dt of the last imex_rk call. */
int sflow_post_step(sflow_handle* h, SflowStepStats* stats);

/*
 * One iteration of the driver loop (IMEX_SfloW2D.f90:395-505): check_solve,
 * timestep, the dt clamps (:417-439), imex_RK_solver, erosion/deposition,
 * t += dt, post-step maxima.  dt is computed and clamped on the device; the
 * call does not synchronise.  Returns status bits seen so far.
 */
int sflow_step(sflow_handle* h);
/*
 * Run driver iterations until t >= t_stop (or t_end) or max_steps are done.
 * Steps are launched as CUDA-graph replays in chunks; the call returns after
 * the device has finished.  stats (may be NULL) receives the last step's log
 * scalars.
 */
int sflow_advance(sflow_handle* h, double t_stop, int64_t max_steps, SflowStepStats* stats);
/* Synchronise and read the log scalars of the last completed step. */
int sflow_get_stats(sflow_handle* h, SflowStepStats* stats);
int sflow_status(sflow_handle* h, uint32_t* flags);
int sflow_clear_status(sflow_handle* h);

/*
 * Timing support.  sflow_advance_timed runs `steps` driver iterations one
 * at a time, each bracketed by CUDA events on the handle's stream, and
 * returns the summed device time in ms; with flush_l2 != 0 a buffer larger
 * than L2 is written between steps, outside the timed intervals.
 * sflow_profile_kernels does the same with events between the four kernels
 * of a step and returns the summed ms of each (mask, flux, dt, stage).
 */
int sflow_advance_timed(sflow_handle* h, int64_t steps, int32_t flush_l2, double* device_ms);
int sflow_profile_kernels(sflow_handle* h, int64_t steps, int32_t flush_l2, double* ms4);

/* Number of kernel launches issued by this handle since creation (for the
 * benchmark's launch count). */
int64_t sflow_launch_count(const sflow_handle* h);

/* Device bytes held by the handle. */
int64_t sflow_device_bytes(const sflow_handle* h);

/*
 * Tile shape and its autotuner (no counterpart in the reference, whose loops
 * run over cells: the tiling is how this library maps the step onto the
 * GPU).  The tiled kernels work on tiles of 32 x tile_h cells; the results
 * of a step are the same for every tile height.  Heights with compiled
 * kernels: 8, 16 and 4 in the FP32 bulk form, 8 in the FP64 plain form
 * (sflow_tile_shapes lists them; the default is 8).
 *
 * sflow_set_tile_shape  switch a run between steps (SFLOW_EINVAL for a
 *                       height without kernels)
 * sflow_autotune        runs `steps_per_shape` steps of the run (after one
 *                       untimed 16-step graph chunk) with each candidate
 *                       height, times them with CUDA events, keeps the
 *                       fastest per active-cell update (a later candidate
 *                       only when it is more than 2 % faster than the best
 *                       before it) and returns it in *best; ms_per_mcu[i] (n entries, candidates in the
 *                       order of sflow_tile_shapes' full list 8, 16, 4) gets
 *                       the ms per 10^6 cell updates, -1 where not
 *                       compiled or nothing ran.  The steps advance the run.
 * sflow_batch_set_tile_shape  height of the batch's runs; only while the
 *                       batch holds no run (SFLOW_ESTATE otherwise)
 */
/* Self-check of the device's integer-pipe float <-> double conversions
 * (used by the FP32 form's FP64 Newton step and FP64 sums) against the
 * hardware conversions on n seeded bit patterns; *mismatches must be 0. */
int sflow_check_conversions(int64_t n, uint64_t seed, int64_t* mismatches);

/* The FP64 pow (which 0), log (1) and cos (2) that the FP64 kernels use for
 * the settling, entrainment and inlet-ramp closures -- functions of this
 * library that give the same bits on the device as on the host -- and
 * CUDA's pow, log, cos (3, 4, 5), evaluated on the device for n host
 * arguments (y only for pow).  For tests of those functions. */
int sflow_eval_math(int32_t which, int64_t n, const double* x, const double* y, double* out);

#define SFLOW_TILE_CANDIDATES 3
int sflow_tile_shapes(int32_t precision, int32_t* heights, int32_t capacity, int32_t* count);
int sflow_set_tile_shape(sflow_handle* h, int32_t tile_h);
int sflow_get_tile_shape(const sflow_handle* h, int32_t* tile_h);
int sflow_autotune(sflow_handle* h, int64_t steps_per_shape, int32_t* best, double* ms_per_mcu, int32_t n);

/* Work counters since the last upload: cell updates (sum over steps of the
 * active cells), steps, Newton iterations and the largest per-cell count. */
int sflow_counters(sflow_handle* h, int64_t* cell_updates, int64_t* steps,
                   int64_t* newton_iters, int32_t* newton_max);
/* dry-border part of the cell updates (see sflow_batch_dry_border_updates) */
int sflow_dry_border_updates(sflow_handle* h, int64_t* n);

/*
 * Host-side set-up of a domain without touching the GPU (for tests and
 * tools).  Fills out (nx*ny doubles, column-major) with one derived field:
 * 0 B'_x  1 B'_y  2 B''_xx  3 B''_xy  4 B''_yy (topography_reconstruction,
 * geometry_2d.f90:555-895), 5 grav_coeff  6 d grav_coeff/dx
 * 7 d grav_coeff/dy, 8 ring inlet perimeter  9 its normal x  10 normal y
 * (init_source, geometry_2d.f90:907-1323), 11 source_cell (0, 1, 2),
 * 12 ring face flags (E | W<<1 | N<<2 | S<<3), 13 bottom radial source
 * cell fraction (compute_cell_fract, geometry_2d.f90:1899-1994).
 */
int sflow_host_geometry(const SflowParams* p, const double* B_cent, int32_t which, double* out);
/* out[0] = h_source (inpout_2d.f90:4745), out[1] = rho_m and out[2] = c_p of
 * the inlet state, out[3] = eps_sing (geometry_2d.f90:300-310). */
int sflow_host_scalars(const SflowParams* p, const double* B_cent, double* out4);

/*
 * Log-line sums (mass, volume, wet area, solid mass -- the four values of
 * SflowStepStats, IMEX_SfloW2D.f90:535-542) of a state that the caller
 * already holds in device memory, computed without allocating anything.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc where they need the sums, such as a host framework that owns
 * all device memory through its own pool and forbids raw allocations by
 * the libraries it loads.  Call it from ordinary host code.
 *   p        parameters of the domain (grid size, n_solid and the carrier /
 *            energy constants are read; rejected like sflow_create rejects
 *            them, SFLOW_EINVAL)
 *   q_dev    device pointer, q(1:n_vars,1:nx,1:ny) doubles, reference layout
 *   sums_dev device pointer to 4 doubles, written asynchronously
 *   stream   cudaStream_t to launch on (NULL = default stream)
 * Scratch: one fixed 128 KiB device array inside the library, held by every
 * GPU that loads the library until the process exits.  Domains above
 * 67,108,864 cells (8192 x 8192) are rejected with SFLOW_ERANGE.  The first
 * call on a device looks up the array's address with that device current;
 * make that first call before any stream capture.  All calls share the
 * array: calls whose kernels may overlap on the GPU (different streams
 * without ordering) race and can return wrong sums; calls on one stream are
 * safe.  The sums are compensated (Neumaier) within each thread, block and
 * across blocks.  Argument errors: sflow_log_sums_noalloc_error() (cleared
 * at every call); an error of the kernels themselves shows up at the
 * caller's next synchronisation of the stream.
 */
int sflow_log_sums_noalloc(const SflowParams* p, const double* q_dev, double* sums_dev, void* stream);
const char* sflow_log_sums_noalloc_error(void);

/*
 * Batched runs.  No counterpart in the reference, which runs ensembles as
 * separate processes (EXAMPLES/EXAMPLE_ENSEMBLE_ETNA/launch_jobs.py): many
 * independent runs -- uneven grid sizes, parameters and solid-class counts
 * -- stay resident on one GPU and advance together, five kernel launches
 * per batch step for all runs of a class count (persistent kernels over a
 * device-built queue of active tiles, replayed as CUDA graphs of 16 steps).
 * Each run follows the N_RK = 2 time step of sflow_step exactly (bitwise the
 * same result as its own handle, alone or in any mix).  Runs can be
 * submitted and collected between sflow_batch_advance calls (continuous
 * batching); a run stops at its t_end, after max_steps steps or at a
 * SFLOW_S_FATAL status (its co-resident runs go on unaffected).
 *
 *   sflow_batch_create   precision SFLOW_PREC_FP32 or _FP64 of every run;
 *                        max_runs slots per class count; max_cells bounds
 *                        the summed cells of resident runs (tile lists)
 *   sflow_batch_submit   set-up (as sflow_create) + upload of q (reference
 *                        layout); SFLOW_EBUSY when no slot, list capacity
 *                        or device memory (free memory minus 1 GiB) is
 *                        available now; the run id is returned in *run_id
 *   sflow_batch_advance  `steps` batch steps; *finished = runs that have
 *                        stopped and are not yet collected
 *   sflow_batch_poll     log scalars of the run and whether it has stopped
 *   sflow_batch_download copy of the run's q (reference layout)
 *   sflow_batch_collect  optional download, then frees the run's slot
 */
typedef struct sflow_batch sflow_batch;
int sflow_batch_create(int32_t precision, int32_t max_runs, int64_t max_cells, sflow_batch** out);
void sflow_batch_destroy(sflow_batch* b);
int sflow_batch_submit(sflow_batch* b, const SflowParams* p, const double* B_cent, const double* q_aos,
                       int64_t max_steps, int32_t* run_id);
/* The host part of sflow_batch_submit on its own: validation, topography
 * terms and ring-inlet geometry of a run (no GPU work, no batch), so that a
 * request loop can prepare arriving runs on other threads while the batch
 * advances; sflow_batch_submit_setup then allocates and uploads the run.
 * A setup is read-only after creation and can be submitted to any batch of
 * its precision, any number of times. */
typedef struct sflow_setup sflow_setup;
int sflow_setup_create(const SflowParams* p, const double* B_cent, sflow_setup** out);
void sflow_setup_destroy(sflow_setup* s);
int sflow_batch_submit_setup(sflow_batch* b, const sflow_setup* s, const double* q_aos, int64_t max_steps,
                             int32_t* run_id);
/* sflow_batch_submit_setup that hands the setup's host arrays over to the
 * run instead of copying them (for a request loop that submits each setup
 * once).  After SFLOW_OK the setup is spent: only sflow_setup_destroy may
 * follow.  After SFLOW_EBUSY or an argument error it is unchanged and can
 * be submitted again; after a device failure it is spent. */
int sflow_batch_submit_setup_take(sflow_batch* b, sflow_setup* s, const double* q_aos, int64_t max_steps,
                                  int32_t* run_id);
/* sflow_batch_collect of n runs: q_aos[i] receives run ids[i]'s q (q_aos
 * NULL or q_aos[i] NULL: no download); the downloads run on `threads` host
 * threads (<= 0: the host's hardware threads, at most 64), the slots are
 * freed in order.  status[i] receives each run's result; returns SFLOW_OK or
 * the first failure (sflow_last_error names the run id); a run whose
 * download failed is not collected. */
int sflow_batch_collect_many(sflow_batch* b, int32_t n, const int32_t* ids, double* const* q_aos, int32_t threads,
                             int32_t* status);
/* n runs at once: params[i], B_cent[i], q_aos[i] and max_steps[i] (NULL:
 * no step limit) as for sflow_batch_submit.  The host set-ups run on
 * `threads` host threads (<= 0: the host's hardware threads, at most 64),
 * which also build on the device the runs whose q is in pinned (page-locked)
 * host memory; the calling thread builds the others and admits every run in
 * order.  At most 2 x threads runs are held ahead at a time, each only while
 * the device has room for it.  run_ids[i] receives the run id, or -1 when
 * run i was not admitted.  Returns SFLOW_OK when every run was admitted,
 * else the code of the first failure in run order (sflow_last_error names
 * the run); the runs that could be admitted are admitted either way.  The
 * runs give the same results as sequential sflow_batch_submit calls. */
int sflow_batch_submit_many(sflow_batch* b, int32_t n, const SflowParams* params, const double* const* B_cent,
                            const double* const* q_aos, const int64_t* max_steps, int32_t* run_ids,
                            int32_t threads);
/* Asynchronous sflow_batch_advance: sflow_batch_launch enqueues `steps`
 * batch steps and returns at once; sflow_batch_wait waits for them and
 * reports finished runs.  Between the two only host work is allowed: every
 * other batch call answers SFLOW_ESTATE until the wait. */
int sflow_batch_launch(sflow_batch* b, int64_t steps);
int sflow_batch_wait(sflow_batch* b, int32_t* finished);
int sflow_batch_advance(sflow_batch* b, int64_t steps, int32_t* finished);
/* sflow_batch_advance with the device time of the steps (CUDA events on the
 * batch's streams) in *device_ms */
int sflow_batch_advance_timed(sflow_batch* b, int64_t steps, int32_t* finished, double* device_ms);
/* `steps` batch steps launched one at a time with CUDA events between the
 * five kernels of a step; ms5 = summed device ms of k_b_cand, k_b_mask,
 * k_b_flux, k_b_dt, k_b_stage2 (for the benchmark's per-kernel roofline) */
int sflow_batch_profile_kernels(sflow_batch* b, int64_t steps, int32_t* finished, double* ms5);
int sflow_batch_poll(sflow_batch* b, int32_t run_id, SflowStepStats* stats, int32_t* done);
int sflow_batch_counters(sflow_batch* b, int32_t run_id, int64_t* cell_updates, int64_t* steps);
/* The part of the cell updates that falls in dry border tiles: tiles active
 * only through the domain's border cells (always in check_solve's mask,
 * solver_2d.f90:351-354) whose 4-cell frame holds no mass and no ring cell.
 * They count as active cells, as in the reference, but the flux and stage
 * kernels skip them (their result is no change). */
int sflow_batch_dry_border_updates(sflow_batch* b, int32_t run_id, int64_t* n);
int sflow_batch_download(sflow_batch* b, int32_t run_id, double* q_aos);
int sflow_batch_collect(sflow_batch* b, int32_t run_id, double* q_aos);
int32_t sflow_batch_live(const sflow_batch* b);
int64_t sflow_batch_launch_count(const sflow_batch* b);
int sflow_batch_set_tile_shape(sflow_batch* b, int32_t tile_h);
/* Caps the device bytes the batch's resident runs may hold (0: no cap but
 * the free memory); a submit that would exceed it answers SFLOW_EBUSY. */
int sflow_batch_set_memory_limit(sflow_batch* b, int64_t bytes);
int sflow_batch_get_tile_shape(const sflow_batch* b, int32_t* tile_h);

/*
 * Host I/O of the reference's files (host only, no GPU needed), so a run
 * keeps its input file, restart files and output formats.  Errors:
 * sflow_io_error().
 *
 * sflow_read_input   IMEX_SfloW2D.inp -> p (from the init_param defaults,
 *                    inpout_2d.f90:408-970) and run; the namelists and
 *                    boundary-condition rules of read_param (986-5134) for
 *                    the subset the GPU path runs; any key that would switch
 *                    on physics outside it is rejected with its line.  A
 *                    restart is required (RESTART = T).  RESTART_FILE is
 *                    accepted as RESTART_FILES(1): the reference's TESTS
 *                    inputs use that name, which the current reference
 *                    namelist no longer declares.
 * sflow_read_dem     ESRI ASCII DEM -> B_cent(nx,ny) at the cell centres
 *                    (bilinear, values clipped at 0) and the no-data mask
 *                    (1 where a surrounding DEM value is NODATA_value);
 *                    nodata may be NULL (inpout_2d.f90:3684-3760,
 *                    geometry_2d.f90:312-350, 1395-1517)
 * sflow_read_q2d     .q_2d restart -> q (reference layout), cells with
 *                    q(1) <= 0 zeroed, negative solids zeroed; the output
 *                    index of the file name (inpout_2d.f90:5674-5722)
 * sflow_write_q2d    .q_2d output (inpout_2d.f90:6000-6110); like the
 *                    reference it sets |q| < 1e-20 to zero in q itself
 * sflow_write_p2d    .p_2d output (inpout_2d.f90:6124-6400) from the
 *                    per-cell fields of sflow_download_phys, B_cent, the
 *                    deposit (may be NULL: zeros) and the maxima maps
 * sflow_write_restart / sflow_read_restart
 *                    restart.bin (inpout_2d.f90:8037-8179), Fortran
 *                    unformatted sequential records with 4-byte markers;
 *                    q records above 2 GiB are refused (SFLOW_ERANGE)
 * sflow_output_name  RUN_NAME_dddd.ext (lettera, inpout_2d.f90:6893-6912)
 */
typedef struct {
  char run_name[128];
  char restart_file[256];
  char topography_file[256];
  int32_t restart;
  int32_t output_cons_flag, output_phys_flag, output_esri_flag, output_netcdf_flag, output_runout_flag;
  int32_t verbose_level;
  int32_t pad;
} SflowRunInfo;

const char* sflow_io_error(void);
int sflow_read_input(const char* path, SflowParams* p, SflowRunInfo* run);
int sflow_read_dem(const char* path, const SflowParams* p, double* B_cent, uint8_t* nodata);
int sflow_read_q2d(const char* path, const SflowParams* p, double* q_aos, int32_t* output_idx);
int sflow_write_q2d(const char* path, const SflowParams* p, double* q_aos);
int sflow_write_p2d(const char* path, const SflowParams* p, const double* phys, const double* B_cent,
                    const double* deposit, const double* hmax, const double* pdynmax, const double* mod_vel_max);
int sflow_write_restart(const char* path, const SflowParams* p, double t, double dt, const double* q_aos,
                        const double* B_cent, const double* deposit, const double* hmax, const double* pdynmax,
                        const double* mod_vel_max);
int sflow_read_restart(const char* path, const SflowParams* p, double* t, double* dt, double* q_aos, double* B_cent,
                       double* deposit, double* hmax, double* pdynmax, double* mod_vel_max);
int sflow_output_name(const char* run_name, int32_t index, const char* ext, char* out, int32_t out_len);

/*
 * Device-side fields for the writers and for restarts:
 *   sflow_download_phys     per cell (reference order) h, u, v, T,
 *                           alphas(1:n_solid), rho_m, red_grav, Ri: the
 *                           qc_to_qp and mixt_var values output_solution
 *                           writes (7 + n_solid doubles per cell)
 *   sflow_download_deposit  deposit(1:nx,1:ny,1:n_solid), the accumulated
 *                           dt * deposition of update_erosion_deposition_cell
 *                           (solver_2d.f90:2476); zeros without settling
 *   sflow_upload_deposit    sets it (restart.bin)
 *   sflow_upload_maps       sets hmax, pdynmax, mod_vel_max (restart.bin);
 *                           a NULL map is left unchanged
 *   sflow_set_output_time   the next output time t_output that the dt clamp
 *                           stops at (IMEX_SfloW2D.f90:417-422); the reference
 *                           sets t_output = t + dt_output after each output
 */
int sflow_download_phys(sflow_handle* h, double* out);
int sflow_download_deposit(sflow_handle* h, double* out);
int sflow_upload_deposit(sflow_handle* h, const double* in);
int sflow_upload_maps(sflow_handle* h, const double* hmax, const double* pdynmax, const double* mod_vel_max);
int sflow_set_output_time(sflow_handle* h, double t_output);

/*
 * Erosion, topography change, B_nodata and the vulnerability table (ABI 2).
 * Planes are nx*ny doubles or bytes with j fastest (the reference's (j,k)
 * order), classes / table entries slowest.
 *   sflow_download_erosion     erosion(:,:,1:n_solid), the accumulated
 *                              dt * erosion_term (solver_2d.f90:2479);
 *                              zeros when EROSION_COEFF = 0
 *   sflow_download_erodible    erodible(1:n_solid,:,:), the erodible solid
 *                              thicknesses left (solver_2d.f90:2482-2488)
 *   sflow_set_erodible         the erodible layer thickness per cell (the
 *                              reference's erodible_init, read from
 *                              ERODIBLE_FILE): class i gets
 *                              erodible_fract(i) * (1 - erodible_porosity)
 *                              of it (inpout_2d.f90:1983-1986).  Kept for
 *                              later sflow_upload_q calls, which otherwise
 *                              reset the layer to INITIAL_ERODIBLE_THICKNESS
 *   sflow_download_topography  B_cent; it changes with TOPO_CHANGE_FLAG
 *                              (B += dt * topo_term, solver_2d.f90:2490)
 *   sflow_set_nodata           B_nodata per cell (nonzero: no data); the
 *                              assembly empties those cells
 *                              (solver_2d.f90:1626).  NULL clears it
 *   sflow_vuln_table_size      n_thk, n_dyn of the table (0, 0: none)
 *   sflow_download_vuln_table  n_thk*n_dyn planes of 0/1 bytes: entry
 *                              (i_thk-1)*n_dyn + i_dyn-1 is vuln_table
 *                              (IMEX_SfloW2D.f90:351, 489)
 */
int sflow_download_erosion(sflow_handle* h, double* out);
int sflow_download_erodible(sflow_handle* h, double* out);
int sflow_set_erodible(sflow_handle* h, const double* thickness);
int sflow_download_topography(sflow_handle* h, double* B_cent);
int sflow_set_nodata(sflow_handle* h, const uint8_t* nodata);
int sflow_vuln_table_size(sflow_handle* h, int32_t* n_thk, int32_t* n_dyn);
int sflow_download_vuln_table(sflow_handle* h, uint8_t* out);

/*
 * Row slabs of one domain (domain decomposition by rows).  A slab handle
 * holds rows k0 .. k0+rows-1 of the whole domain described by p and B_cent
 * (the whole DEM: topography terms, inlet geometry and flags are derived on
 * the whole domain, then cut), of which the local rows own_lo .. own_hi-1
 * are its own: only they enter its CFL minimum (sflow_timestep), its
 * active-cell counts, status bits and log sums.  The other rows are halo:
 * they are computed from the slab's data alone (artificial edges take the
 * domain's boundary conditions) and must be refreshed from the neighbours
 * before each step.  With N_RK = 2 one refresh per step suffices: the flux
 * pass runs once, at the step's start, and reads q up to 2 cells away, and
 * the active mask of those cells reads q up to 2 further; a halo of 4 rows
 * each side gives every own cell the whole domain's update (bitwise), with
 * dt = the minimum over the slabs of sflow_timestep and the driver's clamps
 * applied on the host, through the per-call entry points.
 *   sflow_get_rows / sflow_put_rows  rows k_lo .. k_lo+n-1 of q (local),
 *                                    reference layout, for the exchange
 */
int sflow_create_rows(const SflowParams* p, const double* B_cent, int32_t k0, int32_t rows, int32_t own_lo,
                      int32_t own_hi, sflow_handle** out);
int sflow_get_rows(sflow_handle* h, int32_t k_lo, int32_t n, double* out);
int sflow_put_rows(sflow_handle* h, int32_t k_lo, int32_t n, const double* in);

/* Build information ("fp64+fp32 sm_103a ..."). */
const char* sflow_build_info(void);

#ifdef __cplusplus
}
#endif
#endif /* SFLOW_H */

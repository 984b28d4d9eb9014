// sflow_host.h -- host-side set-up shared by the FP64 and FP32 solvers.
#pragma once
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/sflow.h"

namespace sflow {

// Everything the device solver needs, derived on the host from
// SflowParams + B_cent the way the reference's init sequence does
// (read_param, init_grid, topography_reconstruction, init_source).
struct HostSetup {
  SflowParams p;
  int nx = 0, ny = 0, nv = 0, ns = 0, nrk = 0;
  double dx = 0, dy = 0, eps_sing = 0, eps_sing4 = 0;
  double rho_a_amb = 0, kin_visc_c = 0, rho_c_sub = 0, T_erodible = 300.0;
  double h_source = 0, time_param[4] = {0, 0, 0, 0};
  double src_rho_m = 0, src_cp_mix = 0;
  double pi_g = 0;
  // tableau (solver_2d.f90:399-487), row-major [i][j] of a 4x4 block
  double a_tilde[16] = {0}, a_dirk[16] = {0}, omega_tilde[4] = {0}, omega[4] = {0};
  int take_last = 0;
  // per-cell fields, row-major [k][j] (k = y index)
  std::vector<double> Bx, By, Bxx, Bxy, Byy, gc, dgcx, dgcy;
  std::vector<uint8_t> cflags;                 // source_cell | E<<2 | W<<3 | N<<4 | S<<5 | BSRC<<7
  std::vector<double> arc_perim, arc_nx, arc_ny;
  int64_t ring_cells = 0;
  // update_erosion_deposition_cell runs (settling, entrainment or erosion)
  int exchange = 0;
  // erosion of the erodible layer (inpout_2d.f90:1818-1990)
  double erodible_porosity = 0, coeff_porosity = 0;
  double erodible_fract[SFLOW_MAX_SOLID] = {0, 0, 0, 0};
  double erodible_init = 0;            // uniform initial erodible thickness
  // bottom radial source: fraction of each cell inside the source ellipse
  // (compute_cell_fract, geometry_2d.f90:1899-1994), 0 outside
  std::vector<double> cell_fract;
  int64_t bottom_cells = 0;
  // vulnerability table levels (inpout_2d.f90:3792-3870)
  int n_thk = 0, n_dyn = 0;
  double thk_levels[SFLOW_MAX_LEVELS] = {0}, dyn_levels[SFLOW_MAX_LEVELS] = {0};
  // topography (B_cent), row-major
  std::vector<double> B;
  // row slab of a larger domain (host_setup_rows): rows row0 .. row0+ny-1
  // of it, of which own_lo .. own_hi-1 (local) are this domain's own
  int row0 = 0, own_lo = 0, own_hi = 0;
};

constexpr uint8_t kFlagNodata = 0x40;   // B_nodata cell
constexpr uint8_t kFlagBottom = 0x80;   // cell fraction of the bottom source > 0

// Validates p and fills s; returns 0 or SFLOW_EINVAL with a message in err.
// host_topography = false leaves the topography terms (Bx ... dgcy) empty:
// the solver then derives them from B on the device (the same arithmetic,
// operation by operation), which is how batched runs are set up in bulk.
int host_setup(const SflowParams* p, const double* B_cent, HostSetup& s, std::string& err,
               bool host_topography = true);
// host_setup of the whole domain, then only rows k0 .. k0+rows-1 kept (every
// derived field computed on the whole domain, so a slab's cells carry the
// same topography terms, inlet geometry and flags as in the whole run);
// own_lo .. own_hi-1 are the slab's own rows (local indices)
int host_setup_rows(const SflowParams* p, const double* B_cent, int k0, int rows, int own_lo, int own_hi,
                    HostSetup& s, std::string& err);

// Reference mixt_var (constitutive_2d.f90:1342-1492) in FP64 on the host,
// used for constants of the run (inlet state).
void host_mixt_var(const HostSetup& s, const double* qp, double* rho_m, double* cp_mix);

// Largest float not greater than x: `f > thr` on floats equals the FP64
// test `(double)f > x`.
float float_below(double x);

class SolverBase {
 public:
  virtual ~SolverBase() {}
  virtual int upload(const double* q_aos) = 0;
  virtual int put(const double* q_aos) = 0;
  virtual int set_clock(double t, double dt_old, double dt_old_old) = 0;
  virtual int advance_timed(int64_t steps, int flush, double* ms) = 0;
  virtual int profile_kernels(int64_t steps, int flush, double* ms4) = 0;
  virtual int download(double* q_aos) = 0;
  virtual int download_qp(double* qp_aos) = 0;
  virtual int download_maps(double* h, double* p, double* v) = 0;
  virtual int download_deposit(double* out) = 0;
  virtual int download_phys(double* out) = 0;
  virtual int upload_deposit(const double* in) = 0;
  // which 0: accumulated erosion, 1: erodible layer (n_solid planes)
  virtual int download_erosion(int which, double* out) = 0;
  virtual int download_topography(double* out) = 0;
  virtual int set_erodible(const double* thickness) = 0;
  virtual int set_nodata(const uint8_t* nodata) = 0;
  virtual int vuln_table(int* n_thk, int* n_dyn, uint8_t* out) = 0;
  // rows k_lo .. k_lo+n-1 of the conservative state, reference layout
  virtual int get_rows(int k_lo, int n, double* out) = 0;
  virtual int put_rows(int k_lo, int n, const double* in) = 0;
  virtual int upload_maps(const double* h, const double* p, const double* v) = 0;
  virtual int set_output_time(double t_output) = 0;
  virtual int check_solve(int solve_all) = 0;
  virtual int timestep(double* dt_out) = 0;
  virtual int imex_rk(double t, double dt) = 0;
  virtual int erosion_deposition(double dt) = 0;
  virtual int post_step(SflowStepStats* s) = 0;
  virtual int step() = 0;
  virtual int advance(double t_stop, int64_t max_steps, SflowStepStats* s) = 0;
  virtual int stats(SflowStepStats* s) = 0;
  virtual int status(uint32_t* f) = 0;
  virtual int clear_status() = 0;
  virtual int64_t launches() const = 0;
  virtual int64_t device_bytes() const = 0;
  virtual int newton_stats(int64_t* total, int* maxit) = 0;
  virtual int64_t cells_total() = 0;
  // active-cell updates of dry border tiles (counted, skipped by the kernels)
  virtual int64_t border_total() = 0;
  virtual int tile_shape() const = 0;
  virtual int set_tile_shape(int tile_h) = 0;
  virtual int autotune(int64_t steps, int* best, double* ms_per_mcu) = 0;
  virtual const char* error() const = 0;
};

SolverBase* make_solver_fp64(const HostSetup& s, std::string& err);
SolverBase* make_solver_fp32(const HostSetup& s, std::string& err);

// A batched run whose device state is built but which has not joined the
// batch yet (BatchBase::prepare / commit).
struct PreparedRun {
  virtual ~PreparedRun() {}
};

// Many independent runs advanced together (sflow_batch.cuh).
class BatchBase {
 public:
  virtual ~BatchBase() {}
  // sflow_batch_submit_many: prepare() builds a run's device state and may
  // run on several threads at once (each first calls bind_thread() to
  // select the batch's device); commit() admits prepared runs in order on
  // the submitting thread.  A prepared run that is not admitted (SFLOW_EBUSY
  // and the like) is released with its unique_ptr.
  virtual std::unique_ptr<PreparedRun> prepare(HostSetup&& hs, const double* q_aos, int64_t max_steps, int* rc,
                                               std::string* err) = 0;
  virtual int commit(std::unique_ptr<PreparedRun> pr, int* id) = 0;
  virtual void bind_thread() = 0;
  // host memory the device maps (pinned): runs whose q lives there are
  // built on worker threads; the device reads other host memory fastest
  // from one thread at a time, so those runs are built by the submitter
  virtual bool device_mapped(const void* p) const = 0;
  // takes hs over (its host arrays move into the run)
  virtual int submit(HostSetup&& hs, const double* q_aos, int64_t max_steps, int* id) = 0;
  // start (on) or end of a bulk submission: prepare() then tracks the free
  // device memory across its builds from one fresh query
  virtual void set_bulk(bool on) = 0;
  virtual int advance(int64_t steps, int* finished) = 0;
  // the same with the device time of the steps (CUDA events across the
  // groups' streams) in *ms
  virtual int advance_timed(int64_t steps, int* finished, double* ms) = 0;
  // steps one by one with the device time of each of the five kernels
  virtual int profile_kernels(int64_t steps, int* finished, double* ms5) = 0;
  // asynchronous form of advance: launch returns at once, wait synchronises
  virtual int launch(int64_t steps) = 0;
  virtual int wait(int* finished) = 0;
  virtual int poll(int id, SflowStepStats* s, int* done) = 0;
  virtual int counters(int id, int64_t* cells, int64_t* steps) = 0;
  virtual int border_updates(int id, int64_t* n) = 0;
  virtual int download(int id, double* q_aos) = 0;
  virtual int collect(int id, double* q_aos) = 0;
  // collect() of n runs: the downloads on `threads` host threads (each run
  // on its own stream), the slots freed in order; status[i] per run
  virtual int collect_many(int n, const int32_t* ids, double* const* q_aos, int threads, int32_t* status) = 0;
  virtual int live() const = 0;
  virtual int64_t launches() const = 0;
  virtual int tile_shape() const = 0;
  virtual int set_tile_shape(int tile_h) = 0;
  virtual int set_memory_limit(int64_t bytes) = 0;
  virtual const char* error() const = 0;
};

BatchBase* make_batch_fp64(int max_runs, int64_t max_tiles, std::string& err);
BatchBase* make_batch_fp32(int max_runs, int64_t max_tiles, std::string& err);
// self-check of the integer-pipe float <-> double conversions (sflow_fp32.cu)
int check_conversions(long long n, unsigned long long seed, long long* mismatches);
// the FP64 pow / log / cos of sflow_math.h (and CUDA's) on the device (sflow_fp64.cu)
int eval_math(int which, long long n, const double* x, const double* y, double* out);

}  // namespace sflow

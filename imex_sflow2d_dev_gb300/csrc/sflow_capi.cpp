// sflow_capi.cpp -- the extern "C" boundary declared in include/sflow.h.
#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sflow.h"
#include "sflow_host.h"

using sflow::BatchBase;
using sflow::HostSetup;
using sflow::SolverBase;

struct sflow_batch {
  BatchBase* impl = nullptr;
  int precision = 0;
};

struct sflow_setup {
  HostSetup hs;
  bool spent = false;   // its arrays went to a run (sflow_batch_submit_setup_take)
};

struct sflow_handle {
  SolverBase* solver = nullptr;
  int nx = 0, ny = 0, nv = 0;
  int precision = 0;
};

static thread_local std::string g_err;

static int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CHECK_HANDLE(h)                                         \
  do {                                                          \
    if (!(h) || !(h)->solver) return fail(SFLOW_EINVAL, "null handle"); \
  } while (0)

static std::string last_solver_error(const sflow_handle* h);

extern "C" {

const char* sflow_last_error(void) { return g_err.c_str(); }

int sflow_batch_create(int32_t precision, int32_t max_runs, int64_t max_cells, sflow_batch** out) {
  if (!out) return fail(SFLOW_EINVAL, "out is NULL");
  *out = nullptr;
  if (precision != SFLOW_PREC_FP32 && precision != SFLOW_PREC_FP64) return fail(SFLOW_EINVAL, "unknown precision");
  if (max_cells < 1) return fail(SFLOW_EINVAL, "max_cells must be positive");
  std::string err;
  // tile lists hold one entry per tile (32 x 8 cells at the smallest
  // compiled height); small runs waste part of a tile, so the capacity
  // allows for twice the cells
  const int64_t max_tiles = 2 * ((max_cells + 255) / 256) + 1024;
  BatchBase* b = (precision == SFLOW_PREC_FP32) ? sflow::make_batch_fp32(max_runs, max_tiles, err)
                                                : sflow::make_batch_fp64(max_runs, max_tiles, err);
  if (!b) return fail(SFLOW_EINVAL, err);
  sflow_batch* h = new (std::nothrow) sflow_batch;
  if (!h) {
    delete b;
    return fail(SFLOW_ENOMEM, "out of host memory");
  }
  h->impl = b;
  h->precision = precision;
  *out = h;
  g_err.clear();
  return SFLOW_OK;
}

void sflow_batch_destroy(sflow_batch* b) {
  if (!b) return;
  delete b->impl;
  delete b;
}

#define BATCH_CHECK(b)                                                   \
  do {                                                                   \
    if (!(b) || !(b)->impl) return fail(SFLOW_EINVAL, "null batch");     \
  } while (0)
#define BATCH_FORWARD(b, expr)                                           \
  do {                                                                   \
    int rc_ = (expr);                                                    \
    if (rc_ < 0) return fail(rc_, (b)->impl->error());                   \
    return rc_;                                                          \
  } while (0)

int sflow_batch_submit(sflow_batch* b, const SflowParams* p, const double* B_cent, const double* q_aos,
                       int64_t max_steps, int32_t* run_id) {
  BATCH_CHECK(b);
  if (!p || !q_aos || !run_id) return fail(SFLOW_EINVAL, "NULL argument");
  if (p->precision != b->precision) return fail(SFLOW_EINVAL, "run precision differs from the batch precision");
  HostSetup s;
  std::string err;
  int rc = sflow::host_setup(p, B_cent, s, err);
  if (rc != SFLOW_OK) return fail(rc, err);
  int id = -1;
  rc = b->impl->submit(std::move(s), q_aos, max_steps, &id);
  if (rc < 0) return fail(rc, b->impl->error());
  *run_id = id;
  return SFLOW_OK;
}

int sflow_setup_create(const SflowParams* p, const double* B_cent, sflow_setup** out) {
  if (!p || !out) return fail(SFLOW_EINVAL, "NULL argument");
  *out = nullptr;
  sflow_setup* s = new (std::nothrow) sflow_setup();
  if (!s) return fail(SFLOW_ENOMEM, "host allocation failed");
  std::string err;
  const int rc = sflow::host_setup(p, B_cent, s->hs, err);
  if (rc != SFLOW_OK) {
    delete s;
    return fail(rc, err);
  }
  *out = s;
  return SFLOW_OK;
}

void sflow_setup_destroy(sflow_setup* s) { delete s; }

int sflow_batch_submit_setup(sflow_batch* b, const sflow_setup* s, const double* q_aos, int64_t max_steps,
                             int32_t* run_id) {
  BATCH_CHECK(b);
  if (!s || !q_aos || !run_id) return fail(SFLOW_EINVAL, "NULL argument");
  if (s->spent) return fail(SFLOW_EINVAL, "the setup was handed to a run");
  if (s->hs.p.precision != b->precision) return fail(SFLOW_EINVAL, "run precision differs from the batch precision");
  int id = -1;
  HostSetup copy = s->hs;   // a setup can be submitted again
  const int rc = b->impl->submit(std::move(copy), q_aos, max_steps, &id);
  if (rc < 0) return fail(rc, b->impl->error());
  *run_id = id;
  return SFLOW_OK;
}

int sflow_batch_submit_many(sflow_batch* b, int32_t n, const SflowParams* params, const double* const* B_cent,
                            const double* const* q_aos, const int64_t* max_steps, int32_t* run_ids,
                            int32_t threads) {
  BATCH_CHECK(b);
  if (n < 0) return fail(SFLOW_EINVAL, "n must be >= 0");
  if (n > 0 && (!params || !B_cent || !q_aos || !run_ids)) return fail(SFLOW_EINVAL, "NULL argument");
  for (int32_t i = 0; i < n; ++i) run_ids[i] = -1;
  if (n == 0) return SFLOW_OK;
  int nt = threads > 0 ? threads : (int)std::thread::hardware_concurrency();
  nt = std::min(std::max(1, std::min(nt, 64)), (int)n);
  const int window = 2 * nt;

  // Each run is set up on the host and built on the device by a worker
  // (BatchBase::prepare), then admitted in run order by this thread.
  struct Item {
    std::unique_ptr<sflow::PreparedRun> run;   // built on the device (pinned q)
    HostSetup hs;                              // host set-up only (other q)
    int rc = SFLOW_OK;
    std::string err;
    bool ready = false;
  };
  std::vector<Item> items((size_t)n);
  auto make = [&](int i, Item& it, bool build) {
    try {
      HostSetup hs;
      if (!B_cent[i] || !q_aos[i]) {
        it.rc = SFLOW_EINVAL;
        it.err = "NULL argument";
      } else if (params[i].precision != b->precision) {
        it.rc = SFLOW_EINVAL;
        it.err = "run precision differs from the batch precision";
      } else {
        // topography terms on the device (Solver::init): the host part is
        // validation, inlet geometry and flags
        it.rc = sflow::host_setup(&params[i], B_cent[i], hs, it.err, false);
      }
      if (it.rc == SFLOW_OK && build && b->impl->device_mapped(q_aos[i])) {
        it.run = b->impl->prepare(std::move(hs), q_aos[i], max_steps ? max_steps[i] : 0, &it.rc, &it.err);
        if (!it.run && it.rc == SFLOW_OK) it.rc = SFLOW_ECUDA;
      } else if (it.rc == SFLOW_OK) {
        it.hs = std::move(hs);
      }
    } catch (const std::bad_alloc&) {
      it.run.reset();
      it.hs = HostSetup();
      it.rc = SFLOW_ENOMEM;
      it.err = "host allocation failed";
    }
  };
  std::mutex mu;
  std::condition_variable cv_ready, cv_room;
  int next = 0, taken = 0;
  auto work = [&]() {
    b->impl->bind_thread();
    for (;;) {
      int i;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_room.wait(lk, [&] { return next >= n || next < taken + window; });
        if (next >= n) return;
        i = next++;
      }
      Item tmp;
      make(i, tmp, true);
      {
        std::lock_guard<std::mutex> lk(mu);
        items[(size_t)i] = std::move(tmp);
        items[(size_t)i].ready = true;
      }
      cv_ready.notify_all();
    }
  };
  b->impl->set_bulk(true);
  std::vector<std::thread> pool;
  try {
    for (int t = 0; t < nt; ++t) pool.emplace_back(work);
  } catch (const std::exception&) {
    // fewer threads than asked (at worst none: the runs are made below)
  }
  int first_rc = SFLOW_OK;
  std::string first_err;
  for (int32_t i = 0; i < n; ++i) {
    Item it;
    if (pool.empty()) {
      make(i, it, false);
    } else {
      std::unique_lock<std::mutex> lk(mu);
      cv_ready.wait(lk, [&] { return items[(size_t)i].ready; });
      it = std::move(items[(size_t)i]);
      items[(size_t)i] = Item();
      taken = i + 1;
    }
    cv_room.notify_all();
    int rc = it.rc;
    std::string err = it.err;
    if (rc == SFLOW_OK) {
      int id = -1;
      rc = it.run ? b->impl->commit(std::move(it.run), &id)
                  : b->impl->submit(std::move(it.hs), q_aos[i], max_steps ? max_steps[i] : 0, &id);
      if (rc < 0) err = b->impl->error();
      else run_ids[i] = id;
    }
    if (rc < 0 && first_rc == SFLOW_OK) {
      first_rc = rc;
      first_err = "run " + std::to_string(i) + ": " + err;
    }
  }
  for (auto& t : pool) t.join();
  b->impl->set_bulk(false);
  if (first_rc != SFLOW_OK) return fail(first_rc, first_err);
  return SFLOW_OK;
}

int sflow_batch_submit_setup_take(sflow_batch* b, sflow_setup* s, const double* q_aos, int64_t max_steps,
                                  int32_t* run_id) {
  BATCH_CHECK(b);
  if (!s || !q_aos || !run_id) return fail(SFLOW_EINVAL, "NULL argument");
  if (s->spent) return fail(SFLOW_EINVAL, "the setup was handed to a run");
  if (s->hs.p.precision != b->precision) return fail(SFLOW_EINVAL, "run precision differs from the batch precision");
  const size_t n = (size_t)s->hs.nx * s->hs.ny;
  int id = -1;
  const int rc = b->impl->submit(std::move(s->hs), q_aos, max_steps, &id);
  // the arrays move into the run once admission passed (B is always set up)
  if (rc == SFLOW_OK || s->hs.B.size() != n) s->spent = true;
  if (rc < 0) return fail(rc, b->impl->error());
  *run_id = id;
  return SFLOW_OK;
}

int sflow_batch_collect_many(sflow_batch* b, int32_t n, const int32_t* ids, double* const* q_aos, int32_t threads,
                             int32_t* status) {
  BATCH_CHECK(b);
  if (n < 0) return fail(SFLOW_EINVAL, "n must be >= 0");
  if (n > 0 && (!ids || !status)) return fail(SFLOW_EINVAL, "NULL argument");
  if (n == 0) return SFLOW_OK;
  const int rc = b->impl->collect_many(n, ids, q_aos, threads, status);
  if (rc < 0) return fail(rc, b->impl->error());
  return SFLOW_OK;
}

int sflow_batch_launch(sflow_batch* b, int64_t steps) {
  BATCH_CHECK(b);
  if (steps < 0) return fail(SFLOW_EINVAL, "steps must be >= 0");
  BATCH_FORWARD(b, b->impl->launch(steps));
}

int sflow_batch_wait(sflow_batch* b, int32_t* finished) {
  BATCH_CHECK(b);
  int nf = 0;
  const int rc = b->impl->wait(&nf);
  if (rc < 0) return fail(rc, b->impl->error());
  if (finished) *finished = nf;
  return SFLOW_OK;
}

int sflow_batch_advance_timed(sflow_batch* b, int64_t steps, int32_t* finished, double* device_ms) {
  BATCH_CHECK(b);
  if (steps < 0) return fail(SFLOW_EINVAL, "steps must be >= 0");
  if (!device_ms) return fail(SFLOW_EINVAL, "device_ms is NULL");
  int nf = 0;
  int rc = b->impl->advance_timed(steps, &nf, device_ms);
  if (rc < 0) return fail(rc, b->impl->error());
  if (finished) *finished = nf;
  return SFLOW_OK;
}

int sflow_batch_profile_kernels(sflow_batch* b, int64_t steps, int32_t* finished, double* ms5) {
  BATCH_CHECK(b);
  if (steps < 0) return fail(SFLOW_EINVAL, "steps must be >= 0");
  if (!ms5) return fail(SFLOW_EINVAL, "ms5 is NULL");
  int nf = 0;
  int rc = b->impl->profile_kernels(steps, &nf, ms5);
  if (rc < 0) return fail(rc, b->impl->error());
  if (finished) *finished = nf;
  return SFLOW_OK;
}

int sflow_batch_dry_border_updates(sflow_batch* b, int32_t run_id, int64_t* n) {
  BATCH_CHECK(b);
  if (!n) return fail(SFLOW_EINVAL, "n is NULL");
  BATCH_FORWARD(b, b->impl->border_updates(run_id, n));
}

int sflow_batch_advance(sflow_batch* b, int64_t steps, int32_t* finished) {
  BATCH_CHECK(b);
  if (steps < 0) return fail(SFLOW_EINVAL, "steps must be >= 0");
  int nf = 0;
  int rc = b->impl->advance(steps, &nf);
  if (rc < 0) return fail(rc, b->impl->error());
  if (finished) *finished = nf;
  return SFLOW_OK;
}

int sflow_batch_poll(sflow_batch* b, int32_t run_id, SflowStepStats* stats, int32_t* done) {
  BATCH_CHECK(b);
  int d = 0;
  int rc = b->impl->poll(run_id, stats, &d);
  if (rc < 0) return fail(rc, b->impl->error());
  if (done) *done = d;
  return SFLOW_OK;
}

int sflow_batch_counters(sflow_batch* b, int32_t run_id, int64_t* cell_updates, int64_t* steps) {
  BATCH_CHECK(b);
  BATCH_FORWARD(b, b->impl->counters(run_id, cell_updates, steps));
}

int sflow_batch_download(sflow_batch* b, int32_t run_id, double* q_aos) {
  BATCH_CHECK(b);
  if (!q_aos) return fail(SFLOW_EINVAL, "q is NULL");
  BATCH_FORWARD(b, b->impl->download(run_id, q_aos));
}

int sflow_batch_collect(sflow_batch* b, int32_t run_id, double* q_aos) {
  BATCH_CHECK(b);
  BATCH_FORWARD(b, b->impl->collect(run_id, q_aos));
}

int32_t sflow_batch_live(const sflow_batch* b) { return (b && b->impl) ? b->impl->live() : 0; }

int64_t sflow_batch_launch_count(const sflow_batch* b) { return (b && b->impl) ? b->impl->launches() : 0; }

int sflow_batch_set_tile_shape(sflow_batch* b, int32_t tile_h) {
  BATCH_CHECK(b);
  BATCH_FORWARD(b, b->impl->set_tile_shape(tile_h));
}

int sflow_batch_set_memory_limit(sflow_batch* b, int64_t bytes) {
  BATCH_CHECK(b);
  BATCH_FORWARD(b, b->impl->set_memory_limit(bytes));
}

int sflow_batch_get_tile_shape(const sflow_batch* b, int32_t* tile_h) {
  if (!b || !b->impl) return fail(SFLOW_EINVAL, "null batch");
  if (!tile_h) return fail(SFLOW_EINVAL, "tile_h is NULL");
  *tile_h = b->impl->tile_shape();
  return SFLOW_OK;
}

int sflow_check_conversions(int64_t n, uint64_t seed, int64_t* mismatches) {
  if (!mismatches || n < 0) return fail(SFLOW_EINVAL, "bad argument");
  long long m = 0;
  const int rc = sflow::check_conversions((long long)n, (unsigned long long)seed, &m);
  if (rc != SFLOW_OK) return fail(rc, "conversion check failed to run");
  *mismatches = (int64_t)m;
  return SFLOW_OK;
}

int sflow_eval_math(int32_t which, int64_t n, const double* x, const double* y, double* out) {
  if (which < 0 || which > 5 || n < 0 || (n > 0 && (!x || !out)) || ((which == 0 || which == 3) && n > 0 && !y))
    return fail(SFLOW_EINVAL, "bad argument");
  const int rc = sflow::eval_math(which, (long long)n, x, y, out);
  if (rc != SFLOW_OK) return fail(rc, "device evaluation failed");
  return SFLOW_OK;
}

int sflow_tile_shapes(int32_t precision, int32_t* heights, int32_t capacity, int32_t* count) {
  if (!count) return fail(SFLOW_EINVAL, "count is NULL");
  if (precision != SFLOW_PREC_FP32 && precision != SFLOW_PREC_FP64) return fail(SFLOW_EINVAL, "unknown precision");
  // the compiled heights, in the autotuner's candidate order
  const int32_t fp32[3] = {8, 16, 4}, fp64[1] = {8};
  const int32_t* v = (precision == SFLOW_PREC_FP32) ? fp32 : fp64;
  const int32_t n = (precision == SFLOW_PREC_FP32) ? 3 : 1;
  for (int32_t i = 0; i < n && i < capacity && heights; ++i) heights[i] = v[i];
  *count = n;
  return SFLOW_OK;
}

const char* sflow_build_info(void) {
  return "sflow GB300: FP64 plain form + FP32 bulk form, N_RK=2, KT fluxes, sm_103a";
}

void sflow_default_params(SflowParams* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->abi_version = SFLOW_ABI_VERSION;
  p->precision = SFLOW_PREC_FP64;
  p->comp_cells_x = 1000;
  p->comp_cells_y = 1;
  p->cell_size = 1.0e-3;
  p->gas_flag = 1;
  p->solver_scheme = SFLOW_SCHEME_KT;
  p->n_rk = 2;
  p->dt0 = 1.0e-4;
  p->max_dt = 1.0e-3;
  p->cfl = 0.24;
  p->theta = 1.0;
  p->reconstr_coeff = 1.0;
  for (int i = 0; i < SFLOW_MAX_VARS; ++i) p->limiter[i] = 1;
  for (int s = 0; s < 4; ++s)
    for (int i = 0; i < SFLOW_MAX_VARS; ++i) {
      p->bc[s][i].flag = 1;
      p->bc[s][i].value = 0.0;
    }
  p->grav = 9.81;
  p->maximum_solid_packing = 0.64;
  p->A_drag = -1.0;
  p->B_drag = -1.0;
  p->r2_source = -1.0;
  p->arc_width_source = 360.0;
  p->h_source = -1.0;
  p->mfr_source = -1.0;
  for (int i = 0; i < 4; ++i) p->time_param[i] = -1.0;
  p->t_end = 5.0e-2;
  p->dt_output = 5.0e-3;
  for (int i = 0; i < SFLOW_MAX_LEVELS; ++i) p->thickness_levels[i] = p->dyn_pres_levels[i] = -1.0;
  p->erodible_porosity = p->T_erodible = p->initial_erodible_thickness = -1.0;
  for (int i = 0; i < SFLOW_MAX_SOLID; ++i) p->erodible_fract[i] = -1.0;
  for (int i = 0; i < SFLOW_MAX_INTERVALS; ++i) p->t_intervals[i] = p->vel_intervals[i] = -1.0;
  p->mu_s = p->mu_2 = p->I_0 = p->muI_inf = -1.0;
}

static int create_from(const SflowParams* p, HostSetup& s, sflow_handle** out);

int sflow_create(const SflowParams* p, const double* B_cent, sflow_handle** out) {
  if (!out) return fail(SFLOW_EINVAL, "out is NULL");
  *out = nullptr;
  HostSetup s;
  std::string err;
  int rc = sflow::host_setup(p, B_cent, s, err);
  if (rc != SFLOW_OK) return fail(rc, err);
  return create_from(p, s, out);
}

int sflow_create_rows(const SflowParams* p, const double* B_cent, int32_t k0, int32_t rows, int32_t own_lo,
                      int32_t own_hi, sflow_handle** out) {
  if (!out) return fail(SFLOW_EINVAL, "out is NULL");
  *out = nullptr;
  HostSetup s;
  std::string err;
  int rc = sflow::host_setup_rows(p, B_cent, k0, rows, own_lo, own_hi, s, err);
  if (rc != SFLOW_OK) return fail(rc, err);
  return create_from(p, s, out);
}

static int create_from(const SflowParams* p, HostSetup& s, sflow_handle** out) {
  std::string err;
  SolverBase* sv = (p->precision == SFLOW_PREC_FP32) ? sflow::make_solver_fp32(s, err)
                                                     : sflow::make_solver_fp64(s, err);
  if (!sv) return fail(SFLOW_ECUDA, err.empty() ? "device set-up failed" : err);
  sflow_handle* h = new (std::nothrow) sflow_handle;
  if (!h) {
    delete sv;
    return fail(SFLOW_ENOMEM, "out of host memory");
  }
  h->solver = sv;
  h->nx = s.nx;
  h->ny = s.ny;
  h->nv = s.nv;
  h->precision = p->precision;
  *out = h;
  g_err.clear();
  return SFLOW_OK;
}

void sflow_destroy(sflow_handle* h) {
  if (!h) return;
  delete h->solver;
  delete h;
}

#define FORWARD(expr)                                                  \
  do {                                                                 \
    int rc_ = (expr);                                                  \
    if (rc_ < 0) return fail(rc_, last_solver_error(h));               \
    return rc_;                                                        \
  } while (0)

}  // extern "C"

static std::string last_solver_error(const sflow_handle* h) {
  const char* e = h->solver->error();
  return (e && *e) ? std::string(e) : std::string("solver error");
}

extern "C" {

int sflow_upload_q(sflow_handle* h, const double* q) {
  CHECK_HANDLE(h);
  if (!q) return fail(SFLOW_EINVAL, "q is NULL");
  FORWARD(h->solver->upload(q));
}
int sflow_put_q(sflow_handle* h, const double* q) {
  CHECK_HANDLE(h);
  if (!q) return fail(SFLOW_EINVAL, "q is NULL");
  FORWARD(h->solver->put(q));
}
int sflow_set_clock(sflow_handle* h, double t, double dt_old, double dt_old_old) {
  CHECK_HANDLE(h);
  FORWARD(h->solver->set_clock(t, dt_old, dt_old_old));
}
int sflow_advance_timed(sflow_handle* h, int64_t steps, int32_t flush_l2, double* ms) {
  CHECK_HANDLE(h);
  if (!ms || steps < 0) return fail(SFLOW_EINVAL, "bad arguments");
  FORWARD(h->solver->advance_timed(steps, flush_l2, ms));
}
int sflow_profile_kernels(sflow_handle* h, int64_t steps, int32_t flush_l2, double* ms4) {
  CHECK_HANDLE(h);
  if (!ms4 || steps < 0) return fail(SFLOW_EINVAL, "bad arguments");
  FORWARD(h->solver->profile_kernels(steps, flush_l2, ms4));
}
int sflow_download_q(sflow_handle* h, double* q) {
  CHECK_HANDLE(h);
  if (!q) return fail(SFLOW_EINVAL, "q is NULL");
  FORWARD(h->solver->download(q));
}
int sflow_download_qp(sflow_handle* h, double* qp) {
  CHECK_HANDLE(h);
  if (!qp) return fail(SFLOW_EINVAL, "qp is NULL");
  FORWARD(h->solver->download_qp(qp));
}
int sflow_download_phys(sflow_handle* h, double* out) {
  CHECK_HANDLE(h);
  if (!out) return fail(SFLOW_EINVAL, "out is NULL");
  FORWARD(h->solver->download_phys(out));
}

int sflow_download_deposit(sflow_handle* h, double* out) {
  CHECK_HANDLE(h);
  if (!out) return fail(SFLOW_EINVAL, "out is NULL");
  FORWARD(h->solver->download_deposit(out));
}

int sflow_upload_deposit(sflow_handle* h, const double* in) {
  CHECK_HANDLE(h);
  if (!in) return fail(SFLOW_EINVAL, "in is NULL");
  FORWARD(h->solver->upload_deposit(in));
}

int sflow_get_rows(sflow_handle* h, int32_t k_lo, int32_t n, double* out) {
  CHECK_HANDLE(h);
  if (!out) return fail(SFLOW_EINVAL, "out is NULL");
  FORWARD(h->solver->get_rows(k_lo, n, out));
}

int sflow_put_rows(sflow_handle* h, int32_t k_lo, int32_t n, const double* in) {
  CHECK_HANDLE(h);
  if (!in) return fail(SFLOW_EINVAL, "in is NULL");
  FORWARD(h->solver->put_rows(k_lo, n, in));
}

int sflow_download_erosion(sflow_handle* h, double* out) {
  CHECK_HANDLE(h);
  if (!out) return fail(SFLOW_EINVAL, "out is NULL");
  FORWARD(h->solver->download_erosion(0, out));
}
int sflow_download_erodible(sflow_handle* h, double* out) {
  CHECK_HANDLE(h);
  if (!out) return fail(SFLOW_EINVAL, "out is NULL");
  FORWARD(h->solver->download_erosion(1, out));
}
int sflow_set_erodible(sflow_handle* h, const double* thickness) {
  CHECK_HANDLE(h);
  if (!thickness) return fail(SFLOW_EINVAL, "thickness is NULL");
  FORWARD(h->solver->set_erodible(thickness));
}
int sflow_download_topography(sflow_handle* h, double* B_cent) {
  CHECK_HANDLE(h);
  if (!B_cent) return fail(SFLOW_EINVAL, "B_cent is NULL");
  FORWARD(h->solver->download_topography(B_cent));
}
int sflow_set_nodata(sflow_handle* h, const uint8_t* nodata) {
  CHECK_HANDLE(h);
  FORWARD(h->solver->set_nodata(nodata));
}
int sflow_vuln_table_size(sflow_handle* h, int32_t* n_thk, int32_t* n_dyn) {
  CHECK_HANDLE(h);
  int a = 0, b = 0;
  int rc = h->solver->vuln_table(&a, &b, nullptr);
  if (n_thk) *n_thk = a;
  if (n_dyn) *n_dyn = b;
  return rc;
}
int sflow_download_vuln_table(sflow_handle* h, uint8_t* out) {
  CHECK_HANDLE(h);
  if (!out) return fail(SFLOW_EINVAL, "out is NULL");
  FORWARD(h->solver->vuln_table(nullptr, nullptr, out));
}

int sflow_upload_maps(sflow_handle* h, const double* hmax, const double* pdynmax, const double* mod_vel_max) {
  CHECK_HANDLE(h);
  FORWARD(h->solver->upload_maps(hmax, pdynmax, mod_vel_max));
}

int sflow_set_output_time(sflow_handle* h, double t_output) {
  CHECK_HANDLE(h);
  FORWARD(h->solver->set_output_time(t_output));
}

int sflow_download_maps(sflow_handle* h, double* a, double* b, double* c) {
  CHECK_HANDLE(h);
  FORWARD(h->solver->download_maps(a, b, c));
}
int sflow_check_solve(sflow_handle* h, int32_t solve_all) {
  CHECK_HANDLE(h);
  FORWARD(h->solver->check_solve(solve_all));
}
int sflow_timestep(sflow_handle* h, double* dt) {
  CHECK_HANDLE(h);
  FORWARD(h->solver->timestep(dt));
}
int sflow_imex_rk(sflow_handle* h, double t, double dt) {
  CHECK_HANDLE(h);
  if (!(dt > 0.0)) return fail(SFLOW_EINVAL, "dt must be > 0");
  FORWARD(h->solver->imex_rk(t, dt));
}
int sflow_erosion_deposition(sflow_handle* h, double dt) {
  CHECK_HANDLE(h);
  FORWARD(h->solver->erosion_deposition(dt));
}
int sflow_post_step(sflow_handle* h, SflowStepStats* s) {
  CHECK_HANDLE(h);
  FORWARD(h->solver->post_step(s));
}
int sflow_step(sflow_handle* h) {
  CHECK_HANDLE(h);
  int rc = h->solver->step();
  if (rc < 0) return fail(rc, last_solver_error(h));
  uint32_t f = 0;
  rc = h->solver->status(&f);
  if (rc < 0) return fail(rc, last_solver_error(h));
  return (int)f;
}
int sflow_advance(sflow_handle* h, double t_stop, int64_t max_steps, SflowStepStats* s) {
  CHECK_HANDLE(h);
  int rc = h->solver->advance(t_stop, max_steps, s);
  if (rc < 0) return fail(rc, last_solver_error(h));
  uint32_t f = 0;
  rc = h->solver->status(&f);
  if (rc < 0) return fail(rc, last_solver_error(h));
  return (int)f;
}
int sflow_get_stats(sflow_handle* h, SflowStepStats* s) {
  CHECK_HANDLE(h);
  if (!s) return fail(SFLOW_EINVAL, "stats is NULL");
  FORWARD(h->solver->stats(s));
}
int sflow_status(sflow_handle* h, uint32_t* f) {
  CHECK_HANDLE(h);
  if (!f) return fail(SFLOW_EINVAL, "flags is NULL");
  FORWARD(h->solver->status(f));
}
int sflow_clear_status(sflow_handle* h) {
  CHECK_HANDLE(h);
  FORWARD(h->solver->clear_status());
}
int sflow_set_tile_shape(sflow_handle* h, int32_t tile_h) {
  CHECK_HANDLE(h);
  FORWARD(h->solver->set_tile_shape(tile_h));
}
int sflow_get_tile_shape(const sflow_handle* h, int32_t* tile_h) {
  CHECK_HANDLE(h);
  if (!tile_h) return fail(SFLOW_EINVAL, "tile_h is NULL");
  *tile_h = h->solver->tile_shape();
  return SFLOW_OK;
}
int sflow_autotune(sflow_handle* h, int64_t steps_per_shape, int32_t* best, double* ms_per_mcu, int32_t n) {
  CHECK_HANDLE(h);
  if (!best) return fail(SFLOW_EINVAL, "best is NULL");
  double v[SFLOW_TILE_CANDIDATES];
  int b = 0;
  const int rc = h->solver->autotune(steps_per_shape, &b, v);
  if (rc < 0) return fail(rc, last_solver_error(h));
  *best = b;
  for (int32_t i = 0; i < n && i < SFLOW_TILE_CANDIDATES && ms_per_mcu; ++i) ms_per_mcu[i] = v[i];
  return SFLOW_OK;
}

int64_t sflow_launch_count(const sflow_handle* h) {
  return (h && h->solver) ? h->solver->launches() : -1;
}
int64_t sflow_device_bytes(const sflow_handle* h) {
  return (h && h->solver) ? h->solver->device_bytes() : -1;
}
int sflow_host_geometry(const SflowParams* p, const double* B_cent, int32_t which, double* out) {
  if (!out) return fail(SFLOW_EINVAL, "out is NULL");
  HostSetup s;
  std::string err;
  int rc = sflow::host_setup(p, B_cent, s, err);
  if (rc != SFLOW_OK) return fail(rc, err);
  const std::vector<double>* f[11] = {&s.Bx, &s.By, &s.Bxx, &s.Bxy, &s.Byy, &s.gc, &s.dgcx, &s.dgcy,
                                      &s.arc_perim, &s.arc_nx, &s.arc_ny};
  const size_t N = (size_t)s.nx * s.ny;
  if (which >= 0 && which <= 10) {
    for (size_t i = 0; i < N; ++i) out[i] = (*f[which])[i];
  } else if (which == 11) {
    for (size_t i = 0; i < N; ++i) out[i] = (double)(s.cflags[i] & 0x3);
  } else if (which == 12) {
    for (size_t i = 0; i < N; ++i) {
      uint8_t c = s.cflags[i];
      out[i] = (double)(((c >> 2) & 1) | (((c >> 3) & 1) << 1) | (((c >> 4) & 1) << 2) | (((c >> 5) & 1) << 3));
    }
  } else if (which == 13) {
    for (size_t i = 0; i < N; ++i) out[i] = s.cell_fract.empty() ? 0.0 : s.cell_fract[i];
  } else {
    return fail(SFLOW_EINVAL, "which must be in 0..13");
  }
  return SFLOW_OK;
}

int sflow_host_scalars(const SflowParams* p, const double* B_cent, double* out4) {
  if (!out4) return fail(SFLOW_EINVAL, "out is NULL");
  HostSetup s;
  std::string err;
  int rc = sflow::host_setup(p, B_cent, s, err);
  if (rc != SFLOW_OK) return fail(rc, err);
  out4[0] = s.h_source;
  out4[1] = s.src_rho_m;
  out4[2] = s.src_cp_mix;
  out4[3] = s.eps_sing;
  return SFLOW_OK;
}

int sflow_dry_border_updates(sflow_handle* h, int64_t* n) {
  CHECK_HANDLE(h);
  if (!n) return fail(SFLOW_EINVAL, "n is NULL");
  const int64_t v = h->solver->border_total();
  if (v < 0) return fail(SFLOW_ECUDA, "could not read the run state");
  *n = v;
  return SFLOW_OK;
}

int sflow_counters(sflow_handle* h, int64_t* cell_updates, int64_t* steps, int64_t* newton_iters,
                   int32_t* newton_max) {
  CHECK_HANDLE(h);
  SflowStepStats s;
  int rc = h->solver->stats(&s);
  if (rc < 0) return fail(rc, last_solver_error(h));
  int64_t tot = 0;
  int mx = 0;
  rc = h->solver->newton_stats(&tot, &mx);
  if (rc < 0) return fail(rc, last_solver_error(h));
  if (cell_updates) *cell_updates = h->solver->cells_total();
  if (steps) *steps = s.steps;
  if (newton_iters) *newton_iters = tot;
  if (newton_max) *newton_max = mx;
  return SFLOW_OK;
}

}  // extern "C"

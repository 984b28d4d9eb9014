// sflow_batch.cuh -- host side of the batched engine: many independent runs
// (uneven grid sizes and parameters) resident on one GPU and advanced
// together by the persistent kernels of sflow_batch_kernels.cuh.
//
// Runs are grouped by solid-class count (a template parameter of the heavy
// kernels); each group has its own stream, tile lists and CUDA graph of
// kChunk batch steps.  The graph's kernel arguments point at device tables
// (run arguments, run slots, lists, counters), so the same graph serves any
// membership: runs are admitted and collected between graph launches
// without re-capturing.  Admission checks a free slot, the tile-list
// capacity and the free device memory (cudaMemGetInfo) against the run's
// footprint.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <memory>
#include <mutex>
#include <thread>
#include <string>
#include <vector>

#include "sflow_batch_kernels.cuh"
#include "sflow_solver.cuh"

namespace sflow {

template <class R>
class Batch : public BatchBase {
 public:
  static constexpr int kChunk = 16;
  static constexpr int kStepLaunches = 5;   // k_b_cand, k_b_mask, k_b_flux, k_b_dt, k_b_stage2

  Batch(int max_runs, int64_t max_tiles) : max_runs_(max_runs), max_tiles_(max_tiles) {
    if (cudaGetDevice(&dev_) != cudaSuccess) {
      cudaGetLastError();
      dev_ = 0;
    }
  }
  ~Batch() override {
    for (auto& g : groups_)
      if (g) g->release();
    if (tstream_) {
      cudaStreamSynchronize(tstream_);
      cudaEventDestroy(ev0_);
      cudaEventDestroy(ev1_);
      for (auto& e : evg_)
        if (e) cudaEventDestroy(e);
      cudaStreamDestroy(tstream_);
    }
  }
  std::string err_;

  // A run's device state built off the batch's tables (sflow_batch_submit
  // builds it in place; sflow_batch_submit_many on its worker threads).
  struct Prepared : PreparedRun {
    std::unique_ptr<Solver<R>> sv;
    uint32_t* cand = nullptr;      // per-tile candidate flags (zeroed)
    uint8_t* tile_seed = nullptr;  // per-tile seed flags
    bool flags_owned = false;      // own allocations (else in the solver's)
    int64_t tiles = 0;
    int ns = 0;
    double max_dt = 0.0, t_end = 0.0;
    ~Prepared() override {
      if (flags_owned) {
        if (cand) cudaFree(cand);
        if (tile_seed) cudaFree(tile_seed);
      }
    }
  };

  // what a run must satisfy whatever the batch holds
  int check_run(const HostSetup& hs, std::string& err) const {
    if (hs.nrk != 2) { err = "batched runs use the N_RK = 2 tableau"; return SFLOW_EINVAL; }
    if (hs.ns < kMinSolidBuilt || hs.ns > kMaxSolidBuilt) { err = "n_solid out of range"; return SFLOW_EINVAL; }
    if (hs.p.erosion_coeff != 0.0 || hs.p.bottom_radial_source_flag || hs.n_thk * hs.n_dyn > 0) {
      // their per-step work (source factors, topography) and results
      // (erosion, vulnerability table) belong to the single-run solver
      err = "erosion, the bottom radial source and the vulnerability table run on the single-run solver";
      return SFLOW_EINVAL;
    }
    return SFLOW_OK;
  }
  int64_t run_tiles(const HostSetup& hs) const {
    return (int64_t)((hs.nx + TX - 1) / TX) * ((hs.ny + tile_h_ - 1) / tile_h_);
  }
  static int64_t run_need(const HostSetup& hs, int tile_h) {
    return Solver<R>::batch_bytes(hs, tile_h) +
           (int64_t)sizeof(double) * hs.nx * hs.ny * (hs.nv + 3);   // staging, freed after upload
  }

  // Builds the run's device state: solver, upload of q, limits, the
  // candidate and seed flags.  Touches no table of the batch, so worker
  // threads may run it for different runs at once.
  std::unique_ptr<Prepared> build(HostSetup&& hs, const double* q_aos, int64_t max_steps, int* rc,
                                  std::string& err) const {
    std::unique_ptr<Prepared> pr(new Prepared());
    pr->ns = hs.ns;
    pr->max_dt = hs.p.max_dt;
    pr->t_end = hs.p.t_end;
    pr->tiles = run_tiles(hs);
    pr->sv.reset(new Solver<R>(std::move(hs), tile_h_));
    Solver<R>& sv = *pr->sv;
    sv.reserve_extra(sizeof(uint32_t) * (size_t)pr->tiles);
    sv.reserve_extra((size_t)pr->tiles);
    *rc = sv.init();
    if (*rc == SFLOW_OK) *rc = sv.upload(q_aos);
    if (*rc == SFLOW_OK) *rc = sv.limits(pr->t_end, max_steps > 0 ? max_steps : -1);
    if (*rc != SFLOW_OK) {
      err = sv.err_;
      return nullptr;
    }
    sv.trim_stage();
    const std::vector<uint8_t> ts = sv.tile_seed_host();
    pr->cand = static_cast<uint32_t*>(sv.carve(sizeof(uint32_t) * pr->tiles));
    pr->tile_seed = static_cast<uint8_t*>(sv.carve(ts.size()));
    if (!pr->cand || !pr->tile_seed) {
      // no room left in the run's allocation: allocations of their own
      pr->cand = nullptr;
      pr->tile_seed = nullptr;
      pr->flags_owned = true;
      if (cudaMalloc((void**)&pr->cand, sizeof(uint32_t) * pr->tiles) != cudaSuccess ||
          cudaMalloc((void**)&pr->tile_seed, ts.size()) != cudaSuccess) {
        cudaGetLastError();
        *rc = SFLOW_ENOMEM;
        err = "cudaMalloc failed";
        return nullptr;
      }
    }
    if (cudaMemsetAsync(pr->cand, 0, sizeof(uint32_t) * pr->tiles, sv.stream()) != cudaSuccess ||
        cudaMemcpyAsync(pr->tile_seed, ts.data(), ts.size(), cudaMemcpyHostToDevice, sv.stream()) != cudaSuccess ||
        cudaStreamSynchronize(sv.stream()) != cudaSuccess) {
      *rc = SFLOW_ECUDA;
      err = "cudaMemcpy failed";
      return nullptr;
    }
    return pr;
  }

  // The run joins the batch: a free slot, list capacity and the memory
  // limit are checked, then its arguments go into the device tables.
  int admit(std::unique_ptr<Prepared> pr, int* id) {
    Group* g = group(pr->ns);
    if (!g) return SFLOW_ECUDA;
    int slot = -1;
    for (int i = 0; i < max_runs_; ++i)
      if (!g->slots[i].solver) { slot = i; break; }
    if (slot < 0) { err_ = "no free run slot"; return SFLOW_EBUSY; }
    const int64_t tiles = pr->tiles;
    if (g->tiles_live + g->tiles_draining + tiles > max_tiles_) {
      err_ = "tile-list capacity of the batch is in use";
      return SFLOW_EBUSY;
    }
    Solver<R>& sv = *pr->sv;
    const int64_t bytes = sv.device_bytes() + (pr->flags_owned ? (int64_t)sizeof(uint32_t) * tiles + tiles : 0);
    if (mem_limit_ > 0 && held_ + bytes > mem_limit_) { err_ = "the batch's memory limit is in use"; return SFLOW_EBUSY; }
    if (g->smem_flux < sv.smem_flux()) { err_ = "flux shared memory mismatch"; return SFLOW_EINVAL; }
    Slot& s = g->slots[slot];
    const unsigned gen = (s.gen + 1u) & 0xffffu;
    BatchRun br;
    br.st = sv.state_dev();
    br.cand = pr->cand;
    br.tile_wet = sv.tile_wet_dev();
    br.tile_count = sv.tile_count_dev();
    br.tile_seed = pr->tile_seed;
    br.tiles_x = sv.tiles_x();
    br.tiles_y = sv.tiles_y();
    br.gen = gen;
    br.live = 1;
    br.max_dt = pr->max_dt;
    const KArgs<R> ka = sv.kargs();
    if (ka.g.lim_all != 1 && g->lim == 1) {
      // the group needs the generic limiter kernel from now on: re-capture
      g->lim = -1;
      if (g->graph_exec) cudaGraphExecDestroy(g->graph_exec);
      if (g->graph) cudaGraphDestroy(g->graph);
      g->graph_exec = nullptr;
      g->graph = nullptr;
    }
    // the batch stream is idle here (every advance ends synchronised)
    if (cudaMemcpy(g->d_args + slot, &ka, sizeof(ka), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(g->d_runs + slot, &br, sizeof(br), cudaMemcpyHostToDevice) != cudaSuccess) {
      err_ = "cudaMemcpy failed";
      return SFLOW_ECUDA;
    }
    cudaError_t e = g->tab.b_admit(g->args, g->stream, slot, gen, (unsigned)tiles);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) { err_ = cudaGetErrorString(e); return SFLOW_ECUDA; }
    ++g->launches;
    s.gen = gen;
    s.cand = pr->cand;
    s.tile_seed = pr->tile_seed;
    s.flags_owned = pr->flags_owned;
    pr->cand = nullptr;
    pr->tile_seed = nullptr;
    s.tiles = tiles;
    s.bytes = bytes;
    held_ += s.bytes;
    s.solver = std::move(pr->sv);
    s.done = false;
    g->tiles_live += tiles;
    g->live += 1;
    const int rid = (int)recs_.size();
    recs_.push_back(Rec{pr->ns, slot, true});
    s.rec = rid;
    *id = rid;
    return SFLOW_OK;
  }

  int submit(HostSetup&& hs, const double* q_aos, int64_t max_steps, int* id) override {
    if (launched_) { err_ = "steps are in flight: wait first"; return SFLOW_ESTATE; }
    int rc = check_run(hs, err_);
    if (rc != SFLOW_OK) return rc;
    // admission before anything is allocated: slot, list capacity, memory
    Group* g = group(hs.ns);
    if (!g) return SFLOW_ECUDA;
    bool free_slot = false;
    for (int i = 0; i < max_runs_ && !free_slot; ++i) free_slot = !g->slots[i].solver;
    if (!free_slot) { err_ = "no free run slot"; return SFLOW_EBUSY; }
    if (g->tiles_live + g->tiles_draining + run_tiles(hs) > max_tiles_) {
      err_ = "tile-list capacity of the batch is in use";
      return SFLOW_EBUSY;
    }
    const int64_t need = run_need(hs, tile_h_);
    if (bulk_) {
      // inside sflow_batch_submit_many: the shared estimate of reserve_room
      rc = reserve_room(need, err_);
      if (rc != SFLOW_OK) return rc;
    } else {
      size_t free_b = 0, total_b = 0;
      if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) { err_ = "cudaMemGetInfo failed"; return SFLOW_ECUDA; }
      if ((int64_t)free_b < need + kReserve) { err_ = "not enough free device memory for the run now"; return SFLOW_EBUSY; }
    }
    if (mem_limit_ > 0 && held_ + need > mem_limit_) { err_ = "the batch's memory limit is in use"; return SFLOW_EBUSY; }
    std::unique_ptr<Prepared> pr = build(std::move(hs), q_aos, max_steps, &rc, err_);
    if (!pr) return rc;
    return admit(std::move(pr), id);
  }

  // sflow_batch_submit_many: prepare() on worker threads (each bound to the
  // batch's device), commit() in run order on the submitting thread.  A
  // worker builds a run only while the device has room for it (free memory
  // minus the reserve), so runs built ahead never exhaust the device.
  std::unique_ptr<PreparedRun> prepare(HostSetup&& hs, const double* q_aos, int64_t max_steps, int* rc,
                                       std::string* err) override {
    *rc = check_run(hs, *err);
    if (*rc != SFLOW_OK) return nullptr;
    *rc = reserve_room(run_need(hs, tile_h_), *err);
    if (*rc != SFLOW_OK) return nullptr;
    return build(std::move(hs), q_aos, max_steps, rc, *err);
  }
  int commit(std::unique_ptr<PreparedRun> pr, int* id) override {
    if (launched_) { err_ = "steps are in flight: wait first"; return SFLOW_ESTATE; }
    std::unique_ptr<Prepared> p(static_cast<Prepared*>(pr.release()));
    return admit(std::move(p), id);
  }
  void bind_thread() override { cudaSetDevice(dev_); }
  bool device_mapped(const void* p) const override { return Solver<R>::is_mapped_host(p); }

  // Room on the device for a run built by prepare(): the free memory is
  // queried once per bulk submission, every 32 builds and whenever the
  // estimate nears the need; each build takes its need off the estimate.
  int reserve_room(int64_t need, std::string& err) {
    std::lock_guard<std::mutex> lk(room_mu_);
    if (room_free_ < 0 || room_since_ >= 32 || room_free_ < need + kReserve + (int64_t(4) << 30)) {
      size_t free_b = 0, total_b = 0;
      if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        err = "cudaMemGetInfo failed";
        return SFLOW_ECUDA;
      }
      room_free_ = (int64_t)free_b;
      room_since_ = 0;
    }
    if (room_free_ < need + kReserve) {
      err = "not enough free device memory for the run now";
      return SFLOW_EBUSY;
    }
    room_free_ -= need;
    ++room_since_;
    return SFLOW_OK;
  }

  void set_bulk(bool on) override {
    std::lock_guard<std::mutex> lk(room_mu_);
    bulk_ = on;
    room_free_ = -1;   // a new bulk submission queries afresh
  }

  int advance(int64_t steps, int* finished) override { return advance_impl(steps, finished, nullptr); }

  // Device time of `steps` batch steps: an event on a timing stream that
  // every group's stream waits for, the groups' steps, one event per group
  // that the timing stream waits for, and a last event there.
  int advance_timed(int64_t steps, int* finished, double* ms) override {
    if (!ms) { err_ = "ms is NULL"; return SFLOW_EINVAL; }
    *ms = 0.0;
    if (!tstream_) {
      cudaError_t e = cudaStreamCreateWithFlags(&tstream_, cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreate(&ev0_);
      if (e == cudaSuccess) e = cudaEventCreate(&ev1_);
      for (int i = 0; e == cudaSuccess && i <= kMaxSolidBuilt; ++i)
        e = cudaEventCreateWithFlags(&evg_[i], cudaEventDisableTiming);
      if (e != cudaSuccess) { err_ = cudaGetErrorString(e); return SFLOW_ECUDA; }
    }
    return advance_impl(steps, finished, ms);
  }

  // `steps` batch steps launched one by one without programmatic dependent
  // launch, with events between the five kernels; ms5 gets the summed
  // device time of k_b_cand, k_b_mask, k_b_flux, k_b_dt, k_b_stage2 over
  // the steps and the groups
  int profile_kernels(int64_t steps, int* finished, double* ms5) override {
    if (launched_) { err_ = "steps are in flight: wait first"; return SFLOW_ESTATE; }
    for (int i = 0; i < 5; ++i) ms5[i] = 0.0;
    cudaEvent_t ev[6];
    for (int i = 0; i < 6; ++i)
      if (cudaEventCreate(&ev[i]) != cudaSuccess) { err_ = "cudaEventCreate failed"; return SFLOW_ECUDA; }
    int rc = SFLOW_OK;
    for (auto& gp : groups_) {
      Group* g = gp.get();
      if (!g || g->live == 0) continue;
      for (int64_t st = 0; st < steps && rc == SFLOW_OK; ++st) {
        cudaError_t e = g->tab.b_step(g->args, g->stream, g->grids, g->smem_flux, g->lim, 0, ev);
        if (e == cudaSuccess) e = cudaEventSynchronize(ev[5]);
        for (int i = 0; i < 5 && e == cudaSuccess; ++i) {
          float f = 0.0f;
          e = cudaEventElapsedTime(&f, ev[i], ev[i + 1]);
          ms5[i] += f;
        }
        if (e != cudaSuccess) { err_ = cudaGetErrorString(e); rc = SFLOW_ECUDA; }
        g->launches += kStepLaunches;
      }
    }
    for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
    if (rc != SFLOW_OK) return rc;
    return advance_impl(0, finished, nullptr);
  }

  int advance_impl(int64_t steps, int* finished, double* ms) {
    if (launched_) { err_ = "steps are in flight: wait first"; return SFLOW_ESTATE; }
    int rc = launch_impl(steps, ms != nullptr);
    if (rc != SFLOW_OK) return rc;
    return wait_impl(finished, ms);
  }

  // Enqueue `steps` batch steps on the groups' streams and return at once.
  int launch(int64_t steps) override {
    if (launched_) { err_ = "steps already launched: wait first"; return SFLOW_ESTATE; }
    return launch_impl(steps, false);
  }
  // Wait for the launched steps, read the runs' summaries.
  int wait(int* finished) override { return wait_impl(finished, nullptr); }

  int launch_impl(int64_t steps, bool timed) {
    if (timed) {
      cudaError_t e = cudaEventRecord(ev0_, tstream_);
      for (auto& gp : groups_)
        if (e == cudaSuccess && gp && gp->live > 0) e = cudaStreamWaitEvent(gp->stream, ev0_, 0);
      if (e != cudaSuccess) { err_ = cudaGetErrorString(e); return SFLOW_ECUDA; }
    }
    for (auto& gp : groups_) {
      Group* g = gp.get();
      if (!g || g->live == 0) continue;
      int64_t left = steps;
      while (left >= kChunk) {
        if (!g->graph_exec) {
          cudaError_t e = g->capture();
          if (e != cudaSuccess) { err_ = cudaGetErrorString(e); return SFLOW_ECUDA; }
        }
        cudaError_t e = cudaGraphLaunch(g->graph_exec, g->stream);
        if (e != cudaSuccess) { err_ = cudaGetErrorString(e); return SFLOW_ECUDA; }
        g->launches += kStepLaunches * kChunk;
        left -= kChunk;
      }
      for (; left > 0; --left) {
        cudaError_t e = g->tab.b_step(g->args, g->stream, g->grids, g->smem_flux, g->lim, g->pdl, nullptr);
        if (e != cudaSuccess) { err_ = cudaGetErrorString(e); return SFLOW_ECUDA; }
        g->launches += kStepLaunches;
      }
    }
    launched_ = true;
    return SFLOW_OK;
  }

  int wait_impl(int* finished, double* ms) {
    int nfin = 0;
    launched_ = false;
    if (ms) {
      cudaError_t e = cudaSuccess;
      for (int i = 0; i <= kMaxSolidBuilt; ++i) {
        Group* g = groups_[i].get();
        if (!g || g->live == 0) continue;
        if (e == cudaSuccess) e = cudaEventRecord(evg_[i], g->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(tstream_, evg_[i], 0);
      }
      if (e == cudaSuccess) e = cudaEventRecord(ev1_, tstream_);
      if (e == cudaSuccess) e = cudaEventSynchronize(ev1_);
      float f = 0.0f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&f, ev0_, ev1_);
      if (e != cudaSuccess) { err_ = cudaGetErrorString(e); return SFLOW_ECUDA; }
      *ms = (double)f;
    }
    // groups run concurrently on their streams; wait for all, then read the
    // per-slot summaries
    for (auto& gp : groups_) {
      Group* g = gp.get();
      if (!g || g->live == 0) continue;
      cudaError_t e = g->tab.b_summary(g->args, g->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(g->h_summary, g->d_summary, sizeof(BatchSummary) * max_runs_,
                            cudaMemcpyDeviceToHost, g->stream);
      BatchCtl ctl;
      if (e == cudaSuccess) e = cudaMemcpyAsync(&ctl, g->d_ctl, sizeof(ctl), cudaMemcpyDeviceToHost, g->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
      if (e != cudaSuccess) { err_ = cudaGetErrorString(e); return SFLOW_ECUDA; }
      if (ctl.overflow) { err_ = "active-cell list overflow (internal error)"; return SFLOW_ECUDA; }
      ++g->launches;
      g->tiles_draining = 0;   // entries of collected runs left the lists
      for (int i = 0; i < max_runs_; ++i) {
        Slot& s = g->slots[i];
        if (!s.solver) continue;
        if (!g->h_summary[i].running) s.done = true;
        if (s.done) ++nfin;
      }
    }
    if (finished) *finished = nfin;
    return SFLOW_OK;
  }

  int poll(int id, SflowStepStats* st, int* done) override {
    if (launched_) { err_ = "steps are in flight: wait first"; return SFLOW_ESTATE; }
    Slot* s = lookup(id);
    if (!s) return SFLOW_EINVAL;
    if (st) {
      int rc = s->solver->stats(st);
      if (rc != SFLOW_OK) { err_ = s->solver->error(); return rc; }
    }
    if (done) *done = s->done ? 1 : 0;
    return SFLOW_OK;
  }

  int counters(int id, int64_t* cells, int64_t* steps) override {
    if (launched_) { err_ = "steps are in flight: wait first"; return SFLOW_ESTATE; }
    Slot* s = lookup(id);
    if (!s) return SFLOW_EINVAL;
    RunState h;
    int rc = s->solver->run_state(&h);
    if (rc != SFLOW_OK) { err_ = s->solver->error(); return rc; }
    if (cells) *cells = h.cells_total;
    if (steps) *steps = h.steps;
    return SFLOW_OK;
  }

  int border_updates(int id, int64_t* n) override {
    if (launched_) { err_ = "steps are in flight: wait first"; return SFLOW_ESTATE; }
    Slot* s = lookup(id);
    if (!s) return SFLOW_EINVAL;
    *n = s->solver->border_total();
    return SFLOW_OK;
  }

  int collect(int id, double* q_aos) override {
    if (launched_) { err_ = "steps are in flight: wait first"; return SFLOW_ESTATE; }
    Slot* s = lookup(id);
    if (!s) return SFLOW_EINVAL;
    Group* g = group(recs_[id].ns);
    if (q_aos) {
      int rc = s->solver->download(q_aos);
      if (rc != SFLOW_OK) { err_ = s->solver->error(); return rc; }
    }
    BatchRun br;
    std::memset(&br, 0, sizeof(br));
    br.live = 0;
    br.gen = s->gen;
    if (cudaMemcpy(g->d_runs + recs_[id].slot, &br, sizeof(br), cudaMemcpyHostToDevice) != cudaSuccess) {
      err_ = "cudaMemcpy failed";
      return SFLOW_ECUDA;
    }
    if (s->flags_owned) {
      cudaFree(s->cand);
      cudaFree(s->tile_seed);
    }
    s->solver.reset();   // frees the run's allocation (flags included unless owned)
    held_ -= s->bytes;
    s->bytes = 0;
    s->cand = nullptr;
    s->tile_seed = nullptr;
    s->flags_owned = false;
    g->tiles_live -= s->tiles;
    g->tiles_draining += s->tiles;
    g->live -= 1;
    s->done = false;
    recs_[id].alive = false;
    if (g->live == 0) {
      // no run left: start the group's lists afresh (drops stale entries)
      if (cudaMemset(g->d_ctl, 0, sizeof(BatchCtl)) != cudaSuccess) {
        err_ = "cudaMemset failed";
        return SFLOW_ECUDA;
      }
      g->tiles_draining = 0;
    }
    return SFLOW_OK;
  }

  int collect_many(int n, const int32_t* ids, double* const* q_aos, int threads, int32_t* status) override {
    if (launched_) { err_ = "steps are in flight: wait first"; return SFLOW_ESTATE; }
    std::vector<Solver<R>*> sv((size_t)n, nullptr);
    int first = SFLOW_OK;
    std::string first_err;
    auto note = [&](int i, int rc, const std::string& e) {
      status[i] = rc;
      if (rc < 0 && first == SFLOW_OK) {
        first = rc;
        first_err = "run " + std::to_string(ids[i]) + ": " + e;
      }
    };
    for (int i = 0; i < n; ++i) {
      status[i] = SFLOW_OK;
      for (int j = 0; j < i; ++j)
        if (ids[j] == ids[i]) { note(i, SFLOW_EINVAL, "run id given twice"); break; }
      if (status[i] != SFLOW_OK) continue;
      Slot* s = lookup(ids[i]);
      if (!s) note(i, SFLOW_EINVAL, err_);
      else sv[(size_t)i] = s->solver.get();
    }
    // downloads: independent solvers, their own streams
    std::vector<int> drc((size_t)n, SFLOW_OK);
    std::vector<std::string> derr((size_t)n);
    std::atomic<int> next{0};
    auto work = [&]() {
      cudaSetDevice(dev_);
      for (int i = next.fetch_add(1); i < n; i = next.fetch_add(1)) {
        if (!sv[(size_t)i] || !q_aos || !q_aos[i]) continue;
        drc[(size_t)i] = sv[(size_t)i]->download(q_aos[i]);
        if (drc[(size_t)i] != SFLOW_OK) derr[(size_t)i] = sv[(size_t)i]->error();
      }
    };
    const int nt = std::max(1, std::min(threads > 0 ? threads : (int)std::thread::hardware_concurrency(),
                                        std::min(n, 64)));
    std::vector<std::thread> pool;
    try {
      for (int t = 1; t < nt; ++t) pool.emplace_back(work);
    } catch (const std::exception&) {
      // fewer threads: this one takes the rest
    }
    int prev_dev = dev_;
    if (cudaGetDevice(&prev_dev) != cudaSuccess) cudaGetLastError();
    work();   // this thread too (it selects the batch's device meanwhile)
    cudaSetDevice(prev_dev);
    for (auto& t : pool) t.join();
    for (int i = 0; i < n; ++i) {
      if (!sv[(size_t)i]) continue;
      if (drc[(size_t)i] != SFLOW_OK) {
        note(i, drc[(size_t)i], derr[(size_t)i]);
        continue;
      }
      const int rc = collect(ids[i], nullptr);
      if (rc != SFLOW_OK) note(i, rc, err_);
    }
    if (first != SFLOW_OK) err_ = first_err;
    return first;
  }

  int download(int id, double* q_aos) override {
    if (launched_) { err_ = "steps are in flight: wait first"; return SFLOW_ESTATE; }
    Slot* s = lookup(id);
    if (!s) return SFLOW_EINVAL;
    int rc = s->solver->download(q_aos);
    if (rc != SFLOW_OK) { err_ = s->solver->error(); return rc; }
    s->solver->trim_stage();
    return SFLOW_OK;
  }

  // Tile height of every run admitted from now on; only while the batch
  // holds no run (the groups' lists and graphs are made for one height).
  int set_memory_limit(int64_t bytes) override {
    if (bytes < 0) { err_ = "memory limit must be >= 0"; return SFLOW_EINVAL; }
    mem_limit_ = bytes;
    return SFLOW_OK;
  }
  int set_tile_shape(int th) override {
    if (th == tile_h_) return SFLOW_OK;
    if (!tile_h_built<R>(th)) { err_ = "no kernels built for this tile height"; return SFLOW_EINVAL; }
    if (live() > 0 || launched_) { err_ = "the tile height changes only while the batch holds no run"; return SFLOW_ESTATE; }
    for (auto& g : groups_)
      if (g) {
        g->release();
        g.reset();
      }
    tile_h_ = th;
    return SFLOW_OK;
  }
  int tile_shape() const override { return tile_h_; }

  int live() const override {
    int n = 0;
    for (auto& g : groups_)
      if (g) n += g->live;
    return n;
  }
  int64_t launches() const override {
    int64_t n = 0;
    for (auto& g : groups_)
      if (g) n += g->launches;
    return n;
  }
  const char* error() const override { return err_.c_str(); }

 private:
  static constexpr int64_t kReserve = (int64_t)1 << 30;   // device memory kept free
  int64_t mem_limit_ = 0;   // cap on the resident runs' device bytes (0: none)
  int64_t held_ = 0;        // device bytes of the resident runs
  bool bulk_ = false;       // inside sflow_batch_submit_many (set_bulk)
  std::mutex room_mu_;      // reserve_room(), called by prepare() on worker threads
  int64_t room_free_ = -1;  // free device memory: last query minus the needs built since (-1: query)
  int room_since_ = 0;      // builds since that query

  struct Slot {
    std::unique_ptr<Solver<R>> solver;
    uint32_t* cand = nullptr;
    uint8_t* tile_seed = nullptr;
    bool flags_owned = false;   // cand / tile_seed allocated on their own
    int64_t tiles = 0;
    int64_t bytes = 0;   // device bytes the run holds
    unsigned gen = 0;
    bool done = false;
    int rec = -1;
  };
  struct Rec {
    int ns, slot;
    bool alive;
  };
  struct Group {
    KernelTable<R> tab;
    cudaStream_t stream = nullptr;
    KArgs<R>* d_args = nullptr;
    BatchRun* d_runs = nullptr;
    BatchCtl* d_ctl = nullptr;
    unsigned long long *d_list0 = nullptr, *d_list1 = nullptr, *d_cand = nullptr;
    unsigned long long *d_dlist0 = nullptr, *d_dlist1 = nullptr;
    unsigned long long* d_cells = nullptr;
    BatchSummary* d_summary = nullptr;
    BatchSummary* h_summary = nullptr;
    BatchArgs<R> args;
    int grids[4] = {0, 0, 0, 0};
    size_t smem_flux = 0;
    int lim = 1;   // 1 while every submitted run uses minmod everywhere, else -1
    int pdl = 1;   // programmatic dependent launch of the step kernels (SFLOW_PDL=0: off)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    std::vector<Slot> slots;
    int64_t tiles_live = 0, tiles_draining = 0, launches = 0;
    int live = 0;

    cudaError_t capture() {
      cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
      if (e != cudaSuccess) return e;
      for (int i = 0; i < kChunk; ++i) {
        e = tab.b_step(args, stream, grids, smem_flux, lim, pdl, nullptr);
        if (e != cudaSuccess) {
          cudaGraph_t g0 = nullptr;
          cudaStreamEndCapture(stream, &g0);
          if (g0) cudaGraphDestroy(g0);
          return e;
        }
      }
      e = cudaStreamEndCapture(stream, &graph);
      if (e != cudaSuccess) return e;
      return cudaGraphInstantiate(&graph_exec, graph, 0);
    }
    void release() {
      if (stream) cudaStreamSynchronize(stream);
      for (auto& s : slots) {
        if (s.flags_owned) {
          if (s.cand) cudaFree(s.cand);
          if (s.tile_seed) cudaFree(s.tile_seed);
        }
        s.solver.reset();
        s.cand = nullptr;
        s.tile_seed = nullptr;
        s.flags_owned = false;
      }
      if (graph_exec) cudaGraphExecDestroy(graph_exec);
      if (graph) cudaGraphDestroy(graph);
      void* bufs[10] = {d_args, d_runs, d_ctl, d_list0, d_list1, d_dlist0, d_dlist1, d_cand, d_cells, d_summary};
      for (void* p : bufs)
        if (p) cudaFree(p);
      if (h_summary) cudaFreeHost(h_summary);
      if (stream) cudaStreamDestroy(stream);
      stream = nullptr;
    }
  };

  Slot* lookup(int id) {
    if (id < 0 || id >= (int)recs_.size() || !recs_[id].alive) {
      err_ = "unknown or collected run id";
      return nullptr;
    }
    Group* g = groups_[recs_[id].ns].get();
    return &g->slots[recs_[id].slot];
  }

  Group* group(int ns) {
    if (groups_[ns]) return groups_[ns].get();
    std::unique_ptr<Group> g(new Group());
    g->tab = kernel_table<R>(ns, tile_h_);
    {
      const char* pdl_env = std::getenv("SFLOW_PDL");
      g->pdl = (pdl_env && pdl_env[0] == '0') ? 0 : 1;
    }
    if (!g->tab.b_step) { err_ = "no batch kernels for this class count and tile height"; return nullptr; }
    g->slots.resize(max_runs_);
    // shared memory of the flux kernel for this class count (the largest
    // any run of the group needs: it depends on n_vars only)
    g->smem_flux = Solver<R>::flux_smem_bytes(4 + ns, tile_h_);
    auto fail = [&](cudaError_t e) -> Group* {
      err_ = cudaGetErrorString(e);
      g->release();
      return nullptr;
    };
    cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return fail(e);
    if ((e = g->tab.b_setup(g->smem_flux, g->grids)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&g->d_args, sizeof(KArgs<R>) * max_runs_)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&g->d_runs, sizeof(BatchRun) * max_runs_)) != cudaSuccess) return fail(e);
    if ((e = cudaMemset(g->d_runs, 0, sizeof(BatchRun) * max_runs_)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&g->d_ctl, sizeof(BatchCtl))) != cudaSuccess) return fail(e);
    if ((e = cudaMemset(g->d_ctl, 0, sizeof(BatchCtl))) != cudaSuccess) return fail(e);
    const size_t lb = sizeof(unsigned long long) * (size_t)max_tiles_;
    if ((e = cudaMalloc((void**)&g->d_list0, lb)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&g->d_list1, lb)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&g->d_cand, lb)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&g->d_dlist0, lb)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&g->d_dlist1, lb)) != cudaSuccess) return fail(e);
    // active cells: at most every cell of the tiles the active list holds
    const size_t cap = (size_t)max_tiles_ * TX * tile_h_;
    if (cap > 0xffffffffull) { err_ = "max_cells too large for the active-cell list"; g->release(); return nullptr; }
    if ((e = cudaMalloc((void**)&g->d_cells, sizeof(unsigned long long) * cap)) != cudaSuccess) return fail(e);
    if ((e = cudaMalloc((void**)&g->d_summary, sizeof(BatchSummary) * max_runs_)) != cudaSuccess) return fail(e);
    if ((e = cudaMallocHost((void**)&g->h_summary, sizeof(BatchSummary) * max_runs_)) != cudaSuccess) return fail(e);
    g->args.args = g->d_args;
    g->args.runs = g->d_runs;
    g->args.ctl = g->d_ctl;
    g->args.list0 = g->d_list0;
    g->args.list1 = g->d_list1;
    g->args.cand = g->d_cand;
    g->args.dlist0 = g->d_dlist0;
    g->args.dlist1 = g->d_dlist1;
    g->args.cells = g->d_cells;
    g->args.cells_cap = (unsigned)cap;
    g->args.summary = g->d_summary;
    g->args.max_runs = max_runs_;
    groups_[ns] = std::move(g);
    return groups_[ns].get();
  }

  int max_runs_;
  int64_t max_tiles_;
  int dev_ = 0;                      // the device the batch lives on
  int tile_h_ = kTileHDefault;
  cudaStream_t tstream_ = nullptr;   // timing stream of advance_timed
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr, evg_[kMaxSolidBuilt + 1] = {};
  bool launched_ = false;            // launch() called, wait() not yet
  std::unique_ptr<Group> groups_[kMaxSolidBuilt + 1];
  std::vector<Rec> recs_;
};

template <class R>
BatchBase* make_batch_impl(int max_runs, int64_t max_tiles, std::string& err) {
  if (max_runs < 1 || max_runs > 65535) { err = "max_runs must be 1..65535"; return nullptr; }
  if (max_tiles < 1 || max_tiles > ((int64_t)1 << 31)) { err = "max_cells out of range"; return nullptr; }
  return new Batch<R>(max_runs, max_tiles);
}

}  // namespace sflow

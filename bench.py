"""Benchmark of the IMEX_SfloW2D time step on GB300.

Headline workload (the configuration the metric is quoted on): the batched
ensemble -- 256 independent ring-inlet currents, grid sides log-uniform in
[128, 1024] (dx 5-20 m), each on its own seeded Gaussian-cone + fBm DEM,
per-run Voellmy mu in [0.05, 0.3] and xi in [200, 2000], inlet radius
20-200 m, inlet temperature 600-1200 K, particle volume fractions
0.005-0.05 of 2 classes, settling on (workloads.ensemble_params), each run
2000 steps from the empty state with N_RK = 2, KT fluxes, minmod.  All runs
are resident together and advanced by the batch engine (persistent kernels
over a device-built tile queue and active-cell list, CUDA graphs of 16
steps).

One bench step is one chunk of 2000 / K batch steps (every run advances
that many time steps), so the K timed steps cover the runs' 2000 steps.

Metric: cell-updates/s = sum over runs and steps of the active cells
(solve_cells of the reference's check_solve) / time.
  value        FP32 bulk form with FP64 Newton, device time (CUDA events on
               the batch's streams) of the K steps, inputs resident in HBM
  fp64_plain   the same ensemble in the plain FP64 form (same batch
               engine), the same K steps: the same-workload comparator
  e2e          the same ensemble through the C ABI from host buffers:
               sflow_batch_submit_many of every run (host set-ups and
               device builds on the host's threads),
               the K steps, sflow_batch_collect_many with the download of every
               run's q, host wall clock
  cpu_baseline the oracle (C restatement of the reference time step) built
               with the reference's compiler flags (-fopenmp -Ofast
               -funroll-all-loops) on a bounded sample of the ensemble, one
               single-threaded process per member on the host cores, as the
               reference runs ensembles (one job per process)
  error_vs_oracle  FP32 against the oracle (FP64) on the 8 smallest members
               after their 2000 steps, per member; for a member above the
               1e-4 L1 bar on h, the oracle's own FP32 rounding band (its
               run with the state rounded to FP32 after every step)
The working set (every run's state, increments, topography and maps,
~6 GB) and the per-step traffic of the active tiles (~1.4 M cells x ~150 B)
exceed the 129 MB L2, so no flush is needed between steps.

Further legs (keys of the same JSON line; a zero size switches each off):
  current_1024  the single 1024^2 current from a seeded developed state,
                FP32 vs FP64, per-kernel times and the k_flux roofline
  served        Poisson arrivals (20/s) of 200 dam-break and ring-inlet
                jobs through the request loop, p50/p99 time to solution,
                beside the stream served one job at a time by the plain
                FP64 form (service times measured per job)
  large_domain  one 8192^2 domain (3 classes, entrainment)

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from imex_sflow2d_dev_gb300 import workloads as W  # noqa: E402
from imex_sflow2d_dev_gb300.params import PREC_FP32, PREC_FP64  # noqa: E402

METRIC = ("cell-updates/s (batched FP32 vs plain FP64 GPU, ≤1e-4 L1 err) ; "
          "p50/p99 solve latency")
UNIT = "cell-updates/s"
ENS_RUNS, ENS_STEPS = 256, 2000
H_L1_BAR = 1e-4                # the relative L1 bar on h of the FP32 form against the oracle
WORKLOAD = (f"batched ensemble: {ENS_RUNS} ring-inlet runs x {ENS_STEPS} steps, sides 128-1024 "
            "log-uniform, dx 5-20 m, own cone+fBm DEMs, per-run mu/xi/inlet draws, 2 classes, N_RK=2")
CPU_SAMPLE_EVERY = 16          # cpu sample: members 0, 16, 32, ...
CPU_SAMPLE_STEPS = 200         # time steps per sampled member across the K bench steps


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Replica runs on N GPUs: no data exchange, only a barrier around the
    timed region and a max over ranks of the measured time."""

    def __init__(self):
        self.ws, self.rank, self.local = dist_env()
        self.pg = None
        if self.ws > 1:
            import torch
            import torch.distributed as dist
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.dist = dist
            self.torch = torch

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def max(self, x):
        if self.ws == 1:
            return x
        t = self.torch.tensor([float(x)], dtype=self.torch.float64,
                              device="cuda" if self.torch.cuda.is_available() else "cpu")
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if self.ws == 1:
            return x
        t = self.torch.tensor([float(x)], dtype=self.torch.float64,
                              device="cuda" if self.torch.cuda.is_available() else "cpu")
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


def aggregate(d, cells, ms):
    """Whole-job rate of the replicas: cells of all ranks over the slowest
    rank's time (ms).  Returns (cell-updates/s, max ms)."""
    ms_max = d.max(ms)
    return d.sum(cells) / (ms_max / 1e3), ms_max


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def read_profile(name):
    """A committed ncu summary (profiles/<name>.json), or None."""
    try:
        with open(os.path.join(ROOT, "profiles", name + ".json")) as fh:
            return json.load(fh)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                   "reasons": sorted(reasons), "samples": len(sm)}
        return out


# ---------------------------------------------------------------------------
# errors of the FP32 form
# ---------------------------------------------------------------------------

def field_errors(p, qp_test, qp_ref):
    """Relative L1 / Linf of h, hu, hv, T and each alpha_s of qp_test
    against qp_ref (physical variables, reference layout).  T over the cells
    thicker than 1e-3 of the deepest (a film whose energy is almost all
    kinetic carries the rounding of its fluxes a thousandfold); a solid class
    that has settled out is scaled by at least 1e-6 of h."""
    nv, nx, ny = p.n_vars, p.comp_cells_x, p.comp_cells_y
    G, O = W.from_aos(qp_test, nv + 2, nx, ny), W.from_aos(qp_ref, nv + 2, nx, ny)
    thick = O[0] > 1e-3 * max(O[0].max(), 1e-300)
    out = {}
    names = ["h", "hu", "hv", "T"] + [f"alpha_s{i + 1}" for i in range(p.n_solid)]
    for i, n in enumerate(names):
        a, r = (G[i][thick], O[i][thick]) if n == "T" else (G[i], O[i])
        ref1 = np.abs(r).sum()
        refi = np.abs(r).max() if r.size else 0.0
        if i >= 4:
            ref1 = max(ref1, 1e-6 * np.abs(O[0]).sum())
            refi = max(refi, 1e-6 * np.abs(O[0]).max())
        d = np.abs(a - r)
        out[n] = {"l1_rel": float(d.sum() / ref1) if ref1 > 0 else float(d.sum()),
                  "linf_rel": (float(d.max() / refi) if refi > 0 else float(d.max())) if d.size else 0.0}
    return out


def worst(errs_list):
    """Largest L1 and Linf of each field over several results."""
    out = {}
    for e in errs_list:
        for n, v in e.items():
            o = out.setdefault(n, {"l1_rel": 0.0, "linf_rel": 0.0})
            o["l1_rel"] = max(o["l1_rel"], v["l1_rel"])
            o["linf_rel"] = max(o["linf_rel"], v["linf_rel"])
    return out


def qp_of_state(p, B, q_aos):
    """Physical variables (h, hu, hv, T, alpha_s..., u, v) of a state by the
    oracle's FP64 closure (qc_to_qp), for the error norms."""
    import oracle
    pp = p.copy()
    pp.precision = PREC_FP64
    o = oracle.Oracle(pp, B)
    o.set_q(q_aos)
    qp = o.qp()
    o.close()
    return qp


# ---------------------------------------------------------------------------
# CPU side (spawned processes: no fork after a CUDA context)
# ---------------------------------------------------------------------------

def _cpu_member_worker(args):
    """One ensemble member on one host core with the oracle's timing build:
    `warm` untimed steps, then (after the barrier) `chunks` x `chunk` steps.
    Returns (cell updates of the timed steps, seconds)."""
    index, warm, chunks, chunk, barrier = args
    import oracle
    oracle.set_threads(1, timing=True)
    p, B, q, _ = W.ensemble_params(index, PREC_FP64, ENS_STEPS)
    o = oracle.Oracle(p, B, timing=True)
    o.set_q(W.to_aos(q))
    for _ in range(warm):
        o.step()
    barrier.wait()
    cells = 0
    t0 = time.perf_counter()
    for _ in range(chunks * chunk):
        o.step()
        cells += o.stats().solve_cells
    dt = time.perf_counter() - t0
    o.close()
    return cells, dt


def cpu_ensemble_sample(K, warmup_steps):
    """The reference's CPU path on a bounded sample of the ensemble: members
    0, 16, ..., 240, one single-threaded process each (the reference runs an
    ensemble as one job per process, EXAMPLES/EXAMPLE_ENSEMBLE_ETNA/
    launch_jobs.py), all started together after `warmup_steps` untimed steps;
    the K bench steps cover CPU_SAMPLE_STEPS time steps of each member.
    Rate = cell updates of all members / wall time of the slowest."""
    members = list(range(0, ENS_RUNS, CPU_SAMPLE_EVERY))
    chunk = max(1, CPU_SAMPLE_STEPS // K)
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        barrier = mgr.Barrier(len(members) + 1)
        with ctx.Pool(processes=len(members)) as pool:
            res = pool.map_async(_cpu_member_worker,
                                 [(m, warmup_steps, K, chunk, barrier) for m in members])
            barrier.wait()
            t0 = time.perf_counter()
            out = res.get()
            wall = time.perf_counter() - t0
    cells = sum(c for c, _ in out)
    return {"value": cells / wall, "unit": UNIT, "cores": min(cores, len(members)), "kind": "port",
            "sample": (f"members {members[0]}..{members[-1]} every {CPU_SAMPLE_EVERY} ({len(members)} runs, "
                       f"one single-threaded process each) x {K * chunk} steps after {warmup_steps} "
                       f"untimed steps: {cells} cell updates in {wall:.2f} s; oracle C restatement "
                       f"built -Ofast -funroll-all-loops -fopenmp (the reference's flags)"),
            "steps": K, "chunk_steps": chunk, "seconds": wall, "cell_updates": cells}


def _oracle_member_worker(index):
    """One member over its 2000 steps with the oracle's parity build (one
    host core); returns (index, q)."""
    import oracle
    oracle.set_threads(1)
    p, B, q, steps = W.ensemble_params(index, PREC_FP64, ENS_STEPS)
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    o.run(max_steps=steps)
    qo = o.q()
    o.close()
    return index, qo


def _band_member_worker(index):
    """The FP32 rounding band of one member: the oracle's parity build run
    over the member's 2000 steps with its state rounded to FP32 after every
    step (one host core); returns (index, q).  Its distance from the
    unrounded oracle run is the error any form that stores the state in
    FP32 carries on this member, before its own arithmetic adds any."""
    import oracle
    oracle.set_threads(1)
    p, B, q, steps = W.ensemble_params(index, PREC_FP64, ENS_STEPS)
    o = oracle.Oracle(p, B)
    o.set_q(W.to_aos(q))
    for _ in range(steps):
        if o.run(max_steps=1)[0] == 0:
            break
        o.replace_q(o.q().astype(np.float32).astype(np.float64))
    qo = o.q()
    o.close()
    return index, qo


# ---------------------------------------------------------------------------
# GPU ensemble legs
# ---------------------------------------------------------------------------

def ensemble_members(precision, n_runs):
    return [W.ensemble_params(i, precision, ENS_STEPS) for i in range(n_runs)]


def ensemble_batch(lib, precision, members, tile_h):
    cells = sum(m[0].comp_cells_x * m[0].comp_cells_y for m in members)
    b = lib.Batch(precision, max_runs=len(members), max_cells=int(cells * 1.2) + 4096)
    if tile_h:
        b.set_tile_shape(tile_h)
    return b


def ensemble_submit(b, members):
    ids = b.submit_many([(p, B, W.to_aos(q), st) for p, B, q, st in members])
    if any(rid is None for rid in ids):
        raise RuntimeError("ensemble member not admitted")
    return ids


def ensemble_timed(lib, precision, members, K, chunk, tile_h, keep=()):
    """Submit every member (untimed), then the K bench steps of `chunk`
    batch steps each, device-timed.  Returns the record and the final q of
    the members in `keep`."""
    b = ensemble_batch(lib, precision, members, tile_h)
    ids = ensemble_submit(b, members)
    l0 = b.launch_count()
    ms = []
    for _ in range(K):
        _, m = b.advance_timed(chunk)
        ms.append(m)
    launches = b.launch_count() - l0
    cu = sum(b.counters(i)["cell_updates"] for i in ids)
    border = sum(b.dry_border_updates(i) for i in ids)
    steps = [b.counters(i)["steps"] for i in ids]
    status = 0
    for i in ids:
        st, _ = b.poll(i)
        status |= int(st.status)
    kept = {k: b.download(ids[k]) for k in keep}
    b.close()
    dense = sum(m[0].comp_cells_x * m[0].comp_cells_y for m in members) * ENS_STEPS
    tot_ms = float(sum(ms))
    return {"runs": len(members), "steps_per_run": ENS_STEPS, "bench_steps": K,
            "batch_steps_per_bench_step": chunk,
            "cell_updates": cu, "dry_border_updates": border, "computed_cell_updates": cu - border,
            "dense_cell_steps": dense, "active_fraction": cu / dense,
            "device_ms": tot_ms, "ms_per_bench_step": tot_ms / K, "value": cu / (tot_ms / 1e3),
            "computed_value": (cu - border) / (tot_ms / 1e3), "unit": UNIT,
            "gpu_launches": launches, "min_steps_done": min(steps), "status_bits": status}, kept


def ensemble_profile(lib, members, tile_h, at_step, steps):
    """Per-kernel device time of `steps` batch steps of the FP32 ensemble
    from batch step `at_step` (events between the five kernels)."""
    b = ensemble_batch(lib, PREC_FP32, members, tile_h)
    ids = ensemble_submit(b, members)
    b.advance(at_step)
    c0 = sum(b.counters(i)["cell_updates"] for i in ids)
    d0 = sum(b.dry_border_updates(i) for i in ids)
    ms = b.profile_kernels(steps)
    c1 = sum(b.counters(i)["cell_updates"] for i in ids)
    d1 = sum(b.dry_border_updates(i) for i in ids)
    b.close()
    return ms, (c1 - c0) / steps, ((c1 - c0) - (d1 - d0)) / steps


def ensemble_e2e(lib, members, K, chunk, tile_h):
    """The ensemble through the C ABI from host buffers: submit (host set-up
    and upload), K bench steps, collect with the download of q; wall clock.
    Every run's q comes from and goes to pinned host memory (allocated and
    filled before the timed region), the topography from ordinary host
    arrays."""
    import torch
    b = ensemble_batch(lib, PREC_FP32, members, tile_h)
    pins_in, pins_out = [], []
    for _, _, q, _ in members:
        qa = W.to_aos(q)
        t_in = torch.empty(qa.size, dtype=torch.float64, pin_memory=True)
        t_in.numpy()[:] = qa
        pins_in.append(t_in)
        pins_out.append(torch.empty(qa.size, dtype=torch.float64, pin_memory=True))
    qs = [t.numpy() for t in pins_in]
    outs = [t.numpy() for t in pins_out]
    t0 = time.perf_counter()
    ids = b.submit_many([(p, B, qa, st) for (p, B, _, st), qa in zip(members, qs)])
    if any(rid is None for rid in ids):
        raise RuntimeError("ensemble member not admitted")
    t1 = time.perf_counter()
    for _ in range(K):
        b.advance(chunk)
    t2 = time.perf_counter()
    cu = sum(b.counters(rid)["cell_updates"] for rid in ids)
    qs_out = b.collect_many(ids, outs=outs)
    out_bytes = sum(q.nbytes for q in qs_out)
    t3 = time.perf_counter()
    wall = t3 - t0
    b.close()
    in_bytes = sum(qa.nbytes + B.size * 8 for (p, B, _, _), qa in zip(members, qs))
    return {"value": cu / wall, "unit": UNIT, "h2d_bytes_per_step": in_bytes / K,
            "d2h_bytes_per_step": out_bytes / K, "seconds": wall, "steps": K,
            "split_s": {"submit": t1 - t0, "steps": t2 - t1, "collect": t3 - t2},
            "path": "sflow_batch_submit_many (host set-ups and device builds on the host's threads) of "
                    "every run, sflow_batch_advance, sflow_batch_collect_many with every q downloaded; q in "
                    "and out through pinned host buffers, topography from pageable host arrays; wall clock",
            "host_threads": os.cpu_count()}


def warm_up(lib, precision, members, tile_h, steps):
    """Untimed: a scratch batch of every 8th member advanced `steps` batch
    steps (graph capture, module loading, allocator and cache warm-up)."""
    sample = members[::8]
    b = ensemble_batch(lib, precision, sample, tile_h)
    ensemble_submit(b, sample)
    b.advance(steps)
    b.close()


# ---------------------------------------------------------------------------
# single 1024^2 current
# ---------------------------------------------------------------------------

def current_workload(precision):
    p, B, _ = W.pyroclastic(nx=1024, ny=1024, dx=10.0, settling=False, precision=precision,
                            t_end=1.0e9)
    q = W.developed_current_state(p, B)
    return p, B, q


def autotune_run(s, qa, warmup, steps):
    """Tile-shape autotuner on the run itself (sflow_autotune), from the
    start state after `warmup` steps; the run is then reset to the start
    state and keeps the chosen tile height."""
    t0 = time.perf_counter()
    s.upload_q(qa)
    s.advance(max_steps=warmup)
    best, tab = s.autotune(steps)
    s.upload_q(qa)
    return {"tile_h": best, "ms_per_mcu": {str(k): v for k, v in tab.items()},
            "steps_per_height": steps, "seconds": time.perf_counter() - t0,
            "tuner": "sflow_autotune (CUDA events over graph-replayed steps of this run)"}


def timed_form(lib, p, B, q, steps, warmup, flush=True, tile_h=None):
    s = lib.Solver(p, B)
    if tile_h:
        s.set_tile_shape(tile_h)
    s.upload_q(W.to_aos(q))
    s.advance(max_steps=warmup)
    c0 = s.counters()
    l0 = s.launch_count()
    ms = s.advance_timed(steps, flush_l2=flush)
    c1 = s.counters()
    l1 = s.launch_count()
    cells = c1["cell_updates"] - c0["cell_updates"]
    return s, {"ms": ms, "cells": cells, "steps": c1["steps"] - c0["steps"],
               "launches": l1 - l0, "newton_iters": c1["newton_iters"] - c0["newton_iters"],
               "newton_max": c1["newton_max"], "tile_h": s.tile_shape()}


def current_leg(lib, steps, warmup, tune_steps, peak, peak_kind):
    """The single 1024^2 current (the benchmark configurations' second case)
    from a seeded developed state: FP32 and FP64 forms, event-timed single
    steps with L2 flushed between them, per-kernel times, k_flux roofline,
    and e2e through sflow_put_q / sflow_step / sflow_download_q from pinned
    host memory."""
    p32, B, q = current_workload(PREC_FP32)
    p64 = p32.copy()
    p64.precision = PREC_FP64
    nx, ny, nv = p32.comp_cells_x, p32.comp_cells_y, p32.n_vars
    tune = None
    if tune_steps > 0:
        st = lib.Solver(p32, B)
        tune = autotune_run(st, W.to_aos(q), warmup, tune_steps)
        st.close()
    th = tune["tile_h"] if tune else None
    s32, r32 = timed_form(lib, p32, B, q, steps, warmup, tile_h=th)
    s32.close()
    s64, r64 = timed_form(lib, p64, B, q, max(steps // 5, 3), warmup)
    s64.close()
    v32 = r32["cells"] / (r32["ms"] / 1e3)
    v64 = r64["cells"] / (r64["ms"] / 1e3)
    pk = lib.Solver(p32, B)
    pk.set_tile_shape(r32["tile_h"])
    pk.upload_q(W.to_aos(q))
    pk.advance(max_steps=warmup)
    c0 = pk.counters()
    kms = pk.profile_kernels(max(steps // 2, 3), flush_l2=True)
    c1 = pk.counters()
    pk.close()
    pk_steps = max(c1["steps"] - c0["steps"], 1)
    pk_cells = (c1["cell_updates"] - c0["cell_updates"]) / pk_steps
    alg = (2 * nv + 5) * 4 + 2       # q, 5 topography terms, flag + mask bytes, write divFlux - expl
    dur_s = kms["flux"] / 1e3 / pk_steps
    achieved = alg * pk_cells / dur_s / 1e9
    prof = read_profile("k_flux_pyroclastic_traffic")
    traffic = prof["bytes_per_active_cell"] * pk_cells if prof and prof.get("bytes_per_active_cell") else None
    out = {"workload": "pyroclastic current 1024x1024 dx=10m, ring inlet 1e6 kg/s, 2 classes, Voellmy, "
                       "N_RK=2, seeded developed state, L2 flushed between event-timed steps",
           "fp32": {"value": v32, "ms_per_step": r32["ms"] / max(r32["steps"], 1), "steps": r32["steps"],
                    "active_cells_per_step": r32["cells"] / max(r32["steps"], 1), "tile_h": r32["tile_h"],
                    "newton_iters_per_cell": r32["newton_iters"] / max(r32["cells"], 1)},
           "fp64_plain": {"value": v64, "ms_per_step": r64["ms"] / max(r64["steps"], 1), "steps": r64["steps"]},
           "speedup_fp32_over_fp64": v32 / v64 if v64 else None, "autotune": tune,
           "kernel_ms_per_step": {k: v / pk_steps for k, v in kms.items()},
           "roofline_k_flux": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                               "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                               "alg_bytes_per_active_cell": alg}}
    try:
        import torch
        pinned = torch.empty(nx * ny * nv, dtype=torch.float64, pin_memory=True)
        pinned.numpy()[:] = W.to_aos(q)
        se = lib.Solver(p32, B)
        se.set_tile_shape(r32["tile_h"])
        se.upload_q(W.to_aos(q))
        se.advance(max_steps=warmup)
        ptr = pinned.data_ptr()
        ne = max(steps // 5, 3)
        c0 = se.counters()
        se.download_q_ptr(ptr)
        t0 = time.perf_counter()
        for _ in range(ne):
            se.put_q_ptr(ptr)
            se.step()
            se.download_q_ptr(ptr)
        te = time.perf_counter() - t0
        c1 = se.counters()
        se.close()
        nbytes = nx * ny * nv * 8
        out["e2e"] = {"value": (c1["cell_updates"] - c0["cell_updates"]) / te, "unit": UNIT,
                      "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes, "steps": ne,
                      "path": "sflow_put_q + sflow_step + sflow_download_q, pinned host buffers"}
    except Exception as exc:  # pragma: no cover - reported, not hidden
        out["e2e"] = {"value": None, "error": str(exc)}
    return out


# ---------------------------------------------------------------------------
# large domain and served legs
# ---------------------------------------------------------------------------

def large_leg(lib, n, steps, warmup, tune_steps=16):
    """One n x n domain, dx = 2 m, diamond-square DEM (Hurst 0.8, relief
    2000 m, seed 5), 3 particle classes, entrainment and settling, one ring
    inlet, from a seeded developed current; timed back to back (the ~12 GB
    working set is far larger than L2)."""
    ts = time.perf_counter()
    p32, B, _ = W.large_domain(n=n, precision=PREC_FP32)
    q = W.developed_current_state(p32, B, radius=min(3500.0, 0.2 * n * p32.cell_size))
    qa = W.to_aos(q)
    del q
    out = {"cells": n * n, "workload": f"{n}x{n} dx=2m diamond-square DEM, 3 classes, entrainment + "
                                       f"settling, ring inlet, developed current"}
    res = {}
    # FP32: the configuration's `steps` steps; FP64 (~0.6 s a step): 3
    for name, prec, nst in (("fp32", PREC_FP32, steps), ("fp64_plain", PREC_FP64, min(steps, 3))):
        pp = p32.copy()
        pp.precision = prec
        s = lib.Solver(pp, B)
        if prec == PREC_FP32 and tune_steps > 0:
            out["autotune"] = autotune_run(s, qa, warmup, tune_steps)
        s.upload_q(qa)
        s.advance(max_steps=warmup)
        c0 = s.counters()
        ms = s.advance_timed(nst, flush_l2=False)
        c1 = s.counters()
        cu = c1["cell_updates"] - c0["cell_updates"]
        out[name] = {"value": cu / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / nst, "steps": nst,
                     "active_cells_per_step": cu / nst, "tile_h": s.tile_shape()}
        s.close()
    out["speedup_fp32_over_fp64"] = out["fp32"]["value"] / out["fp64_plain"]["value"]
    # FP32 against FP64 after 10 steps from the same state
    err_steps = min(steps, 10)
    for prec in (PREC_FP32, PREC_FP64):
        pp = p32.copy()
        pp.precision = prec
        s = lib.Solver(pp, B)
        s.upload_q(qa)
        s.advance(max_steps=err_steps)
        res[prec] = s.download_qp()
        s.close()
    out["error_vs_fp64"] = {"steps": err_steps, **field_errors(p32, res[PREC_FP32], res[PREC_FP64])}
    out["seconds"] = time.perf_counter() - ts
    return out


def served_leg(lib, n_requests, rate, probe_steps, tile_h=None):
    """Served solves: Poisson arrivals (mean `rate` per s) of dam-break and
    ring-inlet jobs (side log-uniform in [64, 2048], 1-3 classes, 500-5000
    steps; workloads.served_job) through the request loop (continuous
    batching, host preparation on worker threads).  Job inputs are built
    before the clock starts; time to solution = finish - arrival.

    Beside it, the same stream served one job at a time by the plain FP64
    form through a handle: every job's FP64 service time is measured on its
    own first `probe_steps` steps (set-up, upload and graph-replayed steps,
    wall clock) and scaled to its step count, and the stream is queued first
    come first served on those times.  Running the stream itself one job at
    a time would take ~20 minutes; a few jobs small enough to run whole in a
    few seconds are run whole, and their measured and scaled service times
    are reported together as a check of the scaling."""
    from imex_sflow2d_dev_gb300 import serve as S
    jobs = [W.served_job(i, PREC_FP32) for i in range(n_requests)]
    arr = W.poisson_arrivals(n_requests, rate)
    reqs = [S.Request(i, arr[i], p, B, q, st, kind) for i, (p, B, q, st, kind) in enumerate(jobs)]
    cells = sum(p.comp_cells_x * p.comp_cells_y for p, *_ in jobs)
    tuned = None
    if tile_h is None:
        # the stream's own tile height (untimed), tuned on the jobs that
        # carry most of its work: the largest by cells x steps, up to half
        # of the stream's cell-steps (at most 12 jobs)
        from imex_sflow2d_dev_gb300 import autotune as A
        t0 = time.perf_counter()
        work = [p.comp_cells_x * p.comp_cells_y * st for p, _, _, st, _ in jobs]
        order = sorted(range(len(jobs)), key=lambda i: -work[i])
        pick, acc = [], 0
        for i in order:
            if acc >= 0.5 * sum(work) or len(pick) >= 12:
                break
            pick.append(i)
            acc += work[i]
        sample = [(jobs[i][0], jobs[i][1], W.to_aos(jobs[i][2])) for i in pick]
        tile_h, rates = A.tune_batch(PREC_FP32, sample, steps=64, warm=256)
        tuned = {"tile_h": tile_h, "cell_updates_per_s": {str(k): v for k, v in rates.items()},
                 "sample": f"the {len(sample)} largest jobs ({acc / sum(work):.0%} of the stream's cell-steps), "
                           "256 + 64 batch steps per height",
                 "seconds": time.perf_counter() - t0}
    loop = S.RequestLoop(PREC_FP32, max_runs=64, max_cells=int(cells * 1.2) + 4096, chunk=16,
                         tile_h=tile_h)
    recs = loop.run(reqs)
    launches = loop.batch.launch_count()
    loop.close()
    out = S.summarize(recs)
    out.update({"rate_per_s": rate, "gpu_launches": launches, "tile_h": tile_h or 8, "autotune": tuned})
    # one job at a time, plain FP64 form
    t0 = time.perf_counter()
    service = []
    check = []
    for i, (p, B, q, st, kind) in enumerate(jobs):
        p64 = p.copy()
        p64.precision = PREC_FP64
        n = min(probe_steps, st)
        ts = time.perf_counter()
        s = lib.Solver(p64, B)
        s.upload_q(W.to_aos(q))
        s.advance(max_steps=n)
        probe = time.perf_counter() - ts
        est = probe * st / n
        if p.comp_cells_x <= 128 and len(check) < 6:
            s.advance(max_steps=st - n)
            whole = time.perf_counter() - ts
            check.append({"request": i, "steps": st, "measured_s": whole, "scaled_s": est})
        s.close()
        service.append(est)
    clock = 0.0
    tts = []
    for i in np.argsort(arr, kind="stable"):
        clock = max(clock, arr[i]) + service[i]
        tts.append(clock - arr[i])
    tts = np.array(tts)
    total_cu = sum(r["cell_updates"] for r in recs)
    span = clock - float(arr.min())
    out["fp64_one_at_a_time"] = {
        "requests": n_requests, "p50_s": float(np.percentile(tts, 50)), "p99_s": float(np.percentile(tts, 99)),
        "makespan_s": span, "cell_updates_per_s": total_cu / max(span, 1e-12),
        "probe_steps": probe_steps, "probe_seconds": time.perf_counter() - t0,
        "whole_job_check": check,
        "basis": ("each job's plain-FP64 service time measured over its first steps (set-up, upload, "
                  "graph-replayed steps) and scaled to its step count; FCFS queue on the stream's "
                  "arrival times")}
    out["jobs"] = [{k: r[k] for k in ("kind", "cells", "n_solid", "steps", "tts_s")} for r in recs]
    return out


# ---------------------------------------------------------------------------
# arms
# ---------------------------------------------------------------------------

def run_reference(args, d):
    """The reference arm: the reference's CPU path (the oracle, built with
    the reference's compiler flags) on a bounded sample of the same
    ensemble, same K and W."""
    if d.rank != 0:
        return 0
    cb = cpu_ensemble_sample(args.steps, args.warmup * max(1, CPU_SAMPLE_STEPS // args.steps))
    line = {
        "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * cb["seconds"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded DEMs and per-run draws)",
        "config": {"workload": WORKLOAD, "precision": "FP64 CPU",
                   "bench_step": f"{cb['chunk_steps']} time steps of every sampled member",
                   "implementation": "oracle/sflow_oracle.c (C restatement of the Fortran reference, "
                                     "which has no compiler on this box), reference compiler flags"},
        "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def log(msg):
    print(f"[bench] {msg}", file=sys.stderr, flush=True)


def run_gb300(args, d):
    from imex_sflow2d_dev_gb300 import lib
    lib.load()
    K, Wm = args.steps, args.warmup
    chunk = int(math.ceil(ENS_STEPS / K))
    peak, peak_kind = read_peaks()
    n_runs = args.ensemble_runs

    cb = None
    if d.rank == 0 and not args.no_cpu_baseline:
        cb = cpu_ensemble_sample(K, Wm * max(1, CPU_SAMPLE_STEPS // K))
        log(f"cpu baseline {cb['value']:.3e}")

    members32 = ensemble_members(PREC_FP32, n_runs)
    members64 = ensemble_members(PREC_FP64, n_runs)
    tuned = None
    th = args.tile_h or None
    if not th and args.tune_steps > 0:
        from imex_sflow2d_dev_gb300 import autotune as A
        t0 = time.perf_counter()
        sample = [(p, B, W.to_aos(q)) for p, B, q, _ in members32[::8]]
        # timed from batch step 1000 of the 2000: the currents have grown
        # to their typical size (the first steps see small ones only)
        best, rates = A.tune_batch(PREC_FP32, sample, steps=128, warm=1000)
        tuned = {"tile_h": best, "cell_updates_per_s": {str(k): v for k, v in rates.items()},
                 "sample": f"{len(sample)} runs (every 8th member), 1000 + 128 batch steps per height, "
                           "device time; 32x8 kept unless another height is > 2 % faster",
                 "seconds": time.perf_counter() - t0, "tuner": "autotune.tune_batch"}
        th = best
    warm_up(lib, PREC_FP32, members32, th, Wm * chunk)

    # timed region: the FP32 ensemble, K bench steps
    err_members = sorted(range(n_runs), key=lambda i: members32[i][0].comp_cells_x)[:args.oracle_members]
    clocks = ClockSampler(d.local)
    d.barrier()
    clocks.start()
    t_wall0 = time.perf_counter()
    r32, q32 = ensemble_timed(lib, PREC_FP32, members32, K, chunk, th, keep=err_members)
    t_wall1 = time.perf_counter()
    clk = clocks.stop()
    d.barrier()
    value, ms_max = aggregate(d, r32["cell_updates"], r32["device_ms"])
    log(f"ensemble fp32 {value:.3e} ({r32['device_ms']:.1f} ms)")

    # the oracle on the smallest members (host cores) while the GPU runs FP64
    pool = res_or = None
    if d.rank == 0 and args.oracle_members > 0:
        ctx = mp.get_context("spawn")
        pool = ctx.Pool(processes=len(err_members))
        res_or = pool.map_async(_oracle_member_worker, err_members)
    warm_up(lib, PREC_FP64, members64, None, 16)
    r64, q64 = ensemble_timed(lib, PREC_FP64, members64, K, chunk, None, keep=err_members)
    value64 = r64["value"]
    log(f"ensemble fp64 {value64:.3e} ({r64['device_ms']:.1f} ms)")
    err_fp64, err_oracle = [], []
    if res_or is not None:
        orc = dict(res_or.get())
        pool.close()
        pool.join()
        for k in err_members:
            p, B = members64[k][0], members64[k][1]
            err_oracle.append(field_errors(p, qp_of_state(p, B, q32[k]), qp_of_state(p, B, orc[k])))
            err_fp64.append(float(np.abs(q64[k] - orc[k]).max() / max(np.abs(orc[k]).max(), 1e-300)))

    # e2e through the C ABI from host buffers
    e2e = ensemble_e2e(lib, members32, K, chunk, th)
    log(f"ensemble e2e {e2e['value']:.3e}")

    # members above the h bar: the oracle's own FP32 rounding band (spawned
    # processes, while the GPU runs the legs below)
    over = [k for k, e in zip(err_members, err_oracle) if e["h"]["l1_rel"] > H_L1_BAR]
    band_res = None
    if over:
        pool = mp.get_context("spawn").Pool(processes=len(over))
        band_res = pool.map_async(_band_member_worker, over)

    # per-kernel device times of the developed ensemble and the roofline of
    # its dominant kernel (algorithmic bytes per computed cell: the dry
    # border tiles are counted but not touched)
    kms, cells_launch, computed_launch = ensemble_profile(lib, members32, th, ENS_STEPS // 2, 16)
    dom = max(kms, key=lambda k: kms[k])
    nv = 6
    alg_bytes = {"flux": (2 * nv + 5) * 4 + 2,           # q, 5 topography terms, flags, write divFlux - expl
                 "stage": (3 * nv + 3 + 6) * 4 + 1 + 32,  # q, increment, 3 topography, maps rw, mask, deposit rw
                 "mask": 4 + 1 + 1, "cand": 0, "dt": 0}
    launch_s = kms[dom] / 1e3 / 16
    achieved = alg_bytes[dom] * computed_launch / launch_s / 1e9
    prof = read_profile("k_b_flux_ensemble_64") if dom == "flux" else None
    traffic = (prof["dram_bytes_per_computed_cell"] * computed_launch
               if prof and prof.get("dram_bytes_per_computed_cell") else None)
    roofline = {"bound": "hbm", "kernel": "k_b_" + dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                "alg_bytes_per_computed_cell": alg_bytes[dom],
                "computed_cells_per_launch": computed_launch, "active_cells_per_launch": cells_launch,
                "kernel_ms_per_step": {k: v / 16 for k, v in kms.items()},
                "kernel_share": {k: v / sum(kms.values()) for k, v in kms.items()},
                "profile_window": f"16 batch steps from step {ENS_STEPS // 2}, events between kernels"}
    if prof:
        roofline["traffic_source"] = (f"profiles/k_b_flux_ensemble_64.json: ncu DRAM bytes per computed cell "
                                      f"({prof['tile']} tiles) x computed cells of this launch")
    if prof and prof.get("warp_inst_per_computed_cell") and prof.get("issue_peak_warp_inst_per_s"):
        roofline["issue_frac"] = (prof["warp_inst_per_computed_cell"] * computed_launch / launch_s
                                  / prof["issue_peak_warp_inst_per_s"])
    log(f"profile {roofline['kernel_ms_per_step']}")

    per_member = {}
    for k, e in zip(err_members, err_oracle):
        per_member[str(k)] = {"h_l1": e["h"]["l1_rel"], "h_linf": e["h"]["linf_rel"]}
    if band_res is not None:
        for k, qb in band_res.get():
            p, B = members64[k][0], members64[k][1]
            band = field_errors(p, qp_of_state(p, B, qb), qp_of_state(p, B, orc[k]))
            per_member[str(k)]["fp32_rounding_band_h_l1"] = band["h"]["l1_rel"]
            per_member[str(k)]["fp32_rounding_band_h_linf"] = band["h"]["linf_rel"]
        pool.close()
        pool.join()

    cur = None
    if d.rank == 0 and args.current_steps > 0:
        cur = current_leg(lib, args.current_steps, Wm, args.tune_steps, peak, peak_kind)
        log(f"current 1024 {cur['fp32']['value']:.3e}")
    large = None
    if d.rank == 0 and args.large_n > 0:
        large = large_leg(lib, args.large_n, args.large_steps, Wm, tune_steps=16 if args.tune_steps > 0 else 0)
        log(f"large {large['fp32']['value']:.3e}")
    srv = None
    if d.rank == 0 and args.served_requests > 0:
        srv = served_leg(lib, args.served_requests, args.served_rate, args.served_probe_steps,
                         tile_h=args.tile_h or (None if args.tune_steps > 0 else 8))
        log(f"served p50 {srv['p50_s']:.2f} p99 {srv['p99_s']:.2f}")

    if d.rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": K, "warmup": Wm, "ms_per_step": ms_max / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded cone+fBm DEMs, per-run draws; empty initial states)",
            "config": {"workload": WORKLOAD, "runs": n_runs, "steps_per_run": ENS_STEPS,
                       "bench_step": f"{chunk} batch steps of all runs",
                       "form": "FP32 bulk + FP64 implicit Newton, FP64 log sums and wet/dry tests",
                       "l2": "inputs larger than L2 (~6 GB resident; ~200 MB of active tiles per step)",
                       "parallelism": f"replicas x{args.gpus}", "tile": f"32x{th or 8} cells",
                       "dense_cell_steps": r32["dense_cell_steps"],
                       "active_fraction": r32["active_fraction"],
                       "computed_cell_updates_per_s": aggregate(d, r32["computed_cell_updates"],
                                                                r32["device_ms"])[0],
                       "computed_note": "active cells minus the dry border tiles the kernels skip "
                                        "(counted as active, as in the reference)"},
            "ensemble_fp32": r32,
            "fp64_plain": {"value": value64, "same_workload": True, **{k: r64[k] for k in (
                "device_ms", "ms_per_bench_step", "cell_updates", "gpu_launches", "min_steps_done")}},
            "speedup_fp32_over_fp64": value / value64 if value64 else None,
            "error_vs_oracle": ({"members": err_members, "steps": ENS_STEPS,
                                 "fp32_worst": worst(err_oracle),
                                 "h_l1_bar": H_L1_BAR,
                                 "members_within_h_bar": sum(e["h"]["l1_rel"] <= H_L1_BAR for e in err_oracle),
                                 "per_member": per_member,
                                 "band_note": "fp32_rounding_band_*: the oracle with its state rounded to FP32 "
                                              "after every step against the unrounded oracle (members above "
                                              "the bar only)",
                                 "fp64_max_rel_q": max(err_fp64) if err_fp64 else None}
                                if err_oracle else None),
            "autotune": tuned,
            "roofline": roofline,
            "cpu_baseline": ({k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
                             if cb else None),
            "e2e": e2e,
            "gpu_launches": r32["gpu_launches"],
            "current_1024": cur,
            "served": srv,
            "large_domain": large,
            "clocks": clk,
            "wall_s_timed_region": t_wall1 - t_wall0,
        }
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ensemble-runs", type=int, default=ENS_RUNS)
    ap.add_argument("--oracle-members", type=int, default=8,
                    help="smallest members checked against the oracle over their 2000 steps")
    ap.add_argument("--current-steps", type=int, default=20)
    ap.add_argument("--served-requests", type=int, default=200)
    ap.add_argument("--served-rate", type=float, default=20.0)
    ap.add_argument("--served-probe-steps", type=int, default=16,
                    help="steps of each job run by the plain FP64 form to measure its service time")
    ap.add_argument("--large-n", type=int, default=8192)
    ap.add_argument("--large-steps", type=int, default=200,
                    help="FP32 steps of the large-domain leg (the configuration's run length)")
    ap.add_argument("--tune-steps", type=int, default=64,
                    help="steps per tile height of the autotuners (0: default 32x8 tiles)")
    ap.add_argument("--tile-h", type=int, default=0, choices=[0, 8, 16, 4],
                    help="FP32 tile height of the ensemble without the autotuner (0: autotune)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    d = Dist()
    try:
        if args.impl == "reference":
            return run_reference(args, d)
        return run_gb300(args, d)
    finally:
        d.close()


if __name__ == "__main__":
    sys.exit(main())

"""Request loop over the batched engine (continuous batching).

Independent solves arrive over time.  Each arrived request is prepared on
a worker thread (validation, topography terms and ring-inlet geometry on
the host: sflow_setup_create, which needs no GPU), while the GPU advances
the resident runs.  At every chunk boundary the loop admits the prepared
requests in arrival order while the batch accepts them -- a free slot,
tile-list capacity and free device memory, checked by
sflow_batch_submit_setup_take, which answers SFLOW_EBUSY otherwise and
otherwise hands the prepared host arrays to the run without a copy -- launches
`chunk` batch steps of every resident run (one CUDA-graph replay per
solid-class count, the groups on their own streams; sflow_batch_launch
returns at once), waits for the device (sflow_batch_wait; the worker
threads keep preparing meanwhile) and collects the runs that have stopped
(sflow_batch_collect_many).
A request that arrives while others are on the GPU joins them at the next
chunk boundary; its state stays resident until it is collected.

Per request it records arrival, preparation, admission and finish times,
the time to solution (finish - arrival), steps and cell updates.  No
counterpart in the reference, which runs one job per process.
"""
import concurrent.futures as cf
import time

import numpy as np

from . import lib as L
from . import workloads as W


class Request:
    def __init__(self, rid, arrival_s, params, B_cent, q, max_steps, kind=""):
        self.rid = rid
        self.arrival_s = float(arrival_s)
        self.params = params
        self.B = B_cent
        self.q_aos = W.to_aos(q) if q.ndim == 3 else q
        self.max_steps = int(max_steps)
        self.kind = kind


class RequestLoop:
    def __init__(self, precision, max_runs=256, max_cells=1 << 28, chunk=16, keep_results=False,
                 tile_h=None, prep_threads=4):
        self.precision = precision
        self.batch = L.Batch(precision, max_runs=max_runs, max_cells=max_cells)
        if tile_h:
            self.batch.set_tile_shape(tile_h)
        self.chunk = chunk
        self.keep = keep_results
        self.prep_threads = prep_threads

    def close(self):
        self.batch.close()

    def _prepare(self, r, t0):
        st = L.Setup(r.params, r.B, precision=self.precision)
        return st, time.perf_counter() - t0

    def run(self, requests):
        """Serve `requests` (arrival times relative to the start of the
        call); returns one record per request, in request order."""
        pending = sorted(requests, key=lambda r: r.arrival_s)
        recs = {}
        live = {}
        queue = []          # (request, future): being prepared or prepared, arrival order
        t0 = time.perf_counter()
        i = 0
        with cf.ThreadPoolExecutor(max_workers=self.prep_threads) as pool:
            while i < len(pending) or queue or live:
                now = time.perf_counter() - t0
                # every arrived request starts its host preparation at once
                while i < len(pending) and pending[i].arrival_s <= now:
                    queue.append((pending[i], pool.submit(self._prepare, pending[i], t0)))
                    i += 1
                # admit prepared requests in arrival order while the batch accepts
                while queue and queue[0][1].done():
                    r, fut = queue[0]
                    setup, prep_s = fut.result()
                    bid = self.batch.submit_setup(setup, r.q_aos, max_steps=r.max_steps, take=True)
                    if bid is None:
                        if not live:
                            raise RuntimeError(f"request {r.rid} does not fit an empty batch")
                        break
                    setup.close()
                    queue.pop(0)
                    live[bid] = r
                    recs[r.rid] = {"rid": r.rid, "kind": r.kind, "arrival_s": r.arrival_s,
                                   "prepared_s": prep_s, "admitted_s": time.perf_counter() - t0,
                                   "cells": r.params.comp_cells_x * r.params.comp_cells_y,
                                   "n_solid": r.params.n_solid, "max_steps": r.max_steps}
                if not live:
                    # idle: wait for a preparation or the next arrival
                    if queue:
                        cf.wait([queue[0][1]], timeout=0.05)
                    elif i < len(pending):
                        time.sleep(max(0.0, min(0.05, pending[i].arrival_s - (time.perf_counter() - t0))))
                    continue
                self.batch.launch(self.chunk)
                finished = self.batch.wait()
                if finished:
                    done = [b for b in live if self.batch.done(b)]
                    stats = [(self.batch.counters(b), self.batch.poll(b)[0]) for b in done]
                    qs = self.batch.collect_many(done, want_q=self.keep)
                    t_fin = time.perf_counter() - t0
                    for bid, (c, st), q in zip(done, stats, qs):
                        r = live.pop(bid)
                        rec = recs[r.rid]
                        rec["finished_s"] = t_fin
                        rec["tts_s"] = rec["finished_s"] - r.arrival_s
                        rec["steps"] = c["steps"]
                        rec["cell_updates"] = c["cell_updates"]
                        rec["status"] = int(st.status)
                        if self.keep:
                            rec["q"] = q
        return [recs[r.rid] for r in requests]


def summarize(records):
    tts = np.array([r["tts_s"] for r in records])
    cells = sum(r["cell_updates"] for r in records)
    t_first = min(r["arrival_s"] for r in records)
    t_last = max(r["finished_s"] for r in records)
    return {"requests": len(records), "p50_s": float(np.percentile(tts, 50)),
            "p99_s": float(np.percentile(tts, 99)), "max_s": float(tts.max()),
            "cell_updates": int(cells), "makespan_s": t_last - t_first,
            "cell_updates_per_s": cells / max(t_last - t_first, 1e-12)}

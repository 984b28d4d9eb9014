"""Tile-shape autotuner.

The tiled kernels (check_solve, flux, stage) work on tiles of 32 x TH cells.
The tile height TH trades halo work against skipped dry area and
occupancy: a tall tile recomputes fewer halo cells and faces per cell and
fits the large wet current of one big domain, a short tile skips more of
the dry ground around the small currents of an ensemble.  Which wins depends
on the workload and is measured, not guessed:

  * a single run: ``Solver.autotune(steps)`` (C ABI ``sflow_autotune``)
    times graph-replayed steps of the run itself with every compiled height
    and keeps the fastest per active-cell update (a height other than the
    default 32 x 8 only when it is more than 2 % faster).  The results of a
    step do not depend on the height, so the tuning steps are ordinary
    steps.
  * a batch: ``tune_batch`` advances a sample of the batch's runs in a
    scratch batch once per height and returns the height with the most
    cell-updates/s (with the same 2 % margin); the real batch is then made
    with ``Batch.set_tile_shape``.

``TuneCache`` keeps the choices in a JSON file keyed by device, precision,
solid classes and a size class, so a service tunes a workload class once.
"""
import json
import math
import os

from . import lib as L


def size_class(cells):
    """log2 bucket of a domain size (cells)."""
    return int(math.floor(math.log2(max(int(cells), 1))))


def tune_solver(solver, steps=64):
    """Tune a single run in place; returns (height, {height: ms per 10^6
    cell updates})."""
    return solver.autotune(steps)


def tune_batch(precision, members, steps=128, warm=16, heights=None, max_cells=None, margin=0.02):
    """Time `members` ((params, B_cent, q_aos) triples) in a scratch batch
    once per tile height: `warm` untimed batch steps, then `steps` timed
    ones (device time of the steps, CUDA events).  The first height (the
    default, 32 x 8) is kept unless another one is faster by more than
    `margin` (a near tie is measurement noise, not a better shape).
    Returns (chosen height, {height: cell-updates/s})."""
    heights = list(heights or L.tile_shapes(precision))
    cells = sum(p.comp_cells_x * p.comp_cells_y for p, _, _ in members)
    if max_cells is None:
        max_cells = int(cells * 1.2) + 4096
    rates = {}
    for th in heights:
        b = L.Batch(precision, max_runs=len(members), max_cells=max_cells)
        try:
            b.set_tile_shape(th)
            ids = []
            for p, B, q in members:
                rid = b.submit(p, B, q, max_steps=warm + steps)
                if rid is None:
                    raise RuntimeError("autotune sample does not fit the device")
                ids.append(rid)
            b.advance(warm)
            c0 = sum(b.counters(i)["cell_updates"] for i in ids)
            _, ms = b.advance_timed(steps)
            c1 = sum(b.counters(i)["cell_updates"] for i in ids)
            rates[th] = (c1 - c0) / (ms * 1e-3) if ms > 0 else 0.0
        finally:
            b.close()
    return choose(heights, rates, margin), rates


def choose(heights, rates, margin=0.02):
    """The height to keep from measured rates (higher is better): the first
    height (the default) unless a later one beats the best so far by more
    than `margin`."""
    best = heights[0]
    for th in heights[1:]:
        if rates[th] > rates[best] * (1.0 + margin):
            best = th
    return best


class TuneCache:
    """Chosen tile heights in a JSON file: {key: {"tile_h": h, "score": {...}}}."""

    def __init__(self, path):
        self.path = path
        self.data = {}
        if path and os.path.exists(path):
            with open(path) as f:
                self.data = json.load(f)

    @staticmethod
    def key(kind, precision, n_solid, cells, device=""):
        return f"{device}|{kind}|p{int(precision)}|ns{int(n_solid)}|s{size_class(cells)}"

    def get(self, key):
        e = self.data.get(key)
        return e["tile_h"] if e else None

    def put(self, key, tile_h, score):
        self.data[key] = {"tile_h": int(tile_h), "score": {str(k): v for k, v in score.items()}}
        if self.path:
            tmp = self.path + ".tmp"
            with open(tmp, "w") as f:
                json.dump(self.data, f, indent=1, sort_keys=True)
            os.replace(tmp, self.path)

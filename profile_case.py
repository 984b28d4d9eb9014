"""A short run of the benchmark workloads for profilers (ncu), beside
bench.py: the commands recorded under profiles/ run it.

    python profile_case.py --n 2048 --steps 6 --precision fp32
    python profile_case.py --ensemble 256 --steps 64

--ensemble N: the first N members of the batched ensemble (side
log-uniform in [128, 1024], own DEM and parameters) submitted to one batch
and advanced `steps` batch steps (FP32 bulk form), for a launch list of the
batched kernels.

Otherwise: builds the n x n version of the benchmark workload (cone + fBm DEM with
dx = 10240/n m, seeded developed-current state), uploads it and runs
`steps` driver iterations one at a time (no graph, so every kernel is a
separate launch).  With n = 2048 the FP32 working set (~400 MB) exceeds the
126 MB L2, so DRAM counters of a single launch are meaningful.
"""
import argparse
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from imex_sflow2d_dev_gb300 import lib  # noqa: E402
from imex_sflow2d_dev_gb300 import workloads as W  # noqa: E402
from imex_sflow2d_dev_gb300.params import PREC_FP32, PREC_FP64  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--ensemble", type=int, default=0)
    ap.add_argument("--tile-h", type=int, default=8, help="tile height (8, or 16 in FP32)")
    a = ap.parse_args()
    if a.ensemble > 0:
        members = [W.ensemble_params(i, PREC_FP32, 100000) for i in range(a.ensemble)]
        cells = sum(m[0].comp_cells_x * m[0].comp_cells_y for m in members)
        b = lib.Batch(PREC_FP32, max_runs=a.ensemble, max_cells=int(cells * 1.2) + 4096)
        b.set_tile_shape(a.tile_h)
        ids = [b.submit(p, B, W.to_aos(q), max_steps=st) for p, B, q, st in members]
        b.advance(a.steps)
        cu = sum(b.counters(i)["cell_updates"] for i in ids)
        border = sum(b.dry_border_updates(i) for i in ids)
        print(f"ensemble runs={a.ensemble} cells={cells} steps={a.steps} cell_updates={cu} "
              f"dry_border_updates={border} computed_cell_updates={cu - border}")
        b.close()
        return
    prec = PREC_FP32 if a.precision == "fp32" else PREC_FP64
    p, B, _ = W.pyroclastic(nx=a.n, ny=a.n, dx=10240.0 / a.n, settling=False, precision=prec,
                            t_end=1.0e9)
    q = W.developed_current_state(p, B)
    s = lib.Solver(p, B)
    s.set_tile_shape(a.tile_h)
    s.upload_q(W.to_aos(q))
    for _ in range(a.steps):
        s.step()
    st = s.stats()
    c = s.counters()
    print(f"n={a.n} precision={a.precision} tile=32x{a.tile_h} steps={st.steps} t={st.t:.4f} "
          f"active/step={c['cell_updates'] / max(c['steps'], 1):.0f} status={st.status}")
    s.close()


if __name__ == "__main__":
    main()

"""One domain split into row slabs (domain decomposition by rows).

Each slab is a handle of `sflow_create_rows`: it holds its own rows plus a
halo of `halo` rows on each inner side, derives its topography terms, inlet
geometry and flags on the whole domain, and counts only its own rows in its
CFL minimum, active cells, status bits and log sums.  A step is the
reference driver's call sequence (IMEX_SfloW2D.f90:395-505) on every slab:

    check_solve(.FALSE.)                           each slab
    timestep                                       each slab: CFL minimum of its own rows
    dt = min over the slabs                        the reduction of solver_2d.f90:995-996
         + the driver's clamps (IMEX_SfloW2D.f90:417-439)
    imex_RK_solver, update_erosion_deposition_cell, post-step maxima
    halo exchange: each slab's `halo` own rows next to a neighbour go to
                   that neighbour's halo

With N_RK = 2 the flux pass runs once per step, at the step's start; it
reads q up to 2 rows away, and the active mask of those rows reads q up to
2 rows further, so a 4-row halo refreshed once per step gives every own cell
the undivided domain's update, bit for bit in the plain FP64 form.

Two exchanges: `LocalExchange` keeps every slab in this process (one GPU;
rows travel through host memory), `DistExchange` gives each rank of a
torch.distributed group one slab (rows and the dt minimum through the
group's send/recv and all_reduce).  No counterpart in the reference, which
runs one domain in one process (OpenMP).
"""
import numpy as np

from . import lib as L


def partition(ny, parts, halo):
    """Own and held rows of `parts` slabs over ny rows: [(own_a, own_b,
    held_lo, held_hi)] with every slab owning at least `halo` rows."""
    if parts < 1 or ny // parts < max(halo, 5):
        raise ValueError("too many slabs for the rows (each must own >= max(halo, 5) rows)")
    cuts = [ny * i // parts for i in range(parts + 1)]
    out = []
    for i in range(parts):
        a, b = cuts[i], cuts[i + 1]
        out.append((a, b, max(0, a - halo), min(ny, b + halo)))
    return out


def clamp_dt(dt, t, t_end, t_output, dt_old, dt_old_old):
    """The driver's dt clamps (IMEX_SfloW2D.f90:417-439), in the device's
    order and FP64 arithmetic; returns (dt, t_output)."""
    if t_end - t_output < 1.0e-7:
        t_output = t_end
    if t + dt > t_end:
        dt = t_end - t
    if t + dt > t_output:
        dt = t_output - t
    lim = 1.1 * 0.5 * (dt_old + dt_old_old)
    if lim < dt:
        dt = lim
    return dt, t_output


class LocalExchange:
    """Every slab in this process."""

    def __init__(self, parts):
        self.ranks = list(range(parts))

    def min(self, values):
        return min(values.values())

    def sum(self, values):
        return sum(values.values())

    def swap(self, slabs, send):
        """send[(i, j)] = rows slab i gives slab j; returns recv[(j, i)]."""
        return {(j, i): rows for (i, j), rows in send.items()}


class DistExchange:
    """One slab per rank of a torch.distributed process group."""

    def __init__(self, rank, world):
        import torch
        import torch.distributed as dist
        self.torch, self.dist = torch, dist
        self.rank, self.world = rank, world
        self.ranks = [rank]

    def _reduce(self, value, op):
        t = self.torch.tensor([float(value)], dtype=self.torch.float64)
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def min(self, values):
        return self._reduce(values[self.rank], self.dist.ReduceOp.MIN)

    def sum(self, values):
        return self._reduce(values[self.rank], self.dist.ReduceOp.SUM)

    def swap(self, slabs, send):
        torch, dist = self.torch, self.dist
        reqs, recv = [], {}
        for (i, j), rows in send.items():
            reqs.append(dist.isend(torch.from_numpy(np.ascontiguousarray(rows)), dst=j))
        for (j, i), shape in slabs[self.rank].expect.items():
            buf = torch.empty(shape, dtype=torch.float64)
            reqs.append(dist.irecv(buf, src=i))
            recv[(j, i)] = buf
        for r in reqs:
            r.wait()
        return {k: v.numpy() for k, v in recv.items()}


class Slab:
    def __init__(self, index, own, held, engine):
        self.index = index
        self.own_a, self.own_b = own
        self.lo, self.hi = held
        self.engine = engine
        self.expect = {}


def solver_engine(params, B, slab_rows):
    """GPU engine: a row-slab handle (sflow_create_rows)."""
    k0, n, lo, hi = slab_rows
    return L.Solver(params, B, rows=(k0, n, lo, hi))


class RowSlabs:
    """A domain of `params` / `B` advanced as `parts` row slabs.

    engine(params, B, (k0, rows, own_lo, own_hi)) makes one slab's solver
    (default: a GPU slab handle); it must offer check_solve, timestep,
    imex_rk_solver, update_erosion_deposition_cell, post_step, upload_q,
    get_rows and put_rows as lib.Solver does."""

    def __init__(self, params, B, q_aos, parts, halo=4, exchange=None, engine=solver_engine):
        self.p = params.copy()
        self.nx, self.ny, self.nv = params.comp_cells_x, params.comp_cells_y, params.n_vars
        self.halo = halo
        self.parts = partition(self.ny, parts, halo)
        self.x = exchange or LocalExchange(parts)
        q = np.ascontiguousarray(q_aos, dtype=np.float64).reshape(self.ny, self.nx, self.nv)
        self.slabs = {}
        for i in self.x.ranks:
            a, b, lo, hi = self.parts[i]
            eng = engine(self.p, B, (lo, hi - lo, a - lo, b - lo))
            eng.upload_q(q[lo:hi].reshape(-1))
            self.slabs[i] = Slab(i, (a, b), (lo, hi), eng)
        for i, s in self.slabs.items():
            for j in (i - 1, i + 1):
                if 0 <= j < len(self.parts):
                    rows = self._halo_rows(i, j)[1] - self._halo_rows(i, j)[0]
                    s.expect[(i, j)] = (rows * self.nx * self.nv,)
        self.t = params.t_start
        self.dt_old = self.dt_old_old = params.dt0
        self.t_output = params.t_start + params.dt_output
        self.steps = 0

    def _halo_rows(self, i, j):
        """Global rows of slab i's halo that slab j owns (j = i +- 1)."""
        a, b, lo, hi = self.parts[i]
        return (lo, a) if j < i else (b, hi)

    def step(self):
        p = self.p
        if not (self.t < p.t_end):
            return None
        for s in self.slabs.values():
            s.engine.check_solve(False)
        dt = self.x.min({i: s.engine.timestep() for i, s in self.slabs.items()})
        dt, self.t_output = clamp_dt(dt, self.t, p.t_end, self.t_output, self.dt_old, self.dt_old_old)
        self.dt_old_old, self.dt_old = self.dt_old, dt
        stats = {}
        for i, s in self.slabs.items():
            s.engine.imex_rk_solver(self.t, dt)
            s.engine.update_erosion_deposition_cell(dt)
            stats[i] = s.engine.post_step()
        self.t = stats[next(iter(stats))].t
        self.steps += 1
        self._exchange()
        return stats

    def _exchange(self):
        send = {}
        for i, s in self.slabs.items():
            for j in (i - 1, i + 1):
                if not 0 <= j < len(self.parts):
                    continue
                r0, r1 = self._halo_rows(j, i)          # rows of j's halo that i owns
                send[(i, j)] = s.engine.get_rows(r0 - s.lo, r1 - r0)
        recv = self.x.swap(self.slabs, send)
        for (j, i), rows in recv.items():
            s = self.slabs[j]
            r0, r1 = self._halo_rows(j, i)
            s.engine.put_rows(r0 - s.lo, r1 - r0, rows)

    def run(self, steps):
        for _ in range(steps):
            if self.step() is None:
                break

    def own_q(self):
        """{slab: own rows of q (reference layout)} of the slabs held here."""
        out = {}
        for i, s in self.slabs.items():
            out[i] = s.engine.get_rows(s.own_a - s.lo, s.own_b - s.own_a)
        return out

    def gather_q(self):
        """The whole domain's q (reference layout), local exchange only."""
        own = self.own_q()
        return np.concatenate([own[i] for i in sorted(own)])

"""A small CPU stand-in for a slab solver (test helper): an explicit
two-row-radius stencil on numpy arrays with the per-call interface of
lib.Solver, so the row-slab driver's partition, halo exchange and dt
reduction can be checked on CPU ranks without a GPU.  Its dt depends on the
whole own state (a global reduction is needed) and its update reads q two
rows away (one halo refresh per step is needed)."""
import numpy as np


class _Stats:
    def __init__(self, t, dt, steps):
        self.t, self.dt, self.steps = t, dt, steps


class StencilEngine:
    def __init__(self, params, B, slab_rows=None):
        self.nx, self.nv = params.comp_cells_x, params.n_vars
        if slab_rows is None:
            self.k0, self.n, self.lo, self.hi = 0, params.comp_cells_y, 0, params.comp_cells_y
        else:
            self.k0, self.n, self.lo, self.hi = slab_rows
        self.t, self.steps = params.t_start, 0
        self.q = None

    def upload_q(self, q_aos):
        self.q = np.array(q_aos, dtype=np.float64).reshape(self.n, self.nx, self.nv)

    def check_solve(self, solve_all=False):
        pass

    def timestep(self):
        own = self.q[self.lo:self.hi]
        return 0.5 / (1.0 + np.abs(own).max())

    def imex_rk_solver(self, t, dt):
        q = self.q
        pad = np.concatenate([q[:1], q[:1], q, q[-1:], q[-1:]])      # edge rows repeated
        lap = pad[:-4] + pad[4:] + 2.0 * (pad[1:-3] + pad[3:-1]) - 6.0 * q
        side = np.roll(q, 1, axis=1) - q
        self.q = q + dt * (0.1 * lap + 0.05 * side * np.tanh(q))
        self._dt = dt

    def update_erosion_deposition_cell(self, dt):
        pass

    def post_step(self):
        self.t = self.t + self._dt
        self.steps += 1
        return _Stats(self.t, self._dt, self.steps)

    def get_rows(self, k_lo, n):
        return self.q[k_lo:k_lo + n].reshape(-1).copy()

    def put_rows(self, k_lo, n, rows):
        self.q[k_lo:k_lo + n] = np.asarray(rows).reshape(n, self.nx, self.nv)


def engine(params, B, slab_rows):
    return StencilEngine(params, B, slab_rows)

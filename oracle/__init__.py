"""Python handle on the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package.  It wraps oracle/libsflow_oracle.so, a C restatement of the
reference time step (see the header of sflow_oracle.c for its status).
"""
import ctypes as C
import os

import numpy as np

from .build import LIB, LIB_FAST, build_oracle

_lib = None
_lib_fast = None


def _load(timing=False):
    """The parity build, or with timing=True the build with the reference's
    compiler flags (used only to time the CPU baseline)."""
    global _lib, _lib_fast
    if timing and _lib_fast is not None:
        return _lib_fast
    if not timing and _lib is not None:
        return _lib
    build_oracle()
    lib = C.CDLL(LIB_FAST if timing else LIB)
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.c_int
    lib.sflow_oracle_create.restype = vp
    lib.sflow_oracle_create.argtypes = [vp, dp]
    lib.sflow_oracle_destroy.argtypes = [vp]
    lib.sflow_oracle_set_q.argtypes = [vp, dp]
    lib.sflow_oracle_replace_q.argtypes = [vp, dp]
    lib.sflow_oracle_replace_q.restype = None
    lib.sflow_oracle_step.argtypes = [vp]
    lib.sflow_oracle_run.restype = ip
    lib.sflow_oracle_run.argtypes = [vp, C.c_double, C.c_int64, C.POINTER(C.c_int64)]
    for f in ("get_q", "get_qp"):
        getattr(lib, "sflow_oracle_" + f).argtypes = [vp, dp]
    lib.sflow_oracle_get_maps.argtypes = [vp, dp, dp, dp]
    lib.sflow_oracle_get_mask.argtypes = [vp, C.POINTER(C.c_uint8)]
    lib.sflow_oracle_get_deposit.argtypes = [vp, dp]
    lib.sflow_oracle_get_geometry.argtypes = [vp, ip, dp]
    lib.sflow_oracle_stats.argtypes = [vp, vp]
    lib.sflow_oracle_time.restype = C.c_double
    lib.sflow_oracle_time.argtypes = [vp]
    lib.sflow_oracle_h_source.restype = C.c_double
    lib.sflow_oracle_h_source.argtypes = [vp]
    lib.sflow_oracle_max_newton.argtypes = [vp]
    lib.sflow_oracle_newton_total.restype = C.c_int64
    lib.sflow_oracle_newton_total.argtypes = [vp]
    lib.sflow_oracle_threads.restype = ip
    lib.sflow_oracle_set_threads.argtypes = [ip]
    lib.sflow_oracle_qc_to_qp.argtypes = [vp, dp, dp, dp]
    lib.sflow_oracle_qp_to_qc.argtypes = [vp, dp, dp]
    lib.sflow_oracle_mixt_var.argtypes = [vp, dp, dp]
    lib.sflow_oracle_fluxes.argtypes = [vp, dp, dp, C.c_double, ip, dp]
    lib.sflow_oracle_settling_velocity.restype = C.c_double
    lib.sflow_oracle_settling_velocity.argtypes = [vp] + [C.c_double] * 4
    lib.sflow_oracle_implicit_terms.argtypes = [vp, C.c_double, C.c_double, dp, dp]
    lib.sflow_oracle_newton.restype = ip
    lib.sflow_oracle_newton.argtypes = [vp, C.c_double, C.c_double, C.c_double, C.c_double,
                                        dp, dp, dp]
    lib.oracle_minmod.restype = C.c_double
    lib.oracle_minmod.argtypes = [C.c_double, C.c_double]
    lib.oracle_limit.restype = C.c_double
    lib.oracle_limit.argtypes = [dp, dp, ip, C.c_double]
    lib.sflow_oracle_eval_math.argtypes = [ip, C.c_int64, dp, dp, dp]
    u8p = C.POINTER(C.c_uint8)
    lib.sflow_oracle_get_erosion.argtypes = [vp, ip, dp]
    lib.sflow_oracle_get_topography.argtypes = [vp, dp]
    lib.sflow_oracle_get_cell_fract.argtypes = [vp, dp]
    lib.sflow_oracle_set_erodible.argtypes = [vp, dp]
    lib.sflow_oracle_set_nodata.argtypes = [vp, u8p]
    lib.sflow_oracle_vuln_size.argtypes = [vp, C.POINTER(ip), C.POINTER(ip)]
    lib.sflow_oracle_get_vuln.argtypes = [vp, u8p]
    if timing:
        _lib_fast = lib
    else:
        _lib = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def minmod(a, b):
    return _load().oracle_minmod(a, b)


def limit(v, z, limiter, theta=1.0):
    v = np.ascontiguousarray(v, dtype=np.float64)
    z = np.ascontiguousarray(z, dtype=np.float64)
    return _load().oracle_limit(_dp(v), _dp(z), limiter, theta)


def eval_math(name, x, y=None):
    """The shared FP64 pow / log / cos (sflow_math.h) as the host computes
    them, over the arrays x (and y for pow)."""
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
    out = np.empty_like(x)
    yy = np.ascontiguousarray(np.broadcast_to(np.asarray(0.0 if y is None else y, dtype=np.float64), x.shape))
    _load().sflow_oracle_eval_math({"pow": 0, "log": 1, "cos": 2}[name], x.size, _dp(x), _dp(yy), _dp(out))
    return out


def set_threads(n, timing=False):
    _load(timing).sflow_oracle_set_threads(int(n))


def threads(timing=False):
    return _load(timing).sflow_oracle_threads()


class Oracle:
    """One oracle solver over (params, B_cent)."""

    def __init__(self, params, B, timing=False):
        self.lib = _load(timing)
        self.p = params.copy()
        self.nx, self.ny = params.comp_cells_x, params.comp_cells_y
        self.nv = params.n_vars
        self._B = np.ascontiguousarray(B, dtype=np.float64).reshape(-1)
        assert self._B.size == self.nx * self.ny
        self.h = self.lib.sflow_oracle_create(C.byref(self.p), _dp(self._B))
        if not self.h:
            raise ValueError("oracle rejected the parameter set")

    def close(self):
        if self.h:
            self.lib.sflow_oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_q(self, q_aos):
        q = np.ascontiguousarray(q_aos, dtype=np.float64).reshape(-1)
        assert q.size == self.nx * self.ny * self.nv
        self.lib.sflow_oracle_set_q(self.h, _dp(q))

    def replace_q(self, q_aos):
        """Replace q in place, keeping the time, dt history and maps."""
        q = np.ascontiguousarray(q_aos, dtype=np.float64).reshape(-1)
        assert q.size == self.nx * self.ny * self.nv
        self.lib.sflow_oracle_replace_q(self.h, _dp(q))

    def step(self):
        return self.lib.sflow_oracle_step(self.h)

    def run(self, t_stop=1e300, max_steps=1 << 62):
        cells = C.c_int64(0)
        n = self.lib.sflow_oracle_run(self.h, t_stop, max_steps, C.byref(cells))
        return n, cells.value

    def q(self):
        out = np.empty(self.nx * self.ny * self.nv)
        self.lib.sflow_oracle_get_q(self.h, _dp(out))
        return out

    def qp(self):
        out = np.empty(self.nx * self.ny * (self.nv + 2))
        self.lib.sflow_oracle_get_qp(self.h, _dp(out))
        return out

    def maps(self):
        a = [np.empty(self.nx * self.ny) for _ in range(3)]
        self.lib.sflow_oracle_get_maps(self.h, *[_dp(x) for x in a])
        return a

    def deposit(self):
        """deposit(1:nx,1:ny,1:n_solid), column-major (class slowest)."""
        out = np.empty(self.nx * self.ny * (self.nv - 4))
        self.lib.sflow_oracle_get_deposit(self.h, _dp(out))
        return out

    def erosion(self):
        """Accumulated erosion per class (class slowest)."""
        out = np.empty(self.nx * self.ny * (self.nv - 4))
        self.lib.sflow_oracle_get_erosion(self.h, 0, _dp(out))
        return out

    def erodible(self):
        out = np.empty(self.nx * self.ny * (self.nv - 4))
        self.lib.sflow_oracle_get_erosion(self.h, 1, _dp(out))
        return out

    def topography(self):
        out = np.empty(self.nx * self.ny)
        self.lib.sflow_oracle_get_topography(self.h, _dp(out))
        return out

    def cell_fract(self):
        out = np.empty(self.nx * self.ny)
        self.lib.sflow_oracle_get_cell_fract(self.h, _dp(out))
        return out

    def set_erodible(self, thickness):
        t = np.ascontiguousarray(thickness, dtype=np.float64).reshape(-1)
        self.lib.sflow_oracle_set_erodible(self.h, _dp(t))

    def set_nodata(self, nodata):
        if nodata is None:
            self.lib.sflow_oracle_set_nodata(self.h, None)
            return
        m = np.ascontiguousarray(nodata, dtype=np.uint8).reshape(-1)
        self.lib.sflow_oracle_set_nodata(self.h, m.ctypes.data_as(C.POINTER(C.c_uint8)))

    def vuln_table(self):
        a, b = C.c_int(0), C.c_int(0)
        self.lib.sflow_oracle_vuln_size(self.h, C.byref(a), C.byref(b))
        n = a.value * b.value
        if n == 0:
            return None
        out = np.empty(n * self.nx * self.ny, dtype=np.uint8)
        self.lib.sflow_oracle_get_vuln(self.h, out.ctypes.data_as(C.POINTER(C.c_uint8)))
        return a.value, b.value, out.reshape(n, self.ny, self.nx)

    def mask(self):
        m = np.empty(self.nx * self.ny, dtype=np.uint8)
        self.lib.sflow_oracle_get_mask(self.h, m.ctypes.data_as(C.POINTER(C.c_uint8)))
        return m

    def geometry(self, which):
        out = np.empty(self.nx * self.ny)
        self.lib.sflow_oracle_get_geometry(self.h, which, _dp(out))
        return out

    def stats(self):
        from imex_sflow2d_dev_gb300.params import SflowStepStats
        s = SflowStepStats()
        self.lib.sflow_oracle_stats(self.h, C.byref(s))
        return s

    @property
    def t(self):
        return self.lib.sflow_oracle_time(self.h)

    @property
    def h_source(self):
        return self.lib.sflow_oracle_h_source(self.h)

    def max_newton(self):
        return self.lib.sflow_oracle_max_newton(self.h)

    def newton_total(self):
        return self.lib.sflow_oracle_newton_total(self.h)

    # unit-level helpers -------------------------------------------------
    def qc_to_qp(self, qc):
        qc = np.ascontiguousarray(qc, dtype=np.float64)
        qp = np.empty(self.nv + 2)
        pd = C.c_double(0.0)
        self.lib.sflow_oracle_qc_to_qp(self.h, _dp(qc), _dp(qp), C.byref(pd))
        return qp, pd.value

    def qp_to_qc(self, qp):
        qp = np.ascontiguousarray(qp, dtype=np.float64)
        qc = np.empty(self.nv)
        self.lib.sflow_oracle_qp_to_qc(self.h, _dp(qp), _dp(qc))
        return qc

    def mixt_var(self, qp):
        qp = np.ascontiguousarray(qp, dtype=np.float64)
        out = np.empty(6)
        self.lib.sflow_oracle_mixt_var(self.h, _dp(qp), _dp(out))
        return dict(zip(("Ri", "rho_m", "rho_c", "red_grav", "cp_c", "cp_mix"), out))

    def fluxes(self, qc, qp, gc, direction):
        qc = np.ascontiguousarray(qc, dtype=np.float64)
        qp = np.ascontiguousarray(qp, dtype=np.float64)
        f = np.empty(self.nv)
        self.lib.sflow_oracle_fluxes(self.h, _dp(qc), _dp(qp), gc, direction, _dp(f))
        return f

    def settling_velocity(self, diam, rhos, rhoc, inv_kin_visc):
        return self.lib.sflow_oracle_settling_velocity(self.h, diam, rhos, rhoc, inv_kin_visc)

    def implicit_terms(self, Bx, By, q):
        q = np.ascontiguousarray(q, dtype=np.float64)
        nh = np.empty(self.nv)
        self.lib.sflow_oracle_implicit_terms(self.h, Bx, By, _dp(q), _dp(nh))
        return nh

    def newton(self, dt, a_diag, Bx, By, q_old, Rj, q_guess):
        q_old = np.ascontiguousarray(q_old, dtype=np.float64)
        Rj = np.ascontiguousarray(Rj, dtype=np.float64)
        q = np.ascontiguousarray(q_guess, dtype=np.float64).copy()
        it = self.lib.sflow_oracle_newton(self.h, dt, a_diag, Bx, By, _dp(q_old), _dp(Rj), _dp(q))
        return q, it

"""ctypes binding of libsflow_gb300.so (the C ABI of include/sflow.h).

The library is built in-tree by imex_sflow2d_dev_gb300.build; there is no
CPU fallback: if the library is missing or cannot be loaded, every entry
point raises.
"""
import ctypes as C
import os

import numpy as np

from .params import SflowParams, SflowRunInfo, SflowStepStats

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsflow_gb300.so")

_lib = None


class SflowError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"sflow error {code}: {msg}")
        self.code = code


def load(build_if_missing=True):
    """Load libsflow_gb300.so (building it in-tree first if needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        from .build import build
        build()
    if not os.path.exists(LIB_PATH):
        raise SflowError(-3, f"{LIB_PATH} is missing; run imex_sflow2d_dev_gb300.build.build()")
    lib = C.CDLL(LIB_PATH)
    vp, dp, i32, i64 = C.c_void_p, C.POINTER(C.c_double), C.c_int32, C.c_int64
    P = C.POINTER(SflowParams)
    S = C.POINTER(SflowStepStats)
    sigs = {
        "sflow_last_error": (C.c_char_p, []),
        "sflow_build_info": (C.c_char_p, []),
        "sflow_default_params": (None, [P]),
        "sflow_create": (C.c_int, [P, dp, C.POINTER(vp)]),
        "sflow_destroy": (None, [vp]),
        "sflow_upload_q": (C.c_int, [vp, dp]),
        "sflow_download_q": (C.c_int, [vp, dp]),
        "sflow_download_qp": (C.c_int, [vp, dp]),
        "sflow_download_maps": (C.c_int, [vp, dp, dp, dp]),
        "sflow_check_solve": (C.c_int, [vp, i32]),
        "sflow_timestep": (C.c_int, [vp, dp]),
        "sflow_imex_rk": (C.c_int, [vp, C.c_double, C.c_double]),
        "sflow_erosion_deposition": (C.c_int, [vp, C.c_double]),
        "sflow_post_step": (C.c_int, [vp, S]),
        "sflow_step": (C.c_int, [vp]),
        "sflow_advance": (C.c_int, [vp, C.c_double, i64, S]),
        "sflow_get_stats": (C.c_int, [vp, S]),
        "sflow_status": (C.c_int, [vp, C.POINTER(C.c_uint32)]),
        "sflow_clear_status": (C.c_int, [vp]),
        "sflow_launch_count": (i64, [vp]),
        "sflow_device_bytes": (i64, [vp]),
        "sflow_counters": (C.c_int, [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64),
                                     C.POINTER(i32)]),
        "sflow_put_q": (C.c_int, [vp, dp]),
        "sflow_set_clock": (C.c_int, [vp, C.c_double, C.c_double, C.c_double]),
        "sflow_advance_timed": (C.c_int, [vp, i64, i32, dp]),
        "sflow_profile_kernels": (C.c_int, [vp, i64, i32, dp]),
        "sflow_log_sums_noalloc": (C.c_int, [P, vp, vp, vp]),
        "sflow_log_sums_noalloc_error": (C.c_char_p, []),
        "sflow_host_geometry": (C.c_int, [P, dp, i32, dp]),
        "sflow_host_scalars": (C.c_int, [P, dp, dp]),
        "sflow_io_error": (C.c_char_p, []),
        "sflow_read_input": (C.c_int, [C.c_char_p, P, C.POINTER(SflowRunInfo)]),
        "sflow_read_dem": (C.c_int, [C.c_char_p, P, dp, C.POINTER(C.c_uint8)]),
        "sflow_read_q2d": (C.c_int, [C.c_char_p, P, dp, C.POINTER(i32)]),
        "sflow_write_q2d": (C.c_int, [C.c_char_p, P, dp]),
        "sflow_write_p2d": (C.c_int, [C.c_char_p, P, dp, dp, dp, dp, dp, dp]),
        "sflow_write_restart": (C.c_int, [C.c_char_p, P, C.c_double, C.c_double, dp, dp, dp, dp, dp, dp]),
        "sflow_read_restart": (C.c_int, [C.c_char_p, P, dp, dp, dp, dp, dp, dp, dp, dp]),
        "sflow_output_name": (C.c_int, [C.c_char_p, i32, C.c_char_p, C.c_char_p, i32]),
        "sflow_download_phys": (C.c_int, [vp, dp]),
        "sflow_download_deposit": (C.c_int, [vp, dp]),
        "sflow_upload_deposit": (C.c_int, [vp, dp]),
        "sflow_upload_maps": (C.c_int, [vp, dp, dp, dp]),
        "sflow_set_output_time": (C.c_int, [vp, C.c_double]),
        "sflow_create_rows": (C.c_int, [P, dp, i32, i32, i32, i32, C.POINTER(vp)]),
        "sflow_get_rows": (C.c_int, [vp, i32, i32, dp]),
        "sflow_put_rows": (C.c_int, [vp, i32, i32, dp]),
        "sflow_download_erosion": (C.c_int, [vp, dp]),
        "sflow_download_erodible": (C.c_int, [vp, dp]),
        "sflow_set_erodible": (C.c_int, [vp, dp]),
        "sflow_download_topography": (C.c_int, [vp, dp]),
        "sflow_set_nodata": (C.c_int, [vp, C.POINTER(C.c_uint8)]),
        "sflow_vuln_table_size": (C.c_int, [vp, C.POINTER(i32), C.POINTER(i32)]),
        "sflow_download_vuln_table": (C.c_int, [vp, C.POINTER(C.c_uint8)]),
        "sflow_batch_create": (C.c_int, [i32, i32, i64, C.POINTER(vp)]),
        "sflow_batch_destroy": (None, [vp]),
        "sflow_batch_submit": (C.c_int, [vp, P, dp, dp, i64, C.POINTER(i32)]),
        "sflow_batch_advance": (C.c_int, [vp, i64, C.POINTER(i32)]),
        "sflow_batch_advance_timed": (C.c_int, [vp, i64, C.POINTER(i32), dp]),
        "sflow_batch_profile_kernels": (C.c_int, [vp, i64, C.POINTER(i32), dp]),
        "sflow_setup_create": (C.c_int, [P, dp, C.POINTER(vp)]),
        "sflow_setup_destroy": (None, [vp]),
        "sflow_batch_submit_setup": (C.c_int, [vp, vp, dp, i64, C.POINTER(i32)]),
        "sflow_batch_submit_setup_take": (C.c_int, [vp, vp, dp, i64, C.POINTER(i32)]),
        "sflow_batch_collect_many": (C.c_int, [vp, i32, C.POINTER(i32), C.POINTER(dp), i32, C.POINTER(i32)]),
        "sflow_batch_submit_many": (C.c_int, [vp, i32, P, C.POINTER(dp), C.POINTER(dp), C.POINTER(i64),
                                               C.POINTER(i32), i32]),
        "sflow_batch_launch": (C.c_int, [vp, i64]),
        "sflow_batch_wait": (C.c_int, [vp, C.POINTER(i32)]),
        "sflow_batch_dry_border_updates": (C.c_int, [vp, i32, C.POINTER(i64)]),
        "sflow_dry_border_updates": (C.c_int, [vp, C.POINTER(i64)]),
        "sflow_batch_poll": (C.c_int, [vp, i32, S, C.POINTER(i32)]),
        "sflow_batch_counters": (C.c_int, [vp, i32, C.POINTER(i64), C.POINTER(i64)]),
        "sflow_batch_download": (C.c_int, [vp, i32, dp]),
        "sflow_batch_collect": (C.c_int, [vp, i32, dp]),
        "sflow_batch_live": (i32, [vp]),
        "sflow_batch_launch_count": (i64, [vp]),
        "sflow_tile_shapes": (C.c_int, [i32, C.POINTER(i32), i32, C.POINTER(i32)]),
        "sflow_check_conversions": (C.c_int, [i64, C.c_uint64, C.POINTER(i64)]),
        "sflow_eval_math": (C.c_int, [i32, i64, dp, dp, dp]),
        "sflow_set_tile_shape": (C.c_int, [vp, i32]),
        "sflow_get_tile_shape": (C.c_int, [vp, C.POINTER(i32)]),
        "sflow_autotune": (C.c_int, [vp, i64, C.POINTER(i32), dp, i32]),
        "sflow_batch_set_tile_shape": (C.c_int, [vp, i32]),
        "sflow_batch_set_memory_limit": (C.c_int, [vp, i64]),
        "sflow_batch_get_tile_shape": (C.c_int, [vp, C.POINTER(i32)]),
    }
    for name, (res, args) in sigs.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return ["sflow_last_error", "sflow_build_info", "sflow_default_params", "sflow_create",
            "sflow_destroy", "sflow_upload_q", "sflow_download_q", "sflow_download_qp",
            "sflow_download_maps", "sflow_check_solve", "sflow_timestep", "sflow_imex_rk",
            "sflow_erosion_deposition", "sflow_post_step", "sflow_step", "sflow_advance",
            "sflow_get_stats", "sflow_status", "sflow_clear_status", "sflow_launch_count",
            "sflow_device_bytes", "sflow_counters", "sflow_host_geometry", "sflow_host_scalars",
            "sflow_put_q", "sflow_set_clock", "sflow_advance_timed", "sflow_profile_kernels",
            "sflow_log_sums_noalloc", "sflow_log_sums_noalloc_error", "sflow_batch_create",
            "sflow_batch_destroy", "sflow_batch_submit", "sflow_batch_advance", "sflow_batch_poll",
            "sflow_batch_counters", "sflow_batch_download", "sflow_batch_collect",
            "sflow_batch_live", "sflow_batch_launch_count", "sflow_io_error", "sflow_read_input",
            "sflow_read_dem", "sflow_read_q2d", "sflow_write_q2d", "sflow_write_p2d",
            "sflow_write_restart", "sflow_read_restart", "sflow_output_name",
            "sflow_download_phys", "sflow_download_deposit", "sflow_upload_deposit",
            "sflow_upload_maps", "sflow_set_output_time", "sflow_tile_shapes",
            "sflow_set_tile_shape", "sflow_get_tile_shape", "sflow_autotune",
            "sflow_batch_set_tile_shape", "sflow_batch_get_tile_shape", "sflow_check_conversions",
            "sflow_eval_math", "sflow_batch_advance_timed", "sflow_batch_profile_kernels",
            "sflow_setup_create", "sflow_setup_destroy", "sflow_batch_submit_setup", "sflow_batch_submit_many", "sflow_batch_submit_setup_take",
            "sflow_batch_collect_many",
            "sflow_batch_launch", "sflow_batch_wait", "sflow_batch_dry_border_updates",
            "sflow_dry_border_updates", "sflow_download_erosion", "sflow_download_erodible",
            "sflow_set_erodible", "sflow_download_topography", "sflow_set_nodata",
            "sflow_vuln_table_size", "sflow_download_vuln_table", "sflow_batch_set_memory_limit",
            "sflow_create_rows", "sflow_get_rows", "sflow_put_rows"]


TILE_CANDIDATES = (8, 16, 4)   # the candidate order of sflow_autotune


def check_conversions(n=1 << 22, seed=12345):
    """Mismatches of the integer-pipe float <-> double conversions against
    the hardware conversions on n seeded bit patterns (0 expected)."""
    lib = load()
    m = C.c_int64(-1)
    _check(lib.sflow_check_conversions(int(n), int(seed), C.byref(m)))
    return m.value


MATH_FUNCS = {"pow": 0, "log": 1, "cos": 2, "cuda_pow": 3, "cuda_log": 4, "cuda_cos": 5}


def eval_math(name, x, y=None):
    """The library's FP64 pow / log / cos (or CUDA's, 'cuda_*') evaluated on
    the device over the arrays x (and y for pow)."""
    lib = load()
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
    out = np.empty_like(x)
    yp = None
    if y is not None:
        y = np.ascontiguousarray(np.broadcast_to(np.asarray(y, dtype=np.float64), x.shape))
        yp = _dp(y)
    _check(lib.sflow_eval_math(MATH_FUNCS[name], x.size, _dp(x), yp, _dp(out)))
    return out


def tile_shapes(precision):
    """Tile heights (cells per tile column) with compiled kernels."""
    lib = load()
    h = (C.c_int32 * 8)()
    n = C.c_int32(0)
    _check(lib.sflow_tile_shapes(precision, h, 8, C.byref(n)))
    return [h[i] for i in range(n.value)]


def log_sums_noalloc(params, q_dev_ptr, sums_dev_ptr, stream_ptr=0):
    """Mass, volume, wet area and solid mass of a device-resident state
    (reference layout) into 4 device doubles, without any device allocation
    (see include/sflow.h).  Pointers are integers (device addresses)."""
    lib = load()
    p = params.copy()
    rc = lib.sflow_log_sums_noalloc(C.byref(p), C.c_void_p(q_dev_ptr), C.c_void_p(sums_dev_ptr),
                                    C.c_void_p(stream_ptr))
    if rc < 0:
        raise SflowError(rc, lib.sflow_log_sums_noalloc_error().decode())
    return rc


def host_geometry(params, B_cent, which):
    """Derived per-cell field of the host set-up (no GPU needed)."""
    lib = load()
    p = params.copy()
    B = np.ascontiguousarray(B_cent, dtype=np.float64).reshape(-1)
    out = np.empty(params.comp_cells_x * params.comp_cells_y)
    _check(lib.sflow_host_geometry(C.byref(p), _dp(B), which, _dp(out)))
    return out


def host_scalars(params, B_cent):
    lib = load()
    p = params.copy()
    B = np.ascontiguousarray(B_cent, dtype=np.float64).reshape(-1)
    out = np.empty(4)
    _check(lib.sflow_host_scalars(C.byref(p), _dp(B), _dp(out)))
    return {"h_source": out[0], "src_rho_m": out[1], "src_cp_mix": out[2], "eps_sing": out[3]}


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _io_check(rc):
    if rc < 0:
        raise SflowError(rc, _lib.sflow_io_error().decode())
    return rc


def _path(p):
    return os.fsencode(p)


# --- host I/O of the reference's files (no GPU needed) ----------------------
def read_input(path):
    """IMEX_SfloW2D.inp -> (SflowParams, run info dict)."""
    lib = load()
    p = SflowParams()
    r = SflowRunInfo()
    _io_check(lib.sflow_read_input(_path(path), C.byref(p), C.byref(r)))
    run = {f: getattr(r, f) for f, _ in SflowRunInfo._fields_ if f != "pad"}
    for k in ("run_name", "restart_file", "topography_file"):
        run[k] = run[k].decode()
    return p, run


def read_dem(path, params):
    """ESRI ASCII DEM -> (B_cent (ny, nx), nodata mask (ny, nx) bool)."""
    lib = load()
    nx, ny = params.comp_cells_x, params.comp_cells_y
    B = np.empty(nx * ny)
    nd = np.zeros(nx * ny, dtype=np.uint8)
    _io_check(lib.sflow_read_dem(_path(path), C.byref(params), _dp(B),
                                 nd.ctypes.data_as(C.POINTER(C.c_uint8))))
    return B.reshape(ny, nx), nd.reshape(ny, nx).astype(bool)


def read_q2d(path, params):
    """.q_2d restart -> (q in reference layout (flat), output index)."""
    lib = load()
    q = np.empty(params.n_vars * params.comp_cells_x * params.comp_cells_y)
    idx = C.c_int32(0)
    _io_check(lib.sflow_read_q2d(_path(path), C.byref(params), _dp(q), C.byref(idx)))
    return q, idx.value


def write_q2d(path, params, q_aos):
    """Writes .q_2d; like the reference, zeroes |q| < 1e-20 in q_aos itself."""
    lib = load()
    if q_aos.dtype != np.float64 or not q_aos.flags.c_contiguous:
        raise ValueError("q_aos must be a contiguous float64 array")
    _io_check(lib.sflow_write_q2d(_path(path), C.byref(params), _dp(q_aos)))


def write_p2d(path, params, phys, B_cent, deposit, hmax, pdynmax, mod_vel_max):
    lib = load()
    arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) if a is not None else None
            for a in (phys, B_cent, deposit, hmax, pdynmax, mod_vel_max)]
    _io_check(lib.sflow_write_p2d(_path(path), C.byref(params), *[_dp(a) for a in arrs]))


def write_restart(path, params, t, dt, q_aos, B_cent, deposit, hmax, pdynmax, mod_vel_max):
    lib = load()
    arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) if a is not None else None
            for a in (q_aos, B_cent, deposit, hmax, pdynmax, mod_vel_max)]
    _io_check(lib.sflow_write_restart(_path(path), C.byref(params), float(t), float(dt),
                                      *[_dp(a) for a in arrs]))


def read_restart(path, params):
    lib = load()
    nx, ny, nv, ns = params.comp_cells_x, params.comp_cells_y, params.n_vars, params.n_solid
    N = nx * ny
    t, dt = C.c_double(), C.c_double()
    q, B, dep = np.empty(N * nv), np.empty(N), np.empty(N * ns)
    h, pd, v = np.empty(N), np.empty(N), np.empty(N)
    _io_check(lib.sflow_read_restart(_path(path), C.byref(params), C.byref(t), C.byref(dt), _dp(q),
                                     _dp(B), _dp(dep), _dp(h), _dp(pd), _dp(v)))
    return {"t": t.value, "dt": dt.value, "q": q, "B_cent": B.reshape(ny, nx), "deposit": dep,
            "hmax": h, "pdynmax": pd, "mod_vel_max": v}


def output_name(run_name, index, ext):
    lib = load()
    buf = C.create_string_buffer(512)
    _io_check(lib.sflow_output_name(run_name.encode(), index, ext.encode(), buf, 512))
    return buf.value.decode()


def _check(rc):
    if rc < 0:
        raise SflowError(rc, _lib.sflow_last_error().decode())
    return rc


class Solver:
    """One domain on the GPU.  Method names follow the reference driver's
    call sites (src/IMEX_SfloW2D.f90:395-505)."""

    def __init__(self, params, B_cent, rows=None):
        """rows = (k0, n, own_lo, own_hi): a row slab of the domain (rows
        k0 .. k0+n-1, own rows own_lo .. own_hi-1 local), see
        sflow_create_rows; B_cent is then the whole domain's."""
        self.lib = load()
        self.p = params.copy()
        self.nx, self.ny = params.comp_cells_x, params.comp_cells_y
        self.nv = params.n_vars
        B = np.ascontiguousarray(B_cent, dtype=np.float64).reshape(-1)
        if B.size != self.nx * self.ny:
            raise ValueError("B_cent must have nx*ny values")
        h = C.c_void_p()
        if rows is None:
            _check(self.lib.sflow_create(C.byref(self.p), _dp(B), C.byref(h)))
        else:
            k0, n, lo, hi = (int(x) for x in rows)
            _check(self.lib.sflow_create_rows(C.byref(self.p), _dp(B), k0, n, lo, hi, C.byref(h)))
            self.ny = n
            self.p.comp_cells_y = n
        self.h = h

    def get_rows(self, k_lo, n):
        """Rows k_lo .. k_lo+n-1 of q (local rows), reference layout."""
        out = np.empty(n * self.nx * self.nv)
        _check(self.lib.sflow_get_rows(self.h, int(k_lo), int(n), _dp(out)))
        return out

    def put_rows(self, k_lo, n, q_rows):
        q = np.ascontiguousarray(q_rows, dtype=np.float64).reshape(-1)
        if q.size != n * self.nx * self.nv:
            raise ValueError("q_rows must have n*nx*n_vars values")
        _check(self.lib.sflow_put_rows(self.h, int(k_lo), int(n), _dp(q)))

    def close(self):
        if getattr(self, "h", None):
            self.lib.sflow_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # state -------------------------------------------------------------
    def upload_q(self, q_aos):
        q = np.ascontiguousarray(q_aos, dtype=np.float64).reshape(-1)
        if q.size != self.nx * self.ny * self.nv:
            raise ValueError("q must have n_vars*nx*ny values")
        _check(self.lib.sflow_upload_q(self.h, _dp(q)))

    def put_q(self, q_aos):
        """Replace the state, keeping time, dt history, maxima and counters."""
        q = np.ascontiguousarray(q_aos, dtype=np.float64).reshape(-1)
        if q.size != self.nx * self.ny * self.nv:
            raise ValueError("q must have n_vars*nx*ny values")
        _check(self.lib.sflow_put_q(self.h, _dp(q)))

    def put_q_ptr(self, addr):
        """put_q from a raw host address (e.g. pinned memory)."""
        _check(self.lib.sflow_put_q(self.h, C.cast(addr, C.POINTER(C.c_double))))

    def download_q_ptr(self, addr):
        _check(self.lib.sflow_download_q(self.h, C.cast(addr, C.POINTER(C.c_double))))

    def set_clock(self, t, dt_old, dt_old_old):
        _check(self.lib.sflow_set_clock(self.h, t, dt_old, dt_old_old))

    def advance_timed(self, steps, flush_l2=True):
        ms = C.c_double(0.0)
        _check(self.lib.sflow_advance_timed(self.h, steps, 1 if flush_l2 else 0, C.byref(ms)))
        return ms.value

    def profile_kernels(self, steps, flush_l2=True):
        out = np.zeros(4)
        _check(self.lib.sflow_profile_kernels(self.h, steps, 1 if flush_l2 else 0, _dp(out)))
        return dict(zip(("mask", "flux", "dt", "stage"), out.tolist()))

    def download_q(self, out=None):
        if out is None:
            out = np.empty(self.nx * self.ny * self.nv)
        _check(self.lib.sflow_download_q(self.h, _dp(out)))
        return out

    def download_qp(self):
        out = np.empty(self.nx * self.ny * (self.nv + 2))
        _check(self.lib.sflow_download_qp(self.h, _dp(out)))
        return out

    def maps(self):
        a = [np.empty(self.nx * self.ny) for _ in range(3)]
        _check(self.lib.sflow_download_maps(self.h, *[_dp(x) for x in a]))
        return a

    # reference call sites ---------------------------------------------
    def check_solve(self, solve_all=False):
        return _check(self.lib.sflow_check_solve(self.h, 1 if solve_all else 0))

    def timestep(self):
        dt = C.c_double(0.0)
        _check(self.lib.sflow_timestep(self.h, C.byref(dt)))
        return dt.value

    def imex_rk_solver(self, t, dt):
        return _check(self.lib.sflow_imex_rk(self.h, t, dt))

    def update_erosion_deposition_cell(self, dt):
        return _check(self.lib.sflow_erosion_deposition(self.h, dt))

    def post_step(self):
        s = SflowStepStats()
        _check(self.lib.sflow_post_step(self.h, C.byref(s)))
        return s

    # fused driver --------------------------------------------------------
    def step(self):
        return _check(self.lib.sflow_step(self.h))

    def advance(self, t_stop=1e300, max_steps=1 << 62):
        s = SflowStepStats()
        _check(self.lib.sflow_advance(self.h, t_stop, max_steps, C.byref(s)))
        return s

    def stats(self):
        s = SflowStepStats()
        _check(self.lib.sflow_get_stats(self.h, C.byref(s)))
        return s

    def status(self):
        f = C.c_uint32(0)
        _check(self.lib.sflow_status(self.h, C.byref(f)))
        return f.value

    def clear_status(self):
        _check(self.lib.sflow_clear_status(self.h))

    def counters(self):
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        d = C.c_int32()
        _check(self.lib.sflow_counters(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        e = C.c_int64(0)
        _check(self.lib.sflow_dry_border_updates(self.h, C.byref(e)))
        return {"cell_updates": a.value, "steps": b.value, "newton_iters": c.value,
                "newton_max": d.value, "dry_border_updates": e.value}

    def launch_count(self):
        return self.lib.sflow_launch_count(self.h)

    def download_phys(self):
        """Per cell h, u, v, T, alphas, rho_m, red_grav, Ri (the .p_2d fields)."""
        nx, ny = self.p.comp_cells_x, self.p.comp_cells_y
        out = np.empty(nx * ny * (7 + self.p.n_solid))
        _check(self.lib.sflow_download_phys(self.h, _dp(out)))
        return out

    def download_deposit(self):
        out = np.empty(self.p.comp_cells_x * self.p.comp_cells_y * self.p.n_solid)
        _check(self.lib.sflow_download_deposit(self.h, _dp(out)))
        return out

    def upload_deposit(self, dep):
        d = np.ascontiguousarray(dep, dtype=np.float64).reshape(-1)
        _check(self.lib.sflow_upload_deposit(self.h, _dp(d)))

    def _cells(self):
        return self.p.comp_cells_x * self.p.comp_cells_y

    def download_erosion(self):
        """Accumulated erosion per class (class slowest, nx*ny each)."""
        out = np.empty(self._cells() * self.p.n_solid)
        _check(self.lib.sflow_download_erosion(self.h, _dp(out)))
        return out

    def download_erodible(self):
        """Erodible solid thickness left per class."""
        out = np.empty(self._cells() * self.p.n_solid)
        _check(self.lib.sflow_download_erodible(self.h, _dp(out)))
        return out

    def set_erodible(self, thickness):
        """Erodible layer thickness per cell (ERODIBLE_FILE's field)."""
        t = np.ascontiguousarray(thickness, dtype=np.float64).reshape(-1)
        _check(self.lib.sflow_set_erodible(self.h, _dp(t)))

    def download_topography(self):
        out = np.empty(self._cells())
        _check(self.lib.sflow_download_topography(self.h, _dp(out)))
        return out

    def set_nodata(self, nodata):
        """B_nodata per cell (None clears)."""
        if nodata is None:
            _check(self.lib.sflow_set_nodata(self.h, None))
            return
        m = np.ascontiguousarray(nodata, dtype=np.uint8).reshape(-1)
        _check(self.lib.sflow_set_nodata(self.h, m.ctypes.data_as(C.POINTER(C.c_uint8))))

    def vuln_table(self):
        """(n_thk, n_dyn, table as uint8 [n_thk*n_dyn, ny, nx]) or None."""
        a, b = C.c_int32(0), C.c_int32(0)
        _check(self.lib.sflow_vuln_table_size(self.h, C.byref(a), C.byref(b)))
        n = a.value * b.value
        if n == 0:
            return None
        out = np.empty(n * self._cells(), dtype=np.uint8)
        _check(self.lib.sflow_download_vuln_table(self.h, out.ctypes.data_as(C.POINTER(C.c_uint8))))
        return a.value, b.value, out.reshape(n, self.p.comp_cells_y, self.p.comp_cells_x)

    def upload_maps(self, hmax=None, pdynmax=None, mod_vel_max=None):
        arrs = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) if a is not None else None
                for a in (hmax, pdynmax, mod_vel_max)]
        _check(self.lib.sflow_upload_maps(self.h, *[_dp(a) for a in arrs]))

    def set_output_time(self, t_output):
        _check(self.lib.sflow_set_output_time(self.h, float(t_output)))

    def device_bytes(self):
        return self.lib.sflow_device_bytes(self.h)

    def tile_shape(self):
        v = C.c_int32(0)
        _check(self.lib.sflow_get_tile_shape(self.h, C.byref(v)))
        return v.value

    def set_tile_shape(self, tile_h):
        _check(self.lib.sflow_set_tile_shape(self.h, int(tile_h)))

    def autotune(self, steps_per_shape=64):
        """Time the compiled tile heights on this run (the steps advance
        the run) and keep the fastest; returns (best height, {height: ms
        per 10^6 cell updates})."""
        best = C.c_int32(0)
        v = (C.c_double * len(TILE_CANDIDATES))()
        _check(self.lib.sflow_autotune(self.h, int(steps_per_shape), C.byref(best), v, len(TILE_CANDIDATES)))
        return best.value, {th: v[i] for i, th in enumerate(TILE_CANDIDATES) if v[i] >= 0}


EBUSY = -6


class Setup:
    """The host part of a batch submission (validation, topography terms,
    ring-inlet geometry) of one run, made without touching the GPU
    (sflow_setup_create); safe to build on worker threads."""

    def __init__(self, params, B_cent, precision=None):
        self.lib = load()
        p = params.copy()
        if precision is not None:
            p.precision = precision
        self.p = p
        B = np.ascontiguousarray(B_cent, dtype=np.float64).reshape(-1)
        if B.size != p.comp_cells_x * p.comp_cells_y:
            raise ValueError("B_cent must have nx*ny values")
        self.h = C.c_void_p()
        _check(self.lib.sflow_setup_create(C.byref(p), _dp(B), C.byref(self.h)))

    def close(self):
        if self.h:
            self.lib.sflow_setup_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent runs resident on the GPU and advanced together
    (sflow_batch_* of include/sflow.h).  submit() returns a run id, or None
    when the batch has no slot, list capacity or device memory for the run
    now (SFLOW_EBUSY); collect() returns the run's q and frees its slot."""

    def __init__(self, precision, max_runs=256, max_cells=1 << 28):
        self.lib = load()
        self.h = C.c_void_p()
        self.precision = precision
        _check(self.lib.sflow_batch_create(precision, max_runs, max_cells, C.byref(self.h)))
        self._shape = {}

    def close(self):
        if self.h:
            self.lib.sflow_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, params, B_cent, q_aos, max_steps=0):
        p = params.copy()
        p.precision = self.precision
        B = np.ascontiguousarray(B_cent, dtype=np.float64).reshape(-1)
        q = np.ascontiguousarray(q_aos, dtype=np.float64).reshape(-1)
        if B.size != p.comp_cells_x * p.comp_cells_y:
            raise ValueError("B_cent must have nx*ny values")
        if q.size != p.n_vars * p.comp_cells_x * p.comp_cells_y:
            raise ValueError("q must have n_vars*nx*ny values")
        rid = C.c_int32(-1)
        rc = self.lib.sflow_batch_submit(self.h, C.byref(p), _dp(B), _dp(q), int(max_steps), C.byref(rid))
        if rc == EBUSY:
            return None
        _check(rc)
        self._shape[rid.value] = p.n_vars * p.comp_cells_x * p.comp_cells_y
        return rid.value

    def submit_setup(self, setup, q_aos, max_steps=0, take=False):
        """submit() of a run prepared as a Setup (the GPU part only).  With
        take=True the setup's host arrays move into the run (no copy) and an
        admitted setup is spent (sflow_batch_submit_setup_take); a setup
        that was not admitted (None) can be submitted again."""
        p = setup.p
        q = np.ascontiguousarray(q_aos, dtype=np.float64).reshape(-1)
        if q.size != p.n_vars * p.comp_cells_x * p.comp_cells_y:
            raise ValueError("q must have n_vars*nx*ny values")
        rid = C.c_int32(-1)
        fn = self.lib.sflow_batch_submit_setup_take if take else self.lib.sflow_batch_submit_setup
        rc = fn(self.h, setup.h, _dp(q), int(max_steps), C.byref(rid))
        if rc == EBUSY:
            return None
        _check(rc)
        self._shape[rid.value] = p.n_vars * p.comp_cells_x * p.comp_cells_y
        return rid.value

    def submit_many(self, runs, threads=0):
        """Submit [(params, B_cent, q_aos, max_steps)] at once, the host
        set-ups on `threads` host threads (0: every hardware thread) while
        the runs are uploaded in order (sflow_batch_submit_many).  Returns
        the run ids, None for a run not admitted for want of room (EBUSY);
        any other failure raises SflowError, whose run_ids attribute holds
        the ids of the runs that were admitted."""
        n = len(runs)
        m = max(n, 1)
        ps = (SflowParams * m)()
        Bs, qs, keep = (C.POINTER(C.c_double) * m)(), (C.POINTER(C.c_double) * m)(), []
        ms = (C.c_int64 * m)()
        for i, (params, B_cent, q_aos, max_steps) in enumerate(runs):
            p = params.copy()
            p.precision = self.precision
            B = np.ascontiguousarray(B_cent, dtype=np.float64).reshape(-1)
            q = np.ascontiguousarray(q_aos, dtype=np.float64).reshape(-1)
            if B.size != p.comp_cells_x * p.comp_cells_y:
                raise ValueError("B_cent must have nx*ny values")
            if q.size != p.n_vars * p.comp_cells_x * p.comp_cells_y:
                raise ValueError("q must have n_vars*nx*ny values")
            ps[i] = p
            Bs[i], qs[i], ms[i] = _dp(B), _dp(q), int(max_steps or 0)
            keep.append((B, q, p))
        ids = (C.c_int32 * m)()
        rc = self.lib.sflow_batch_submit_many(self.h, n, ps, Bs, qs, ms, ids, int(threads))
        out = []
        for i in range(n):
            rid = ids[i]
            if rid >= 0:
                p = keep[i][2]
                self._shape[rid] = p.n_vars * p.comp_cells_x * p.comp_cells_y
            out.append(rid if rid >= 0 else None)
        if rc < 0 and rc != EBUSY:
            err = SflowError(rc, self.lib.sflow_last_error().decode())
            err.run_ids = out
            raise err
        return out

    def advance(self, steps):
        f = C.c_int32(0)
        _check(self.lib.sflow_batch_advance(self.h, int(steps), C.byref(f)))
        return f.value

    def advance_timed(self, steps):
        """advance() with the device time of the steps: (finished, ms)."""
        f = C.c_int32(0)
        ms = C.c_double(0.0)
        _check(self.lib.sflow_batch_advance_timed(self.h, int(steps), C.byref(f), C.byref(ms)))
        return f.value, ms.value

    def profile_kernels(self, steps):
        """steps batch steps one at a time; summed device ms per kernel."""
        f = C.c_int32(0)
        out = np.zeros(5)
        _check(self.lib.sflow_batch_profile_kernels(self.h, int(steps), C.byref(f), _dp(out)))
        return dict(zip(("cand", "mask", "flux", "dt", "stage"), out.tolist()))

    def launch(self, steps):
        """Enqueue steps and return at once (wait() before any other call)."""
        _check(self.lib.sflow_batch_launch(self.h, int(steps)))

    def wait(self):
        f = C.c_int32(0)
        _check(self.lib.sflow_batch_wait(self.h, C.byref(f)))
        return f.value

    def dry_border_updates(self, rid):
        n = C.c_int64(0)
        _check(self.lib.sflow_batch_dry_border_updates(self.h, rid, C.byref(n)))
        return n.value

    def poll(self, rid):
        s = SflowStepStats()
        d = C.c_int32(0)
        _check(self.lib.sflow_batch_poll(self.h, rid, C.byref(s), C.byref(d)))
        return s, bool(d.value)

    def done(self, rid):
        d = C.c_int32(0)
        _check(self.lib.sflow_batch_poll(self.h, rid, None, C.byref(d)))
        return bool(d.value)

    def counters(self, rid):
        a, b = C.c_int64(), C.c_int64()
        _check(self.lib.sflow_batch_counters(self.h, rid, C.byref(a), C.byref(b)))
        return {"cell_updates": a.value, "steps": b.value}

    def download(self, rid, out=None):
        """The run's q (reference layout), into `out` when given (a float64
        array of the run's size, e.g. a view of pinned host memory)."""
        out = self._out(rid, out)
        _check(self.lib.sflow_batch_download(self.h, rid, _dp(out)))
        return out

    def collect(self, rid, want_q=True, out=None):
        out = self._out(rid, out) if want_q else None
        _check(self.lib.sflow_batch_collect(self.h, rid, _dp(out) if want_q else None))
        del self._shape[rid]
        return out

    def collect_many(self, rids, outs=None, want_q=True, threads=0):
        """collect() of several runs at once (sflow_batch_collect_many: the
        downloads on host threads).  outs: optional arrays (one per run) to
        receive q.  Returns the q arrays (None where want_q is False); a
        failure raises SflowError."""
        n = len(rids)
        m = max(n, 1)
        ids = (C.c_int32 * m)(*[int(r) for r in rids])
        ptrs = (C.POINTER(C.c_double) * m)()
        res = []
        for i, rid in enumerate(rids):
            if want_q and rid in self._shape:
                o = self._out(rid, outs[i] if outs is not None else None)
                ptrs[i] = _dp(o)
                res.append(o)
            else:
                res.append(None)   # no download (an unknown id is reported by the call)
        status = (C.c_int32 * m)()
        rc = self.lib.sflow_batch_collect_many(self.h, n, ids, ptrs if want_q else None, int(threads), status)
        for i, rid in enumerate(rids):
            if status[i] == 0:
                self._shape.pop(rid, None)
        _check(rc)
        return res

    def _out(self, rid, out):
        if out is None:
            return np.empty(self._shape[rid])
        if out.dtype != np.float64 or out.size != self._shape[rid] or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous float64 array of the run's size")
        return out

    def live(self):
        return self.lib.sflow_batch_live(self.h)

    def launch_count(self):
        return self.lib.sflow_batch_launch_count(self.h)

    def tile_shape(self):
        v = C.c_int32(0)
        _check(self.lib.sflow_batch_get_tile_shape(self.h, C.byref(v)))
        return v.value

    def set_tile_shape(self, tile_h):
        """Tile height of the runs admitted from now on (no run may be live)."""
        _check(self.lib.sflow_batch_set_tile_shape(self.h, int(tile_h)))

    def set_memory_limit(self, nbytes):
        """Cap on the device bytes of the resident runs (0: none); a submit
        past it returns None (SFLOW_EBUSY)."""
        _check(self.lib.sflow_batch_set_memory_limit(self.h, int(nbytes)))

"""ctypes mirror of the C-ABI structs in include/sflow.h.

The field names follow the IMEX_SfloW2D.inp namelist keys (reference
src/inpout_2d.f90:326-391 and 1017-1039) so that a parsed input file maps
onto SflowParams one to one.
"""
import ctypes as C

SFLOW_ABI_VERSION = 2
MAX_SOLID = 4
MAX_VARS = 4 + MAX_SOLID
MAX_LEVELS = 10
MAX_INTERVALS = 100

PREC_FP64 = 0
PREC_FP32 = 1
SCHEME_KT = 0
SCHEME_UP = 1
W, E, S, N = 0, 1, 2, 3

S_NAN = 0x1
S_NEG_H = 0x2
S_NEG_ALPHA = 0x4
S_LOW_T = 0x8
S_SOLID_GT_MASS = 0x10
S_NEWTON_MAXIT = 0x20
S_EROSION = 0x40
# a run stops at the end of the step that raised one of these
S_FATAL = S_NAN | S_NEG_H | S_NEG_ALPHA | S_EROSION

STATUS_NAMES = {
    S_NAN: "NaN", S_NEG_H: "negative thickness", S_NEG_ALPHA: "negative solid mass",
    S_LOW_T: "T < 273 K", S_SOLID_GT_MASS: "solid mass > total mass",
    S_NEWTON_MAXIT: "Newton max iterations", S_EROSION: "erosion check",
}


class SflowBC(C.Structure):
    _fields_ = [("flag", C.c_int32), ("pad", C.c_int32), ("value", C.c_double)]


class SflowParams(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("precision", C.c_int32),
        ("comp_cells_x", C.c_int32), ("comp_cells_y", C.c_int32),
        ("x0", C.c_double), ("y0", C.c_double), ("cell_size", C.c_double),
        ("n_solid", C.c_int32),
        ("gas_flag", C.c_int32), ("liquid_flag", C.c_int32), ("energy_flag", C.c_int32),
        ("alpha_flag", C.c_int32), ("rheology_flag", C.c_int32),
        ("slope_correction_flag", C.c_int32), ("curvature_term_flag", C.c_int32),
        ("radial_source_flag", C.c_int32),
        ("solver_scheme", C.c_int32), ("n_rk", C.c_int32),
        ("dt0", C.c_double), ("max_dt", C.c_double), ("cfl", C.c_double),
        ("theta", C.c_double), ("reconstr_coeff", C.c_double),
        ("limiter", C.c_int32 * MAX_VARS),
        ("bc", (SflowBC * MAX_VARS) * 4),
        ("grav", C.c_double),
        ("rheology_model", C.c_int32), ("pad0", C.c_int32),
        ("mu", C.c_double), ("xi", C.c_double), ("friction_factor", C.c_double),
        ("pres", C.c_double), ("sp_heat_a", C.c_double), ("sp_gas_const_a", C.c_double),
        ("kin_visc_a", C.c_double), ("T_ambient", C.c_double),
        ("entrainment_flag", C.c_int32), ("pad1", C.c_int32),
        ("rho_l", C.c_double), ("sp_heat_l", C.c_double), ("kin_visc_l", C.c_double),
        ("loss_rate", C.c_double),
        ("rho_s", C.c_double * MAX_SOLID), ("diam_s", C.c_double * MAX_SOLID),
        ("sp_heat_s", C.c_double * MAX_SOLID),
        ("settling_flag", C.c_int32), ("collective_settling_flag", C.c_int32),
        ("alphastot_min", C.c_double), ("maximum_solid_packing", C.c_double),
        ("A_drag", C.c_double), ("B_drag", C.c_double),
        ("erosion_coeff", C.c_double),
        ("x_source", C.c_double), ("y_source", C.c_double), ("r_source", C.c_double),
        ("r2_source", C.c_double),
        ("vel_source", C.c_double), ("T_source", C.c_double), ("h_source", C.c_double),
        ("mfr_source", C.c_double),
        ("alphas_source", C.c_double * MAX_SOLID),
        ("time_param", C.c_double * 4),
        ("azimuth_source", C.c_double), ("arc_width_source", C.c_double),
        ("t_start", C.c_double), ("t_end", C.c_double), ("dt_output", C.c_double),
        # ABI version 2
        ("thickness_levels", C.c_double * MAX_LEVELS), ("dyn_pres_levels", C.c_double * MAX_LEVELS),
        ("erodible_porosity", C.c_double), ("T_erodible", C.c_double),
        ("initial_erodible_thickness", C.c_double), ("erodible_fract", C.c_double * MAX_SOLID),
        ("erodible_deposit_flag", C.c_int32), ("topo_change_flag", C.c_int32),
        ("bottom_radial_source_flag", C.c_int32), ("n_intervals", C.c_int32),
        ("angle_source", C.c_double),
        ("t_intervals", C.c_double * MAX_INTERVALS), ("vel_intervals", C.c_double * MAX_INTERVALS),
        ("fp32_newton_fp64", C.c_int32), ("pad2", C.c_int32),
        ("mu_s", C.c_double), ("mu_2", C.c_double), ("I_0", C.c_double), ("muI_inf", C.c_double),
    ]

    @property
    def n_vars(self):
        return 4 + self.n_solid

    def copy(self):
        c = SflowParams()
        C.memmove(C.addressof(c), C.addressof(self), C.sizeof(SflowParams))
        return c

    def set_bc_all(self, flag, value=0.0):
        for s in range(4):
            for i in range(MAX_VARS):
                self.bc[s][i].flag = flag
                self.bc[s][i].value = value


def params_to_dict(p):
    """Plain-Python copy of SflowParams (arrays as lists, BCs as
    [side][var] = [flag, value])."""
    out = {}
    for name, _ in SflowParams._fields_:
        v = getattr(p, name)
        if name == "bc":
            out[name] = [[[v[s][i].flag, v[s][i].value] for i in range(MAX_VARS)] for s in range(4)]
        elif hasattr(v, "__len__"):
            out[name] = list(v)
        else:
            out[name] = v
    return out


def params_from_dict(d):
    """SflowParams from params_to_dict output; keys the dict does not hold
    (fields added after it was made) keep the defaults, and the ABI version
    is this library's."""
    p = default_params()
    for name, _ in SflowParams._fields_:
        if name not in d or name == "abi_version":
            continue
        v = d[name]
        if name == "bc":
            for s in range(4):
                for i in range(MAX_VARS):
                    p.bc[s][i].flag, p.bc[s][i].value = int(v[s][i][0]), float(v[s][i][1])
        elif isinstance(v, list):
            arr = getattr(p, name)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(p, name, v)
    return p


class SflowRunInfo(C.Structure):
    _fields_ = [
        ("run_name", C.c_char * 128), ("restart_file", C.c_char * 256),
        ("topography_file", C.c_char * 256), ("restart", C.c_int32),
        ("output_cons_flag", C.c_int32), ("output_phys_flag", C.c_int32),
        ("output_esri_flag", C.c_int32), ("output_netcdf_flag", C.c_int32),
        ("output_runout_flag", C.c_int32), ("verbose_level", C.c_int32), ("pad", C.c_int32),
    ]


class SflowStepStats(C.Structure):
    _fields_ = [
        ("t", C.c_double), ("dt", C.c_double), ("mass", C.c_double),
        ("volume", C.c_double), ("area", C.c_double), ("solid_mass", C.c_double),
        ("solve_cells", C.c_int64), ("steps", C.c_int64),
        ("status", C.c_uint32), ("pad", C.c_uint32),
    ]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "pad"}


def default_params():
    """Defaults of init_param (reference src/inpout_2d.f90:408-985)."""
    p = SflowParams()
    p.abi_version = SFLOW_ABI_VERSION
    p.precision = PREC_FP64
    p.comp_cells_x, p.comp_cells_y, p.cell_size = 1000, 1, 1.0e-3
    p.gas_flag = 1
    p.solver_scheme, p.n_rk = SCHEME_KT, 2
    p.dt0, p.max_dt, p.cfl, p.theta, p.reconstr_coeff = 1.0e-4, 1.0e-3, 0.24, 1.0, 1.0
    for i in range(MAX_VARS):
        p.limiter[i] = 1
    p.set_bc_all(1, 0.0)
    p.grav = 9.81
    p.maximum_solid_packing = 0.64
    p.A_drag = p.B_drag = -1.0
    p.r2_source, p.arc_width_source, p.h_source, p.mfr_source = -1.0, 360.0, -1.0, -1.0
    for i in range(4):
        p.time_param[i] = -1.0
    p.t_end, p.dt_output = 5.0e-2, 5.0e-3
    for i in range(MAX_LEVELS):
        p.thickness_levels[i] = p.dyn_pres_levels[i] = -1.0
    p.erodible_porosity = p.T_erodible = p.initial_erodible_thickness = -1.0
    for i in range(MAX_SOLID):
        p.erodible_fract[i] = -1.0
    for i in range(MAX_INTERVALS):
        p.t_intervals[i] = p.vel_intervals[i] = -1.0
    return p


def status_text(bits):
    return ", ".join(v for k, v in STATUS_NAMES.items() if bits & k) or "ok"

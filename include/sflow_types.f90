! sflow_types.f90 -- ISO_C_BINDING layouts of the C ABI's structs
! (include/sflow.h): SflowBC, SflowParams and SflowStepStats, member for
! member in the C order, for a Fortran host that fills the parameters from
! its namelist variables and passes C_LOC(params) to sflow_create.  C arrays
! [a][b] are Fortran arrays (b, a): bc(ivar, side) is bc[side][ivar].
! tests/test_fortran_layout.py checks the offsets this declaration implies
! against offsetof() of the C structs.
MODULE sflow_types
  USE, INTRINSIC :: ISO_C_BINDING
  IMPLICIT NONE

  INTEGER(C_INT32_T), PARAMETER :: SFLOW_ABI_VERSION = 2
  INTEGER, PARAMETER :: SFLOW_MAX_SOLID = 4
  INTEGER, PARAMETER :: SFLOW_MAX_VARS = 4 + SFLOW_MAX_SOLID
  INTEGER, PARAMETER :: SFLOW_MAX_LEVELS = 10
  INTEGER, PARAMETER :: SFLOW_MAX_INTERVALS = 100

  TYPE, BIND(C) :: sflow_bc
     INTEGER(C_INT32_T) :: flag
     INTEGER(C_INT32_T) :: pad
     REAL(C_DOUBLE) :: value
  END TYPE sflow_bc

  TYPE, BIND(C) :: sflow_params
     INTEGER(C_INT32_T) :: abi_version
     INTEGER(C_INT32_T) :: precision
     INTEGER(C_INT32_T) :: comp_cells_x
     INTEGER(C_INT32_T) :: comp_cells_y
     REAL(C_DOUBLE) :: x0
     REAL(C_DOUBLE) :: y0
     REAL(C_DOUBLE) :: cell_size
     INTEGER(C_INT32_T) :: n_solid
     INTEGER(C_INT32_T) :: gas_flag
     INTEGER(C_INT32_T) :: liquid_flag
     INTEGER(C_INT32_T) :: energy_flag
     INTEGER(C_INT32_T) :: alpha_flag
     INTEGER(C_INT32_T) :: rheology_flag
     INTEGER(C_INT32_T) :: slope_correction_flag
     INTEGER(C_INT32_T) :: curvature_term_flag
     INTEGER(C_INT32_T) :: radial_source_flag
     INTEGER(C_INT32_T) :: solver_scheme
     INTEGER(C_INT32_T) :: n_rk
     REAL(C_DOUBLE) :: dt0
     REAL(C_DOUBLE) :: max_dt
     REAL(C_DOUBLE) :: cfl
     REAL(C_DOUBLE) :: theta
     REAL(C_DOUBLE) :: reconstr_coeff
     INTEGER(C_INT32_T) :: limiter(SFLOW_MAX_VARS)
     TYPE(sflow_bc) :: bc(SFLOW_MAX_VARS, 4)
     REAL(C_DOUBLE) :: grav
     INTEGER(C_INT32_T) :: rheology_model
     INTEGER(C_INT32_T) :: pad0
     REAL(C_DOUBLE) :: mu
     REAL(C_DOUBLE) :: xi
     REAL(C_DOUBLE) :: friction_factor
     REAL(C_DOUBLE) :: pres
     REAL(C_DOUBLE) :: sp_heat_a
     REAL(C_DOUBLE) :: sp_gas_const_a
     REAL(C_DOUBLE) :: kin_visc_a
     REAL(C_DOUBLE) :: T_ambient
     INTEGER(C_INT32_T) :: entrainment_flag
     INTEGER(C_INT32_T) :: pad1
     REAL(C_DOUBLE) :: rho_l
     REAL(C_DOUBLE) :: sp_heat_l
     REAL(C_DOUBLE) :: kin_visc_l
     REAL(C_DOUBLE) :: loss_rate
     REAL(C_DOUBLE) :: rho_s(SFLOW_MAX_SOLID)
     REAL(C_DOUBLE) :: diam_s(SFLOW_MAX_SOLID)
     REAL(C_DOUBLE) :: sp_heat_s(SFLOW_MAX_SOLID)
     INTEGER(C_INT32_T) :: settling_flag
     INTEGER(C_INT32_T) :: collective_settling_flag
     REAL(C_DOUBLE) :: alphastot_min
     REAL(C_DOUBLE) :: maximum_solid_packing
     REAL(C_DOUBLE) :: A_drag
     REAL(C_DOUBLE) :: B_drag
     REAL(C_DOUBLE) :: erosion_coeff
     REAL(C_DOUBLE) :: x_source
     REAL(C_DOUBLE) :: y_source
     REAL(C_DOUBLE) :: r_source
     REAL(C_DOUBLE) :: r2_source
     REAL(C_DOUBLE) :: vel_source
     REAL(C_DOUBLE) :: T_source
     REAL(C_DOUBLE) :: h_source
     REAL(C_DOUBLE) :: mfr_source
     REAL(C_DOUBLE) :: alphas_source(SFLOW_MAX_SOLID)
     REAL(C_DOUBLE) :: time_param(4)
     REAL(C_DOUBLE) :: azimuth_source
     REAL(C_DOUBLE) :: arc_width_source
     REAL(C_DOUBLE) :: t_start
     REAL(C_DOUBLE) :: t_end
     REAL(C_DOUBLE) :: dt_output
     REAL(C_DOUBLE) :: thickness_levels(SFLOW_MAX_LEVELS)
     REAL(C_DOUBLE) :: dyn_pres_levels(SFLOW_MAX_LEVELS)
     REAL(C_DOUBLE) :: erodible_porosity
     REAL(C_DOUBLE) :: T_erodible
     REAL(C_DOUBLE) :: initial_erodible_thickness
     REAL(C_DOUBLE) :: erodible_fract(SFLOW_MAX_SOLID)
     INTEGER(C_INT32_T) :: erodible_deposit_flag
     INTEGER(C_INT32_T) :: topo_change_flag
     INTEGER(C_INT32_T) :: bottom_radial_source_flag
     INTEGER(C_INT32_T) :: n_intervals
     REAL(C_DOUBLE) :: angle_source
     REAL(C_DOUBLE) :: t_intervals(SFLOW_MAX_INTERVALS)
     REAL(C_DOUBLE) :: vel_intervals(SFLOW_MAX_INTERVALS)
     INTEGER(C_INT32_T) :: fp32_newton_fp64
     INTEGER(C_INT32_T) :: pad2
     REAL(C_DOUBLE) :: mu_s
     REAL(C_DOUBLE) :: mu_2
     REAL(C_DOUBLE) :: I_0
     REAL(C_DOUBLE) :: muI_inf
  END TYPE sflow_params

  TYPE, BIND(C) :: sflow_step_stats
     REAL(C_DOUBLE) :: t
     REAL(C_DOUBLE) :: dt
     REAL(C_DOUBLE) :: mass
     REAL(C_DOUBLE) :: volume
     REAL(C_DOUBLE) :: area
     REAL(C_DOUBLE) :: solid_mass
     INTEGER(C_INT64_T) :: solve_cells
     INTEGER(C_INT64_T) :: steps
     INTEGER(C_INT32_T) :: status
     INTEGER(C_INT32_T) :: pad
  END TYPE sflow_step_stats

END MODULE sflow_types

// sflow_types.cuh -- parameter blocks shared by host and device code.
#pragma once
#include <cstdint>

#include "../../include/sflow.h"

namespace sflow {

constexpr int kMaxSolid = SFLOW_MAX_SOLID;
constexpr int kMaxVars = SFLOW_MAX_VARS;   // conservative variables
constexpr int kMaxNewton = 100;            // max_nl_iter (parameters_2d.f90:362)

// Physical constants and model flags, in the bulk arithmetic type R.  A
// double copy always exists for the FP64 parts (Newton, epilogue).
template <class R>
struct Phys {
  int nv, ns, nrk;
  int gas, liquid, energy, alpha, rheo, rheo_model, slope_corr, curv;
  int settling, entrain, collective, radial_source, scheme;
  double eps_sing_d;          // thresholds are always tested in FP64
  // FP64 thresholds as R: for R = float these are the largest floats not
  // above the FP64 value, so `x > thr` on a float x gives the same answer
  // as the FP64 test (double)x > value.
  R thr_eps, thr_eps_sing, thr_neg1e7, thr_neg1e10, thr_1em10, thr_1em7, thr_1em3, thr_273;
  R eps_sing4, inv_eps_sing, sqrt2;
  R grav, pres, inv_pres, sp_heat_a, sp_gas_const_a, T_ambient, rho_a_amb;
  R rho_l, inv_rho_l, sp_heat_l;
  R rho_s[kMaxSolid], inv_rho_s[kMaxSolid], sp_heat_s[kMaxSolid];
  R h_source, vel_source, T_source, alphas_source[kMaxSolid], cell_area;
  R src_rho_m, src_cp_mix;    // mixt_var of the inlet state (constant per run)
  // FP64-only physics (semi-implicit, Newton, mass exchange)
  R mu, xi, friction_factor, kin_visc_c, loss_rate;
  R mu_s, mu_2, I_0, muI_inf;   // mu(I) rheology (model 11)
  R diam_s[kMaxSolid];
  R alphastot_min, max_packing, A_drag, B_drag, coeff_porosity, rho_c_sub, T_erodible,
      erodible_porosity;
  // erosion of the erodible layer (constitutive_2d.f90:4732-4760)
  R erosion_coeff, erodible_fract[kMaxSolid];
  int erodible_deposit, topo_change;
  // bottom radial source (constitutive_2d.f90:3149-3307)
  int bottom_source;
  int nodata;     // some cell is B_nodata (emptied by the assembly)
  int newton64;   // FP32 form: implicit friction solve with FP64 coefficients and iterations
  int exchange;   // update_erosion_deposition_cell runs: settling, entrainment or erosion
  // vulnerability table (IMEX_SfloW2D.f90:351, 489): levels as R (for the
  // FP32 form the smallest float not below the FP64 level, so that a float
  // compares with it as its FP64 value would)
  int n_thk, n_dyn;
  R thk_levels[SFLOW_MAX_LEVELS], dyn_levels[SFLOW_MAX_LEVELS];
};

// Topography terms of one cell.
template <class R>
struct Geo {
  R Bx, By, Bxx, Bxy, Byy, gc, dgcx, dgcy;
};

// Boundary conditions per side / variable, in R.
template <class R>
struct BC {
  int flag[4][kMaxVars];
  R value[4][kMaxVars];
};

// Grid and numerics of one domain.
template <class R>
struct Grid {
  int nx, ny;
  int pitch;        // row stride of every cell plane (elements)
  int64_t plane;    // stride between variable planes
  int tiles_x, tiles_y;
  double x0, y0, dx, dy;   // coordinates in FP64 (x_stag = x0 + j*dx)
  R x0r, y0r, rdx, rdy, dx2, dy2, one_by_dx, one_by_dy;
  R rc, theta;
  R cfl_dx, cfl_dy;
  int limiter[kMaxVars + 2];
  double cfl, max_dt;
  int dry_bc;       // every boundary condition is (Neumann, 0): a dry inside keeps dry ghosts
  int lim_all;      // the limiter of every variable when they are all equal, else -1
  int pdl;          // launch the step kernels with programmatic dependent launch
  // rows of a larger domain (row slabs): this domain's row k is row
  // k + k_off of the whole one (coordinates); the CFL minimum, the active
  // counts, the status bits and the log sums take only rows own_lo .. own_hi-1
  int k_off, own_lo, own_hi;
  int whole;        // own_lo == 0 && own_hi == ny
};

// Device-resident run state (one per domain).
struct RunState {
  double t, dt, dt_old, dt_old_old, t_output, t_end, t_stop, t_prev;
  unsigned long long cells_acc[2];  // active-cell counts of the running step
  unsigned long long dtmin_bits;   // atomicMin over positive doubles
  unsigned int status;             // SFLOW_S_* bits
  int run_step;                    // 1 when this step's dt is valid
  long long steps;
  long long step_limit;             // steps stop at this count
  long long cells_total;           // sum over steps of active cells
  long long last_cells;            // active cells of the last step
  long long newton_iters;          // sum of Newton iterations
  int newton_max;
  int pad;
  double src_t_coeff;              // ring inlet time factor at this step's t
  float src_t_coeff_f;
  int pad2;
  double tp[4];                    // time_param
  double pi_g;
  // bottom radial source at this step's t: time factor and inflow velocity
  // (constitutive_2d.f90:3151-3187)
  double bsrc_t_coeff, bsrc_vel;
  float bsrc_t_coeff_f, bsrc_vel_f;
  // active cells of dry border tiles (tile code 3: counted, not computed)
  unsigned long long border_acc[2];
  long long border_total;
};

}  // namespace sflow

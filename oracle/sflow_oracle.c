/*
 * sflow_oracle.c -- CPU FP64 restatement of the IMEX_SfloW2D time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GPU
 * path and the CPU baseline of the benchmark.  It is never linked into the
 * product library; only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg load it.
 *
 * Parity status: UNPINNED.  The reference is Fortran 90 and no Fortran
 * compiler exists on either machine available to this project, and the
 * reference's own tests (TESTS/run_tests.sh) only check that an output file
 * is written, so there are no golden vectors to pin against.  The oracle
 * is therefore pinned by (a) known-answer tests derived by hand from the
 * reference formulas (tests/golden/) and (b) physical invariants (mass
 * conservation, lake at rest, x/y mirror symmetry, the Ritter dam-break
 * solution).  The implicit friction term is differentiated by complex step
 * as the reference does (solver_2d.f90:2302-2367 with complexify.f90), with
 * the complex arithmetic written out (the GPU's plain FP64 form spells the
 * same formulas, so both compute the same Jacobian).
 *
 * Every routine names the reference routine it restates (path:line inside
 * the reference project).  The arithmetic follows the reference operation
 * order; compile with -ffp-contract=off so no FMA is introduced.
 *
 * Documented departures from the reference (all of them also hold for the
 * GPU path, so GPU and oracle implement the same semantics):
 *  D1  Cells outside the active set (solve_mask) are read as the dry state
 *      (h = 0, T = T_ambient) by their active neighbours, and interface
 *      values on their side of a face are zero.  The reference reads
 *      whatever it left there the last time the cell was active; that is the
 *      same thing unless a wet region vanished in one step (lift-off).
 *  D2  d_grav_coeff_dy is 0 when SLOPE_CORRECTION_FLAG = F; the reference
 *      leaves it unset (geometry_2d.f90:884-886 assigns dx twice).
 *  D3  The reference pauses on READ(*,*) on a NaN / negative thickness /
 *      T < 273 K; here a status bit is raised and the step continues.
 *  D4  A non-finite Newton residual ends the Newton solve at once (the
 *      reference iterates to its iteration limits on such a cell).
 *  D5  With ERODIBLE_DEPOSIT_FLAG the erodible layer's temperature in the
 *      energy exchange is the cell's own temperature.  The reference
 *      assigns its module-wide T_erodible = r_T just before that use in
 *      eval_mass_exchange_terms (constitutive_2d.f90:5044), so each cell
 *      sees its own value there too; only the stored global differs.
 *  Scope: n_add_gas = 0, no stochastic / pore-pressure / vertical-profile
 *  terms, rheology models 1 (Voellmy-Salm) and 6, SOLVER_SCHEME KT or UP;
 *  erosion with a uniform or user-given erodible layer, topography change,
 *  the bottom radial source, B_nodata cells and the vulnerability table.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/sflow.h"
/* pow, log and cos of the FP64 closures: the same functions, and so the
 * same bits, as the GPU kernels (double-double evaluation, see the header) */
#include "../imex_sflow2d_dev_gb300/csrc/sflow_math.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#define EPS DBL_EPSILON /* EPSILON(1.0_wp) */
#define MAXV (SFLOW_MAX_VARS + 2)
#define MAXS SFLOW_MAX_SOLID

/* Complex numbers of the complex-step Jacobian, with the arithmetic written
 * out (the GPU's plain FP64 form uses the same formulas, so both compute
 * the same Jacobian bits): products by the textbook formula, quotients by
 * Smith's algorithm (R. L. Smith, CACM 5(8), 1962), the square root by the
 * principal-branch formula sqrt((|z| + |x|)/2).  A real operand is a complex
 * number with zero imaginary part; for such operands every operation gives
 * the real result exactly, so the real calls of the closure (eval_f) equal
 * real arithmetic. */
typedef struct {
  double re, im;
} cplx;
static cplx cx(double re, double im) {
  cplx z;
  z.re = re;
  z.im = im;
  return z;
}
static cplx cr(double re) { return cx(re, 0.0); }
static cplx c_add(cplx a, cplx b) { return cx(a.re + b.re, a.im + b.im); }
static cplx c_sub(cplx a, cplx b) { return cx(a.re - b.re, a.im - b.im); }
static cplx c_mul(cplx a, cplx b) { return cx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static cplx c_div(cplx a, cplx b) {
  if (fabs(b.re) >= fabs(b.im)) {
    const double r = b.im / b.re, den = b.re + b.im * r;
    return cx((a.re + a.im * r) / den, (a.im - a.re * r) / den);
  }
  const double r = b.re / b.im, den = b.re * r + b.im;
  return cx((a.re * r + a.im) / den, (a.im * r - a.re) / den);
}
static cplx c_sqrt(cplx z) {
  const double ar = fabs(z.re), ai = fabs(z.im);
  if (ar == 0.0 && ai == 0.0) return cx(0.0, z.im);
  double m;
  if (ai == 0.0) m = ar;
  else if (ar == 0.0) m = ai;
  else if (ar >= ai) { const double t = ai / ar; m = ar * sqrt(1.0 + t * t); }
  else { const double t = ar / ai; m = ai * sqrt(1.0 + t * t); }
  const double t = sqrt((ar + m) * 0.5);
  if (z.re >= 0.0) return cx(t, z.im / (2.0 * t));
  return cx(ai / (2.0 * t), copysign(t, z.im));
}

/* ------------------------------------------------------------------------ */
/* physical constants and flags (constitutive_2d.f90:25-275 module data)     */
/* ------------------------------------------------------------------------ */
typedef struct {
  int nv, ns, nrk;
  int gas, liquid, energy, alpha, rheo, rheo_model, slope_corr, curv;
  int settling, entrain, collective, radial_source, scheme;
  double grav, mu, xi, friction_factor;
  double mu_s, mu_2, I_0, muI_inf; /* mu(I) rheology 11 */
  double pres, inv_pres, sp_heat_a, sp_gas_const_a, T_ambient, rho_a_amb;
  double kin_visc_c;
  double rho_l, inv_rho_l, sp_heat_l, loss_rate;
  double rho_s[MAXS], inv_rho_s[MAXS], diam_s[MAXS], sp_heat_s[MAXS];
  double alphastot_min, max_packing, A_drag, B_drag;
  double coeff_porosity, rho_c_sub, T_erodible, erodible_porosity, erosion_coeff;
  double eps_sing, eps_sing4;
  double theta, reconstr_coeff;
  int limiter[MAXV];
  double x_source, y_source, r_source, r2_source, vel_source, T_source, h_source;
  double alphas_source[MAXS], time_param[4], pi_g;
  /* erosion (constitutive_2d.f90:225-232; inpout_2d.f90:1818-1990) */
  double erodible_fract[MAXS], erodible_init;
  int erodible_deposit, topo_change, exchange;
  /* bottom radial source (constitutive_2d.f90:3149-3307) */
  int bottom_source, n_intervals;
  double angle_source, t_intervals[SFLOW_MAX_INTERVALS], vel_intervals[SFLOW_MAX_INTERVALS];
  /* vulnerability table (inpout_2d.f90:3808-3866) */
  int n_thk, n_dyn;
  double thk_levels[SFLOW_MAX_LEVELS], dyn_levels[SFLOW_MAX_LEVELS];
} phys_t;

/* ------------------------------------------------------------------------ */
/* small helpers mirroring Fortran intrinsics on the arrays used here        */
/* ------------------------------------------------------------------------ */
static double sumv(const double* a, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += a[i];
  return s;
}
static double dotv(const double* a, const double* b, int n) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}
static double dmin(double a, double b) { return a < b ? a : b; }
static double dmax(double a, double b) { return a > b ? a : b; }
static double sq(double a) { return a * a; }

/* ------------------------------------------------------------------------ */
/* geometry_2d.f90:1855-1876 minmod, 1878-1897 maxmod, 1776-1841 limit       */
/* ------------------------------------------------------------------------ */
double oracle_minmod(double a, double b) {
  if (dmin(fabs(a), fabs(b)) <= 0.0) return 0.0;
  double sa = a / fabs(a), sb = b / fabs(b);
  return 0.5 * (sa + sb) * dmin(fabs(a), fabs(b));
}
static double maxmod(double a, double b) {
  if (fabs(a * b) <= 0.0) return 0.0;
  double sa = a / fabs(a), sb = b / fabs(b);
  return 0.5 * (sa + sb) * dmax(fabs(a), fabs(b));
}
double oracle_limit(const double v[3], const double z[3], int limiter, double theta) {
  double a = (v[2] - v[1]) / (z[2] - z[1]);
  double b = (v[1] - v[0]) / (z[1] - z[0]);
  double c = (v[2] - v[0]) / (z[2] - z[0]);
  switch (limiter) {
    case 0: return 0.0;
    case 1: return oracle_minmod(a, b);
    case 2: {
      double s1 = oracle_minmod(a, 2.0 * b), s2 = oracle_minmod(2.0 * a, b);
      return maxmod(s1, s2);
    }
    case 3: return oracle_minmod(c, theta * oracle_minmod(a, b));
    case 4: return oracle_minmod(c, 2.0 * oracle_minmod(a, b));
    case 5: return c;
    case 6: return a;
    case 7: return b;
  }
  return 0.0;
}

/* ------------------------------------------------------------------------ */
/* constitutive_2d.f90:550-976 r_phys_var (vertical profiles off)            */
/* ------------------------------------------------------------------------ */
typedef struct {
  double h, u, v, alphas[MAXS], rho_m, T, red_grav, p_dyn;
} physv_t;

static void r_phys_var(const phys_t* P, const double* q, physv_t* o) {
  const int ns = P->ns;
  double xs[MAXS], inv_qj1;
  if (q[0] > EPS) {
    inv_qj1 = 1.0 / q[0];
    for (int i = 0; i < ns; ++i) xs[i] = q[4 + i] * inv_qj1;
    if (sumv(q + 4, ns) == q[0]) {
      double s = sumv(xs, ns);
      for (int i = 0; i < ns; ++i) xs[i] = xs[i] / s;
    }
  } else {
    o->h = 0.0; o->u = 0.0; o->v = 0.0;
    for (int i = 0; i < ns; ++i) o->alphas[i] = 0.0;
    o->rho_m = P->rho_a_amb; o->T = P->T_ambient; o->red_grav = 0.0; o->p_dyn = 0.0;
    return;
  }
  double xs_tot = sumv(xs, ns);
  double xc = 1.0 - xs_tot;
  double cbyxc;
  if (P->gas) cbyxc = ((xc - 0.0) * P->sp_heat_a + 0.0);
  else cbyxc = P->sp_heat_l * xc;
  double cmix = dotv(xs, P->sp_heat_s, ns) + cbyxc;
  double T;
  if (q[0] > P->eps_sing) {
    if (P->energy)
      T = (q[3] - 0.5 * (sq(q[1]) + sq(q[2])) * inv_qj1) / (q[0] * cmix);
    else
      T = q[3] / (q[0] * cmix);
    if (T <= 0.0) T = P->T_ambient;
  } else {
    T = P->T_ambient;
  }
  double inv_rho_c;
  if (P->gas) {
    double Rc;
    if (xc > EPS) Rc = ((xc - 0.0) * P->sp_gas_const_a + 0.0) / xc;
    else Rc = P->sp_gas_const_a;
    inv_rho_c = Rc * T * P->inv_pres;
  } else {
    inv_rho_c = P->inv_rho_l;
  }
  double inv_rhom = dotv(xs, P->inv_rho_s, ns) + xc * inv_rho_c;
  double rho_m = 1.0 / inv_rhom;
  for (int i = 0; i < ns; ++i) o->alphas[i] = xs[i] * rho_m * P->inv_rho_s[i];
  o->h = q[0] * inv_rhom;
  o->red_grav = (rho_m - P->rho_a_amb) * inv_rhom * P->grav;
  if (q[0] > P->eps_sing) {
    o->u = q[1] * inv_qj1;
    o->v = q[2] * inv_qj1;
  } else {
    double q12 = q[0] * q[0];
    double den = sqrt(q12 * q12 + P->eps_sing4);
    o->u = sqrt(2.0) * q[0] * q[1] / den;
    o->v = sqrt(2.0) * q[0] * q[2] / den;
  }
  o->p_dyn = 0.5 * rho_m * (sq(o->u) + sq(o->v));
  o->rho_m = rho_m;
  o->T = T;
}

/* constitutive_2d.f90:1637-1690 qc_to_qp */
void oracle_qc_to_qp_p(const phys_t* P, const double* qc, double* qp, double* p_dyn) {
  physv_t o;
  r_phys_var(P, qc, &o);
  const int nv = P->nv, ns = P->ns;
  qp[0] = o.h;
  qp[1] = o.h * o.u;
  qp[2] = o.h * o.v;
  qp[3] = o.T;
  for (int i = 0; i < ns; ++i) qp[4 + i] = P->alpha ? o.alphas[i] : o.alphas[i] * o.h;
  qp[nv] = o.u;
  qp[nv + 1] = o.v;
  if (p_dyn) *p_dyn = o.p_dyn;
}

/* constitutive_2d.f90:1718-2149 qp_to_qc (vertical profiles off) */
void oracle_qp_to_qc_p(const phys_t* P, const double* qp, double* qc) {
  const int nv = P->nv, ns = P->ns;
  double r_h = qp[0], r_hu, r_hv, r_u, r_v;
  if (r_h > EPS) {
    r_hu = qp[1]; r_hv = qp[2]; r_u = qp[nv]; r_v = qp[nv + 1];
  } else {
    for (int i = 0; i < nv; ++i) qc[i] = 0.0;
    return;
  }
  double r_T = qp[3];
  double alphas[MAXS], arhos[MAXS];
  for (int i = 0; i < ns; ++i) alphas[i] = P->alpha ? qp[4 + i] : qp[4 + i] / qp[0];
  double at = sumv(alphas, ns);
  for (int i = 0; i < ns; ++i) arhos[i] = alphas[i] * P->rho_s[i];
  double rho_c;
  if (P->gas) {
    double rho_a = P->pres / (P->sp_gas_const_a * r_T);
    rho_c = ((1.0 - 0.0 - at - 0.0) * rho_a + 0.0) / (1.0 - 0.0 - at);
  } else {
    rho_c = P->rho_l;
  }
  /* the rescaling of r_alphas (constitutive_2d.f90:1912-1920) does not
   * reach r_alphas_rhos, which was formed before it; nothing to do here */
  double alphac = 1.0 - at;
  double rho_m = alphac * rho_c + sumv(arhos, ns);
  double inv_rhom = 1.0 / rho_m;
  double xs[MAXS];
  for (int i = 0; i < ns; ++i) xs[i] = arhos[i] * inv_rhom;
  double xc = alphac * rho_c * inv_rhom;
  double cp_c;
  if (P->gas) {
    if (xc > EPS) cp_c = ((xc - 0.0) * P->sp_heat_a + 0.0) / xc;
    else cp_c = P->sp_heat_a;
  } else {
    cp_c = P->sp_heat_l;
  }
  double cmix = dotv(xs, P->sp_heat_s, ns) + xc * cp_c;
  qc[0] = rho_m * r_h;
  qc[1] = rho_m * r_hu;
  qc[2] = rho_m * r_hv;
  if (P->energy) {
    if (r_h > 0.0) qc[3] = r_h * rho_m * (cmix * r_T + 0.5 * (sq(r_u) + sq(r_v)));
    else qc[3] = 0.0;
  } else {
    qc[3] = r_h * rho_m * cmix * r_T;
  }
  for (int i = 0; i < ns; ++i) qc[4 + i] = xs[i] * qc[0];
}

/* constitutive_2d.f90:2164-2188 qp_to_qp2 */
static void qp_to_qp2(const double* qp, double B, double* qp2) {
  qp2[0] = qp[0] + B;
  if (qp[0] <= 0.0) { qp2[1] = 0.0; qp2[2] = 0.0; }
  else { qp2[1] = qp[1] / qp[0]; qp2[2] = qp[2] / qp[0]; }
}

/* constitutive_2d.f90:1513-1607 eval_sp_heat (gas xor liquid carrier) */
static void eval_sp_heat(const phys_t* P, const double* alphas, double inv_rhom,
                         double* cp_c, double* cp_mix) {
  const int ns = P->ns;
  double xs[MAXS];
  for (int i = 0; i < ns; ++i) xs[i] = alphas[i] * P->rho_s[i] * inv_rhom;
  double xc = 1.0 - sumv(xs, ns);
  *cp_c = 0.0;
  if (P->gas) {
    if (xc > EPS) *cp_c = ((xc - 0.0) * P->sp_heat_a + 0.0) / xc;
    else *cp_c = P->sp_heat_a;
  } else {
    *cp_c = P->sp_heat_l;
  }
  *cp_mix = dotv(xs, P->sp_heat_s, ns) + xc * *cp_c;
}

/* constitutive_2d.f90:1342-1492 mixt_var */
typedef struct { double Ri, rho_m, rho_c, red_grav, cp_c, cp_mix; } mixt_t;

static void mixt_var(const phys_t* P, const double* qpj, int sp_heat_flag, mixt_t* m) {
  const int nv = P->nv, ns = P->ns;
  double r_h = qpj[0];
  if (qpj[0] <= EPS) {
    m->red_grav = 0.0; m->rho_m = P->rho_a_amb; m->rho_c = P->rho_a_amb;
    if (P->liquid) { m->cp_c = P->sp_heat_l; m->cp_mix = P->sp_heat_l; }
    else { m->cp_c = P->sp_heat_a; m->cp_mix = P->sp_heat_a; }
    m->Ri = 0.0;
    return;
  }
  double r_u = qpj[nv], r_v = qpj[nv + 1], r_T = qpj[3];
  double alphas[MAXS];
  for (int i = 0; i < ns; ++i) alphas[i] = P->alpha ? qpj[4 + i] : qpj[4 + i] / qpj[0];
  double at = sumv(alphas, ns);
  double rho_c;
  if (P->gas) {
    double rho_a = P->pres / (P->sp_gas_const_a * r_T);
    rho_c = ((1.0 - 0.0 - at - 0.0) * rho_a + 0.0) / (1.0 - 0.0 - at);
  } else {
    rho_c = P->rho_l;
  }
  double rho_m = (1.0 - at) * rho_c + dotv(alphas, P->rho_s, ns);
  double inv_rhom = 1.0 / rho_m;
  double red_grav = (rho_m - P->rho_a_amb) / rho_m * P->grav;
  double u2 = sq(r_u) + sq(r_v);
  m->Ri = (u2 > 0.0) ? dmin(1.0e15, red_grav * r_h / u2) : 0.0;
  m->rho_m = rho_m;
  m->rho_c = rho_c;
  m->red_grav = red_grav;
  m->cp_c = 0.0; m->cp_mix = 0.0;
  if (sp_heat_flag) eval_sp_heat(P, alphas, inv_rhom, &m->cp_c, &m->cp_mix);
}

/* constitutive_2d.f90:2203-2307 eval_local_speeds_x / _y */
static void local_speeds(const phys_t* P, const double* qpj, double gc, int dir,
                         double* vmin, double* vmax) {
  mixt_t m;
  mixt_var(P, qpj, 0, &m);
  double r_h = qpj[0];
  double vel = (dir == 1) ? qpj[P->nv] : qpj[P->nv + 1];
  if (m.red_grav * r_h < 0.0) {
    *vmin = vel; *vmax = vel;
  } else {
    double c = (dir == 1) ? sqrt(m.red_grav * r_h * gc) : sqrt(gc * m.red_grav * r_h);
    *vmin = vel - c; *vmax = vel + c;
  }
}

/* constitutive_2d.f90:2325-2518 eval_fluxes (vertical profiles off) */
void oracle_eval_fluxes_p(const phys_t* P, const double* qcj, const double* qpj,
                          double gc, int dir, double* flux) {
  const int nv = P->nv, ns = P->ns;
  if (qpj[0] > EPS) {
    double r_h = qpj[0], r_u = qpj[nv], r_v = qpj[nv + 1];
    mixt_t m;
    mixt_var(P, qpj, 0, &m);
    double vel = (dir == 1) ? r_u : r_v;
    double pterm = 0.5 * m.rho_m * gc * m.red_grav * sq(r_h);
    flux[0] = vel * qcj[0] * 1.0;
    if (dir == 1) {
      flux[1] = vel * qcj[1] * 1.0 + pterm;
      flux[2] = vel * qcj[2] * 1.0;
    } else {
      flux[1] = vel * qcj[1] * 1.0;
      flux[2] = vel * qcj[2] * 1.0 + pterm;
    }
    if (P->energy) flux[3] = vel * (qcj[3] * 1.0 + pterm);
    else flux[3] = vel * qcj[3] * 1.0;
    for (int i = 0; i < ns; ++i) flux[4 + i] = vel * qcj[4 + i] * 1.0;
    if (ns > 0 && flux[0] > 0.0) {
      double s = sumv(flux + 4, ns);
      if (s / flux[0] > 1.0) {
        for (int i = 0; i < ns; ++i) flux[4 + i] = flux[4 + i] / s * flux[0];
      }
    }
  } else {
    for (int i = 0; i < nv; ++i) flux[i] = 0.0;
  }
}

/* ------------------------------------------------------------------------ */
/* constitutive_2d.f90:1154-1322 c_phys_var and 3513-4009                    */
/* eval_implicit_terms (rheology 1 and 6), complex arithmetic: the reference */
/* evaluates the implicit terms in complex variables for the real residual   */
/* as well as for the complex-step Jacobian.  DOT_PRODUCT conjugates its     */
/* first (complex) argument; the implicit columns hu, hv leave the solid     */
/* mass fractions real, so the conjugation changes no digit and is omitted.  */
/* ------------------------------------------------------------------------ */
static void c_phys_var(const phys_t* P, const cplx* q, cplx* h, cplx* u, cplx* v,
                       cplx* T, cplx* rho_m) {
  const int ns = P->ns;
  cplx inv_cqj1;
  if (q[0].re > EPS) {
    inv_cqj1 = c_div(cr(1.0), q[0]);
  } else {
    *h = cr(0.0); *u = cr(0.0); *v = cr(0.0); *T = cr(P->T_ambient); *rho_m = cr(P->rho_a_amb);
    return;
  }
  cplx xs_tot = cr(0.0), dcp = cr(0.0), dinv = cr(0.0);
  for (int i = 0; i < ns; ++i) xs_tot = c_add(xs_tot, c_mul(q[4 + i], inv_cqj1));
  for (int i = 0; i < ns; ++i) {
    const cplx xs = c_mul(q[4 + i], inv_cqj1);
    dcp = c_add(dcp, c_mul(xs, cr(P->sp_heat_s[i])));
    dinv = c_add(dinv, c_mul(xs, cr(P->inv_rho_s[i])));
  }
  const cplx xc = c_sub(cr(1.0), xs_tot);
  cplx cp_c;
  if (P->gas) cp_c = c_div(c_add(c_mul(c_sub(xc, cr(0.0)), cr(P->sp_heat_a)), cr(0.0)), xc);
  else cp_c = cr(P->sp_heat_l);
  const cplx cmix = c_add(dcp, c_mul(xc, cp_c));
  if (q[0].re > P->eps_sing) {
    if (P->energy)
      *T = c_div(c_sub(q[3], c_mul(c_mul(cr(0.5), c_add(c_mul(q[1], q[1]), c_mul(q[2], q[2]))), inv_cqj1)),
                 c_mul(q[0], cmix));
    else
      *T = c_div(q[3], c_mul(q[0], cmix));
    if (T->re <= 0.0) *T = cr(P->T_ambient);
  } else {
    *T = cr(P->T_ambient);
  }
  cplx inv_rho_c;
  if (P->gas) {
    const cplx Rc = c_div(c_add(c_mul(c_sub(xc, cr(0.0)), cr(P->sp_gas_const_a)), cr(0.0)), xc);
    inv_rho_c = c_mul(c_mul(Rc, *T), cr(P->inv_pres));
  } else {
    inv_rho_c = cr(P->inv_rho_l);
  }
  const cplx inv_rhom = c_add(dinv, c_mul(xc, inv_rho_c));
  *rho_m = c_div(cr(1.0), inv_rhom);
  *h = c_mul(q[0], inv_rhom);
  if (q[0].re > P->eps_sing) {
    *u = c_mul(q[1], inv_cqj1);
    *v = c_mul(q[2], inv_cqj1);
  } else {
    cplx q4 = c_mul(q[0], q[0]);
    q4 = c_mul(q4, q4);
    const cplx den = c_sqrt(c_add(q4, cr(P->eps_sing4)));
    *u = c_div(c_mul(c_mul(cr(sqrt(2.0)), q[0]), q[1]), den);
    *v = c_div(c_mul(c_mul(cr(sqrt(2.0)), q[0]), q[2]), den);
  }
}

static void c_implicit_terms(const phys_t* P, double Bx, double By, const cplx* q, cplx* nh) {
  for (int i = 0; i < P->nv; ++i) nh[i] = cr(0.0);
  if (!P->rheo) return;
  cplx h, u, v, T, rho_m;
  c_phys_var(P, q, &h, &u, &v, &T, &rho_m);
  if (!(q[0].re > EPS)) return;   /* h = u = v = 0: no friction */
  const cplx red_grav = c_mul(c_div(c_sub(rho_m, cr(P->rho_a_amb)), rho_m), cr(P->grav));
  const cplx w = P->slope_corr ? c_add(c_mul(u, cr(Bx)), c_mul(v, cr(By))) : cr(0.0);
  const cplx mod_vel2 = c_add(c_add(c_mul(u, u), c_mul(v, v)), c_mul(w, w));
  const cplx mod_vel = c_sqrt(mod_vel2);
  if (mod_vel.re != 0.0) {
    if (P->rheo_model == 1) {
      const cplx turb = c_mul(c_div(c_mul(rho_m, red_grav), cr(P->xi)), mod_vel2);
      nh[1] = c_sub(nh[1], c_mul(turb, c_div(u, mod_vel)));
      nh[2] = c_sub(nh[2], c_mul(turb, c_div(v, mod_vel)));
    } else if (P->rheo_model == 6) {
      const cplx mod_vel_hor = c_sqrt(c_add(c_mul(u, u), c_mul(v, v)));
      nh[1] = c_sub(nh[1], c_mul(c_mul(c_mul(rho_m, c_div(u, mod_vel_hor)), cr(P->friction_factor)), mod_vel2));
      nh[2] = c_sub(nh[2], c_mul(c_mul(c_mul(rho_m, c_div(v, mod_vel_hor)), cr(P->friction_factor)), mod_vel2));
    }
  }
}

/* real call of eval_implicit_terms (r_qj path): complex with zero imag */
static void r_implicit_terms(const phys_t* P, double Bx, double By, const double* q, double* nh) {
  cplx cq[SFLOW_MAX_VARS], cn[SFLOW_MAX_VARS];
  for (int i = 0; i < SFLOW_MAX_VARS; ++i) cq[i] = cr((i < P->nv) ? q[i] : 0.0);
  c_implicit_terms(P, Bx, By, cq, cn);
  for (int i = 0; i < P->nv; ++i) nh[i] = cn[i].re;
}

/* constitutive_2d.f90:4027-4547 eval_nh_semi_impl_terms (rheology 1) */
static void semi_impl_terms(const phys_t* P, double Bx, double By, double Bxx, double Bxy,
                            double Byy, double gc, const double* qpj, double* si) {
  const int nv = P->nv;
  for (int i = 0; i < nv; ++i) si[i] = 0.0;
  if (!P->rheo) return;
  double r_h = qpj[0], r_u = qpj[nv], r_v = qpj[nv + 1];
  mixt_t m;
  mixt_var(P, qpj, 0, &m);
  double r_w = P->slope_corr ? (r_u * Bx + r_v * By) : 0.0;
  double mod_vel = sqrt(sq(r_u) + sq(r_v) + sq(r_w));
  if (P->rheo_model == 1) {
    if (mod_vel > 0.0) {
      double centr = P->curv ? (Bxx * sq(r_u) + 2.0 * Bxy * r_u * r_v + Byy * sq(r_v)) : 0.0;
      double tt = P->mu * m.rho_m * (m.red_grav + centr) * r_h * sqrt(gc);
      tt = dmax(0.0, tt);
      tt = dmax(0.0, tt);
      si[1] = si[1] - tt * r_u / mod_vel;
      si[2] = si[2] - tt * r_v / mod_vel;
    }
  } else if (P->rheo_model == 11) {
    /* constitutive_2d.f90:4384-4458, mu(I) rheology */
    if (mod_vel > 0.0) {
      const int ns = P->ns;
      double diam, rho_p;
      if (ns > 1) {
        double al[MAXS];
        for (int i = 0; i < ns; ++i) al[i] = P->alpha ? qpj[4 + i] : qpj[4 + i] / qpj[0];
        /* sauter_diameter, average_density_solids (constitutive_2d.f90:387-416) */
        if (sumv(al, ns) < EPS) {
          diam = sumv(P->diam_s, ns) / ns;
          rho_p = sumv(P->rho_s, ns) / ns;
        } else {
          double q[MAXS], r[MAXS];
          for (int i = 0; i < ns; ++i) { q[i] = al[i] / P->diam_s[i]; r[i] = al[i] * P->rho_s[i]; }
          diam = sumv(al, ns) / sumv(q, ns);
          rho_p = sumv(r, ns) / sumv(al, ns);
        }
      } else {
        diam = P->diam_s[0];
        rho_p = P->rho_s[0];
      }
      if (r_h < EPS) r_h = EPS;
      double centr = P->curv ? (Bxx * sq(r_u) + 2.0 * Bxy * r_u * r_v + Byy * sq(r_v)) : 0.0;
      double vert = m.rho_m * (m.red_grav + centr) * r_h;
      vert = dmax(vert, 0.0);
      double eff = dmax(0.0, vert * sqrt(gc));
      if (eff < EPS) eff = EPS;
      double shear = 5.0 / 2.0 * mod_vel / (r_h * sqrt(gc));
      double I = diam * shear / sqrt(eff / rho_p);
      double mu_I = (P->mu_s * P->I_0 + P->mu_2 * I + P->muI_inf * (I * I)) / (P->I_0 + I);
      double tt = mu_I * eff;
      si[1] = si[1] - tt * (r_u / mod_vel);
      si[2] = si[2] - tt * (r_v / mod_vel);
    }
  }
}

/* ------------------------------------------------------------------------ */
/* solver_2d.f90:2245-2284 eval_f, 2302-2367 eval_jacobian,                  */
/* 2021-2226 lnsrch, 1662-1996 solve_rk_step  (n_nh = 2: hu, hv implicit)    */
/* ------------------------------------------------------------------------ */
typedef struct {
  const phys_t* P;
  double dt, a_diag, Bx, By;
  const double* q_old;
  const double* Rj;
} newton_ctx;

static void eval_f(const newton_ctx* c, const double* qj, double* f, double* scal_f) {
  const int nv = c->P->nv;
  double nh[SFLOW_MAX_VARS], Rj;
  r_implicit_terms(c->P, c->Bx, c->By, qj, nh);
  double s = 0.0;
  for (int i = 0; i < nv; ++i) {
    Rj = c->Rj[i] - c->a_diag * nh[i];
    f[i] = qj[i] - c->q_old[i] + c->dt * Rj;
    f[i] = 1.0 * f[i];
  }
  for (int i = 0; i < nv; ++i) s += f[i] * f[i];
  *scal_f = 0.5 * s;
}

/* left_matrix(i,j) stored row-major L[i*nv+j]; columns 1, 2 (hu, hv) by
 * complex step with h = n_vars EPSILON on the normalised unknowns */
static void eval_jacobian(const newton_ctx* c, const double* qj_rel, const double* qj_org,
                          double* L) {
  const int nv = c->P->nv;
  const double h = nv * EPS, one_by_h = 1.0 / h;
  for (int i = 0; i < nv * nv; ++i) L[i] = 0.0;
  cplx qc[SFLOW_MAX_VARS], nh[SFLOW_MAX_VARS];
  for (int i = 0; i < nv; ++i) {
    L[i * nv + i] = 1.0 * qj_org[i];
    if (i == 1 || i == 2) {
      for (int k = 0; k < nv; ++k) qc[k] = cr(qj_rel[k] * qj_org[k]);
      qc[i] = c_mul(cx(qj_rel[i], h), cr(qj_org[i]));
      c_implicit_terms(c->P, c->Bx, c->By, qc, nh);
      for (int k = 0; k < nv; ++k) {
        double jr = 1.0 * nh[k].im * one_by_h;
        L[k * nv + i] = L[k * nv + i] - c->dt * c->a_diag * jr;
      }
    }
  }
}

static void lnsrch(const newton_ctx* c, const double* x_old, const double* qj_org,
                   double f_old, const double* g, double* p, double* x, double* fval,
                   double* right_term, double stpmax, int* check) {
  const int nv = c->P->nv;
  const double TOLX = EPS, ALF = 1.0e-4;
  (void)ALF;
  double alam, alam2 = 0.0, alamin, a, b, disc, f2 = 0.0, rhs1, rhs2, slope, tmplam = 0.0;
  double qj[SFLOW_MAX_VARS];
  *check = 0;
  double nrm = 0.0;
  for (int i = 0; i < nv; ++i) nrm += p[i] * p[i];
  nrm = sqrt(nrm);
  if (nrm > stpmax)
    for (int i = 0; i < nv; ++i) p[i] = p[i] * stpmax / nrm;
  slope = dotv(g, p, nv);
  double mx = 0.0;
  for (int i = 0; i < nv; ++i) {
    double t = fabs(p[i]) / dmax(fabs(x_old[i]), 1.0);
    if (i == 0 || t > mx) mx = t;
  }
  alamin = TOLX / mx;
  if (alamin == 0.0) {
    for (int i = 0; i < nv; ++i) x[i] = x_old[i];
    return;
  }
  alam = 1.0;
  for (int it = 0; it < 100000; ++it) {
    for (int i = 0; i < nv; ++i) {
      x[i] = x_old[i] + alam * p[i];
      qj[i] = x[i] * qj_org[i];
    }
    eval_f(c, qj, right_term, fval);
    if (*fval <= 0.9 * f_old) {
      return;
    } else if (alam < alamin) {
      for (int i = 0; i < nv; ++i) x[i] = x_old[i];
      *fval = f_old;
      *check = 1;
      return;
    } else {
      if (alam == 1.0) {
        tmplam = -slope / (2.0 * (*fval - f_old - slope));
      } else {
        rhs1 = *fval - f_old - alam * slope;
        rhs2 = f2 - f_old - alam2 * slope;
        a = (rhs1 / sq(alam) - rhs2 / sq(alam2)) / (alam - alam2);
        b = (-alam2 * rhs1 / sq(alam) + alam * rhs2 / sq(alam2)) / (alam - alam2);
        if (a == 0.0) {
          tmplam = -slope / (2.0 * b);
        } else {
          disc = b * b - 3.0 * a * slope;
          if (disc < 0.0) tmplam = 0.5 * alam;
          else if (b <= 0.0) tmplam = (-b + sqrt(disc)) / (3.0 * a);
          else tmplam = -slope / (b + sqrt(disc));
        }
        if (tmplam > 0.5 * alam) tmplam = 0.5 * alam;
      }
    }
    alam2 = alam;
    f2 = *fval;
    alam = dmax(tmplam, 0.5 * alam);
  }
}

/* returns number of Newton iterations done (max_nl_iter+1 if exhausted) */
static int solve_rk_step(const newton_ctx* c, double* qj) {
  const int nv = c->P->nv;
  const int max_nl_iter = 100;
  const double STPMX = 100.0, TOLF = 1.0e-10, TOLMIN = 1.0e-6;
  double qj_org[SFLOW_MAX_VARS], qj_rel[SFLOW_MAX_VARS], right_term[SFLOW_MAX_VARS];
  double L[SFLOW_MAX_VARS * SFLOW_MAX_VARS], desc_dir[SFLOW_MAX_VARS], grad_f[SFLOW_MAX_VARS];
  double qj_rel_old[SFLOW_MAX_VARS];
  double scal_f, scal_f_old;
  int check = 0;
  for (int i = 0; i < nv; ++i) grad_f[i] = 0.0;
  for (int i = 0; i < nv; ++i) qj_org[i] = dmax(fabs(qj[i]), 1.0e-3);
  for (int i = 0; i < nv; ++i) qj_rel[i] = qj[i] / qj_org[i];
  int nl_iter;
  for (nl_iter = 1; nl_iter <= max_nl_iter; ++nl_iter) {
    const double TOLX = EPS;
    eval_f(c, qj, right_term, &scal_f);
    double mf = 0.0;
    for (int i = 0; i < nv; ++i) mf = dmax(mf, fabs(right_term[i]));
    if (mf < TOLF) return nl_iter;
    if (!isfinite(scal_f)) return max_nl_iter + 1; /* D4: NaN/Inf state */
    eval_jacobian(c, qj_rel, qj_org, L);
    /* explicit block: diagonal (mask11), coupling mask21 is identically 0
     * for a Jacobian with only implicit columns filled */
    double d1[SFLOW_MAX_VARS];
    for (int i = 0; i < nv; ++i) d1[i] = 0.0;
    for (int i = 0; i < nv; ++i)
      if (i != 1 && i != 2) d1[i] = right_term[i] / L[i * nv + i];
    double d2a = right_term[1], d2b = right_term[2];
    for (int i = 0; i < nv; ++i) {
      if (i == 1 || i == 2) continue;
      d2a = d2a - d1[i] * L[1 * nv + i];
      d2b = d2b - d1[i] * L[2 * nv + i];
    }
    double s11 = L[1 * nv + 1], s12 = L[1 * nv + 2], s21 = L[2 * nv + 1], s22 = L[2 * nv + 2];
    double inv_det = 1.0 / (s11 * s22 - s21 * s12);
    double sol1 = (d2a * s22 - d2b * s12) * inv_det;
    double sol2 = (s11 * d2b - s21 * d2a) * inv_det;
    for (int i = 0; i < nv; ++i) desc_dir[i] = -d1[i] + 0.0;
    desc_dir[1] = -sol1 + 0.0;
    desc_dir[2] = -sol2 + 0.0;
    for (int i = 0; i < nv; ++i) qj_rel_old[i] = qj_rel[i];
    scal_f_old = scal_f;
    if (nl_iter > 1) {
      double stpmax = STPMX * dmax(sqrt(dotv(qj_rel, qj_rel, nv)), (double)nv);
      for (int i = 0; i < nv; ++i) {
        double s = 0.0;
        for (int k = 0; k < nv; ++k) s += right_term[k] * L[k * nv + i];
        grad_f[i] = s;
      }
      lnsrch(c, qj_rel_old, qj_org, scal_f_old, grad_f, desc_dir, qj_rel, &scal_f, right_term,
             stpmax, &check);
    } else {
      for (int i = 0; i < nv; ++i) {
        qj_rel[i] = qj_rel_old[i] + desc_dir[i];
        qj[i] = qj_rel[i] * qj_org[i];
      }
      eval_f(c, qj, right_term, &scal_f);
    }
    for (int i = 0; i < nv; ++i) qj[i] = qj_rel[i] * qj_org[i];
    mf = 0.0;
    for (int i = 0; i < nv; ++i) mf = dmax(mf, fabs(right_term[i]));
    if (mf < TOLF) return nl_iter;
    if (check) {
      double mc = 0.0;
      for (int i = 0; i < nv; ++i) {
        double t = fabs(grad_f[i]) * dmax(fabs(qj_rel[i]), 1.0) / dmax(scal_f, 0.5 * nv);
        mc = dmax(mc, t);
      }
      check = mc < TOLMIN;
    }
    double mx = 0.0;
    for (int i = 0; i < nv; ++i) {
      double t = fabs(qj_rel[i] - qj_rel_old[i]) / dmax(fabs(qj_rel[i]), 1.0);
      mx = dmax(mx, t);
    }
    if (mx < TOLX) return nl_iter;
  }
  return max_nl_iter + 1;
}

/* ------------------------------------------------------------------------ */
/* constitutive_2d.f90:3024-3431 eval_expl_terms                             */
/* ------------------------------------------------------------------------ */
static void expl_terms(const phys_t* P, double Bx, double By, double Bxx, double Bxy, double Byy,
                       double gc, double dgcx, double dgcy, const double* qpj, double time,
                       double cell_fract, double arc_perim, double arc_nx, double arc_ny, double area,
                       double* e) {
  const int nv = P->nv, ns = P->ns;
  for (int i = 0; i < nv; ++i) e[i] = 0.0;
  if (qpj[0] <= EPS && cell_fract == 0.0 && arc_perim == 0.0) return;
  if (qpj[0] > EPS) {
    double r_h = qpj[0], r_u = qpj[nv], r_v = qpj[nv + 1];
    mixt_t m;
    mixt_var(P, qpj, 1, &m);
    double centr = P->curv ? (Bxx * sq(r_u) + 2.0 * Bxy * r_u * r_v + Byy * sq(r_v)) : 0.0;
    double tg = m.red_grav + centr;
    e[1] = -gc * m.rho_m * tg * r_h * Bx + 0.5 * m.rho_m * m.red_grav * sq(r_h) * dgcx;
    e[2] = -gc * m.rho_m * tg * r_h * By + 0.5 * m.rho_m * m.red_grav * sq(r_h) * dgcy;
    e[3] = P->energy ? (e[1] * r_u + e[2] * r_v) : 0.0;
  }
  /* bottom radial source (constitutive_2d.f90:3149-3307) */
  if (P->bottom_source && cell_fract > 0.0) {
    const double* tp = P->time_param;
    double t_coeff, h_dot;
    if (P->n_intervals > 0) {
      double vel_local = 0.0;
      for (int i = P->n_intervals - 1; i >= 0; --i)
        if (time >= P->t_intervals[i]) { vel_local = P->vel_intervals[i]; break; }
      t_coeff = vel_local > 0.0 ? 1.0 : 0.0;
      h_dot = cell_fract * vel_local;
    } else {
      double t_rem = fmod(time + tp[3], tp[0]);
      if (tp[2] == 0.0) {
        t_coeff = t_rem <= tp[1] ? 1.0 : 0.0;
      } else {
        if (t_rem <= tp[2]) t_coeff = t_rem / tp[2];
        else if (t_rem <= tp[1] - tp[2]) t_coeff = 1.0;
        else if (t_rem <= tp[1]) t_coeff = 1.0 - (t_rem - tp[1] + tp[2]) / tp[2];
        else t_coeff = 0.0;
      }
      h_dot = cell_fract * P->vel_source;
    }
    double qs[MAXV];
    for (int i = 0; i < nv + 2; ++i) qs[i] = 0.0;
    qs[0] = 1.0;
    qs[3] = P->T_source;
    for (int i = 0; i < ns; ++i) qs[4 + i] = P->alpha ? P->alphas_source[i] : P->alphas_source[i] * qs[0];
    mixt_t m;
    mixt_var(P, qs, 1, &m);
    e[0] = e[0] + t_coeff * h_dot * m.rho_m;
    e[1] = e[1] + 0.0;
    e[2] = e[2] + 0.0;
    e[3] = e[3] + t_coeff * h_dot * m.rho_m * m.cp_mix * P->T_source;
    for (int i = 0; i < ns; ++i) e[4 + i] = e[4 + i] + t_coeff * h_dot * P->alphas_source[i] * P->rho_s[i];
  }
  if (P->radial_source && arc_perim > 0.0 && P->h_source > 0.0) {
    const double* tp = P->time_param;
    double t_coeff;
    if (time >= tp[3]) {
      if (tp[2] > 0.0 && time < tp[3] + tp[2])
        t_coeff = 0.5 * (1.0 + sfm_cos(P->pi_g * (time - tp[3]) / tp[2]));
      else
        t_coeff = 0.0;
    } else {
      double t_rem = fmod(time, tp[0]);
      t_coeff = 0.0;
      if (tp[2] == 0.0) {
        if (t_rem <= tp[1]) t_coeff = 1.0;
      } else {
        if (t_rem < tp[2]) t_coeff = 0.5 * (1.0 - sfm_cos(P->pi_g * t_rem / tp[2]));
        else if (t_rem <= tp[1] - tp[2]) t_coeff = 1.0;
        else if (t_rem <= tp[1])
          t_coeff = 0.5 * (1.0 + sfm_cos(P->pi_g * ((t_rem - tp[1]) / tp[2] + 1.0)));
      }
    }
    if (t_coeff > 0.0) {
      double qs[MAXV];
      for (int i = 0; i < nv + 2; ++i) qs[i] = 0.0;
      qs[0] = 1.0;
      qs[3] = P->T_source;
      for (int i = 0; i < ns; ++i) qs[4 + i] = P->alpha ? P->alphas_source[i] : P->alphas_source[i] * qs[0];
      qs[nv] = 0.0; qs[nv + 1] = 0.0;
      mixt_t m;
      mixt_var(P, qs, 1, &m);
      double h_dot = P->h_source * P->vel_source * arc_perim / area;
      e[0] = e[0] + t_coeff * h_dot * m.rho_m;
      e[1] = e[1] + t_coeff * h_dot * m.rho_m * P->vel_source * arc_nx;
      e[2] = e[2] + t_coeff * h_dot * m.rho_m * P->vel_source * arc_ny;
      e[3] = e[3] + t_coeff * h_dot * m.rho_m * m.cp_mix * P->T_source;
      for (int i = 0; i < ns; ++i)
        e[4 + i] = e[4 + i] + t_coeff * h_dot * P->alphas_source[i] * P->rho_s[i];
    }
  }
}

/* ------------------------------------------------------------------------ */
/* constitutive_2d.f90:5326-5404 settling_velocity                           */
/* ------------------------------------------------------------------------ */
static double settling_velocity(const phys_t* P, double diam, double rhos, double rhoc,
                                double inv_kin_visc) {
  double inv_sqrt_C_D = 1.0, sv, Rey, const_part, sv_old;
  if (rhos <= rhoc) return 0.0;
  const_part = sqrt((4.0 / 3.0) * (rhos / rhoc - 1.0) * diam * P->grav);
  sv = const_part * inv_sqrt_C_D;
  Rey = diam * sv * inv_kin_visc;
  if (Rey <= 1000.0) {
    for (int i = 1; i <= 20; ++i) {
      sv_old = sv;
      if (P->collective)
        inv_sqrt_C_D = sqrt(1.0 / (24.0 * (1.0 + 0.15 * sfm_pow(Rey, 0.687)) / Rey +
                                   P->A_drag * (sfm_log(Rey) - P->B_drag)));
      else
        inv_sqrt_C_D = sqrt(Rey / (24.0 * (1.0 + 0.15 * sfm_pow(Rey, 0.687))));
      sv = const_part * inv_sqrt_C_D;
      if (fabs(sv_old - sv) / sv_old < 1.0e-6) return sv;
      Rey = diam * sv * inv_kin_visc;
    }
  }
  return sv;
}

/* constitutive_2d.f90:4574-5153 eval_mass_exchange_terms (no pore
 * pressure, no vaporisation, no vertical profiles): settling, erosion of the
 * erodible layer, air entrainment; returns deposition / erosion rates, the
 * equation terms and the topography rate */
static void mass_exchange(const phys_t* P, const double* qpj, double Bx, double By,
                          const double* erodible, double dt, double* dep, double* ers, double* eqn,
                          double* topo) {
  const int nv = P->nv, ns = P->ns;
  for (int i = 0; i < ns; ++i) { dep[i] = 0.0; ers[i] = 0.0; }
  for (int i = 0; i < nv; ++i) eqn[i] = 0.0;
  *topo = 0.0;
  if (qpj[0] <= EPS) return;
  const double alpha_max = 0.6, hind_exp = 4.65;
  double r_h = qpj[0], r_u = qpj[nv], r_v = qpj[nv + 1];
  double alphas[MAXS];
  for (int i = 0; i < ns; ++i) alphas[i] = P->alpha ? qpj[4 + i] : qpj[4 + i] / qpj[0];
  double at = sumv(alphas, ns);
  double r_w = P->slope_corr ? (r_u * Bx + r_v * By) : 0.0;
  double mod_vel2 = sq(r_u) + sq(r_v) + sq(r_w);
  double mod_vel = sqrt(mod_vel2);
  double tot_erosion, tot_solid_erosion;
  if (P->erosion_coeff > 0.0) {
    /* Fagents & Baloga (2006), eq. 5, with the solid volume fraction */
    tot_erosion = P->erosion_coeff * mod_vel * r_h * (1.0 - at);
    tot_solid_erosion = tot_erosion * (1.0 - P->erodible_porosity);
    for (int i = 0; i < ns; ++i) ers[i] = P->erodible_fract[i] * tot_solid_erosion;
  } else {
    for (int i = 0; i < ns; ++i) ers[i] = 0.0;
  }
  for (int i = 0; i < ns; ++i) ers[i] = dmax(0.0, dmin(ers[i], erodible[i] / dt));
  tot_solid_erosion = sumv(ers, ns);
  tot_erosion = tot_solid_erosion / (1.0 - P->erodible_porosity);
  double cont_erosion = tot_erosion * P->erodible_porosity;
  if (at <= P->alphastot_min) return;
  double r_T = qpj[3];
  /* ERODIBLE_DEPOSIT_FLAG: T_erodible = r_T (constitutive_2d.f90:5044) */
  const double T_ers = P->erodible_deposit ? r_T : P->T_erodible;
  mixt_t m;
  mixt_var(P, qpj, 1, &m);
  double inv_kin_visc = 1.0 / P->kin_visc_c;
  double rhoc = m.rho_c;
  for (int i = 0; i < ns; ++i) {
    if (alphas[i] > 0.0 && P->settling) {
      double sv = settling_velocity(P, P->diam_s[i], P->rho_s[i], rhoc, inv_kin_visc);
      dep[i] = alphas[i] * sv * 1.0;
      dep[i] = dep[i] * sfm_pow(1.0 - dmin(1.0, at / alpha_max), hind_exp);
      dep[i] = dmin(dep[i], r_h * alphas[i] / dt);
    }
  }
  double cpl = P->liquid ? P->loss_rate : 0.0;
  cpl = cpl + P->coeff_porosity * sumv(dep, ns);
  cpl = dmin(cpl, r_h * dmax(0.0, P->max_packing - sumv(alphas, ns)) / dt);
  cpl = dmin(cpl, (r_h * (1.0 - sumv(alphas, ns)) -
                   P->coeff_porosity * (r_h * sumv(alphas, ns) - dt * sumv(dep, ns))) / dt);
  double air_entr = 0.0;
  if (P->entrain && r_h > 0.0 && m.Ri > 0.0) {
    double entr_coeff = 0.075 / sqrt(1.0 + 718.0 * sfm_pow(m.Ri, 2.4));
    air_entr = entr_coeff * sqrt(mod_vel2);
  }
  double rho_dep_tot = dotv(P->rho_s, dep, ns);
  double rho_ers_tot = dotv(P->rho_s, ers, ns);
  double s_dep = 0.0, s_ers = 0.0;
  for (int i = 0; i < ns; ++i) s_dep += P->rho_s[i] * P->sp_heat_s[i] * dep[i];
  for (int i = 0; i < ns; ++i) s_ers += P->rho_s[i] * P->sp_heat_s[i] * ers[i];
  eqn[0] = P->rho_a_amb * air_entr + rho_ers_tot - rho_dep_tot + P->rho_c_sub * cont_erosion -
           m.rho_c * cpl;
  eqn[1] = -r_u * (rho_dep_tot + m.rho_c * cpl);
  eqn[2] = -r_v * (rho_dep_tot + m.rho_c * cpl);
  if (P->energy)
    eqn[3] = -r_T * (s_dep + m.rho_c * m.cp_c * cpl) -
             0.5 * mod_vel2 * (rho_dep_tot + m.rho_c * cpl) +
             T_ers * (s_ers + P->rho_c_sub * m.cp_c * cont_erosion) +
             P->T_ambient * P->sp_heat_a * P->rho_a_amb * air_entr;
  else
    eqn[3] = -r_T * (s_dep + m.rho_c * m.cp_c * cpl) +
             T_ers * (s_ers + P->rho_c_sub * m.cp_c * cont_erosion) +
             P->T_ambient * P->sp_heat_a * P->rho_a_amb * air_entr;
  for (int i = 0; i < ns; ++i) eqn[4 + i] = P->rho_s[i] * (ers[i] - dep[i]);
  *topo = (sumv(dep, ns) - sumv(ers, ns)) / (1.0 - P->erodible_porosity);
}

/* ======================================================================== */
/* The solver state (solver_2d.f90:65-248 module arrays)                     */
/* ======================================================================== */
typedef struct oracle {
  phys_t P;
  SflowParams prm;
  int nx, ny, N, nix, niy; /* cells; interfaces x = nx+1, y = ny+1 */
  double dx, dy, dx2, dy2, one_by_dx, one_by_dy;
  double *x_comp, *x_stag, *y_comp, *y_stag;
  double *B_cent, *Bx, *By, *Bxx, *Bxy, *Byy, *gc, *dgcx, *dgcy, *gcsx, *gcsy;
  int* source_cell;
  unsigned char *srcE, *srcW, *srcN, *srcS;
  double *arc_perim, *arc_nx, *arc_ny;
  /* state */
  double *q, *q0, *qp, *q_fv, *q_rk, *qp_rk, *divFlux, *NH, *SI, *expl;
  double *qL, *qR, *qB, *qT, *qpL, *qpR, *qpB, *qpT;
  double *axN, *axP, *ayN, *ayP, *Hx, *Hy;
  unsigned char *mask, *mask_tmp, *mask_x, *mask_y;
  int *j_cent, *k_cent, *j_sx, *k_sx, *j_sy, *k_sy;
  int solve_cells, solve_ix, solve_iy;
  double t, dt, dt_old, dt_old_old, t_output;
  double a_tilde_ij[16], a_dirk_ij[16], omega_tilde[4], omega[4];
  double *hmax, *pdynmax, *mod_vel_max, *deposit;
  /* erosion, bottom source, nodata, vulnerability table */
  double *erosion, *erodible, *erodible_thk, *B_init, *cell_fract;
  unsigned char *nodata, *vuln;
  int have_erodible_thk;
  uint32_t status;
  int64_t steps;
  int max_newton_iter_seen;
  int64_t newton_iters_total;
} oracle_t;

#define IDX(j, k) ((size_t)(k) * o->nx + (j))       /* cell (0-based) */
#define IDXX(j, k) ((size_t)(k) * o->nix + (j))     /* x-interface */
#define IDXY(j, k) ((size_t)(k) * o->nx + (j))      /* y-interface, k in 0..ny */

static void* xcalloc(size_t n, size_t s) {
  void* p = calloc(n ? n : 1, s);
  return p;
}

void sflow_oracle_default_params(SflowParams* p) {
  memset(p, 0, sizeof(*p));
  p->abi_version = SFLOW_ABI_VERSION;
  p->precision = SFLOW_PREC_FP64;
  p->comp_cells_x = 1000; p->comp_cells_y = 1; p->cell_size = 1.0e-3;
  p->gas_flag = 1;
  p->solver_scheme = SFLOW_SCHEME_KT; p->n_rk = 2;
  p->dt0 = 1.0e-4; p->max_dt = 1.0e-3; p->cfl = 0.24; p->theta = 1.0; p->reconstr_coeff = 1.0;
  for (int i = 0; i < SFLOW_MAX_VARS; ++i) p->limiter[i] = 1;
  for (int s = 0; s < 4; ++s)
    for (int i = 0; i < SFLOW_MAX_VARS; ++i) { p->bc[s][i].flag = 1; p->bc[s][i].value = 0.0; }
  p->grav = 9.81;
  p->maximum_solid_packing = 0.64;
  p->A_drag = -1.0; p->B_drag = -1.0;
  p->r2_source = -1.0; p->arc_width_source = 360.0; p->h_source = -1.0; p->mfr_source = -1.0;
  for (int i = 0; i < 4; ++i) p->time_param[i] = -1.0;
  p->t_end = 5.0e-2; p->dt_output = 5.0e-3;
}

/* ------------------------------------------------------------------------ */
/* geometry_2d.f90:555-895 topography_reconstruction (hot-path outputs)      */
/* ------------------------------------------------------------------------ */
static void topography_reconstruction(oracle_t* o) {
  const int nx = o->nx, ny = o->ny;
  const double dx = o->dx, dy = o->dy;
  static const double c1[5] = {-2.0, -1.0, 0.0, 1.0, 2.0};
  static const double c2[5] = {2.0, -1.0, -2.0, -1.0, 2.0};
  double norm1_x = 10.0 * dx, norm1_y = 10.0 * dy;
  double norm2_x = 7.0 * sq(dx), norm2_y = 7.0 * sq(dy);
  double norm_xy = (10.0 * dx) * (10.0 * dy);
#define B(j, k) o->B_cent[IDX(j, k)]
  for (int i = 0; i < o->N; ++i) { o->Bx[i] = o->By[i] = o->Bxx[i] = o->Byy[i] = o->Bxy[i] = 0.0; }
  if (ny == 1) {
    int k = 0;
    for (int j = 2; j <= nx - 3; ++j) {
      double px = 0.0, sxx = 0.0;
      for (int kj = 0; kj < 5; ++kj) {
        px = px + c1[kj] * B(j + kj - 2, k);
        sxx = sxx + c2[kj] * B(j + kj - 2, k);
      }
      o->Bx[IDX(j, k)] = px / norm1_x;
      o->By[IDX(j, k)] = 0.0 / norm1_y;
      o->Bxx[IDX(j, k)] = sxx / norm2_x;
      o->Byy[IDX(j, k)] = 0.0 / norm2_y;
      o->Bxy[IDX(j, k)] = 0.0;
    }
  }
  for (int k = 2; k <= ny - 3; ++k) {
    for (int j = 2; j <= nx - 3; ++j) {
      double px = 0.0, py = 0.0, sxx = 0.0, syy = 0.0;
      for (int kj = 0; kj < 5; ++kj) {
        px = px + c1[kj] * B(j + kj - 2, k);
        sxx = sxx + c2[kj] * B(j + kj - 2, k);
      }
      for (int kk = 0; kk < 5; ++kk) {
        py = py + c1[kk] * B(j, k + kk - 2);
        syy = syy + c2[kk] * B(j, k + kk - 2);
      }
      o->Bx[IDX(j, k)] = px / norm1_x;
      o->By[IDX(j, k)] = py / norm1_y;
      o->Bxx[IDX(j, k)] = sxx / norm2_x;
      o->Byy[IDX(j, k)] = syy / norm2_y;
      double ws = 0.0;
      for (int kk = 0; kk < 5; ++kk)
        for (int kj = 0; kj < 5; ++kj) ws = ws + c1[kj] * c1[kk] * B(j + kj - 2, k + kk - 2);
      o->Bxy[IDX(j, k)] = ws / norm_xy;
    }
  }
#undef B
  double* arrs[5] = {o->Bx, o->By, o->Bxx, o->Byy, o->Bxy};
  if (nx >= 3) {
    for (int k = 0; k < ny; ++k)
      for (int a = 0; a < 5; ++a) {
        double* A = arrs[a];
        A[IDX(0, k)] = A[IDX(2, k)];
        A[IDX(1, k)] = A[IDX(2, k)];
        A[IDX(nx - 2, k)] = A[IDX(nx - 3, k)];
        A[IDX(nx - 1, k)] = A[IDX(nx - 3, k)];
      }
  }
  if (ny > 1 && ny >= 3) {
    for (int j = 0; j < nx; ++j)
      for (int a = 0; a < 5; ++a) {
        double* A = arrs[a];
        A[IDX(j, 0)] = A[IDX(j, 2)];
        A[IDX(j, 1)] = A[IDX(j, 2)];
        A[IDX(j, ny - 2)] = A[IDX(j, ny - 3)];
        A[IDX(j, ny - 1)] = A[IDX(j, ny - 3)];
      }
  }
  if (o->P.slope_corr) {
    for (int i = 0; i < o->N; ++i) {
      o->gc[i] = 1.0 / (1.0 + sq(o->Bx[i]) + sq(o->By[i]));
      o->dgcx[i] = -2.0 * sq(o->gc[i]) * (o->Bx[i] * o->Bxx[i] + o->By[i] * o->Bxy[i]);
      o->dgcy[i] = -2.0 * sq(o->gc[i]) * (o->Bx[i] * o->Bxy[i] + o->By[i] * o->Byy[i]);
    }
    for (int k = 0; k < ny; ++k) {
      o->gcsx[IDXX(0, k)] = o->gc[IDX(0, k)];
      for (int j = 1; j < nx; ++j)
        o->gcsx[IDXX(j, k)] = 0.5 * (o->gc[IDX(j - 1, k)] + o->gc[IDX(j, k)]);
      o->gcsx[IDXX(nx, k)] = o->gc[IDX(nx - 1, k)];
    }
    for (int j = 0; j < nx; ++j) {
      o->gcsy[IDXY(j, 0)] = o->gc[IDX(j, 0)];
      for (int k = 1; k < ny; ++k)
        o->gcsy[IDXY(j, k)] = 0.5 * (o->gc[IDX(j, k - 1)] + o->gc[IDX(j, k)]);
      o->gcsy[IDXY(j, ny)] = o->gc[IDX(j, ny - 1)];
    }
  } else {
    for (int i = 0; i < o->N; ++i) { o->gc[i] = 1.0; o->dgcx[i] = 0.0; o->dgcy[i] = 0.0; }
    for (size_t i = 0; i < (size_t)o->nix * ny; ++i) o->gcsx[i] = 1.0;
    for (size_t i = 0; i < (size_t)nx * o->niy; ++i) o->gcsy[i] = 1.0;
  }
}

/* ------------------------------------------------------------------------ */
/* geometry_2d.f90:907-1323 init_source (radial ring, full or arc sector)   */
/* ------------------------------------------------------------------------ */
static void init_source(oracle_t* o) {
  const phys_t* P = &o->P;
  const int nx = o->nx, ny = o->ny;
  double *vEx = xcalloc(o->N, sizeof(double)), *vEy = xcalloc(o->N, sizeof(double));
  double *vWx = xcalloc(o->N, sizeof(double)), *vWy = xcalloc(o->N, sizeof(double));
  double *vNx = xcalloc(o->N, sizeof(double)), *vNy = xcalloc(o->N, sizeof(double));
  double *vSx = xcalloc(o->N, sizeof(double)), *vSy = xcalloc(o->N, sizeof(double));
  const double xs = P->x_source, ys = P->y_source, rs = P->r_source;
  const double* xc = o->x_comp; const double* yc = o->y_comp;
  const double* xst = o->x_stag; const double* yst = o->y_stag;
  for (int k = 1; k <= ny - 2; ++k) {
    for (int j = 1; j <= nx - 2; ++j) {
      if (sq(xc[j] - xs) + sq(yc[k] - ys) <= sq(rs)) {
        o->source_cell[IDX(j, k)] = 1;
        if (sq(xc[j - 1] - xs) + sq(yc[k] - ys) >= sq(rs)) {
          size_t c = IDX(j - 1, k);
          o->source_cell[c] = 2; o->srcE[c] = 1;
          double d = sqrt(sq(xst[j] - xs) + sq(yc[k] - ys));
          vEx[c] = (xst[j] - xs) * rs / sq(d);
          vEy[c] = (yc[k] - ys) * rs / sq(d);
        } else if (sq(xc[j + 1] - xs) + sq(yc[k] - ys) >= sq(rs)) {
          size_t c = IDX(j + 1, k);
          o->source_cell[c] = 2; o->srcW[c] = 1;
          double d = sqrt(sq(xst[j + 1] - xs) + sq(yc[k] - ys));
          vWx[c] = (xst[j + 1] - xs) * rs / sq(d);
          vWy[c] = (yc[k] - ys) * rs / sq(d);
        }
        if (sq(xc[j] - xs) + sq(yc[k - 1] - ys) >= sq(rs)) {
          size_t c = IDX(j, k - 1);
          o->source_cell[c] = 2; o->srcN[c] = 1;
          double d = sqrt(sq(xc[j] - xs) + sq(yst[k] - ys));
          vNx[c] = (xc[j] - xs) * rs / sq(d);
          vNy[c] = (yst[k] - ys) * rs / sq(d);
        } else if (sq(xc[j] - xs) + sq(yc[k + 1] - ys) >= sq(rs)) {
          size_t c = IDX(j, k + 1);
          o->source_cell[c] = 2; o->srcS[c] = 1;
          double d = sqrt(sq(xc[j] - xs) + sq(yst[k + 1] - ys));
          vSx[c] = (xc[j] - xs) * rs / sq(d);
          vSy[c] = (yst[k + 1] - ys) * rs / sq(d);
        }
      }
    }
  }
  if (P->radial_source) {
    double half_arc = 0.5 * o->prm.arc_width_source;
    for (int k = 0; k < ny; ++k) {
      for (int j = 0; j < nx; ++j) {
        size_t c = IDX(j, k);
        if (o->source_cell[c] != 2) continue;
        const unsigned char flags[4] = {o->srcE[c], o->srcW[c], o->srcN[c], o->srcS[c]};
        const double vxs[4] = {vEx[c], vWx[c], vNx[c], vSx[c]};
        const double vys[4] = {vEy[c], vWy[c], vNy[c], vSy[c]};
        const double flen[4] = {o->dy, o->dy, o->dx, o->dx};
        for (int f = 0; f < 4; ++f) {
          if (!flags[f]) continue;
          double vx = vxs[f], vy = vys[f];
          double vmag = sqrt(vx * vx + vy * vy);
          if (vmag > 0.0) {
            double nxv = vx / vmag, nyv = vy / vmag;
            int in_arc;
            if (o->prm.arc_width_source >= 360.0) {
              in_arc = 1;
            } else {
              double ang = 90.0 - atan2(vy, vx) * 180.0 / P->pi_g;
              ang = fmod(ang + 360.0, 360.0);
              double diff = fmod(fabs(ang - o->prm.azimuth_source) + 360.0, 360.0);
              if (diff > 180.0) diff = 360.0 - diff;
              in_arc = diff <= half_arc;
            }
            if (in_arc) {
              o->arc_perim[c] = o->arc_perim[c] + flen[f];
              o->arc_nx[c] = o->arc_nx[c] + flen[f] * nxv;
              o->arc_ny[c] = o->arc_ny[c] + flen[f] * nyv;
            }
          }
        }
        if (o->arc_perim[c] > 0.0) {
          o->arc_nx[c] = o->arc_nx[c] / o->arc_perim[c];
          o->arc_ny[c] = o->arc_ny[c] / o->arc_perim[c];
          double vmag = sqrt(sq(o->arc_nx[c]) + sq(o->arc_ny[c]));
          if (vmag > 0.0) { o->arc_nx[c] /= vmag; o->arc_ny[c] /= vmag; }
        }
      }
    }
    double tot = 0.0;
    for (int k = 0; k < ny; ++k)
      for (int j = 0; j < nx; ++j) tot += o->arc_perim[IDX(j, k)];
    double r1 = P->r_source, r2 = P->r2_source;
    double h_ell = sq(r1 - r2) / sq(r1 + r2);
    double len = P->pi_g * (r1 + r2) *
                 (1.0 + 0.25 * h_ell + sq(h_ell) / 64.0 + h_ell * h_ell * h_ell / 256.0 +
                  sq(sq(h_ell)) * 25.0 / 16384.0 + sq(sq(h_ell)) * h_ell * 49.0 / 65536.0);
    if (o->prm.arc_width_source < 360.0) len = len * (o->prm.arc_width_source / 360.0);
    if (tot > 0.0) {
      double rescale = len / tot;
      for (int i = 0; i < o->N; ++i) o->arc_perim[i] = o->arc_perim[i] * rescale;
    }
  }
  free(vEx); free(vEy); free(vWx); free(vWy); free(vNx); free(vNy); free(vSx); free(vSy);
}

/* inpout_2d.f90:4097-4137, 4526, 4637-4747: ring length and h_source from
 * MFR_SOURCE and VEL_SOURCE; time_param(2) from MFR (4435-4437) */
static void derive_source(oracle_t* o) {
  phys_t* P = &o->P;
  if (!P->radial_source && !P->bottom_source) return;
  if (P->time_param[0] < 0.0 || P->time_param[1] < 0.0 || P->time_param[2] < 0.0 ||
      P->time_param[3] < 0.0) {
    P->time_param[0] = o->prm.t_end; P->time_param[1] = o->prm.t_end;
    P->time_param[2] = 0.0; P->time_param[3] = o->prm.t_end;
  }
  if (P->r2_source <= 0.0) { P->r2_source = P->r_source; P->angle_source = 0.0; }
  if (!P->radial_source) return;
  double r1 = P->r_source, r2 = P->r2_source;
  double h_ell = sq(r1 - r2) / sq(r1 + r2);
  double len = P->pi_g * (r1 + r2) *
               (1.0 + 0.25 * h_ell + sq(h_ell) / 64.0 + h_ell * h_ell * h_ell / 256.0 +
                sq(sq(h_ell)) * 25.0 / 16384.0 + sq(sq(h_ell)) * h_ell * 49.0 / 65536.0);
  if (o->prm.arc_width_source < 360.0) len = len * (o->prm.arc_width_source / 360.0);
  if (o->prm.mfr_source >= 0.0) {
    double qs[MAXV];
    double hs = 1.0;
    for (int i = 0; i < P->nv + 2; ++i) qs[i] = 0.0;
    qs[0] = hs; qs[1] = hs * P->vel_source; qs[2] = 0.0; qs[3] = P->T_source;
    for (int i = 0; i < P->ns; ++i) qs[4 + i] = P->alpha ? P->alphas_source[i] : P->alphas_source[i] * hs;
    qs[P->nv] = P->vel_source; qs[P->nv + 1] = 0.0;
    mixt_t m;
    mixt_var(P, qs, 0, &m);
    P->h_source = o->prm.mfr_source / (len * m.rho_m * P->vel_source * 1.0);
    P->time_param[1] = 1.0e14 / o->prm.mfr_source;
  }
}

/* ------------------------------------------------------------------------ */
/* geometry_2d.f90:1899-1994 compute_cell_fract: 200 x 200 sub-cell points   */
/* per cell inside the rotated ellipse; REAL(count)/n2 in single precision   */
/* ------------------------------------------------------------------------ */
static void compute_cell_fract(oracle_t* o) {
  const phys_t* P = &o->P;
  const int n_points = 200, n_points2 = n_points * n_points;
  const double ang_rad = P->angle_source / 180.0 * atan(1.0) * 4.0;
  const double xs = P->x_source, ys = P->y_source, rs = P->r_source, r2s = P->r2_source;
  const double rmx = dmax(rs, r2s);
  double* xsub = xcalloc(n_points2, 8);
  double* ysub = xcalloc(n_points2, 8);
  for (int h = 1; h <= n_points; ++h) {
    for (int i = h; i <= n_points2; i += n_points) xsub[i - 1] = (double)h;
    for (int i = (h - 1) * n_points + 1; i <= h * n_points; ++i) ysub[i - 1] = (double)h;
  }
  for (int i = 0; i < n_points2; ++i) {
    xsub[i] = (2.0 * xsub[i] - 1.0) / (2.0 * (double)n_points);
    ysub[i] = (2.0 * ysub[i] - 1.0) / (2.0 * (double)n_points);
    xsub[i] = (xsub[i] - 0.5) * o->dx;
    ysub[i] = (ysub[i] - 0.5) * o->dy;
  }
  for (int j = 0; j < o->nx; ++j)
    for (int k = 0; k < o->ny; ++k) {
      double f = 0.0;
      if (!(o->x_stag[j + 1] < xs - rmx || o->x_stag[j] > xs + rmx || o->y_stag[k + 1] < ys - rmx ||
            o->y_stag[k] > ys + rmx)) {
        int cnt = 0;
        for (int i = 0; i < n_points2; ++i) {
          double a = (o->x_comp[j] + xsub[i] - xs) * cos(ang_rad) + (o->y_comp[k] + ysub[i] - ys) * sin(ang_rad);
          double b = -((o->x_comp[j] + xsub[i] - xs) * sin(ang_rad)) + (o->y_comp[k] + ysub[i] - ys) * cos(ang_rad);
          if (sq(a) / sq(rs) + sq(b) / sq(r2s) <= 1.0) ++cnt;
        }
        f = (double)((float)cnt / (float)n_points2);
      }
      o->cell_fract[IDX(j, k)] = f;
    }
  free(xsub);
  free(ysub);
}

/* ------------------------------------------------------------------------ */
/* solver_2d.f90:667-858 check_solve                                         */
/* ------------------------------------------------------------------------ */
static void check_solve(oracle_t* o, int solve_all) {
  const int nx = o->nx, ny = o->ny, nv = o->P.nv;
  unsigned char* m = o->mask;
  for (int k = 1; k < ny - 1; ++k)
    for (int j = 1; j < nx - 1; ++j) m[IDX(j, k)] = solve_all ? 1 : 0;
  for (int k = 0; k < ny; ++k) { m[IDX(0, k)] = 1; m[IDX(nx - 1, k)] = 1; }
  for (int j = 0; j < nx; ++j) { m[IDX(j, 0)] = 1; m[IDX(j, ny - 1)] = 1; }
  for (int k = 1; k < ny - 1; ++k)
    for (int j = 1; j < nx - 1; ++j)
      if (o->q[IDX(j, k) * nv + 0] > 0.0) m[IDX(j, k)] = 1;
  if (o->P.bottom_source)
    for (int i = 0; i < o->N; ++i)
      if (o->cell_fract[i] > 0.0) m[i] = 1;
  if (o->P.radial_source)
    for (int k = 1; k < ny - 1; ++k)
      for (int j = 1; j < nx - 1; ++j)
        if (o->source_cell[IDX(j, k)] == 2) m[IDX(j, k)] = 1;
  for (int i = 0; i < o->P.nrk; ++i) {
    memcpy(o->mask_tmp, m, o->N);
    const unsigned char* t = o->mask_tmp;
    for (int k = 1; k < ny - 1; ++k)
      for (int j = 1; j < nx - 1; ++j) {
        size_t c = IDX(j, k);
        m[c] = m[c] || t[IDX(j - 1, k)] || t[IDX(j + 1, k)] || t[IDX(j, k - 1)] || t[IDX(j, k + 1)];
      }
  }
  if (o->P.radial_source)
    for (int i = 0; i < o->N; ++i)
      if (o->source_cell[i] == 1) m[i] = 0;
  memset(o->mask_x, 0, (size_t)o->nix * ny);
  memset(o->mask_y, 0, (size_t)nx * o->niy);
  int n = 0;
  for (int k = 0; k < ny; ++k)
    for (int j = 0; j < nx; ++j)
      if (m[IDX(j, k)]) {
        o->j_cent[n] = j; o->k_cent[n] = k; ++n;
        o->mask_x[IDXX(j, k)] = 1; o->mask_x[IDXX(j + 1, k)] = 1;
        o->mask_y[IDXY(j, k)] = 1; o->mask_y[IDXY(j, k + 1)] = 1;
      }
  o->solve_cells = n;
  n = 0;
  for (int k = 0; k < ny; ++k)
    for (int j = 0; j < o->nix; ++j)
      if (o->mask_x[IDXX(j, k)]) { o->j_sx[n] = j; o->k_sx[n] = k; ++n; }
  o->solve_ix = n;
  n = 0;
  for (int k = 0; k < o->niy; ++k)
    for (int j = 0; j < nx; ++j)
      if (o->mask_y[IDXY(j, k)]) { o->j_sy[n] = j; o->k_sy[n] = k; ++n; }
  o->solve_iy = n;
}

/* ------------------------------------------------------------------------ */
/* solver_2d.f90:3095-3924 reconstruction                                    */
/* ------------------------------------------------------------------------ */
static void reconstruction(oracle_t* o, const double* q_expl, const double* qp_expl) {
  const phys_t* P = &o->P;
  const int nx = o->nx, ny = o->ny, nv = P->nv, np = nv + 2;
  const SflowBC* bcW = o->prm.bc[SFLOW_W];
  const SflowBC* bcE = o->prm.bc[SFLOW_E];
  const SflowBC* bcS = o->prm.bc[SFLOW_S];
  const SflowBC* bcN = o->prm.bc[SFLOW_N];
  const double rc = P->reconstr_coeff;
  /* D1: faces on the side of cells that are not reconstructed read zero */
  memset(o->qL, 0, sizeof(double) * o->nix * ny * nv);
  memset(o->qR, 0, sizeof(double) * o->nix * ny * nv);
  memset(o->qpL, 0, sizeof(double) * o->nix * ny * np);
  memset(o->qpR, 0, sizeof(double) * o->nix * ny * np);
  memset(o->qB, 0, sizeof(double) * nx * o->niy * nv);
  memset(o->qT, 0, sizeof(double) * nx * o->niy * nv);
  memset(o->qpB, 0, sizeof(double) * nx * o->niy * np);
  memset(o->qpT, 0, sizeof(double) * nx * o->niy * np);
#define QP(i, j, k) qp_expl[IDX(j, k) * np + (i)]
#pragma omp parallel for schedule(static)
  for (int l = 0; l < o->solve_cells; ++l) {
    const int j = o->j_cent[l], k = o->k_cent[l];
    const size_t c = IDX(j, k);
    const int sc = o->source_cell[c];
    const int sE = o->srcE[c], sW = o->srcW[c], sN = o->srcN[c], sS = o->srcS[c];
    double qW[MAXV], qE[MAXV], qS[MAXV], qN[MAXV], sb[MAXV], px[MAXV], py[MAXV];
    double qs[3], xs[3], ys[3], qp2[3], dq;
    for (int i = 0; i < np; ++i) {
      qW[i] = qE[i] = qS[i] = qN[i] = sb[i] = QP(i, j, k);
      px[i] = py[i] = 0.0;
    }
    xs[1] = o->x_comp[j];
    ys[1] = o->y_comp[k];
    xs[0] = xs[2] = ys[0] = ys[2] = 0.0;
    for (int i = 0; i < nv; ++i) {
      qs[1] = QP(i, j, k);
      if (nx > 1) {
        if (j == 0) {
          xs[0] = o->x_stag[0]; xs[2] = o->x_comp[j + 1];
          if (sc == 2) {
            qs[0] = sb[i]; qs[2] = QP(i, j + 1, k);
            px[i] = oracle_limit(qs, xs, P->limiter[i], P->theta);
          } else if (bcW[i].flag == 0) {
            qs[0] = bcW[i].value; qs[2] = QP(i, j + 1, k);
            px[i] = oracle_limit(qs, xs, P->limiter[i], P->theta);
          } else if (bcW[i].flag == 1) {
            px[i] = bcW[i].value;
          } else if (bcW[i].flag == 2) {
            px[i] = (QP(i, 1, k) - QP(i, 0, k)) * o->one_by_dx;
          }
        } else if (j == nx - 1) {
          xs[2] = o->x_stag[o->nix - 1]; xs[0] = o->x_comp[j - 1];
          if (sc == 2) {
            qs[2] = sb[i]; qs[0] = QP(i, j - 1, k);
            px[i] = oracle_limit(qs, xs, P->limiter[i], P->theta);
          } else if (bcE[i].flag == 0) {
            qs[2] = bcE[i].value; qs[0] = QP(i, j - 1, k);
            px[i] = oracle_limit(qs, xs, P->limiter[i], P->theta);
          } else if (bcE[i].flag == 1) {
            px[i] = bcE[i].value;
          } else if (bcE[i].flag == 2) {
            px[i] = (QP(i, nx - 1, k) - QP(i, nx - 2, k)) * o->one_by_dx;
          }
        } else {
          xs[0] = o->x_comp[j - 1]; xs[2] = o->x_comp[j + 1];
          qs[0] = QP(i, j - 1, k); qs[2] = QP(i, j + 1, k);
          if (P->radial_source && sc == 2) {
            if (sE) { xs[2] = o->x_stag[j + 1]; qs[2] = sb[i]; }
            else if (sW) { xs[0] = o->x_stag[j]; qs[0] = sb[i]; }
          }
          px[i] = oracle_limit(qs, xs, P->limiter[i], P->theta);
        }
        dq = rc * o->dx2 * px[i];
        qW[i] = qs[1] - dq;
        qE[i] = qs[1] + dq;
        if (j == 0) {
          if (sc == 2) qW[i] = sb[i];
          else if (bcW[i].flag == 0) qW[i] = bcW[i].value;
          else if (i == 1) qW[i] = dmin(qW[i], 0.0);
        }
        if (j == nx - 1) {
          if (sc == 2) qE[i] = sb[i];
          else if (bcE[i].flag == 0) qE[i] = bcE[i].value;
          else if (i == 1) qE[i] = dmax(qE[i], 0.0);
        }
      }
      if (ny > 1) {
        if (k == 0) {
          ys[0] = o->y_stag[0]; ys[2] = o->y_comp[k + 1];
          if (bcS[i].flag == 0) {
            qs[0] = bcS[i].value; qs[2] = QP(i, j, k + 1);
            py[i] = oracle_limit(qs, ys, P->limiter[i], P->theta);
          } else if (bcS[i].flag == 1) {
            py[i] = bcS[i].value;
          } else if (bcS[i].flag == 2) {
            py[i] = (QP(i, j, 1) - QP(i, j, 0)) * o->one_by_dy;
          }
        } else if (k == ny - 1) {
          ys[0] = o->y_comp[k - 1]; ys[2] = o->y_stag[o->niy - 1];
          if (bcN[i].flag == 0) {
            qs[0] = QP(i, j, k - 1); qs[2] = bcN[i].value;
            py[i] = oracle_limit(qs, ys, P->limiter[i], P->theta);
          } else if (bcN[i].flag == 1) {
            py[i] = bcN[i].value;
          } else if (bcN[i].flag == 2) {
            py[i] = (QP(i, j, ny - 1) - QP(i, j, ny - 2)) * o->one_by_dy;
          }
        } else {
          ys[0] = o->y_comp[k - 1]; ys[2] = o->y_comp[k + 1];
          qs[0] = QP(i, j, k - 1); qs[2] = QP(i, j, k + 1);
          if (P->radial_source && sc == 2) {
            if (sS) { ys[0] = o->y_stag[k]; qs[0] = sb[i]; }
            else if (sN) { ys[2] = o->y_stag[k + 1]; qs[2] = sb[i]; }
          }
          py[i] = oracle_limit(qs, ys, P->limiter[i], P->theta);
        }
        dq = rc * o->dy2 * py[i];
        qS[i] = qs[1] - dq;
        qN[i] = qs[1] + dq;
        if (k == 0) {
          if (bcS[i].flag == 0) qS[i] = bcS[i].value;
          else if (i == 2) qS[i] = dmin(qS[i], 0.0);
        }
        if (k == ny - 1) {
          if (bcN[i].flag == 0) qN[i] = bcN[i].value;
          else if (i == 2) qN[i] = dmax(qN[i], 0.0);
        }
      }
    }
    /* velocities u, v (add_vars_loop, solver_2d.f90:3487-3652) */
    for (int i = nv; i < nv + 2; ++i) {
      if (nx > 1) {
        qs[1] = QP(i, j, k);
        if (j == 0) {
          qp_to_qp2(qW, o->B_cent[c], qp2);
          qs[0] = qp2[i - nv + 1]; qs[2] = QP(i, j + 1, k);
        } else if (j == nx - 1) {
          qp_to_qp2(qE, o->B_cent[c], qp2);
          qs[0] = QP(i, j - 1, k); qs[2] = qp2[i - nv + 1];
        } else {
          qs[0] = QP(i, j - 1, k); qs[2] = QP(i, j + 1, k);
          if (P->radial_source && sc == 2) {
            if (sE) { xs[2] = o->x_stag[j + 1]; qs[2] = sb[i]; }
            else if (sW) { xs[0] = o->x_stag[j]; qs[0] = sb[i]; }
          }
        }
        px[i] = oracle_limit(qs, xs, P->limiter[i], P->theta);
        dq = rc * o->dx2 * px[i];
        qW[i] = qs[1] - dq;
        qE[i] = qs[1] + dq;
        if (j == 0) {
          qp_to_qp2(qW, o->B_cent[c], qp2);
          qW[i] = qp2[i - nv + 1];
        } else if (j == nx - 1) {
          qp_to_qp2(qE, o->B_cent[c], qp2);
          qE[i] = qp2[i - nv + 1];
        } else if (P->radial_source && sc == 2) {
          if (sE) for (int m = 0; m < np; ++m) qE[m] = sb[m];
          else if (sW) for (int m = 0; m < np; ++m) qW[m] = sb[m];
        }
      }
      if (ny > 1) {
        qs[1] = QP(i, j, k);
        if (k == 0) {
          qp_to_qp2(qS, o->B_cent[c], qp2);
          qs[0] = qp2[i - nv + 1]; qs[2] = QP(i, j, k + 1);
        } else if (k == ny - 1) {
          qp_to_qp2(qN, o->B_cent[c], qp2);
          qs[0] = QP(i, j, k - 1); qs[2] = qp2[i - nv + 1];
        } else {
          qs[0] = QP(i, j, k - 1); qs[2] = QP(i, j, k + 1);
          if (P->radial_source && sc == 2) {
            /* the reference writes x_stencil(3) here (solver_2d.f90:3605) */
            if (sS) { ys[0] = o->y_stag[k]; qs[0] = sb[i]; }
            else if (sN) { xs[2] = o->y_stag[k + 1]; qs[2] = sb[i]; }
          }
        }
        py[i] = oracle_limit(qs, ys, P->limiter[i], P->theta);
        dq = rc * o->dy2 * py[i];
        qS[i] = qs[1] - dq;
        qN[i] = qs[1] + dq;
        if (k == 0) {
          qp_to_qp2(qS, o->B_cent[c], qp2);
          qS[i] = qp2[i - nv + 1];
        } else if (k == ny - 1) {
          qp_to_qp2(qN, o->B_cent[c], qp2);
          qN[i] = qp2[i - nv + 1];
        } else if (P->radial_source && sc == 2) {
          if (sS) for (int m = 0; m < np; ++m) qS[m] = sb[m];
          else if (sN) for (int m = 0; m < np; ++m) qN[m] = sb[m];
        }
      }
    }
    /* interface values (solver_2d.f90:3658-3920) */
    if (nx > 1) {
      size_t fr = IDXX(j, k), fl = IDXX(j + 1, k);
      oracle_qp_to_qc_p(P, qW, &o->qR[fr * nv]);
      oracle_qp_to_qc_p(P, qE, &o->qL[fl * nv]);
      for (int m = 0; m < np; ++m) { o->qpR[fr * np + m] = qW[m]; o->qpL[fl * np + m] = qE[m]; }
      if (j == 0) {
        for (int m = 0; m < nv; ++m) o->qL[fr * nv + m] = o->qR[fr * nv + m];
        for (int m = 0; m < np; ++m) o->qpL[fr * np + m] = o->qpR[fr * np + m];
      } else if (j == nx - 1) {
        for (int m = 0; m < nv; ++m) o->qR[fl * nv + m] = o->qL[fl * nv + m];
        for (int m = 0; m < np; ++m) o->qpR[fl * np + m] = o->qpL[fl * np + m];
      } else if (P->radial_source && sc == 2) {
        if (sE) {
          for (int m = 0; m < nv; ++m) o->qR[fl * nv + m] = o->qL[fl * nv + m];
          o->qR[fl * nv + 1] = -o->qL[fl * nv + 1];
          for (int m = 0; m < np; ++m) o->qpR[fl * np + m] = o->qpL[fl * np + m];
          o->qpR[fl * np + nv] = -o->qpL[fl * np + nv];
        } else if (sW) {
          for (int m = 0; m < nv; ++m) o->qL[fr * nv + m] = o->qR[fr * nv + m];
          o->qL[fr * nv + 1] = -o->qR[fr * nv + 1];
          for (int m = 0; m < np; ++m) o->qpL[fr * np + m] = o->qpR[fr * np + m];
          o->qpL[fr * np + nv] = -o->qpR[fr * np + nv];
        }
      }
    } else {
      size_t fr = IDXX(j, k), fl = IDXX(j + 1, k);
      for (int m = 0; m < nv; ++m) { o->qR[fr * nv + m] = q_expl[c * nv + m]; o->qL[fl * nv + m] = q_expl[c * nv + m]; }
      for (int m = 0; m < np; ++m) { o->qpR[fr * np + m] = QP(m, j, k); o->qpL[fl * np + m] = QP(m, j, k); }
    }
    if (ny > 1) {
      size_t ft = IDXY(j, k), fb = IDXY(j, k + 1);
      oracle_qp_to_qc_p(P, qS, &o->qT[ft * nv]);
      oracle_qp_to_qc_p(P, qN, &o->qB[fb * nv]);
      for (int m = 0; m < np; ++m) { o->qpT[ft * np + m] = qS[m]; o->qpB[fb * np + m] = qN[m]; }
      if (k == 0) {
        for (int m = 0; m < nv; ++m) o->qB[ft * nv + m] = o->qT[ft * nv + m];
        for (int m = 0; m < np; ++m) o->qpB[ft * np + m] = o->qpT[ft * np + m];
      } else if (k == ny - 1) {
        for (int m = 0; m < nv; ++m) o->qT[fb * nv + m] = o->qB[fb * nv + m];
        for (int m = 0; m < np; ++m) o->qpT[fb * np + m] = o->qpB[fb * np + m];
      } else if (P->radial_source && sc == 2) {
        if (sS) {
          for (int m = 0; m < nv; ++m) o->qB[ft * nv + m] = o->qT[ft * nv + m];
          o->qB[ft * nv + 2] = -o->qT[ft * nv + 2];
          for (int m = 0; m < np; ++m) o->qpB[ft * np + m] = o->qpT[ft * np + m];
          o->qpB[ft * np + nv + 1] = -o->qpT[ft * np + nv + 1];
        } else if (sN) {
          for (int m = 0; m < nv; ++m) o->qT[fb * nv + m] = o->qB[fb * nv + m];
          o->qT[fb * nv + 2] = -o->qB[fb * nv + 2];
          for (int m = 0; m < np; ++m) o->qpT[fb * np + m] = o->qpB[fb * np + m];
          o->qpT[fb * np + nv + 1] = -o->qpB[fb * np + nv + 1];
        }
      }
    } else {
      size_t ft = IDXY(j, k), fb = IDXY(j, k + 1);
      for (int m = 0; m < nv; ++m) {
        o->qB[ft * nv + m] = o->qT[ft * nv + m] = q_expl[c * nv + m];
        o->qB[fb * nv + m] = o->qT[fb * nv + m] = q_expl[c * nv + m];
      }
      for (int m = 0; m < np; ++m) {
        o->qpB[ft * np + m] = o->qpT[ft * np + m] = QP(m, j, k);
        o->qpB[fb * np + m] = o->qpT[fb * np + m] = QP(m, j, k);
      }
    }
  }
#undef QP
}

/* solver_2d.f90:3937-4014 eval_speeds */
static void eval_speeds(oracle_t* o) {
  const phys_t* P = &o->P;
  const int np = P->nv + 2;
  if (o->nx > 1) {
#pragma omp parallel for schedule(static)
    for (int l = 0; l < o->solve_ix; ++l) {
      size_t f = IDXX(o->j_sx[l], o->k_sx[l]);
      double lmin, lmax, rmin, rmax;
      local_speeds(P, &o->qpL[f * np], o->gcsx[f], 1, &lmin, &lmax);
      local_speeds(P, &o->qpR[f * np], o->gcsx[f], 1, &rmin, &rmax);
      o->axN[f] = dmin(dmin(lmin, rmin), 0.0);
      o->axP[f] = dmax(dmax(lmax, rmax), 0.0);
    }
  }
  if (o->ny > 1) {
#pragma omp parallel for schedule(static)
    for (int l = 0; l < o->solve_iy; ++l) {
      size_t f = IDXY(o->j_sy[l], o->k_sy[l]);
      double bmin, bmax, tmin, tmax;
      local_speeds(P, &o->qpB[f * np], o->gcsy[f], 2, &bmin, &bmax);
      local_speeds(P, &o->qpT[f * np], o->gcsy[f], 2, &tmin, &tmax);
      o->ayN[f] = dmin(dmin(bmin, tmin), 0.0);
      o->ayP[f] = dmax(dmax(bmax, tmax), 0.0);
    }
  }
}

/* solver_2d.f90:2834-3002 eval_flux_KT + 3019-3049 average_KT; the
 * per-equation speeds are all equal (eval_local_speeds_x fills every
 * entry with the same value), so one pair per face is stored */
static void eval_flux_KT(oracle_t* o) {
  const phys_t* P = &o->P;
  const int nv = P->nv, np = nv + 2, ns = P->ns;
  if (o->nx > 1) {
#pragma omp parallel for schedule(static)
    for (int l = 0; l < o->solve_ix; ++l) {
      const int j = o->j_sx[l], k = o->k_sx[l];
      size_t f = IDXX(j, k);
      double fL[SFLOW_MAX_VARS], fR[SFLOW_MAX_VARS], *H = &o->Hx[f * nv];
      oracle_eval_fluxes_p(P, &o->qL[f * nv], &o->qpL[f * np], o->gcsx[f], 1, fL);
      oracle_eval_fluxes_p(P, &o->qR[f * nv], &o->qpR[f * np], o->gcsx[f], 1, fR);
      double a1 = o->axN[f], a2 = o->axP[f];
      for (int i = 0; i < nv; ++i) {
        double avg = (a1 == a2) ? 0.0 : (a2 * fL[i] - a1 * fR[i]) / (a2 - a1);
        if (a1 == a2) H[i] = 0.0;
        else H[i] = avg + (a2 * a1) / (a2 - a1) * (o->qR[f * nv + i] - o->qL[f * nv + i]);
      }
      if (ns > 0) {
        double s = 0.0;
        for (int i = 0; i < ns; ++i) s += H[4 + i] / H[0];
        if (sumv(H + 4, ns) / H[0] >= 1.0)
          for (int i = 0; i < ns; ++i) H[4 + i] = H[4 + i] / s;
      }
      if (o->qpL[f * np + 1] == 0.0 && o->qpR[f * np + 1] == 0.0) {
        H[0] = 0.0;
        for (int i = 3; i < nv; ++i) H[i] = 0.0;
      }
    }
  }
  if (o->ny > 1) {
#pragma omp parallel for schedule(static)
    for (int l = 0; l < o->solve_iy; ++l) {
      const int j = o->j_sy[l], k = o->k_sy[l];
      size_t f = IDXY(j, k);
      double fB[SFLOW_MAX_VARS], fT[SFLOW_MAX_VARS], *H = &o->Hy[f * nv];
      oracle_eval_fluxes_p(P, &o->qB[f * nv], &o->qpB[f * np], o->gcsy[f], 2, fB);
      oracle_eval_fluxes_p(P, &o->qT[f * nv], &o->qpT[f * np], o->gcsy[f], 2, fT);
      double a1 = o->ayN[f], a2 = o->ayP[f];
      for (int i = 0; i < nv; ++i) {
        double avg = (a1 == a2) ? 0.0 : (a2 * fB[i] - a1 * fT[i]) / (a2 - a1);
        if (a1 == a2) H[i] = 0.0;
        else H[i] = avg + (a2 * a1) / (a2 - a1) * (o->qT[f * nv + i] - o->qB[f * nv + i]);
      }
      if (ns > 0) {
        double s = sumv(H + 4, ns);
        if (s / H[0] > 1.0)
          for (int i = 0; i < ns; ++i) H[4 + i] = H[4 + i] / (s / H[0]);
      }
      if (o->qB[f * nv + 2] == 0.0 && o->qT[f * nv + 2] == 0.0) {
        H[0] = 0.0;
        for (int i = 3; i < nv; ++i) H[i] = 0.0;
      }
    }
  }
}

/* solver_2d.f90:2705-2821 eval_flux_UP */
static void eval_flux_UP(oracle_t* o) {
  const phys_t* P = &o->P;
  const int nv = P->nv, np = nv + 2;
  memset(o->Hx, 0, sizeof(double) * o->nix * o->ny * nv);
  memset(o->Hy, 0, sizeof(double) * o->nx * o->niy * nv);
  if (o->nx > 1) {
#pragma omp parallel for schedule(static)
    for (int l = 0; l < o->solve_ix; ++l) {
      size_t f = IDXX(o->j_sx[l], o->k_sx[l]);
      double fL[SFLOW_MAX_VARS], fR[SFLOW_MAX_VARS], *H = &o->Hx[f * nv];
      oracle_eval_fluxes_p(P, &o->qL[f * nv], &o->qpL[f * np], o->gcsx[f], 1, fL);
      oracle_eval_fluxes_p(P, &o->qR[f * nv], &o->qpR[f * np], o->gcsx[f], 1, fR);
      double uL = o->qpL[f * np + nv], uR = o->qpR[f * np + nv];
      for (int i = 0; i < nv; ++i) {
        if (uL > 0.0 && uR >= 0.0) H[i] = fL[i];
        else if (uL <= 0.0 && uR < 0.0) H[i] = fR[i];
        else H[i] = 0.5 * (fL[i] + fR[i]);
      }
      /* q_interfaceL(n_vars+1) is read past the conservative vector in the
       * reference (solver_2d.f90:2771); it aliases qp storage there and is
       * not reproducible, so that zero-velocity fix is left out */
    }
  }
  if (o->ny > 1) {
#pragma omp parallel for schedule(static)
    for (int l = 0; l < o->solve_iy; ++l) {
      size_t f = IDXY(o->j_sy[l], o->k_sy[l]);
      double fB[SFLOW_MAX_VARS], fT[SFLOW_MAX_VARS], *H = &o->Hy[f * nv];
      oracle_eval_fluxes_p(P, &o->qB[f * nv], &o->qpB[f * np], o->gcsy[f], 2, fB);
      oracle_eval_fluxes_p(P, &o->qT[f * nv], &o->qpT[f * np], o->gcsy[f], 2, fT);
      double vB = o->qB[f * nv + 2], vT = o->qT[f * nv + 2];
      for (int i = 0; i < nv; ++i) {
        if (vB > 0.0 && vT >= 0.0) H[i] = fB[i];
        else if (vB <= 0.0 && vT < 0.0) H[i] = fT[i];
        else H[i] = 0.5 * (fB[i] + fT[i]);
      }
      if (vB == 0.0 && vT == 0.0) {
        H[0] = 0.0;
        for (int i = 3; i < nv; ++i) H[i] = 0.0;
      }
    }
  }
}

/* solver_2d.f90:2616-2693 eval_hyperbolic_terms */
static void eval_hyperbolic_terms(oracle_t* o, const double* q_expl, const double* qp_expl,
                                  double* divF) {
  const int nv = o->P.nv;
  reconstruction(o, q_expl, qp_expl);
  eval_speeds(o);
  if (o->P.scheme == SFLOW_SCHEME_UP) eval_flux_UP(o);
  else eval_flux_KT(o);
#pragma omp parallel for schedule(static)
  for (int l = 0; l < o->solve_cells; ++l) {
    const int j = o->j_cent[l], k = o->k_cent[l];
    size_t c = IDX(j, k);
    for (int i = 0; i < nv; ++i) {
      double d = 0.0;
      if (o->nx > 1) d = d + (o->Hx[IDXX(j + 1, k) * nv + i] - o->Hx[IDXX(j, k) * nv + i]) * o->one_by_dx;
      if (o->ny > 1) d = d + (o->Hy[IDXY(j, k + 1) * nv + i] - o->Hy[IDXY(j, k) * nv + i]) * o->one_by_dy;
      divF[c * nv + i] = d;
    }
  }
}

/* dry state (qp = 0, T = T_ambient) */
static void dry_qp(const phys_t* P, double* qp) {
  for (int i = 0; i < P->nv + 2; ++i) qp[i] = 0.0;
  qp[3] = P->T_ambient;
}

/* solver_2d.f90:873-1006 timestep */
static double timestep(oracle_t* o) {
  const phys_t* P = &o->P;
  const int nv = P->nv, np = nv + 2;
  double dt = o->prm.max_dt;
  if (o->prm.cfl != -1.0) {
    /* D1: the reconstruction reads every inactive cell as dry */
    for (int i = 0; i < o->N; ++i)
      if (!o->mask[i]) dry_qp(P, &o->qp[(size_t)i * np]);
#pragma omp parallel for schedule(static)
    for (int l = 0; l < o->solve_cells; ++l) {
      size_t c = IDX(o->j_cent[l], o->k_cent[l]);
      if (o->q[c * nv] > 0.0) oracle_qc_to_qp_p(P, &o->q[c * nv], &o->qp[c * np], NULL);
      else dry_qp(P, &o->qp[c * np]);
    }
    reconstruction(o, o->q, o->qp);
    eval_speeds(o);
    for (int l = 0; l < o->solve_cells; ++l) {
      const int j = o->j_cent[l], k = o->k_cent[l];
      double dti_x, dti_y;
      double ma = dmax(dmax(o->axP[IDXX(j, k)], -o->axN[IDXX(j, k)]),
                       dmax(o->axP[IDXX(j + 1, k)], -o->axN[IDXX(j + 1, k)]));
      if (o->nx == 1) ma = 0.0;
      dti_x = (ma > 0.0) ? o->prm.cfl * o->dx / ma : dt;
      ma = dmax(dmax(o->ayP[IDXY(j, k)], -o->ayN[IDXY(j, k)]),
                dmax(o->ayP[IDXY(j, k + 1)], -o->ayN[IDXY(j, k + 1)]));
      if (o->ny == 1) ma = 0.0;
      dti_y = (ma > 0.0) ? o->prm.cfl * o->dy / ma : dt;
      dt = dmin(dt, dmin(dti_x, dti_y));
    }
  }
  return dt;
}

/* solver_2d.f90:1022-1634 imex_RK_solver */
static void imex_RK_solver(oracle_t* o) {
  const phys_t* P = &o->P;
  const int nv = P->nv, np = nv + 2, nrk = P->nrk, ns = P->ns;
  const double dt = o->dt;
  const size_t N = o->N;
  /* zero the stage arrays (every cell, see D1) */
  for (size_t c = 0; c < N; ++c)
    for (int r = 0; r < nrk; ++r) {
      size_t b = ((size_t)r * N + c);
      for (int i = 0; i < nv; ++i) {
        o->q_rk[b * nv + i] = 0.0; o->divFlux[b * nv + i] = 0.0; o->NH[b * nv + i] = 0.0;
        o->SI[b * nv + i] = 0.0; o->expl[b * nv + i] = 0.0;
      }
      dry_qp(P, &o->qp_rk[b * np]);
    }
  for (int l = 0; l < o->solve_cells; ++l) {
    size_t c = IDX(o->j_cent[l], o->k_cent[l]);
    for (int i = 0; i < nv; ++i) o->q0[c * nv + i] = o->q[c * nv + i];
  }
  for (int irk = 0; irk < nrk; ++irk) {
    double a_tilde[4] = {0, 0, 0, 0}, a_dirk[4] = {0, 0, 0, 0};
    for (int r = 0; r < irk; ++r) {
      a_tilde[r] = o->a_tilde_ij[irk * 4 + r];
      a_dirk[r] = o->a_dirk_ij[irk * 4 + r];
    }
    const double a_diag = o->a_dirk_ij[irk * 4 + irk];
    int iters_max = 0;
    int64_t iters_tot = 0;
    uint32_t st = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(max : iters_max) reduction(+ : iters_tot) reduction(| : st)
    for (int l = 0; l < o->solve_cells; ++l) {
      const int j = o->j_cent[l], k = o->k_cent[l];
      const size_t c = IDX(j, k);
      double q_guess[SFLOW_MAX_VARS], q_si[SFLOW_MAX_VARS], Rj[SFLOW_MAX_VARS];
      double qpc[MAXV];
      double* qfv = &o->q_fv[c * nv];
      const double* q0 = &o->q0[c * nv];
      if (irk == 0)
        for (int i = 0; i < nv; ++i) q_guess[i] = q0[i];
      for (int i = 0; i < nv; ++i) {
        double s1 = 0.0, s2 = 0.0;
        for (int r = 0; r <= irk; ++r) {
          size_t b = ((size_t)r * N + c) * nv + i;
          s1 += (o->divFlux[b] - o->expl[b]) * a_tilde[r];
          s2 += (o->NH[b] + o->SI[b]) * a_dirk[r];
        }
        qfv[i] = q0[i] - dt * (s1 - s2);
      }
      oracle_qc_to_qp_p(P, qfv, qpc, NULL);
      double* SIc = &o->SI[((size_t)irk * N + c) * nv];
      double* NHc = &o->NH[((size_t)irk * N + c) * nv];
      if (a_diag != 0.0) {
        if (qfv[0] > 0.0) {
          semi_impl_terms(P, o->Bx[c], o->By[c], o->Bxx[c], o->Bxy[c], o->Byy[c], o->gc[c], qpc, SIc);
          for (int i = 0; i < nv; ++i) q_si[i] = qfv[i] + dt * a_diag * SIc[i];
          if (sq(qfv[1]) + sq(qfv[2]) == 0.0) {
            q_si[1] = 0.0; q_si[2] = 0.0;
          } else if (q_si[1] * qfv[1] < 0.0 || q_si[2] * qfv[2] < 0.0) {
            q_si[1] = 0.0; q_si[2] = 0.0;
          } else {
            double m1 = sqrt(sq(q_si[1]) + sq(q_si[2])), m0 = sqrt(sq(qfv[1]) + sq(qfv[2]));
            q_si[1] = m1 * qfv[1] / m0;
            q_si[2] = m1 * qfv[2] / m0;
          }
          for (int i = 0; i < nv; ++i) SIc[i] = (q_si[i] - qfv[i]) / (dt * a_diag);
          for (int i = 0; i < nv; ++i) q_guess[i] = q_si[i];
          for (int i = 0; i < nv; ++i) {
            double s1 = 0.0, s2 = 0.0;
            for (int r = 0; r < irk; ++r) {
              size_t b = ((size_t)r * N + c) * nv + i;
              s1 += (o->divFlux[b] - o->expl[b]) * a_tilde[r];
              s2 += (o->NH[b] + o->SI[b]) * a_dirk[r];
            }
            Rj[i] = (s1 - s2) - a_diag * SIc[i];
          }
          newton_ctx nc = {P, dt, a_diag, o->Bx[c], o->By[c], q0, Rj};
          int it = solve_rk_step(&nc, q_guess);
          if (it > 100) st |= SFLOW_S_NEWTON_MAXIT;
          if (it > iters_max) iters_max = it;
          iters_tot += it;
          if (o->ny == 1) q_guess[2] = 0.0;
          if (o->nx == 1) q_guess[1] = 0.0;
          r_implicit_terms(P, o->Bx[c], o->By[c], q_guess, NHc);
          if (sq(q_si[1]) + sq(q_si[2]) == 0.0) {
            q_guess[1] = 0.0; q_guess[2] = 0.0;
          } else if (q_guess[1] * q_si[1] <= 0.0 && q_guess[2] * q_si[2] <= 0.0) {
            q_guess[1] = 0.0; q_guess[2] = 0.0;
          } else {
            double m1 = sqrt(sq(q_guess[1]) + sq(q_guess[2])), m0 = sqrt(sq(q_si[1]) + sq(q_si[2]));
            q_guess[1] = m1 * q_si[1] / m0;
            q_guess[2] = m1 * q_si[2] / m0;
          }
        } else {
          for (int i = 0; i < nv; ++i) { q_guess[i] = qfv[i]; q_si[i] = qfv[i]; SIc[i] = 0.0; NHc[i] = 0.0; }
        }
      }
      if (a_diag != 0.0)
        for (int i = 0; i < nv; ++i) NHc[i] = (q_guess[i] - q_si[i]) / (dt * a_diag);
      double* qrk = &o->q_rk[((size_t)irk * N + c) * nv];
      for (int i = 0; i < nv; ++i) qrk[i] = q_guess[i];
      if (o->omega_tilde[irk] > 0.0) {
        double* qprk = &o->qp_rk[((size_t)irk * N + c) * np];
        if (qrk[0] > 0.0) oracle_qc_to_qp_p(P, qrk, qprk, NULL);
        else dry_qp(P, qprk);
        expl_terms(P, o->Bx[c], o->By[c], o->Bxx[c], o->Bxy[c], o->Byy[c], o->gc[c], o->dgcx[c],
                   o->dgcy[c], qprk, o->t, o->cell_fract[c], o->arc_perim[c], o->arc_nx[c], o->arc_ny[c],
                   o->dx * o->dy, &o->expl[((size_t)irk * N + c) * nv]);
      }
    }
    if (iters_max > o->max_newton_iter_seen) o->max_newton_iter_seen = iters_max;
    o->newton_iters_total += iters_tot;
    o->status |= st;
    if (o->omega_tilde[irk] > 0.0)
      eval_hyperbolic_terms(o, &o->q_rk[(size_t)irk * N * nv], &o->qp_rk[(size_t)irk * N * np],
                            &o->divFlux[(size_t)irk * N * nv]);
  }
  /* assemble_sol (solver_2d.f90:1342-1630) */
  double d1 = 0.0, d2 = 0.0;
  for (int r = 0; r < nrk; ++r) {
    d1 += fabs(o->omega_tilde[r] - o->a_tilde_ij[(nrk - 1) * 4 + r]);
    d2 += fabs(o->omega[r] - o->a_dirk_ij[(nrk - 1) * 4 + r]);
  }
  const int take_last = (d1 == 0.0 && d2 == 0.0);
  uint32_t st = 0;
#pragma omp parallel for schedule(static) reduction(| : st)
  for (int l = 0; l < o->solve_cells; ++l) {
    const size_t c = IDX(o->j_cent[l], o->k_cent[l]);
    double* q = &o->q[c * nv];
    const double* q0 = &o->q0[c * nv];
    double res[SFLOW_MAX_VARS];
    for (int i = 0; i < nv; ++i) {
      double s1 = 0.0, s2 = 0.0;
      for (int r = 0; r < nrk; ++r) {
        size_t b = ((size_t)r * N + c) * nv + i;
        s1 += (o->divFlux[b] - o->expl[b]) * o->omega_tilde[r];
        s2 += (o->NH[b] + o->SI[b]) * o->omega[r];
      }
      res[i] = s1 - s2;
    }
    if (take_last)
      for (int i = 0; i < nv; ++i) q[i] = o->q_rk[((size_t)(nrk - 1) * N + c) * nv + i];
    else
      for (int i = 0; i < nv; ++i) q[i] = q0[i] - dt * res[i];
    for (int i = 0; i < nv; ++i)
      if (isnan(q[i])) st |= SFLOW_S_NAN;
    if (q[0] < EPS) {
      if (q[0] > -1.0e-7) {
        for (int i = 0; i < nv; ++i) q[i] = 0.0;
      } else {
        st |= SFLOW_S_NEG_H;
      }
    }
    int anyneg = 0, anybad = 0;
    for (int i = 0; i < ns; ++i) {
      if (q[4 + i] < 0.0) anyneg = 1;
      if (q[4 + i] <= -1.0e-7) anybad = 1;
    }
    if (anyneg) {
      if (anybad) st |= SFLOW_S_NEG_ALPHA;
      else
        for (int i = 0; i < ns; ++i)
          if (q[4 + i] > -1.0e-7) q[4 + i] = 0.0;
    }
    double qpc[MAXV];
    oracle_qc_to_qp_p(P, q, qpc, NULL);
    if (qpc[3] < 273.0) st |= SFLOW_S_LOW_T;
    double ssum = sumv(q + 4, ns);
    if (ns > 0 && ssum > q[0]) {
      if ((ssum - q[0]) / q[0] < 1.0e-10 || q[0] < EPS) {
        double s = sumv(q + 4, ns);
        for (int i = 0; i < ns; ++i) q[4 + i] = q[4 + i] / s * q[0];
      } else {
        st |= SFLOW_S_SOLID_GT_MASS;
        double s = sumv(q + 4, ns);
        for (int i = 0; i < ns; ++i) q[4 + i] = q[4 + i] / s * q[0];
      }
    }
    /* solver_2d.f90:1626 */
    if (o->nodata[c])
      for (int i = 0; i < nv; ++i) q[i] = 0.0;
  }
  o->status |= st;
}

/* solver_2d.f90:2382-2597 update_erosion_deposition_cell */
static void update_erosion_deposition(oracle_t* o) {
  const phys_t* P = &o->P;
  const int nv = P->nv, np = nv + 2, ns = P->ns;
  const double dt = o->dt;
  if (P->erosion_coeff == 0.0 && !P->settling && !P->entrain) return;
  uint32_t st = 0;
#pragma omp parallel for schedule(static) reduction(| : st)
  for (int l = 0; l < o->solve_cells; ++l) {
    const size_t c = IDX(o->j_cent[l], o->k_cent[l]);
    double* q = &o->q[c * nv];
    double* qp = &o->qp[c * np];
    double dep[MAXS], ers[MAXS], eqn[SFLOW_MAX_VARS], topo, erod[MAXS];
    if (q[0] > 0.0) oracle_qc_to_qp_p(P, q, qp, NULL);
    else dry_qp(P, qp);
    for (int i = 0; i < ns; ++i) erod[i] = o->erodible[c * MAXS + i];
    mass_exchange(P, qp, o->Bx[c], o->By[c], erod, dt, dep, ers, eqn, &topo);
    if (P->bottom_source) {
      const double out_of_source_fraction = 1.0 - o->cell_fract[c];
      for (int i = 0; i < ns; ++i) dep[i] = dep[i] * out_of_source_fraction;
      for (int i = 0; i < ns; ++i) ers[i] = ers[i] * out_of_source_fraction;
      for (int i = 0; i < nv; ++i) eqn[i] = eqn[i] * out_of_source_fraction;
      topo = topo * out_of_source_fraction;
    }
    for (int i = 0; i < nv; ++i) q[i] = q[i] + dt * eqn[i];
    for (int i = 0; i < ns; ++i) q[4 + i] = dmax(0.0, q[4 + i]);
    for (int i = 0; i < ns; ++i) o->deposit[c * MAXS + i] += dt * dep[i];
    for (int i = 0; i < ns; ++i) o->erosion[c * MAXS + i] += dt * ers[i];
    for (int i = 0; i < ns; ++i) o->erodible[c * MAXS + i] = o->erodible[c * MAXS + i] - dt * ers[i];
    if (P->erodible_deposit)
      for (int i = 0; i < ns; ++i) o->erodible[c * MAXS + i] = o->erodible[c * MAXS + i] + dt * dep[i];
    if (P->topo_change) o->B_cent[c] = o->B_cent[c] + dt * topo;
    if (q[0] <= 0.0) {
      if (q[0] > -1.0e-10) {
        for (int i = 0; i < nv; ++i) q[i] = 0.0;
      } else {
        st |= SFLOW_S_EROSION;
      }
    }
    double ssum = sumv(q + 4, ns);
    if (ns > 0 && ssum > q[0]) {
      if (q[0] < 1.0e-10) {
        double s = sumv(q + 4, ns);
        for (int i = 0; i < ns; ++i) q[4 + i] = q[4 + i] / s * q[0];
      } else {
        st |= SFLOW_S_EROSION;
      }
    }
    double red_grav;
    if (q[0] > 0.0) {
      oracle_qc_to_qp_p(P, q, qp, NULL);
      mixt_t m;
      mixt_var(P, qp, 0, &m);
      red_grav = m.red_grav;
    } else {
      dry_qp(P, qp);
      red_grav = 0.0;
    }
    if (red_grav <= 0.0)
      for (int i = 0; i < nv; ++i) q[i] = 0.0;
  }
  o->status |= st;
}

/* IMEX_SfloW2D.f90:339-353, 477-491: entry it*n_dyn + id of the table is
 * h >= thickness level it and p_dyn >= dynamic-pressure level id */
static void vuln_cell(oracle_t* o, size_t c, double h, double p_dyn, int accumulate) {
  const phys_t* P = &o->P;
  const int ne = P->n_thk * P->n_dyn;
  unsigned char* v = &o->vuln[c * SFLOW_MAX_LEVELS * SFLOW_MAX_LEVELS];
  int e = 0;
  for (int it = 0; it < P->n_thk; ++it) {
    int thck = h >= P->thk_levels[it];
    for (int id = 0; id < P->n_dyn; ++id, ++e) {
      int pdyn = p_dyn >= P->dyn_levels[id];
      v[e] = accumulate ? (v[e] || (thck && pdyn)) : (thck && pdyn);
    }
  }
  (void)ne;
}

/* IMEX_SfloW2D.f90:449-505 post-step qc_to_qp and maxima */
static void post_step(oracle_t* o) {
  const phys_t* P = &o->P;
  const int nv = P->nv, np = nv + 2;
#pragma omp parallel for schedule(static)
  for (int l = 0; l < o->solve_cells; ++l) {
    const size_t c = IDX(o->j_cent[l], o->k_cent[l]);
    double* qp = &o->qp[c * np];
    if (o->q[c * nv] > 0.0) {
      double p_dyn;
      oracle_qc_to_qp_p(P, &o->q[c * nv], qp, &p_dyn);
      o->hmax[c] = dmax(o->hmax[c], qp[0]);
      double mv = sqrt(sq(qp[nv]) + sq(qp[nv + 1]));
      if (qp[0] > 0.001) {
        o->pdynmax[c] = dmax(o->pdynmax[c], p_dyn);
        o->mod_vel_max[c] = dmax(o->mod_vel_max[c], mv);
      }
      if (P->n_thk * P->n_dyn > 0) vuln_cell(o, c, qp[0], p_dyn, 1);
    } else {
      dry_qp(P, qp);
    }
  }
}

/* ------------------------------------------------------------------------ */
/* public oracle API                                                         */
/* ------------------------------------------------------------------------ */
static int setup_phys(oracle_t* o, const SflowParams* p) {
  phys_t* P = &o->P;
  memset(P, 0, sizeof(*P));
  P->ns = p->n_solid;
  P->nv = 4 + p->n_solid;
  P->nrk = p->n_rk;
  P->gas = p->gas_flag; P->liquid = p->liquid_flag; P->energy = p->energy_flag;
  P->alpha = p->alpha_flag; P->rheo = p->rheology_flag; P->rheo_model = p->rheology_model;
  P->slope_corr = p->slope_correction_flag; P->curv = p->curvature_term_flag;
  P->settling = p->settling_flag; P->entrain = p->entrainment_flag;
  P->collective = p->collective_settling_flag; P->radial_source = p->radial_source_flag;
  P->scheme = p->solver_scheme;
  P->grav = p->grav; P->mu = p->mu; P->xi = p->xi; P->friction_factor = p->friction_factor;
  P->mu_s = p->mu_s; P->mu_2 = p->mu_2; P->I_0 = p->I_0; P->muI_inf = p->muI_inf;
  P->pres = p->pres; P->inv_pres = 1.0 / p->pres;
  P->sp_heat_a = p->sp_heat_a; P->sp_gas_const_a = p->sp_gas_const_a; P->T_ambient = p->T_ambient;
  P->rho_a_amb = p->pres / (p->sp_gas_const_a * p->T_ambient);
  P->rho_l = p->rho_l; P->inv_rho_l = (p->rho_l != 0.0) ? 1.0 / p->rho_l : 0.0;
  P->sp_heat_l = p->sp_heat_l; P->loss_rate = p->loss_rate;
  P->kin_visc_c = p->gas_flag ? p->kin_visc_a : p->kin_visc_l;
  for (int i = 0; i < P->ns; ++i) {
    P->rho_s[i] = p->rho_s[i]; P->inv_rho_s[i] = 1.0 / p->rho_s[i];
    P->diam_s[i] = p->diam_s[i]; P->sp_heat_s[i] = p->sp_heat_s[i];
    P->alphas_source[i] = p->alphas_source[i];
  }
  P->alphastot_min = p->alphastot_min; P->max_packing = p->maximum_solid_packing;
  P->A_drag = p->A_drag; P->B_drag = p->B_drag;
  /* SOLID_TRANSPORT_PARAMETERS checks (inpout_2d.f90:1818-1990) */
  P->erosion_coeff = p->erosion_coeff;
  if (p->erosion_coeff < 0.0) return -1;
  if (p->erosion_coeff == 0.0) {
    P->erodible_porosity = 0.0;
    for (int i = 0; i < P->ns; ++i) P->erodible_fract[i] = 1.0 / P->ns;
    P->T_erodible = 300.0;
    P->coeff_porosity = 0.0;
    P->erodible_init = 0.0;
  } else {
    if (p->erodible_porosity < 0.0 || p->erodible_porosity > 1.0) return -1;
    P->erodible_porosity = p->erodible_porosity;
    P->coeff_porosity = p->erodible_porosity / (1.0 - p->erodible_porosity);
    if (P->ns == 1) {
      P->erodible_fract[0] = 1.0;
    } else {
      for (int i = 0; i < P->ns; ++i) {
        if (p->erodible_fract[i] < 0.0) return -1;
        P->erodible_fract[i] = p->erodible_fract[i];
      }
      double sum = sumv(P->erodible_fract, P->ns);
      if (sum != 1.0)
        for (int i = 0; i < P->ns; ++i) P->erodible_fract[i] = P->erodible_fract[i] / sum;
    }
    if (p->T_erodible < 0.0) return -1;
    P->T_erodible = p->T_erodible;
    P->erodible_init = p->initial_erodible_thickness >= 0.0 ? p->initial_erodible_thickness : 0.0;
  }
  P->rho_c_sub = p->gas_flag ? p->pres / (p->sp_gas_const_a * P->T_erodible) : p->rho_l;
  P->erodible_deposit = p->erodible_deposit_flag;
  P->topo_change = p->topo_change_flag;
  P->exchange = p->erosion_coeff != 0.0 || p->settling_flag || p->entrainment_flag;
  /* bottom radial source */
  P->bottom_source = p->bottom_radial_source_flag;
  P->n_intervals = p->n_intervals;
  for (int i = 0; i < p->n_intervals && i < SFLOW_MAX_INTERVALS; ++i) {
    P->t_intervals[i] = p->t_intervals[i];
    P->vel_intervals[i] = p->vel_intervals[i];
  }
  P->angle_source = p->angle_source;
  /* VULNERABILITY_TABLE_PARAMETERS (inpout_2d.f90:3808-3866) */
  P->n_thk = 0; P->n_dyn = 0;
  for (int i = 0; i < SFLOW_MAX_LEVELS; ++i) {
    if (p->thickness_levels[i] >= 0.0) P->n_thk++;
    if (p->dyn_pres_levels[i] >= 0.0) P->n_dyn++;
  }
  for (int i = 0; i < P->n_thk; ++i) P->thk_levels[i] = p->thickness_levels[i];
  for (int i = 0; i < P->n_dyn; ++i) P->dyn_levels[i] = p->dyn_pres_levels[i];
  if (P->n_thk > 0 && P->n_dyn <= 0) { P->n_dyn = 1; P->dyn_levels[0] = 0.0; }
  if (P->n_dyn > 0 && P->n_thk <= 0) { P->n_thk = 1; P->thk_levels[0] = 0.0; }
  P->theta = p->theta; P->reconstr_coeff = p->reconstr_coeff;
  for (int i = 0; i < P->nv; ++i) P->limiter[i] = p->limiter[i];
  P->limiter[P->nv] = p->limiter[1];
  P->limiter[P->nv + 1] = p->limiter[2];
  P->x_source = p->x_source; P->y_source = p->y_source; P->r_source = p->r_source;
  P->r2_source = p->r2_source; P->vel_source = p->vel_source; P->T_source = p->T_source;
  P->h_source = p->h_source;
  for (int i = 0; i < 4; ++i) P->time_param[i] = p->time_param[i];
  P->pi_g = 4.0 * atan(1.0);
  return 0;
}

static void set_tableau(oracle_t* o) {
  memset(o->a_tilde_ij, 0, sizeof(o->a_tilde_ij));
  memset(o->a_dirk_ij, 0, sizeof(o->a_dirk_ij));
  memset(o->omega_tilde, 0, sizeof(o->omega_tilde));
  memset(o->omega, 0, sizeof(o->omega));
#define AT(i, j) o->a_tilde_ij[((i)-1) * 4 + (j)-1]
#define AD(i, j) o->a_dirk_ij[((i)-1) * 4 + (j)-1]
  switch (o->P.nrk) {
    case 1: AT(1, 1) = 1.0; o->omega_tilde[0] = 1.0; break;
    case 2:
      AT(2, 1) = 1.0; o->omega_tilde[0] = 1.0; AD(2, 2) = 1.0; o->omega[1] = 1.0; break;
    case 3:
      AT(2, 1) = 0.5; AT(3, 1) = 0.5; AT(3, 2) = 0.5;
      o->omega_tilde[0] = o->omega_tilde[1] = o->omega_tilde[2] = 1.0 / 3.0;
      AD(1, 1) = 0.25; AD(2, 2) = 0.25; AD(3, 1) = 1.0 / 3.0; AD(3, 2) = 1.0 / 3.0; AD(3, 3) = 1.0 / 3.0;
      o->omega[0] = o->omega[1] = o->omega[2] = 1.0 / 3.0;
      break;
    case 4:
      AT(2, 1) = 0.5; AT(3, 1) = 1.0 / 3.0; AT(4, 2) = 1.0;
      o->omega_tilde[1] = 1.0;
      AD(2, 2) = 0.5; AD(3, 3) = 1.0 / 3.0; AD(4, 3) = 0.75; AD(4, 4) = 0.25;
      o->omega[2] = 0.75; o->omega[3] = 0.25;
      break;
  }
#undef AT
#undef AD
}

oracle_t* sflow_oracle_create(const SflowParams* p, const double* B_cent) {
  if (p->n_solid < 0 || p->n_solid > MAXS || p->n_rk < 1 || p->n_rk > 4) return NULL;
  if (p->comp_cells_x < 5) return NULL;
  if (p->comp_cells_y < 5 && p->comp_cells_y != 1) return NULL;
  oracle_t* o = calloc(1, sizeof(oracle_t));
  o->prm = *p;
  if (setup_phys(o, p) != 0) {
    free(o);
    return NULL;
  }
  const int nx = p->comp_cells_x, ny = p->comp_cells_y;
  o->nx = nx; o->ny = ny; o->N = nx * ny; o->nix = nx + 1; o->niy = ny + 1;
  o->dx = nx > 1 ? p->cell_size : 1.0;
  o->dy = ny > 1 ? p->cell_size : 1.0;
  o->dx2 = o->dx / 2.0; o->dy2 = o->dy / 2.0;
  o->one_by_dx = 1.0 / o->dx; o->one_by_dy = 1.0 / o->dy;
  o->P.eps_sing = dmin(dmin(pow(o->dx, 4.0), pow(o->dy, 4.0)), 1.0e-10);
  o->P.eps_sing4 = pow(o->P.eps_sing, 4);
  const size_t N = o->N, NX = (size_t)o->nix * ny, NY = (size_t)nx * o->niy;
  const int nv = o->P.nv, np = nv + 2, nrk = o->P.nrk;
  o->x_comp = xcalloc(nx, 8); o->x_stag = xcalloc(nx + 1, 8);
  o->y_comp = xcalloc(ny, 8); o->y_stag = xcalloc(ny + 1, 8);
  for (int j = 0; j <= nx; ++j) o->x_stag[j] = p->x0 + j * o->dx;
  for (int k = 0; k <= ny; ++k) o->y_stag[k] = p->y0 + k * o->dy;
  for (int j = 0; j < nx; ++j) o->x_comp[j] = 0.5 * (o->x_stag[j] + o->x_stag[j + 1]);
  for (int k = 0; k < ny; ++k) o->y_comp[k] = 0.5 * (o->y_stag[k] + o->y_stag[k + 1]);
  double** geo[] = {&o->B_cent, &o->Bx, &o->By, &o->Bxx, &o->Bxy, &o->Byy, &o->gc, &o->dgcx, &o->dgcy,
                    &o->arc_perim, &o->arc_nx, &o->arc_ny, &o->hmax, &o->pdynmax, &o->mod_vel_max};
  for (size_t i = 0; i < sizeof(geo) / sizeof(geo[0]); ++i) *geo[i] = xcalloc(N, 8);
  o->gcsx = xcalloc(NX, 8); o->gcsy = xcalloc(NY, 8);
  o->deposit = xcalloc(N * MAXS, 8);
  o->erosion = xcalloc(N * MAXS, 8);
  o->erodible = xcalloc(N * MAXS, 8);
  o->erodible_thk = xcalloc(N, 8);
  o->B_init = xcalloc(N, 8);
  o->cell_fract = xcalloc(N, 8);
  o->nodata = xcalloc(N, 1);
  o->vuln = xcalloc(N * SFLOW_MAX_LEVELS * SFLOW_MAX_LEVELS, 1);
  o->source_cell = xcalloc(N, sizeof(int));
  o->srcE = xcalloc(N, 1); o->srcW = xcalloc(N, 1); o->srcN = xcalloc(N, 1); o->srcS = xcalloc(N, 1);
  for (size_t i = 0; i < N; ++i) o->B_cent[i] = B_cent ? B_cent[i] : 0.0;
  memcpy(o->B_init, o->B_cent, sizeof(double) * N);
  o->q = xcalloc(N * nv, 8); o->q0 = xcalloc(N * nv, 8); o->q_fv = xcalloc(N * nv, 8);
  o->qp = xcalloc(N * np, 8);
  for (size_t i = 0; i < N; ++i) o->qp[i * np + 3] = o->P.T_ambient;
  o->q_rk = xcalloc(N * nv * nrk, 8); o->qp_rk = xcalloc(N * np * nrk, 8);
  o->divFlux = xcalloc(N * nv * nrk, 8); o->NH = xcalloc(N * nv * nrk, 8);
  o->SI = xcalloc(N * nv * nrk, 8); o->expl = xcalloc(N * nv * nrk, 8);
  o->qL = xcalloc(NX * nv, 8); o->qR = xcalloc(NX * nv, 8);
  o->qpL = xcalloc(NX * np, 8); o->qpR = xcalloc(NX * np, 8);
  o->qB = xcalloc(NY * nv, 8); o->qT = xcalloc(NY * nv, 8);
  o->qpB = xcalloc(NY * np, 8); o->qpT = xcalloc(NY * np, 8);
  o->axN = xcalloc(NX, 8); o->axP = xcalloc(NX, 8); o->ayN = xcalloc(NY, 8); o->ayP = xcalloc(NY, 8);
  o->Hx = xcalloc(NX * nv, 8); o->Hy = xcalloc(NY * nv, 8);
  o->mask = xcalloc(N, 1); o->mask_tmp = xcalloc(N, 1);
  o->mask_x = xcalloc(NX, 1); o->mask_y = xcalloc(NY, 1);
  o->j_cent = xcalloc(N, sizeof(int)); o->k_cent = xcalloc(N, sizeof(int));
  o->j_sx = xcalloc(NX, sizeof(int)); o->k_sx = xcalloc(NX, sizeof(int));
  o->j_sy = xcalloc(NY, sizeof(int)); o->k_sy = xcalloc(NY, sizeof(int));
  set_tableau(o);
  topography_reconstruction(o);
  derive_source(o);
  if (o->P.radial_source) init_source(o);
  if (o->P.bottom_source) compute_cell_fract(o);
  o->t = p->t_start;
  o->dt = o->dt_old = o->dt_old_old = p->dt0;
  o->t_output = p->t_start + p->dt_output;
  return o;
}

void sflow_oracle_destroy(oracle_t* o) {
  if (!o) return;
  void* ptrs[] = {o->x_comp, o->x_stag, o->y_comp, o->y_stag, o->B_cent, o->Bx, o->By, o->Bxx,
                  o->Bxy, o->Byy, o->gc, o->dgcx, o->dgcy, o->gcsx, o->gcsy, o->source_cell,
                  o->srcE, o->srcW, o->srcN, o->srcS, o->arc_perim, o->arc_nx, o->arc_ny, o->q,
                  o->q0, o->qp, o->q_fv, o->q_rk, o->qp_rk, o->divFlux, o->NH, o->SI, o->expl,
                  o->qL, o->qR, o->qB, o->qT, o->qpL, o->qpR, o->qpB, o->qpT, o->axN, o->axP,
                  o->ayN, o->ayP, o->Hx, o->Hy, o->mask, o->mask_tmp, o->mask_x, o->mask_y,
                  o->j_cent, o->k_cent, o->j_sx, o->k_sx, o->j_sy, o->k_sy, o->hmax, o->pdynmax,
                  o->mod_vel_max, o->deposit, o->erosion, o->erodible, o->erodible_thk, o->B_init,
                  o->cell_fract, o->nodata, o->vuln};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
  free(o);
}

/* IMEX_SfloW2D.f90:263-368: init check_solve(.TRUE.), initial qp and maxima */
/* Replace the conserved variables in place, keeping the time, dt history
 * and every map (test hook: perturbs a running state, e.g. rounds it to
 * FP32 to measure how the run responds to rounding of the state). */
void sflow_oracle_replace_q(oracle_t* o, const double* q) {
  memcpy(o->q, q, sizeof(double) * o->N * o->P.nv);
}

int sflow_oracle_set_q(oracle_t* o, const double* q) {
  const int nv = o->P.nv, np = nv + 2;
  memcpy(o->q, q, sizeof(double) * o->N * nv);
  o->t = o->prm.t_start;
  o->dt = o->dt_old = o->dt_old_old = o->prm.dt0;
  o->t_output = o->prm.t_start + o->prm.dt_output;
  o->status = 0;
  o->steps = 0;
  /* a new run: deposit, erosion and the erodible layer as initialised
   * (inpout_2d.f90:1983-1986), the topography as given */
  const int ns = o->P.ns;
  for (size_t c = 0; c < (size_t)o->N; ++c)
    for (int i = 0; i < ns; ++i) {
      o->deposit[c * MAXS + i] = 0.0;
      o->erosion[c * MAXS + i] = 0.0;
      o->erodible[c * MAXS + i] = o->P.erodible_fract[i] * (1.0 - o->P.erodible_porosity) *
                                  (o->have_erodible_thk ? o->erodible_thk[c] : o->P.erodible_init);
    }
  if (memcmp(o->B_cent, o->B_init, sizeof(double) * o->N) != 0) {
    memcpy(o->B_cent, o->B_init, sizeof(double) * o->N);
    topography_reconstruction(o);
  }
  memset(o->vuln, 0, (size_t)o->N * SFLOW_MAX_LEVELS * SFLOW_MAX_LEVELS);
  check_solve(o, 1);
  for (int i = 0; i < o->N; ++i) { o->hmax[i] = 0.0; o->pdynmax[i] = 0.0; o->mod_vel_max[i] = 0.0; }
  for (int l = 0; l < o->solve_cells; ++l) {
    const size_t c = IDX(o->j_cent[l], o->k_cent[l]);
    double* qp = &o->qp[c * np];
    if (o->q[c * nv] > 0.0) {
      double p_dyn;
      oracle_qc_to_qp_p(&o->P, &o->q[c * nv], qp, &p_dyn);
      o->hmax[c] = qp[0];
      double mv = sqrt(sq(qp[nv]) + sq(qp[nv + 1]));
      if (qp[0] > 0.001) { o->pdynmax[c] = p_dyn; o->mod_vel_max[c] = mv; }
      if (o->P.n_thk * o->P.n_dyn > 0) vuln_cell(o, c, qp[0], p_dyn, 0);
    } else {
      for (int i = 0; i < nv; ++i) qp[i] = 0.0;
      qp[3] = o->P.T_ambient;
    }
  }
  return 0;
}

/* One iteration of the driver loop, IMEX_SfloW2D.f90:395-505 */
int sflow_oracle_step(oracle_t* o) {
  const double t_end = o->prm.t_end;
  if (!(o->t < t_end)) return 0;
  check_solve(o, 0);
  o->dt = timestep(o);
  if (t_end - o->t_output < 1.0e-7) o->t_output = t_end;
  if (o->t + o->dt > t_end) o->dt = t_end - o->t;
  if (o->t + o->dt > o->t_output) o->dt = o->t_output - o->t;
  o->dt = dmin(o->dt, 1.1 * 0.5 * (o->dt_old + o->dt_old_old));
  o->dt_old_old = o->dt_old;
  o->dt_old = o->dt;
  imex_RK_solver(o);
  update_erosion_deposition(o);
  if (o->P.topo_change) topography_reconstruction(o);
  o->t = o->t + o->dt;
  post_step(o);
  o->steps++;
  return (int)o->status;
}

int sflow_oracle_run(oracle_t* o, double t_stop, int64_t max_steps, int64_t* cells_done) {
  int64_t n = 0, cells = 0;
  while (o->t < o->prm.t_end && o->t < t_stop && n < max_steps) {
    sflow_oracle_step(o);
    cells += o->solve_cells;
    ++n;
  }
  if (cells_done) *cells_done = cells;
  return (int)n;
}

void sflow_oracle_get_q(const oracle_t* o, double* q) { memcpy(q, o->q, sizeof(double) * o->N * o->P.nv); }
void sflow_oracle_get_qp(const oracle_t* o, double* qp) {
  memcpy(qp, o->qp, sizeof(double) * o->N * (o->P.nv + 2));
}
void sflow_oracle_get_maps(const oracle_t* o, double* hmax, double* pdynmax, double* mvmax) {
  memcpy(hmax, o->hmax, sizeof(double) * o->N);
  memcpy(pdynmax, o->pdynmax, sizeof(double) * o->N);
  memcpy(mvmax, o->mod_vel_max, sizeof(double) * o->N);
}
void sflow_oracle_get_mask(const oracle_t* o, unsigned char* m) { memcpy(m, o->mask, o->N); }
/* deposit(1:nx,1:ny,1:n_solid), column-major (class slowest) */
void sflow_oracle_get_deposit(const oracle_t* o, double* out) {
  for (int i = 0; i < o->P.ns; ++i)
    for (size_t c = 0; c < (size_t)o->N; ++c) out[(size_t)i * o->N + c] = o->deposit[c * MAXS + i];
}

/* erosion (which 0) or erodible (1), class slowest */
void sflow_oracle_get_erosion(const oracle_t* o, int which, double* out) {
  const double* src = which == 0 ? o->erosion : o->erodible;
  for (int i = 0; i < o->P.ns; ++i)
    for (size_t c = 0; c < (size_t)o->N; ++c) out[(size_t)i * o->N + c] = src[c * MAXS + i];
}
void sflow_oracle_get_topography(const oracle_t* o, double* out) { memcpy(out, o->B_cent, sizeof(double) * o->N); }
void sflow_oracle_get_cell_fract(const oracle_t* o, double* out) {
  memcpy(out, o->cell_fract, sizeof(double) * o->N);
}
/* the erodible layer thickness per cell (erodible_init); used from the next
 * sflow_oracle_set_q */
void sflow_oracle_set_erodible(oracle_t* o, const double* thk) {
  memcpy(o->erodible_thk, thk, sizeof(double) * o->N);
  o->have_erodible_thk = 1;
}
void sflow_oracle_set_nodata(oracle_t* o, const unsigned char* nodata) {
  for (int i = 0; i < o->N; ++i) o->nodata[i] = nodata ? (nodata[i] != 0) : 0;
}
void sflow_oracle_vuln_size(const oracle_t* o, int* n_thk, int* n_dyn) {
  *n_thk = o->P.n_thk;
  *n_dyn = o->P.n_dyn;
}
/* n_thk*n_dyn planes of nx*ny bytes */
void sflow_oracle_get_vuln(const oracle_t* o, unsigned char* out) {
  const int ne = o->P.n_thk * o->P.n_dyn;
  for (int e = 0; e < ne; ++e)
    for (size_t c = 0; c < (size_t)o->N; ++c)
      out[(size_t)e * o->N + c] = o->vuln[c * SFLOW_MAX_LEVELS * SFLOW_MAX_LEVELS + e];
}

/* which: 0 Bx_geom 1 By_geom 2 Bxx 3 Bxy 4 Byy 5 grav_coeff 6 dgc/dx 7 dgc/dy
 * 8 arc_perim 9 arc_nx 10 arc_ny 11 source_cell 12 src flags (E|W<<1|N<<2|S<<3) */
void sflow_oracle_get_geometry(const oracle_t* o, int which, double* out) {
  const double* arrs[] = {o->Bx, o->By, o->Bxx, o->Bxy, o->Byy, o->gc, o->dgcx, o->dgcy,
                          o->arc_perim, o->arc_nx, o->arc_ny};
  for (int i = 0; i < o->N; ++i) {
    if (which <= 10) out[i] = arrs[which][i];
    else if (which == 11) out[i] = o->source_cell[i];
    else out[i] = o->srcE[i] | (o->srcW[i] << 1) | (o->srcN[i] << 2) | (o->srcS[i] << 3);
  }
}

void sflow_oracle_stats(const oracle_t* o, SflowStepStats* s) {
  const int nv = o->P.nv, np = nv + 2, ns = o->P.ns;
  double mass = 0.0, vol = 0.0, solid = 0.0;
  int64_t area = 0;
  for (int i = 0; i < o->N; ++i) {
    mass += o->q[(size_t)i * nv];
    vol += o->qp[(size_t)i * np];
    if (o->q[(size_t)i * nv] > 1.0e-7) ++area;
    for (int k = 0; k < ns; ++k) solid += o->q[(size_t)i * nv + 4 + k];
  }
  s->t = o->t; s->dt = o->dt;
  s->mass = o->dx * o->dy * mass;
  s->volume = o->dx * o->dy * vol;
  s->area = o->dx * o->dy * (double)area;
  s->solid_mass = o->dx * o->dy * solid;
  s->solve_cells = o->solve_cells;
  s->steps = o->steps;
  s->status = o->status;
  s->pad = 0;
}

double sflow_oracle_time(const oracle_t* o) { return o->t; }
double sflow_oracle_h_source(const oracle_t* o) { return o->P.h_source; }
int sflow_oracle_max_newton(const oracle_t* o) { return o->max_newton_iter_seen; }
int64_t sflow_oracle_newton_total(const oracle_t* o) { return o->newton_iters_total; }
int sflow_oracle_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void sflow_oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ---- unit-level entry points for known-answer tests --------------------- */
void sflow_oracle_qc_to_qp(const oracle_t* o, const double* qc, double* qp, double* p_dyn) {
  oracle_qc_to_qp_p(&o->P, qc, qp, p_dyn);
}
void sflow_oracle_qp_to_qc(const oracle_t* o, const double* qp, double* qc) {
  oracle_qp_to_qc_p(&o->P, qp, qc);
}
void sflow_oracle_mixt_var(const oracle_t* o, const double* qp, double* out6) {
  mixt_t m;
  mixt_var(&o->P, qp, 1, &m);
  out6[0] = m.Ri; out6[1] = m.rho_m; out6[2] = m.rho_c; out6[3] = m.red_grav;
  out6[4] = m.cp_c; out6[5] = m.cp_mix;
}
void sflow_oracle_fluxes(const oracle_t* o, const double* qc, const double* qp, double gc, int dir,
                         double* flux) {
  oracle_eval_fluxes_p(&o->P, qc, qp, gc, dir, flux);
}
double sflow_oracle_settling_velocity(const oracle_t* o, double diam, double rhos, double rhoc,
                                      double inv_kin_visc) {
  return settling_velocity(&o->P, diam, rhos, rhoc, inv_kin_visc);
}
void sflow_oracle_implicit_terms(const oracle_t* o, double Bx, double By, const double* q, double* nh) {
  r_implicit_terms(&o->P, Bx, By, q, nh);
}
/* one Newton solve, returns iterations */
int sflow_oracle_newton(const oracle_t* o, double dt, double a_diag, double Bx, double By,
                        const double* q_old, const double* Rj, double* q_inout) {
  newton_ctx nc = {&o->P, dt, a_diag, Bx, By, q_old, Rj};
  return solve_rk_step(&nc, q_inout);
}

/* the shared FP64 functions as the host computes them (tests compare them
 * with correctly rounded values and with the device's bits) */
double sflow_oracle_pow(double x, double y) { return sfm_pow(x, y); }
double sflow_oracle_log(double x) { return sfm_log(x); }
double sflow_oracle_cos(double x) { return sfm_cos(x); }
void sflow_oracle_eval_math(int which, int64_t n, const double* x, const double* y, double* out) {
  for (int64_t i = 0; i < n; ++i)
    out[i] = which == 0 ? sfm_pow(x[i], y[i]) : which == 1 ? sfm_log(x[i]) : sfm_cos(x[i]);
}

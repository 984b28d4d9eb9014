// sflow_setup.cpp -- parameter checks and the init-time geometry of a
// domain: grid constants (init_grid, geometry_2d.f90:186-385), topography
// derivatives and slope factor (topography_reconstruction,
// geometry_2d.f90:555-895), the lateral ring inlet (init_source,
// geometry_2d.f90:907-1323; inlet thickness from MFR_SOURCE,
// inpout_2d.f90:4097-4137, 4526, 4637-4747), and the IMEX tableau
// (solver_2d.f90:399-487).  All in FP64 on the host, once per run.
#include <cfloat>
#include <cmath>
#include <cstring>
#include <type_traits>

#include "sflow_host.h"

namespace sflow {

static inline double sqd(double a) { return a * a; }

float float_below(double x) {
  float f = (float)x;                         // round to nearest
  if ((double)f > x) f = std::nextafterf(f, -INFINITY);
  return f;
}

// constitutive_2d.f90:1342-1492 mixt_var with sp_heat_flag = .TRUE.
void host_mixt_var(const HostSetup& s, const double* qp, double* rho_m_out, double* cp_mix_out) {
  const SflowParams& p = s.p;
  const int ns = s.ns, nv = s.nv;
  if (!(qp[0] > DBL_EPSILON)) {
    *rho_m_out = s.rho_a_amb;
    *cp_mix_out = p.liquid_flag ? p.sp_heat_l : p.sp_heat_a;
    return;
  }
  (void)nv;
  double al[SFLOW_MAX_SOLID], at = 0.0;
  for (int i = 0; i < ns; ++i) {
    al[i] = p.alpha_flag ? qp[4 + i] : qp[4 + i] / qp[0];
    at += al[i];
  }
  double rho_c;
  if (p.gas_flag) {
    double rho_a = p.pres / (p.sp_gas_const_a * qp[3]);
    rho_c = ((1.0 - 0.0 - at - 0.0) * rho_a + 0.0) / (1.0 - 0.0 - at);
  } else {
    rho_c = p.rho_l;
  }
  double d = 0.0;
  for (int i = 0; i < ns; ++i) d += al[i] * p.rho_s[i];
  double rho_m = (1.0 - at) * rho_c + d;
  double inv_rhom = 1.0 / rho_m;
  double xs[SFLOW_MAX_SOLID], sxs = 0.0;
  for (int i = 0; i < ns; ++i) {
    xs[i] = al[i] * p.rho_s[i] * inv_rhom;
    sxs += xs[i];
  }
  double xc = 1.0 - sxs, cp_c;
  if (p.gas_flag) cp_c = (xc > DBL_EPSILON) ? ((xc - 0.0) * p.sp_heat_a + 0.0) / xc : p.sp_heat_a;
  else cp_c = p.sp_heat_l;
  double dcp = 0.0;
  for (int i = 0; i < ns; ++i) dcp += xs[i] * p.sp_heat_s[i];
  *rho_m_out = rho_m;
  *cp_mix_out = dcp + xc * cp_c;
}

static void topography(HostSetup& s, const double* B) {
  const int nx = s.nx, ny = s.ny;
  const size_t N = (size_t)nx * ny;
  const double dx = s.dx, dy = s.dy;
  static const double c1[5] = {-2.0, -1.0, 0.0, 1.0, 2.0};
  static const double c2[5] = {2.0, -1.0, -2.0, -1.0, 2.0};
  const double n1x = 10.0 * dx, n1y = 10.0 * dy, n2x = 7.0 * sqd(dx), n2y = 7.0 * sqd(dy);
  const double nxy = (10.0 * dx) * (10.0 * dy);
  auto Bc = [&](int j, int k) { return B[(size_t)k * nx + j]; };
  auto at = [&](std::vector<double>& v, int j, int k) -> double& { return v[(size_t)k * nx + j]; };
  std::vector<double>* arr[5] = {&s.Bx, &s.By, &s.Bxx, &s.Byy, &s.Bxy};
  for (auto* a : arr) a->assign(N, 0.0);
  // one row: x derivatives only (geometry_2d.f90:600-640)
  if (ny == 1) {
    for (int j = 2; j <= nx - 3; ++j) {
      double px = 0.0, sxx = 0.0;
      for (int m = 0; m < 5; ++m) {
        px = px + c1[m] * Bc(j + m - 2, 0);
        sxx = sxx + c2[m] * Bc(j + m - 2, 0);
      }
      at(s.Bx, j, 0) = px / n1x;
      at(s.By, j, 0) = 0.0 / n1y;
      at(s.Bxx, j, 0) = sxx / n2x;
      at(s.Byy, j, 0) = 0.0 / n2y;
      at(s.Bxy, j, 0) = 0.0;
    }
  }
  // five-point centred derivatives (geometry_2d.f90:730-790)
  for (int k = 2; k <= ny - 3; ++k) {
    for (int j = 2; j <= nx - 3; ++j) {
      double px = 0.0, py = 0.0, sxx = 0.0, syy = 0.0, ws = 0.0;
      for (int m = 0; m < 5; ++m) {
        px = px + c1[m] * Bc(j + m - 2, k);
        sxx = sxx + c2[m] * Bc(j + m - 2, k);
      }
      for (int m = 0; m < 5; ++m) {
        py = py + c1[m] * Bc(j, k + m - 2);
        syy = syy + c2[m] * Bc(j, k + m - 2);
      }
      for (int mm = 0; mm < 5; ++mm)
        for (int m = 0; m < 5; ++m) ws = ws + c1[m] * c1[mm] * Bc(j + m - 2, k + mm - 2);
      at(s.Bx, j, k) = px / n1x;
      at(s.By, j, k) = py / n1y;
      at(s.Bxx, j, k) = sxx / n2x;
      at(s.Byy, j, k) = syy / n2y;
      at(s.Bxy, j, k) = ws / nxy;
    }
  }
  // two-cell frame copied from the nearest computed row/column
  for (int k = 0; k < ny; ++k)
    for (auto* a : arr) {
      at(*a, 0, k) = at(*a, 2, k);
      at(*a, 1, k) = at(*a, 2, k);
      at(*a, nx - 2, k) = at(*a, nx - 3, k);
      at(*a, nx - 1, k) = at(*a, nx - 3, k);
    }
  if (ny >= 3)
    for (int j = 0; j < nx; ++j)
      for (auto* a : arr) {
        at(*a, j, 0) = at(*a, j, 2);
        at(*a, j, 1) = at(*a, j, 2);
        at(*a, j, ny - 2) = at(*a, j, ny - 3);
        at(*a, j, ny - 1) = at(*a, j, ny - 3);
      }
  s.gc.assign(N, 1.0);
  s.dgcx.assign(N, 0.0);
  s.dgcy.assign(N, 0.0);
  if (s.p.slope_correction_flag) {
    for (size_t i = 0; i < N; ++i) {
      s.gc[i] = 1.0 / (1.0 + sqd(s.Bx[i]) + sqd(s.By[i]));
      s.dgcx[i] = -2.0 * sqd(s.gc[i]) * (s.Bx[i] * s.Bxx[i] + s.By[i] * s.Bxy[i]);
      s.dgcy[i] = -2.0 * sqd(s.gc[i]) * (s.Bx[i] * s.Bxy[i] + s.By[i] * s.Byy[i]);
    }
  }
}

static void ring_source(HostSetup& s) {
  const int nx = s.nx, ny = s.ny;
  const size_t N = (size_t)nx * ny;
  const SflowParams& p = s.p;
  s.cflags.assign(N, 0);
  s.arc_perim.assign(N, 0.0);
  s.arc_nx.assign(N, 0.0);
  s.arc_ny.assign(N, 0.0);
  if (!p.radial_source_flag) return;
  std::vector<double> vx[4], vy[4];  // E, W, N, S
  for (int f = 0; f < 4; ++f) { vx[f].assign(N, 0.0); vy[f].assign(N, 0.0); }
  auto xst = [&](int j) { return p.x0 + (double)j * s.dx; };
  auto yst = [&](int k) { return p.y0 + (double)k * s.dy; };
  auto xc = [&](int j) { return 0.5 * (xst(j) + xst(j + 1)); };
  auto yc = [&](int k) { return 0.5 * (yst(k) + yst(k + 1)); };
  const double xs = p.x_source, ys = p.y_source, rs = p.r_source;
  const uint8_t FE = 0x4, FW = 0x8, FN = 0x10, FS = 0x20;
  auto mark2 = [&](int j, int k, uint8_t bit) {
    size_t c = (size_t)k * nx + j;
    s.cflags[c] = (uint8_t)((s.cflags[c] & 0xFC) | 2 | bit);
  };
  for (int k = 1; k <= ny - 2; ++k) {
    for (int j = 1; j <= nx - 2; ++j) {
      if (sqd(xc(j) - xs) + sqd(yc(k) - ys) <= sqd(rs)) {
        size_t c = (size_t)k * nx + j;
        s.cflags[c] = (uint8_t)((s.cflags[c] & 0xFC) | 1);
        if (sqd(xc(j - 1) - xs) + sqd(yc(k) - ys) >= sqd(rs)) {
          size_t e = (size_t)k * nx + (j - 1);
          mark2(j - 1, k, FE);
          double d = std::sqrt(sqd(xst(j) - xs) + sqd(yc(k) - ys));
          vx[0][e] = (xst(j) - xs) * rs / sqd(d);
          vy[0][e] = (yc(k) - ys) * rs / sqd(d);
        } else if (sqd(xc(j + 1) - xs) + sqd(yc(k) - ys) >= sqd(rs)) {
          size_t e = (size_t)k * nx + (j + 1);
          mark2(j + 1, k, FW);
          double d = std::sqrt(sqd(xst(j + 1) - xs) + sqd(yc(k) - ys));
          vx[1][e] = (xst(j + 1) - xs) * rs / sqd(d);
          vy[1][e] = (yc(k) - ys) * rs / sqd(d);
        }
        if (sqd(xc(j) - xs) + sqd(yc(k - 1) - ys) >= sqd(rs)) {
          size_t e = (size_t)(k - 1) * nx + j;
          mark2(j, k - 1, FN);
          double d = std::sqrt(sqd(xc(j) - xs) + sqd(yst(k) - ys));
          vx[2][e] = (xc(j) - xs) * rs / sqd(d);
          vy[2][e] = (yst(k) - ys) * rs / sqd(d);
        } else if (sqd(xc(j) - xs) + sqd(yc(k + 1) - ys) >= sqd(rs)) {
          size_t e = (size_t)(k + 1) * nx + j;
          mark2(j, k + 1, FS);
          double d = std::sqrt(sqd(xc(j) - xs) + sqd(yst(k + 1) - ys));
          vx[3][e] = (xc(j) - xs) * rs / sqd(d);
          vy[3][e] = (yst(k + 1) - ys) * rs / sqd(d);
        }
      }
    }
  }
  const double half_arc = 0.5 * p.arc_width_source;
  const uint8_t bits[4] = {FE, FW, FN, FS};
  const double flen[4] = {s.dy, s.dy, s.dx, s.dx};
  for (int k = 0; k < ny; ++k) {
    for (int j = 0; j < nx; ++j) {
      size_t c = (size_t)k * nx + j;
      if ((s.cflags[c] & 0x3) != 2) continue;
      for (int f = 0; f < 4; ++f) {
        if (!(s.cflags[c] & bits[f])) continue;
        double ux = vx[f][c], uy = vy[f][c];
        double vmag = std::sqrt(ux * ux + uy * uy);
        if (vmag > 0.0) {
          double nxv = ux / vmag, nyv = uy / vmag;
          bool in_arc = true;
          if (p.arc_width_source < 360.0) {
            double ang = 90.0 - std::atan2(uy, ux) * 180.0 / s.pi_g;
            ang = std::fmod(ang + 360.0, 360.0);
            double diff = std::fmod(std::fabs(ang - p.azimuth_source) + 360.0, 360.0);
            if (diff > 180.0) diff = 360.0 - diff;
            in_arc = diff <= half_arc;
          }
          if (in_arc) {
            s.arc_perim[c] = s.arc_perim[c] + flen[f];
            s.arc_nx[c] = s.arc_nx[c] + flen[f] * nxv;
            s.arc_ny[c] = s.arc_ny[c] + flen[f] * nyv;
          }
        }
      }
      if (s.arc_perim[c] > 0.0) {
        s.arc_nx[c] = s.arc_nx[c] / s.arc_perim[c];
        s.arc_ny[c] = s.arc_ny[c] / s.arc_perim[c];
        double vmag = std::sqrt(sqd(s.arc_nx[c]) + sqd(s.arc_ny[c]));
        if (vmag > 0.0) {
          s.arc_nx[c] /= vmag;
          s.arc_ny[c] /= vmag;
        }
      }
    }
  }
  double tot = 0.0;
  for (size_t c = 0; c < N; ++c) tot += s.arc_perim[c];
  const double r1 = p.r_source, r2 = s.p.r2_source;
  const double he = sqd(r1 - r2) / sqd(r1 + r2);
  double len = s.pi_g * (r1 + r2) *
               (1.0 + 0.25 * he + sqd(he) / 64.0 + he * he * he / 256.0 + sqd(sqd(he)) * 25.0 / 16384.0 +
                sqd(sqd(he)) * he * 49.0 / 65536.0);
  if (p.arc_width_source < 360.0) len = len * (p.arc_width_source / 360.0);
  if (tot > 0.0) {
    const double rescale = len / tot;
    for (size_t c = 0; c < N; ++c) s.arc_perim[c] = s.arc_perim[c] * rescale;
  }
  for (size_t c = 0; c < N; ++c)
    if (s.cflags[c] & 0x3) ++s.ring_cells;
}

// compute_cell_fract (geometry_2d.f90:1899-1994): the fraction of 200 x 200
// sub-cell points of each cell inside the source ellipse (semi-axes
// r_source along the rotated x axis and r2_source, rotation angle_source
// degrees); cells outside the ellipse's bounding box are 0.  The quotient
// is taken in single precision, as the reference's REAL(SUM(...))/n2.
static void cell_fractions(HostSetup& s) {
  const SflowParams& p = s.p;
  const int nx = s.nx, ny = s.ny;
  const size_t N = (size_t)nx * ny;
  s.cell_fract.assign(N, 0.0);
  const int n = 200, n2 = n * n;
  const double ang = p.angle_source / 180.0 * std::atan(1.0) * 4.0;
  const double ca = std::cos(ang), sa = std::sin(ang);
  std::vector<double> xsub(n), ysub(n);   // the offsets take n distinct values
  for (int h = 1; h <= n; ++h) {
    double v = (2.0 * (double)h - 1.0) / (2.0 * (double)n);
    xsub[h - 1] = (v - 0.5) * s.dx;
    ysub[h - 1] = (v - 0.5) * s.dy;
  }
  auto xst = [&](int j) { return p.x0 + (double)j * s.dx; };
  auto yst = [&](int k) { return p.y0 + (double)k * s.dy; };
  const double xs = p.x_source, ys = p.y_source, rs = p.r_source, r2s = p.r2_source;
  const double rmx = std::fmax(rs, r2s);
  const double rs2 = rs * rs, r2s2 = r2s * r2s;
  for (int k = 0; k < ny; ++k) {
    for (int j = 0; j < nx; ++j) {
      if (xst(j + 1) < xs - rmx || xst(j) > xs + rmx || yst(k + 1) < ys - rmx || yst(k) > ys + rmx) continue;
      const double xc = 0.5 * (xst(j) + xst(j + 1)), yc = 0.5 * (yst(k) + yst(k + 1));
      int cnt = 0;
      for (int iy = 0; iy < n; ++iy) {
        const double dyv = yc + ysub[iy] - ys;
        for (int ix = 0; ix < n; ++ix) {
          const double dxv = xc + xsub[ix] - xs;
          const double a1 = dxv * ca + dyv * sa;
          const double a2 = -(dxv * sa) + dyv * ca;
          if (a1 * a1 / rs2 + a2 * a2 / r2s2 <= 1.0) ++cnt;
        }
      }
      const double f = (double)((float)cnt / (float)n2);
      s.cell_fract[(size_t)k * nx + j] = f;
      if (f > 0.0) {
        s.cflags[(size_t)k * nx + j] |= kFlagBottom;
        ++s.bottom_cells;
      }
    }
  }
}

int host_setup(const SflowParams* pin, const double* B, HostSetup& s, std::string& err, bool host_topography) {
  if (!pin) { err = "params is NULL"; return SFLOW_EINVAL; }
  s.p = *pin;
  SflowParams& p = s.p;
  if (p.abi_version != SFLOW_ABI_VERSION) { err = "abi_version mismatch"; return SFLOW_EINVAL; }
  if (p.precision != SFLOW_PREC_FP64 && p.precision != SFLOW_PREC_FP32) { err = "precision must be SFLOW_PREC_FP64 or SFLOW_PREC_FP32"; return SFLOW_EINVAL; }
  if (p.comp_cells_x < 5 || (p.comp_cells_y < 5 && p.comp_cells_y != 1)) {
    err = "comp_cells_x must be >= 5 and comp_cells_y 1 or >= 5";
    return SFLOW_EINVAL;
  }
  if (p.comp_cells_y == 1 && (p.radial_source_flag || p.bottom_radial_source_flag)) { err = "a radial source needs comp_cells_y > 1"; return SFLOW_EINVAL; }
  if (p.radial_source_flag && p.bottom_radial_source_flag) {
    // the lateral ring needs H_SOURCE or MFR_SOURCE, which the bottom source forbids
    err = "radial_source_flag and bottom_radial_source_flag exclude each other";
    return SFLOW_EINVAL;
  }
  if ((int64_t)p.comp_cells_x * p.comp_cells_y > (int64_t)1 << 31) { err = "domain larger than 2^31 cells"; return SFLOW_ERANGE; }
  if (p.n_solid < 1 || p.n_solid > 3) { err = "the GPU kernels are built for n_solid = 1, 2 or 3"; return SFLOW_EINVAL; }
  if (p.n_rk < 1 || p.n_rk > 4) { err = "N_RK must be 1, 2, 3 or 4"; return SFLOW_EINVAL; }
  if (p.gas_flag && p.liquid_flag) { err = "gas carrier with a liquid phase is not supported"; return SFLOW_EINVAL; }
  if (!p.gas_flag && !p.liquid_flag) { err = "one of gas_flag / liquid_flag must be set"; return SFLOW_EINVAL; }
  if (p.rheology_flag && p.rheology_model != 1 && p.rheology_model != 6 && p.rheology_model != 11) {
    err = "rheology_model must be 1, 6 or 11";
    return SFLOW_EINVAL;
  }
  if (p.rheology_flag && p.rheology_model == 11 &&
      (p.mu_s < 0.0 || p.mu_2 < 0.0 || p.I_0 < 0.0 || p.muI_inf < 0.0)) {
    // inpout_2d.f90:3592-3611
    err = "rheology_model 11 needs mu_s, mu_2, I_0 and muI_inf >= 0";
    return SFLOW_EINVAL;
  }
  if (p.erosion_coeff < 0.0) { err = "erosion_coeff must be >= 0"; return SFLOW_EINVAL; }
  if (p.solver_scheme != SFLOW_SCHEME_KT && p.solver_scheme != SFLOW_SCHEME_UP) {
    err = "SOLVER_SCHEME must be KT or UP";
    return SFLOW_EINVAL;
  }
  if (!(p.cell_size > 0.0) || !(p.cfl > 0.0) || !(p.max_dt > 0.0) || !(p.dt0 > 0.0)) { err = "cell_size, cfl, max_dt, dt0 must be > 0"; return SFLOW_EINVAL; }
  if (!(p.pres > 0.0) || !(p.sp_gas_const_a > 0.0) || !(p.T_ambient > 0.0)) { err = "pres, sp_gas_const_a, T_ambient must be > 0"; return SFLOW_EINVAL; }
  for (int i = 0; i < p.n_solid; ++i)
    if (!(p.rho_s[i] > 0.0)) { err = "rho_s must be > 0"; return SFLOW_EINVAL; }
  for (int i = 0; i < 4 + p.n_solid; ++i)
    if (p.limiter[i] < 0 || p.limiter[i] > 7) { err = "limiter out of 0..7"; return SFLOW_EINVAL; }
  for (int sd = 0; sd < 4; ++sd)
    for (int i = 0; i < 4 + p.n_solid; ++i)
      if (p.bc[sd][i].flag < 0 || p.bc[sd][i].flag > 2) { err = "boundary flag out of 0..2"; return SFLOW_EINVAL; }
  if (p.liquid_flag && !(p.rho_l > 0.0)) { err = "rho_l must be > 0"; return SFLOW_EINVAL; }
  if ((p.settling_flag) && !((p.gas_flag ? p.kin_visc_a : p.kin_visc_l) > 0.0)) { err = "settling needs a positive kinematic viscosity"; return SFLOW_EINVAL; }
  if (p.entrainment_flag && !p.gas_flag) { err = "entrainment needs a gas carrier"; return SFLOW_EINVAL; }

  s.nx = p.comp_cells_x;
  s.ny = p.comp_cells_y;
  s.ns = p.n_solid;
  s.nv = 4 + p.n_solid;
  s.nrk = p.n_rk;
  s.dx = p.cell_size;
  s.dy = p.comp_cells_y > 1 ? p.cell_size : 1.0;   // geometry_2d.f90:288-298
  s.eps_sing = std::fmin(std::fmin(std::pow(s.dx, 4.0), std::pow(s.dy, 4.0)), 1.0e-10);
  {
    double e2 = s.eps_sing * s.eps_sing;
    s.eps_sing4 = e2 * e2;
  }
  s.pi_g = 4.0 * std::atan(1.0);
  s.rho_a_amb = p.pres / (p.sp_gas_const_a * p.T_ambient);
  s.kin_visc_c = p.gas_flag ? p.kin_visc_a : p.kin_visc_l;
  // erodible layer (inpout_2d.f90:1818-1990)
  if (p.erosion_coeff == 0.0) {
    s.erodible_porosity = 0.0;
    for (int i = 0; i < p.n_solid; ++i) s.erodible_fract[i] = 1.0 / p.n_solid;
    s.T_erodible = 300.0;
    s.coeff_porosity = 0.0;
    s.erodible_init = 0.0;
  } else {
    if (p.erodible_porosity < 0.0 || p.erodible_porosity > 1.0) { err = "erodible_porosity must be in [0, 1]"; return SFLOW_EINVAL; }
    s.erodible_porosity = p.erodible_porosity;
    s.coeff_porosity = p.erodible_porosity / (1.0 - p.erodible_porosity);
    if (p.n_solid == 1) {
      s.erodible_fract[0] = 1.0;
    } else {
      double sum = 0.0;
      for (int i = 0; i < p.n_solid; ++i) {
        if (p.erodible_fract[i] < 0.0) { err = "erodible_fract must be >= 0"; return SFLOW_EINVAL; }
        s.erodible_fract[i] = p.erodible_fract[i];
        sum += p.erodible_fract[i];
      }
      if (sum != 1.0) {
        if (!(sum > 0.0)) { err = "erodible_fract sums to 0"; return SFLOW_EINVAL; }
        for (int i = 0; i < p.n_solid; ++i) s.erodible_fract[i] = s.erodible_fract[i] / sum;
      }
    }
    if (p.T_erodible < 0.0) { err = "T_erodible must be given (>= 0) with erosion"; return SFLOW_EINVAL; }
    s.T_erodible = p.T_erodible;
    s.erodible_init = p.initial_erodible_thickness >= 0.0 ? p.initial_erodible_thickness : 0.0;
  }
  s.rho_c_sub = p.gas_flag ? p.pres / (p.sp_gas_const_a * s.T_erodible) : p.rho_l;
  s.exchange = (p.erosion_coeff != 0.0 || p.settling_flag || p.entrainment_flag) ? 1 : 0;

  // vulnerability table levels (inpout_2d.f90:3808-3866)
  {
    int nt = 0, nd = 0;
    for (int i = 0; i < SFLOW_MAX_LEVELS; ++i) {
      if (p.thickness_levels[i] >= 0.0) ++nt;
      if (p.dyn_pres_levels[i] >= 0.0) ++nd;
    }
    for (int i = 0; i < nt; ++i)
      if (p.thickness_levels[i] < 0.0) { err = "thickness_levels: the levels >= 0 must come first"; return SFLOW_EINVAL; }
    for (int i = 0; i < nd; ++i)
      if (p.dyn_pres_levels[i] < 0.0) { err = "dyn_pres_levels: the levels >= 0 must come first"; return SFLOW_EINVAL; }
    for (int i = 0; i < nt; ++i) s.thk_levels[i] = p.thickness_levels[i];
    for (int i = 0; i < nd; ++i) s.dyn_levels[i] = p.dyn_pres_levels[i];
    if (nt > 0 && nd == 0) { nd = 1; s.dyn_levels[0] = 0.0; }
    if (nd > 0 && nt == 0) { nt = 1; s.thk_levels[0] = 0.0; }
    s.n_thk = nt;
    s.n_dyn = nd;
  }

  // IMEX tableaux (solver_2d.f90:421-487)
  {
    auto AT = [&](int i, int j) -> double& { return s.a_tilde[(i - 1) * 4 + (j - 1)]; };
    auto AD = [&](int i, int j) -> double& { return s.a_dirk[(i - 1) * 4 + (j - 1)]; };
    switch (p.n_rk) {
      case 1:
        AT(1, 1) = 1.0; s.omega_tilde[0] = 1.0;
        break;
      case 2:
        AT(2, 1) = 1.0; s.omega_tilde[0] = 1.0; AD(2, 2) = 1.0; s.omega[1] = 1.0;
        break;
      case 3:
        AT(2, 1) = 0.5; AT(3, 1) = 0.5; AT(3, 2) = 0.5;
        s.omega_tilde[0] = s.omega_tilde[1] = s.omega_tilde[2] = 1.0 / 3.0;
        AD(1, 1) = 0.25; AD(2, 2) = 0.25; AD(3, 1) = 1.0 / 3.0; AD(3, 2) = 1.0 / 3.0; AD(3, 3) = 1.0 / 3.0;
        s.omega[0] = s.omega[1] = s.omega[2] = 1.0 / 3.0;
        break;
      case 4:
        AT(2, 1) = 0.5; AT(3, 1) = 1.0 / 3.0; AT(4, 2) = 1.0;
        s.omega_tilde[1] = 1.0;
        AD(2, 2) = 0.5; AD(3, 3) = 1.0 / 3.0; AD(4, 3) = 0.75; AD(4, 4) = 0.25;
        s.omega[2] = 0.75; s.omega[3] = 0.25;
        break;
    }
    // q = q_rk(n_RK) when the last row equals the weights (solver_2d.f90:1362-1372)
    double d1 = 0.0, d2 = 0.0;
    for (int r = 0; r < p.n_rk; ++r) {
      d1 += std::fabs(s.omega_tilde[r] - s.a_tilde[(p.n_rk - 1) * 4 + r]);
      d2 += std::fabs(s.omega[r] - s.a_dirk[(p.n_rk - 1) * 4 + r]);
    }
    s.take_last = (d1 == 0.0 && d2 == 0.0) ? 1 : 0;
  }

  if (!B) { err = "B_cent is NULL"; return SFLOW_EINVAL; }
  if (host_topography) topography(s, B);
  s.B.assign(B, B + (size_t)s.nx * s.ny);

  // inlet (radial ring / bottom source) constants
  s.h_source = p.h_source;
  for (int i = 0; i < 4; ++i) s.time_param[i] = p.time_param[i];
  if (p.n_intervals != 0) {
    // inpout_2d.f90:4451-4512
    if (!p.bottom_radial_source_flag) { err = "n_intervals needs bottom_radial_source_flag"; return SFLOW_EINVAL; }
    if (p.n_intervals < 0 || p.n_intervals > SFLOW_MAX_INTERVALS) { err = "n_intervals must be in 0..100"; return SFLOW_EINVAL; }
    for (int i = 0; i < p.n_intervals; ++i) {
      if (p.t_intervals[i] < 0.0) { err = "t_intervals must be >= 0"; return SFLOW_EINVAL; }
      if (p.vel_intervals[i] < 0.0) { err = "vel_intervals must be >= 0"; return SFLOW_EINVAL; }
      if (i > 0 && p.t_intervals[i] <= p.t_intervals[i - 1]) { err = "t_intervals must increase"; return SFLOW_EINVAL; }
    }
  }
  if (p.bottom_radial_source_flag) {
    // inpout_2d.f90:4029-4075: the inflow is vel_source over the ellipse
    if (p.h_source >= 0.0 || p.mfr_source >= 0.0) {
      err = "h_source / mfr_source must not be given with bottom_radial_source_flag";
      return SFLOW_EINVAL;
    }
    if (p.vel_source == -1.0) { err = "vel_source must be given with bottom_radial_source_flag"; return SFLOW_EINVAL; }
  }
  if (p.radial_source_flag || p.bottom_radial_source_flag) {
    if (!(p.r_source > 0.0)) { err = "r_source must be > 0"; return SFLOW_EINVAL; }
    if (p.r2_source <= 0.0) { p.r2_source = p.r_source; p.angle_source = 0.0; }
    // inpout_2d.f90:4140-4175: the ring must stay a cell away from the edges
    const double rmax_ = std::fmax(p.r_source, p.r2_source);
    if (p.x_source - rmax_ <= p.x0 + p.cell_size || p.x_source + rmax_ >= p.x0 + (p.comp_cells_x - 1) * p.cell_size ||
        p.y_source - rmax_ <= p.y0 + p.cell_size || p.y_source + rmax_ >= p.y0 + (p.comp_cells_y - 1) * p.cell_size) {
      err = "radial source too close to the domain boundary";
      return SFLOW_EINVAL;
    }
    if (s.time_param[0] < 0.0 || s.time_param[1] < 0.0 || s.time_param[2] < 0.0 || s.time_param[3] < 0.0) {
      s.time_param[0] = p.t_end; s.time_param[1] = p.t_end; s.time_param[2] = 0.0; s.time_param[3] = p.t_end;
    }
    double qs[SFLOW_MAX_VARS + 2] = {0};
    if (p.radial_source_flag && p.mfr_source >= 0.0) {
      // inlet thickness from the mass flow rate over the ring's length
      const double r1 = p.r_source, r2 = p.r2_source;
      const double he = sqd(r1 - r2) / sqd(r1 + r2);
      double len = s.pi_g * (r1 + r2) *
                   (1.0 + 0.25 * he + sqd(he) / 64.0 + he * he * he / 256.0 + sqd(sqd(he)) * 25.0 / 16384.0 +
                    sqd(sqd(he)) * he * 49.0 / 65536.0);
      if (p.arc_width_source < 360.0) len = len * (p.arc_width_source / 360.0);
      if (!(p.vel_source > 0.0)) { err = "vel_source must be > 0 with mfr_source"; return SFLOW_EINVAL; }
      const double hs = 1.0;
      qs[0] = hs; qs[1] = hs * p.vel_source; qs[2] = 0.0; qs[3] = p.T_source;
      for (int i = 0; i < s.ns; ++i) qs[4 + i] = p.alpha_flag ? p.alphas_source[i] : p.alphas_source[i] * hs;
      qs[s.nv] = p.vel_source; qs[s.nv + 1] = 0.0;
      double rho_m, cpm;
      host_mixt_var(s, qs, &rho_m, &cpm);
      s.h_source = p.mfr_source / (len * rho_m * p.vel_source * 1.0);
      s.time_param[1] = 1.0e14 / p.mfr_source;
    }
    // inflow state of eval_expl_terms (constitutive_2d.f90:3192-3225,
    // 3351-3384): h = 1, T_source, alphas_source, at rest
    for (int i = 0; i < SFLOW_MAX_VARS + 2; ++i) qs[i] = 0.0;
    qs[0] = 1.0;
    qs[3] = p.T_source;
    for (int i = 0; i < s.ns; ++i) qs[4 + i] = p.alpha_flag ? p.alphas_source[i] : p.alphas_source[i] * qs[0];
    host_mixt_var(s, qs, &s.src_rho_m, &s.src_cp_mix);
  }
  ring_source(s);
  if (p.bottom_radial_source_flag) cell_fractions(s);
  s.row0 = 0;
  s.own_lo = 0;
  s.own_hi = s.ny;
  return SFLOW_OK;
}

int host_setup_rows(const SflowParams* p, const double* B, int k0, int rows, int own_lo, int own_hi,
                    HostSetup& s, std::string& err) {
  int rc = host_setup(p, B, s, err);
  if (rc != SFLOW_OK) return rc;
  const int nx = s.nx, ny = s.ny;
  if (ny == 1) { err = "row slabs need comp_cells_y > 1"; return SFLOW_EINVAL; }
  if (k0 < 0 || rows < 5 || k0 + rows > ny) { err = "row slab outside the domain (or under 5 rows)"; return SFLOW_EINVAL; }
  if (own_lo < 0 || own_hi > rows || own_lo >= own_hi) { err = "own rows outside the slab"; return SFLOW_EINVAL; }
  auto cut = [&](auto& v) {
    using V = typename std::decay<decltype(v)>::type;
    if (v.empty()) return;
    V w(v.begin() + (size_t)k0 * nx, v.begin() + (size_t)(k0 + rows) * nx);
    v.swap(w);
  };
  cut(s.Bx); cut(s.By); cut(s.Bxx); cut(s.Bxy); cut(s.Byy); cut(s.gc); cut(s.dgcx); cut(s.dgcy);
  cut(s.cflags); cut(s.arc_perim); cut(s.arc_nx); cut(s.arc_ny); cut(s.cell_fract); cut(s.B);
  s.ny = rows;
  s.p.comp_cells_y = rows;   // y0 stays: coordinates count rows from the whole domain's edge
  s.row0 = k0;
  s.own_lo = own_lo;
  s.own_hi = own_hi;
  return SFLOW_OK;
}

}  // namespace sflow

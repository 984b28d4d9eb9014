// sflow_io.cpp -- host I/O of the reference's files, so that a run keeps its
// input file, its initial/restart files and its output format:
//
//   sflow_read_input     IMEX_SfloW2D.inp namelists -> SflowParams + run
//                        information (inpout_2d.f90 init_param 408-970,
//                        read_param 986-5134), the subset the GPU path runs
//   sflow_read_dem       ESRI ASCII DEM -> B_cent and the no-data mask at the
//                        cell centres (inpout_2d.f90:3684-3760, geometry_2d
//                        init_grid 312-350, interp_2d_scalar 1395-1447,
//                        interp_2d_nodata 1463-1517)
//   sflow_read_q2d       .q_2d restart (inpout_2d.f90:5674-5722)
//   sflow_write_q2d      .q_2d output (inpout_2d.f90:6000-6110)
//   sflow_write_p2d      .p_2d output (inpout_2d.f90:6124-6400)
//   sflow_write_restart / sflow_read_restart
//                        restart.bin (inpout_2d.f90:8037-8179), Fortran
//                        unformatted sequential records
//
// Fortran edit descriptors used by the writers are restated from the
// Fortran standard's E and ES editing: Ew.d prints 0.d1d2..dd E+xx (the
// optional leading zero present, as gfortran writes it when the width
// allows), ESw.dEe prints d1.d2..d(d+1) E+xx; both right-justified in w
// characters; an exponent that does not fit prints w asterisks.
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/sflow.h"
#include "sflow_host.h"

namespace sflow {
namespace io {

static thread_local std::string g_io_err;

static int fail(int code, const std::string& msg) {
  g_io_err = msg;
  return code;
}

static std::string upper(std::string s) {
  for (auto& c : s) c = (char)std::toupper((unsigned char)c);
  return s;
}

// ---------------------------------------------------------------------------
// Fortran namelist input (the forms the reference's input files use):
//   &GROUP  name = v, name(i) = v, name%comp = v, name(i)%comp = v,
//           values separated by commas or blanks, r*v repeats, r* nulls,
//           'strings' / "strings", logicals T F .TRUE. .FALSE., reals with
//           E or D exponents, ! comments;  group ended by /
// ---------------------------------------------------------------------------
struct NValue {
  bool null = true;
  std::string text;   // raw token (strings without quotes)
  bool quoted = false;
};

struct NItem {
  std::string name;   // upper case
  int index = 0;      // 1-based element, 0 = whole object
  std::string comp;   // derived-type component (upper case) or ""
  std::vector<NValue> values;
  int line = 0;
};

struct NGroup {
  std::string name;   // upper case
  std::vector<NItem> items;
  bool used = false;
};

class Lexer {
 public:
  explicit Lexer(const std::string& s) : s_(s) {}
  size_t pos = 0;
  int line = 1;
  bool eof() const { return pos >= s_.size(); }
  char peek(size_t k = 0) const { return pos + k < s_.size() ? s_[pos + k] : '\0'; }
  char get() {
    char c = s_[pos++];
    if (c == '\n') ++line;
    return c;
  }
  // blanks, newlines and ! comments
  void skip_ws() {
    while (!eof()) {
      char c = peek();
      if (c == '!') {
        while (!eof() && peek() != '\n') get();
      } else if (std::isspace((unsigned char)c)) {
        get();
      } else {
        break;
      }
    }
  }
  bool ident_start() const { return std::isalpha((unsigned char)peek()) || peek() == '_'; }
  std::string ident() {
    std::string r;
    while (!eof() && (std::isalnum((unsigned char)peek()) || peek() == '_')) r += get();
    return r;
  }
  // does an item designator (name[(i)][%comp] =) start here?
  bool item_ahead() const {
    size_t p = pos;
    auto at = [&](size_t q) { return q < s_.size() ? s_[q] : '\0'; };
    if (!(std::isalpha((unsigned char)at(p)) || at(p) == '_')) return false;
    while (std::isalnum((unsigned char)at(p)) || at(p) == '_') ++p;
    auto blanks = [&]() {
      while (at(p) == ' ' || at(p) == '\t' || at(p) == '\r' || at(p) == '\n') ++p;
    };
    blanks();
    if (at(p) == '(') {
      while (at(p) && at(p) != ')') ++p;
      if (at(p) != ')') return false;
      ++p;
      blanks();
    }
    if (at(p) == '%') {
      ++p;
      blanks();
      while (std::isalnum((unsigned char)at(p)) || at(p) == '_') ++p;
      blanks();
    }
    return at(p) == '=';
  }

 private:
  const std::string& s_;
};

static int parse_namelists(const std::string& text, std::vector<NGroup>& out, std::string& err) {
  Lexer L(text);
  while (true) {
    // find the next '&' outside comments and strings
    bool found = false;
    while (!L.eof()) {
      char c = L.peek();
      if (c == '!') {
        while (!L.eof() && L.peek() != '\n') L.get();
      } else if (c == '&') {
        found = true;
        break;
      } else {
        L.get();
      }
    }
    if (!found) break;
    L.get();
    NGroup g;
    g.name = upper(L.ident());
    if (g.name.empty()) { err = "line " + std::to_string(L.line) + ": '&' without a group name"; return -1; }
    if (g.name == "END") continue;
    bool closed = false;
    while (true) {
      L.skip_ws();
      if (L.eof()) break;
      char c = L.peek();
      if (c == '/') { L.get(); closed = true; break; }
      if (c == '&') {   // &END terminator
        size_t save = L.pos;
        L.get();
        if (upper(L.ident()) == "END") { closed = true; break; }
        L.pos = save;
        err = "line " + std::to_string(L.line) + ": unexpected '&' inside group " + g.name;
        return -1;
      }
      if (c == ',') { L.get(); continue; }
      if (!L.item_ahead()) {
        err = "line " + std::to_string(L.line) + ": expected 'name =' in group " + g.name;
        return -1;
      }
      NItem it;
      it.line = L.line;
      it.name = upper(L.ident());
      L.skip_ws();
      if (L.peek() == '(') {
        L.get();
        std::string num;
        while (!L.eof() && L.peek() != ')') num += L.get();
        L.get();
        char* end = nullptr;
        long v = std::strtol(num.c_str(), &end, 10);
        if (!end || *end != '\0' || v < 1) { err = "line " + std::to_string(it.line) + ": bad index (" + num + ") of " + it.name; return -1; }
        it.index = (int)v;
        L.skip_ws();
      }
      if (L.peek() == '%') {
        L.get();
        L.skip_ws();
        it.comp = upper(L.ident());
        L.skip_ws();
      }
      L.get();   // '='
      // values until the next item designator, '/' or '&'
      bool after_sep = true;   // a separator was seen since the last value
      while (true) {
        L.skip_ws();
        if (L.eof()) break;
        char d = L.peek();
        if (d == '/' || d == '&') break;
        if (d == ',') {
          L.get();
          if (!after_sep) {
            after_sep = true;
          } else {
            it.values.push_back(NValue());   // null value between separators
          }
          continue;
        }
        if (L.item_ahead()) break;
        NValue v;
        if (d == '\'' || d == '"') {
          const char q = L.get();
          std::string sv;
          while (!L.eof()) {
            char e = L.get();
            if (e == q) {
              if (L.peek() == q) { sv += L.get(); continue; }   // doubled quote
              break;
            }
            sv += e;
          }
          v.null = false;
          v.quoted = true;
          v.text = sv;
          it.values.push_back(v);
        } else {
          std::string tok;
          while (!L.eof()) {
            char e = L.peek();
            if (std::isspace((unsigned char)e) || e == ',' || e == '/' || e == '!' || e == '&') break;
            tok += L.get();
          }
          // r*value and r* (null) repeats
          const size_t star = tok.find('*');
          int rep = 1;
          if (star != std::string::npos) {
            char* end = nullptr;
            long r = std::strtol(tok.substr(0, star).c_str(), &end, 10);
            if (star == 0 || !end || *end != '\0' || r < 1) {
              err = "line " + std::to_string(L.line) + ": bad repeat count in '" + tok + "'";
              return -1;
            }
            rep = (int)r;
            tok = tok.substr(star + 1);
          }
          for (int k = 0; k < rep; ++k) {
            NValue w;
            w.null = tok.empty();
            w.text = tok;
            it.values.push_back(w);
          }
        }
        after_sep = false;
      }
      g.items.push_back(it);
    }
    if (!closed) { err = "group " + g.name + " is not terminated by '/'"; return -1; }
    out.push_back(g);
  }
  return 0;
}

// typed conversions of namelist values
static bool to_double(const NValue& v, double& out) {
  if (v.null || v.quoted) return false;
  std::string t = v.text;
  for (auto& c : t)
    if (c == 'd' || c == 'D') c = 'E';
  char* end = nullptr;
  errno = 0;
  double x = std::strtod(t.c_str(), &end);
  if (!end || *end != '\0' || t.empty()) return false;
  out = x;
  return true;
}
static bool to_int(const NValue& v, int& out) {
  if (v.null || v.quoted) return false;
  char* end = nullptr;
  long x = std::strtol(v.text.c_str(), &end, 10);
  if (!end || *end != '\0' || v.text.empty()) return false;
  out = (int)x;
  return true;
}
static bool to_bool(const NValue& v, int& out) {
  if (v.null || v.quoted) return false;
  std::string t = upper(v.text);
  size_t k = (t.size() > 0 && t[0] == '.') ? 1 : 0;
  if (k >= t.size()) return false;
  if (t[k] == 'T') { out = 1; return true; }
  if (t[k] == 'F') { out = 0; return true; }
  return false;
}

}  // namespace io
}  // namespace sflow

namespace sflow {
namespace io {

// ---------------------------------------------------------------------------
// namelist keys -> SflowParams / SflowRunInfo
// ---------------------------------------------------------------------------
enum Kind { K_INT, K_REAL, K_BOOL, K_STR, K_IARR, K_RARR, K_OFF, K_ZERO, K_ACCEPT, K_NOFILE };

struct Key {
  const char* group;
  const char* name;
  Kind kind;
  size_t off;     // offset in SflowParams (or SflowRunInfo when run == true)
  int n;          // array length
  bool run;
};

#define PK(g, n, k, f) {g, n, k, offsetof(SflowParams, f), 1, false}
#define PA(g, n, k, f, len) {g, n, k, offsetof(SflowParams, f), len, false}
#define RK(g, n, k, f, len) {g, n, k, offsetof(SflowRunInfo, f), len, true}
#define XK(g, n, k) {g, n, k, 0, 0, false}

static const Key kKeys[] = {
    // RUN_PARAMETERS (inpout_2d.f90:326-328)
    RK("RUN_PARAMETERS", "RUN_NAME", K_STR, run_name, (int)sizeof(((SflowRunInfo*)0)->run_name)),
    RK("RUN_PARAMETERS", "RESTART", K_BOOL, restart, 1),
    PK("RUN_PARAMETERS", "T_START", K_REAL, t_start),
    PK("RUN_PARAMETERS", "T_END", K_REAL, t_end),
    PK("RUN_PARAMETERS", "DT_OUTPUT", K_REAL, dt_output),
    RK("RUN_PARAMETERS", "OUTPUT_CONS_FLAG", K_BOOL, output_cons_flag, 1),
    RK("RUN_PARAMETERS", "OUTPUT_ESRI_FLAG", K_BOOL, output_esri_flag, 1),
    RK("RUN_PARAMETERS", "OUTPUT_PHYS_FLAG", K_BOOL, output_phys_flag, 1),
    RK("RUN_PARAMETERS", "OUTPUT_NETCDF_FLAG", K_BOOL, output_netcdf_flag, 1),
    RK("RUN_PARAMETERS", "OUTPUT_RUNOUT_FLAG", K_BOOL, output_runout_flag, 1),
    RK("RUN_PARAMETERS", "VERBOSE_LEVEL", K_INT, verbose_level, 1),
    XK("RUN_PARAMETERS", "SERIAL_FLAG", K_ACCEPT),
    // RESTART_PARAMETERS (:330-331); RESTART_FILE is the key of the
    // reference's own test inputs (see sflow_read_input in include/sflow.h)
    RK("RESTART_PARAMETERS", "RESTART_FILES", K_STR, restart_file, (int)sizeof(((SflowRunInfo*)0)->restart_file)),
    RK("RESTART_PARAMETERS", "RESTART_FILE", K_STR, restart_file, (int)sizeof(((SflowRunInfo*)0)->restart_file)),
    XK("RESTART_PARAMETERS", "N_RESTART_FILES", K_ACCEPT),
    XK("RESTART_PARAMETERS", "RELEASE_TIME", K_ACCEPT),
    XK("RESTART_PARAMETERS", "T_INIT", K_ACCEPT),
    PK("RESTART_PARAMETERS", "T_AMBIENT", K_REAL, T_ambient),
    XK("RESTART_PARAMETERS", "U_INIT", K_ACCEPT),
    XK("RESTART_PARAMETERS", "V_INIT", K_ACCEPT),
    XK("RESTART_PARAMETERS", "SED_VOL_PERC", K_ACCEPT),
    // NEWRUN_PARAMETERS (:333-338)
    PK("NEWRUN_PARAMETERS", "N_SOLID", K_INT, n_solid),
    RK("NEWRUN_PARAMETERS", "TOPOGRAPHY_FILE", K_STR, topography_file, (int)sizeof(((SflowRunInfo*)0)->topography_file)),
    PK("NEWRUN_PARAMETERS", "X0", K_REAL, x0),
    PK("NEWRUN_PARAMETERS", "Y0", K_REAL, y0),
    PK("NEWRUN_PARAMETERS", "COMP_CELLS_X", K_INT, comp_cells_x),
    PK("NEWRUN_PARAMETERS", "COMP_CELLS_Y", K_INT, comp_cells_y),
    PK("NEWRUN_PARAMETERS", "CELL_SIZE", K_REAL, cell_size),
    PK("NEWRUN_PARAMETERS", "RHEOLOGY_FLAG", K_BOOL, rheology_flag),
    PK("NEWRUN_PARAMETERS", "ALPHA_FLAG", K_BOOL, alpha_flag),
    PK("NEWRUN_PARAMETERS", "ENERGY_FLAG", K_BOOL, energy_flag),
    PK("NEWRUN_PARAMETERS", "LIQUID_FLAG", K_BOOL, liquid_flag),
    PK("NEWRUN_PARAMETERS", "RADIAL_SOURCE_FLAG", K_BOOL, radial_source_flag),
    PK("NEWRUN_PARAMETERS", "GAS_FLAG", K_BOOL, gas_flag),
    PK("NEWRUN_PARAMETERS", "SLOPE_CORRECTION_FLAG", K_BOOL, slope_correction_flag),
    PK("NEWRUN_PARAMETERS", "CURVATURE_TERM_FLAG", K_BOOL, curvature_term_flag),
    XK("NEWRUN_PARAMETERS", "N_ADD_GAS", K_ZERO),
    XK("NEWRUN_PARAMETERS", "COLLAPSING_VOLUME_FLAG", K_OFF),
    PK("NEWRUN_PARAMETERS", "TOPO_CHANGE_FLAG", K_BOOL, topo_change_flag),
    XK("NEWRUN_PARAMETERS", "SUBTRACT_INIT_FLAG", K_OFF),
    PK("NEWRUN_PARAMETERS", "BOTTOM_RADIAL_SOURCE_FLAG", K_BOOL, bottom_radial_source_flag),
    XK("NEWRUN_PARAMETERS", "VERTICAL_PROFILES_FLAG", K_OFF),
    XK("NEWRUN_PARAMETERS", "LATERAL_SOURCE_FLAG", K_OFF),
    XK("NEWRUN_PARAMETERS", "STOCHASTIC_FLAG", K_OFF),
    XK("NEWRUN_PARAMETERS", "PORE_PRESSURE_FLAG", K_OFF),
    // NUMERIC_PARAMETERS (:343-344)
    XK("NUMERIC_PARAMETERS", "SOLVER_SCHEME", K_STR),
    PK("NUMERIC_PARAMETERS", "DT0", K_REAL, dt0),
    PK("NUMERIC_PARAMETERS", "MAX_DT", K_REAL, max_dt),
    PK("NUMERIC_PARAMETERS", "CFL", K_REAL, cfl),
    PA("NUMERIC_PARAMETERS", "LIMITER", K_IARR, limiter, SFLOW_MAX_VARS),
    PK("NUMERIC_PARAMETERS", "THETA", K_REAL, theta),
    PK("NUMERIC_PARAMETERS", "RECONSTR_COEFF", K_REAL, reconstr_coeff),
    XK("NUMERIC_PARAMETERS", "INTERFACES_RELAXATION", K_OFF),
    PK("NUMERIC_PARAMETERS", "N_RK", K_INT, n_rk),
    // EXPL_TERMS_PARAMETERS (:346)
    PK("EXPL_TERMS_PARAMETERS", "GRAV", K_REAL, grav),
    // RADIAL_SOURCE_PARAMETERS (:348-352)
    PK("RADIAL_SOURCE_PARAMETERS", "X_SOURCE", K_REAL, x_source),
    PK("RADIAL_SOURCE_PARAMETERS", "Y_SOURCE", K_REAL, y_source),
    PK("RADIAL_SOURCE_PARAMETERS", "R_SOURCE", K_REAL, r_source),
    PK("RADIAL_SOURCE_PARAMETERS", "R2_SOURCE", K_REAL, r2_source),
    PK("RADIAL_SOURCE_PARAMETERS", "ANGLE_SOURCE", K_REAL, angle_source),
    PK("RADIAL_SOURCE_PARAMETERS", "VEL_SOURCE", K_REAL, vel_source),
    PK("RADIAL_SOURCE_PARAMETERS", "T_SOURCE", K_REAL, T_source),
    PK("RADIAL_SOURCE_PARAMETERS", "H_SOURCE", K_REAL, h_source),
    PA("RADIAL_SOURCE_PARAMETERS", "ALPHAS_SOURCE", K_RARR, alphas_source, SFLOW_MAX_SOLID),
    XK("RADIAL_SOURCE_PARAMETERS", "ALPHAL_SOURCE", K_ACCEPT),
    XK("RADIAL_SOURCE_PARAMETERS", "ALPHAG_SOURCE", K_ACCEPT),
    PA("RADIAL_SOURCE_PARAMETERS", "TIME_PARAM", K_RARR, time_param, 4),
    XK("RADIAL_SOURCE_PARAMETERS", "RI_SOURCE", K_ACCEPT),
    PK("RADIAL_SOURCE_PARAMETERS", "MFR_SOURCE", K_REAL, mfr_source),
    XK("RADIAL_SOURCE_PARAMETERS", "XS_SOURCE", K_ACCEPT),
    XK("RADIAL_SOURCE_PARAMETERS", "XL_SOURCE", K_ACCEPT),
    XK("RADIAL_SOURCE_PARAMETERS", "XG_SOURCE", K_ACCEPT),
    PK("RADIAL_SOURCE_PARAMETERS", "AZIMUTH_SOURCE", K_REAL, azimuth_source),
    PK("RADIAL_SOURCE_PARAMETERS", "ARC_WIDTH_SOURCE", K_REAL, arc_width_source),
    PK("RADIAL_SOURCE_PARAMETERS", "N_INTERVALS", K_INT, n_intervals),
    PA("RADIAL_SOURCE_PARAMETERS", "T_INTERVALS", K_RARR, t_intervals, SFLOW_MAX_INTERVALS),
    PA("RADIAL_SOURCE_PARAMETERS", "VEL_INTERVALS", K_RARR, vel_intervals, SFLOW_MAX_INTERVALS),
    // TEMPERATURE_PARAMETERS (:368-370): cooling terms, off at their defaults
    XK("TEMPERATURE_PARAMETERS", "EMISSIVITY", K_ZERO),
    XK("TEMPERATURE_PARAMETERS", "ATM_HEAT_TRANSF_COEFF", K_ZERO),
    XK("TEMPERATURE_PARAMETERS", "THERMAL_CONDUCTIVITY", K_ZERO),
    XK("TEMPERATURE_PARAMETERS", "EXP_AREA_FRACT", K_ACCEPT),
    XK("TEMPERATURE_PARAMETERS", "C_P", K_ACCEPT),
    XK("TEMPERATURE_PARAMETERS", "ENNE", K_ACCEPT),
    XK("TEMPERATURE_PARAMETERS", "EMME", K_ACCEPT),
    XK("TEMPERATURE_PARAMETERS", "T_ENV", K_ACCEPT),
    XK("TEMPERATURE_PARAMETERS", "T_GROUND", K_ACCEPT),
    // RHEOLOGY_PARAMETERS (:372-374): models 1 and 6
    PK("RHEOLOGY_PARAMETERS", "RHEOLOGY_MODEL", K_INT, rheology_model),
    PK("RHEOLOGY_PARAMETERS", "MU", K_REAL, mu),
    PK("RHEOLOGY_PARAMETERS", "XI", K_REAL, xi),
    PK("RHEOLOGY_PARAMETERS", "FRICTION_FACTOR", K_REAL, friction_factor),
    XK("RHEOLOGY_PARAMETERS", "TAU", K_ACCEPT), XK("RHEOLOGY_PARAMETERS", "NU_REF", K_ACCEPT),
    XK("RHEOLOGY_PARAMETERS", "VISC_PAR", K_ACCEPT), XK("RHEOLOGY_PARAMETERS", "T_REF", K_ACCEPT),
    XK("RHEOLOGY_PARAMETERS", "ALPHA2", K_ACCEPT), XK("RHEOLOGY_PARAMETERS", "BETA2", K_ACCEPT),
    XK("RHEOLOGY_PARAMETERS", "ALPHA1_REF", K_ACCEPT), XK("RHEOLOGY_PARAMETERS", "BETA1", K_ACCEPT),
    XK("RHEOLOGY_PARAMETERS", "KAPPA", K_ACCEPT), XK("RHEOLOGY_PARAMETERS", "N_TD", K_ACCEPT),
    XK("RHEOLOGY_PARAMETERS", "TAU0", K_ACCEPT), XK("RHEOLOGY_PARAMETERS", "MU_0", K_ACCEPT),
    XK("RHEOLOGY_PARAMETERS", "MU_INF", K_ACCEPT), XK("RHEOLOGY_PARAMETERS", "FR_0", K_ACCEPT),
    XK("RHEOLOGY_PARAMETERS", "U_W", K_ACCEPT), PK("RHEOLOGY_PARAMETERS", "MU_S", K_REAL, mu_s),
    PK("RHEOLOGY_PARAMETERS", "MU_2", K_REAL, mu_2), PK("RHEOLOGY_PARAMETERS", "I_0", K_REAL, I_0),
    PK("RHEOLOGY_PARAMETERS", "MUI_INF", K_REAL, muI_inf),
    // SOLID_TRANSPORT_PARAMETERS (inpout_2d.f90:1033-1037)
    PA("SOLID_TRANSPORT_PARAMETERS", "RHO_S", K_RARR, rho_s, SFLOW_MAX_SOLID),
    PA("SOLID_TRANSPORT_PARAMETERS", "DIAM_S", K_RARR, diam_s, SFLOW_MAX_SOLID),
    PA("SOLID_TRANSPORT_PARAMETERS", "SP_HEAT_S", K_RARR, sp_heat_s, SFLOW_MAX_SOLID),
    XK("SOLID_TRANSPORT_PARAMETERS", "SPHERICITY_S", K_ACCEPT),
    PK("SOLID_TRANSPORT_PARAMETERS", "EROSION_COEFF", K_REAL, erosion_coeff),
    PK("SOLID_TRANSPORT_PARAMETERS", "ERODIBLE_POROSITY", K_REAL, erodible_porosity),
    PK("SOLID_TRANSPORT_PARAMETERS", "SETTLING_FLAG", K_BOOL, settling_flag),
    PK("SOLID_TRANSPORT_PARAMETERS", "T_ERODIBLE", K_REAL, T_erodible),
    // the erodible layer per cell comes through sflow_set_erodible
    XK("SOLID_TRANSPORT_PARAMETERS", "ERODIBLE_FILE", K_NOFILE),
    PA("SOLID_TRANSPORT_PARAMETERS", "ERODIBLE_FRACT", K_RARR, erodible_fract, SFLOW_MAX_SOLID),
    PK("SOLID_TRANSPORT_PARAMETERS", "ALPHASTOT_MIN", K_REAL, alphastot_min),
    PK("SOLID_TRANSPORT_PARAMETERS", "INITIAL_ERODIBLE_THICKNESS", K_REAL, initial_erodible_thickness),
    PK("SOLID_TRANSPORT_PARAMETERS", "ERODIBLE_DEPOSIT_FLAG", K_BOOL, erodible_deposit_flag),
    PK("SOLID_TRANSPORT_PARAMETERS", "MAXIMUM_SOLID_PACKING", K_REAL, maximum_solid_packing),
    PK("SOLID_TRANSPORT_PARAMETERS", "A_DRAG", K_REAL, A_drag),
    PK("SOLID_TRANSPORT_PARAMETERS", "B_DRAG", K_REAL, B_drag),
    PK("SOLID_TRANSPORT_PARAMETERS", "COLLECTIVE_SETTLING_FLAG", K_BOOL, collective_settling_flag),
    // GAS_TRANSPORT_PARAMETERS (:1039-1042)
    PK("GAS_TRANSPORT_PARAMETERS", "SP_HEAT_A", K_REAL, sp_heat_a),
    PK("GAS_TRANSPORT_PARAMETERS", "SP_GAS_CONST_A", K_REAL, sp_gas_const_a),
    PK("GAS_TRANSPORT_PARAMETERS", "KIN_VISC_A", K_REAL, kin_visc_a),
    PK("GAS_TRANSPORT_PARAMETERS", "PRES", K_REAL, pres),
    PK("GAS_TRANSPORT_PARAMETERS", "T_AMBIENT", K_REAL, T_ambient),
    PK("GAS_TRANSPORT_PARAMETERS", "ENTRAINMENT_FLAG", K_BOOL, entrainment_flag),
    XK("GAS_TRANSPORT_PARAMETERS", "SP_HEAT_G", K_ACCEPT),
    XK("GAS_TRANSPORT_PARAMETERS", "SP_GAS_CONST_G", K_ACCEPT),
    XK("GAS_TRANSPORT_PARAMETERS", "LIQUID_VAPORIZATION_FLAG", K_OFF),
    XK("GAS_TRANSPORT_PARAMETERS", "WATER_LEVEL", K_ACCEPT),
    XK("GAS_TRANSPORT_PARAMETERS", "GAMMA_STEAM", K_ACCEPT),
    XK("GAS_TRANSPORT_PARAMETERS", "SUTHERLAND_FLAG", K_OFF),
    XK("GAS_TRANSPORT_PARAMETERS", "TREF_SUTH", K_ACCEPT),
    XK("GAS_TRANSPORT_PARAMETERS", "MUREF_SUTH", K_ACCEPT),
    XK("GAS_TRANSPORT_PARAMETERS", "S_MU", K_ACCEPT),
    // LIQUID_TRANSPORT_PARAMETERS (:379-380)
    PK("LIQUID_TRANSPORT_PARAMETERS", "SP_HEAT_L", K_REAL, sp_heat_l),
    PK("LIQUID_TRANSPORT_PARAMETERS", "RHO_L", K_REAL, rho_l),
    PK("LIQUID_TRANSPORT_PARAMETERS", "KIN_VISC_L", K_REAL, kin_visc_l),
    PK("LIQUID_TRANSPORT_PARAMETERS", "LOSS_RATE", K_REAL, loss_rate),
    // VULNERABILITY_TABLE_PARAMETERS (:380)
    PA("VULNERABILITY_TABLE_PARAMETERS", "THICKNESS_LEVELS0", K_RARR, thickness_levels, SFLOW_MAX_LEVELS),
    PA("VULNERABILITY_TABLE_PARAMETERS", "DYN_PRES_LEVELS0", K_RARR, dyn_pres_levels, SFLOW_MAX_LEVELS),
    // output-only groups: accepted, not used by the solver
    XK("RUNOUT_PARAMETERS", "X0_RUNOUT", K_ACCEPT), XK("RUNOUT_PARAMETERS", "Y0_RUNOUT", K_ACCEPT),
    XK("RUNOUT_PARAMETERS", "DT_RUNOUT", K_ACCEPT), XK("RUNOUT_PARAMETERS", "EPS_STOP", K_ACCEPT),
    XK("RUNOUT_PARAMETERS", "ALPHAS_THRESHOLD", K_ACCEPT),
};

// boundary-condition designators of *_BOUNDARY_CONDITIONS (inpout_2d.f90:1017-1031)
struct BcVar {
  const char* stem;   // key = stem + side letter
  int first;          // first variable index (0-based) it maps to
  bool array;         // one element per solid class
};
static const BcVar kBcVars[] = {{"H_BC", 0, false}, {"HU_BC", 1, false}, {"HV_BC", 2, false},
                                {"T_BC", 3, false}, {"HALPHAS_BC", 4, true}, {"ALPHAS_BC", 4, true}};

template <class T>
static T& field(void* base, size_t off, int i = 0) {
  return reinterpret_cast<T*>(reinterpret_cast<char*>(base) + off)[i];
}

static std::string where(const NGroup& g, const NItem& it) {
  return "line " + std::to_string(it.line) + " (" + g.name + ": " + it.name + ")";
}

// one group's items onto params / run; BC groups onto bcs
static int apply_group(NGroup& g, SflowParams* p, SflowRunInfo* run, SflowBC bcs[4][2][SFLOW_MAX_VARS],
                       std::string& scheme, std::string& err) {
  g.used = true;
  static const char* sides = "WESN";
  int side = -1;
  if (g.name == "WEST_BOUNDARY_CONDITIONS") side = 0;
  if (g.name == "EAST_BOUNDARY_CONDITIONS") side = 1;
  if (g.name == "SOUTH_BOUNDARY_CONDITIONS") side = 2;
  if (g.name == "NORTH_BOUNDARY_CONDITIONS") side = 3;
  for (NItem& it : g.items) {
    if (side >= 0) {
      // <stem><side>[(i)]%FLAG|VALUE ; [0] HALPHAS form, [1] ALPHAS form
      const BcVar* bv = nullptr;
      int form = 0;
      for (const BcVar& b : kBcVars)
        if (it.name == std::string(b.stem) + sides[side]) {
          bv = &b;
          form = (std::string(b.stem) == "ALPHAS_BC") ? 1 : 0;
        }
      if (!bv) {
        err = where(g, it) + ": boundary condition not supported by the GPU path";
        return SFLOW_EINVAL;
      }
      if (it.comp != "FLAG" && it.comp != "VALUE") {
        err = where(g, it) + ": expected %FLAG or %VALUE";
        return SFLOW_EINVAL;
      }
      const int nel = bv->array ? SFLOW_MAX_SOLID : 1;
      int k0 = it.index > 0 ? it.index - 1 : 0;
      for (const NValue& v : it.values) {
        if (k0 >= nel) { err = where(g, it) + ": too many values"; return SFLOW_EINVAL; }
        if (!v.null) {
          SflowBC& b = bcs[side][form][bv->first + k0];
          if (it.comp == "FLAG") {
            int x;
            if (!to_int(v, x)) { err = where(g, it) + ": integer expected"; return SFLOW_EINVAL; }
            b.flag = x;
          } else {
            double x;
            if (!to_double(v, x)) { err = where(g, it) + ": real expected"; return SFLOW_EINVAL; }
            b.value = x;
          }
        }
        ++k0;
      }
      continue;
    }
    const Key* key = nullptr;
    for (const Key& k : kKeys)
      if (g.name == k.group && it.name == k.name) key = &k;
    if (!key) {
      bool known_group = false;
      for (const Key& k : kKeys)
        if (g.name == k.group) known_group = true;
      err = where(g, it) + (known_group ? ": unknown key" : ": group not supported by the GPU path");
      return SFLOW_EINVAL;
    }
    if (!it.comp.empty()) { err = where(g, it) + ": unexpected %component"; return SFLOW_EINVAL; }
    void* base = key->run ? (void*)run : (void*)p;
    const int k0 = it.index > 0 ? it.index - 1 : 0;
    switch (key->kind) {
      case K_INT:
      case K_BOOL:
      case K_REAL:
      case K_STR: {
        if (it.values.size() != 1 || it.index > 1) {
          // a scalar given one value (a trailing null is allowed)
          if (!(it.values.size() == 2 && it.values[1].null)) {
            err = where(g, it) + ": one value expected";
            return SFLOW_EINVAL;
          }
        }
        const NValue& v = it.values[0];
        if (v.null) break;
        if (std::string(key->name) == "SOLVER_SCHEME") {
          scheme = upper(v.text);
          while (!scheme.empty() && scheme.back() == ' ') scheme.pop_back();
          break;
        }
        if (key->kind == K_INT) {
          int x;
          if (!to_int(v, x)) { err = where(g, it) + ": integer expected"; return SFLOW_EINVAL; }
          field<int32_t>(base, key->off) = x;
        } else if (key->kind == K_BOOL) {
          int x;
          if (!to_bool(v, x)) { err = where(g, it) + ": logical expected"; return SFLOW_EINVAL; }
          field<int32_t>(base, key->off) = x;
        } else if (key->kind == K_REAL) {
          double x;
          if (!to_double(v, x)) { err = where(g, it) + ": real expected"; return SFLOW_EINVAL; }
          field<double>(base, key->off) = x;
        } else {
          std::string t = v.text;
          while (!t.empty() && t.back() == ' ') t.pop_back();
          if ((int)t.size() >= key->n) { err = where(g, it) + ": string too long"; return SFLOW_EINVAL; }
          char* dst = &field<char>(base, key->off);
          std::memset(dst, 0, key->n);
          std::memcpy(dst, t.data(), t.size());
        }
        break;
      }
      case K_IARR:
      case K_RARR: {
        int k = k0;
        for (const NValue& v : it.values) {
          if (k >= key->n) {
            if (v.null) continue;
            err = where(g, it) + ": more values than the GPU path supports";
            return SFLOW_EINVAL;
          }
          if (!v.null) {
            if (key->kind == K_IARR) {
              int x;
              if (!to_int(v, x)) { err = where(g, it) + ": integer expected"; return SFLOW_EINVAL; }
              field<int32_t>(base, key->off, k) = x;
            } else {
              double x;
              if (!to_double(v, x)) { err = where(g, it) + ": real expected"; return SFLOW_EINVAL; }
              field<double>(base, key->off, k) = x;
            }
          }
          ++k;
        }
        break;
      }
      case K_OFF:
        for (const NValue& v : it.values) {
          int x = 0;
          if (v.null) continue;
          if (!to_bool(v, x)) { err = where(g, it) + ": logical expected"; return SFLOW_EINVAL; }
          if (x) { err = where(g, it) + " = T: not supported by the GPU path"; return SFLOW_EINVAL; }
        }
        break;
      case K_ZERO:
        for (const NValue& v : it.values) {
          double x = 0.0;
          if (v.null) continue;
          if (!to_double(v, x)) { err = where(g, it) + ": number expected"; return SFLOW_EINVAL; }
          if (x != 0.0) { err = where(g, it) + " /= 0: not supported by the GPU path"; return SFLOW_EINVAL; }
        }
        break;
      case K_ACCEPT:
        break;
      case K_NOFILE:
        for (const NValue& v : it.values) {
          if (v.null) continue;
          std::string t = v.text;
          while (!t.empty() && t.back() == ' ') t.pop_back();
          if (!t.empty()) {
            err = where(g, it) + ": not read by this driver (give the field with sflow_set_erodible)";
            return SFLOW_EINVAL;
          }
        }
        break;
    }
  }
  return SFLOW_OK;
}

static NGroup* find_group(std::vector<NGroup>& gs, const char* name) {
  for (NGroup& g : gs)
    if (g.name == name) return &g;   // the first occurrence, as a READ after REWIND
  return nullptr;
}

int read_input(const char* path, SflowParams* p, SflowRunInfo* run) {
  if (!path || !p || !run) return fail(SFLOW_EINVAL, "NULL argument");
  std::ifstream in(path, std::ios::binary);
  if (!in) return fail(SFLOW_EINVAL, std::string("input file not found: ") + path);
  std::stringstream ss;
  ss << in.rdbuf();
  const std::string text = ss.str();
  std::vector<NGroup> gs;
  std::string err;
  if (parse_namelists(text, gs, err) != 0) return fail(SFLOW_EINVAL, err);

  // init_param defaults (inpout_2d.f90:408-970)
  sflow_default_params(p);
  std::memset(run, 0, sizeof(*run));
  std::snprintf(run->run_name, sizeof(run->run_name), "default");
  std::snprintf(run->topography_file, sizeof(run->topography_file), "topography_dem.asc");
  p->n_solid = -1;
  int n_add_gas_seen = 0;
  (void)n_add_gas_seen;
  // boundary conditions as read: flag -1 = not given; [side][form][var]
  SflowBC bcs[4][2][SFLOW_MAX_VARS];
  for (auto& a : bcs)
    for (auto& b : a)
      for (auto& c : b) {
        c.flag = -1;
        c.pad = 0;
        c.value = 0.0;
      }
  std::string scheme = "KT";

  auto need = [&](const char* name) -> NGroup* {
    NGroup* g = find_group(gs, name);
    if (!g) fail(SFLOW_EINVAL, std::string("namelist ") + name + " missing from " + path);
    return g;
  };
  auto apply = [&](NGroup* g) -> int {
    int rc = apply_group(*g, p, run, bcs, scheme, err);
    if (rc != SFLOW_OK) return fail(rc, err);
    return SFLOW_OK;
  };
  // read_param order (inpout_2d.f90:986-): run, newrun, restart, numeric, BCs, ...
  const char* required[] = {"RUN_PARAMETERS", "NEWRUN_PARAMETERS", "NUMERIC_PARAMETERS", "EXPL_TERMS_PARAMETERS"};
  for (const char* name : required) {
    NGroup* g = need(name);
    if (!g) return SFLOW_EINVAL;
    if (apply(g) != SFLOW_OK) return SFLOW_EINVAL;
  }
  if (p->n_solid < 1 || p->n_solid > 3) return fail(SFLOW_EINVAL, "N_SOLID must be 1, 2 or 3 on the GPU path");
  if (run->restart) {
    NGroup* g = need("RESTART_PARAMETERS");
    if (!g || apply(g) != SFLOW_OK) return SFLOW_EINVAL;
    if (!run->restart_file[0]) return fail(SFLOW_EINVAL, "RESTART_PARAMETERS: no restart file given");
  } else {
    return fail(SFLOW_EINVAL,
                "RESTART = F (a new run from INITIAL_CONDITIONS) is not supported: start from a restart file");
  }
  if (scheme == "KT") p->solver_scheme = SFLOW_SCHEME_KT;
  else if (scheme == "UP") p->solver_scheme = SFLOW_SCHEME_UP;
  else return fail(SFLOW_EINVAL, "SOLVER_SCHEME " + scheme + " is not supported (KT or UP)");
  const int nx = p->comp_cells_x, ny = p->comp_cells_y;
  if (nx > 1) {
    for (const char* name : {"WEST_BOUNDARY_CONDITIONS", "EAST_BOUNDARY_CONDITIONS"}) {
      NGroup* g = need(name);
      if (!g || apply(g) != SFLOW_OK) return SFLOW_EINVAL;
    }
  }
  if (ny > 1) {
    for (const char* name : {"SOUTH_BOUNDARY_CONDITIONS", "NORTH_BOUNDARY_CONDITIONS"}) {
      NGroup* g = need(name);
      if (!g || apply(g) != SFLOW_OK) return SFLOW_EINVAL;
    }
  }
  const char* optional[] = {"TEMPERATURE_PARAMETERS", "RHEOLOGY_PARAMETERS", "SOLID_TRANSPORT_PARAMETERS",
                            "GAS_TRANSPORT_PARAMETERS", "LIQUID_TRANSPORT_PARAMETERS",
                            "RADIAL_SOURCE_PARAMETERS", "VULNERABILITY_TABLE_PARAMETERS", "RUNOUT_PARAMETERS"};
  for (const char* name : optional) {
    NGroup* g = find_group(gs, name);
    if (g && apply(g) != SFLOW_OK) return SFLOW_EINVAL;
  }
  if (p->rheology_flag && !find_group(gs, "RHEOLOGY_PARAMETERS"))
    return fail(SFLOW_EINVAL, "namelist RHEOLOGY_PARAMETERS missing (RHEOLOGY_FLAG = T)");
  if (p->gas_flag && !find_group(gs, "GAS_TRANSPORT_PARAMETERS"))
    return fail(SFLOW_EINVAL, "namelist GAS_TRANSPORT_PARAMETERS missing (GAS_FLAG = T)");
  if (p->liquid_flag && !find_group(gs, "LIQUID_TRANSPORT_PARAMETERS"))
    return fail(SFLOW_EINVAL, "namelist LIQUID_TRANSPORT_PARAMETERS missing (LIQUID_FLAG = T)");
  if (p->radial_source_flag && !find_group(gs, "RADIAL_SOURCE_PARAMETERS"))
    return fail(SFLOW_EINVAL, "namelist RADIAL_SOURCE_PARAMETERS missing (RADIAL_SOURCE_FLAG = T)");
  if (!find_group(gs, "SOLID_TRANSPORT_PARAMETERS"))
    return fail(SFLOW_EINVAL, "namelist SOLID_TRANSPORT_PARAMETERS missing");
  for (const NGroup& g : gs) {
    if (g.used) continue;
    bool known = false;
    for (const Key& k : kKeys)
      if (g.name == k.group) known = true;
    if (g.name == "RESTART_PARAMETERS" || g.name == "INITIAL_CONDITIONS" ||
        g.name.find("_BOUNDARY_CONDITIONS") != std::string::npos)
      known = true;
    if (!known) return fail(SFLOW_EINVAL, "namelist " + g.name + " is not supported by the GPU path");
  }

  // boundary conditions (inpout_2d.f90:2313-3104): the checks and the
  // reference's assignments, including its quirks: hv on the west side is
  // set to (1, 0) whenever ny > 1 (the ELSE of 2356-2372 belongs to the
  // flag test), on the other sides only when the direction is absent
  const int ns = p->n_solid, nv = 4 + ns;
  static const char* side_name[4] = {"WEST", "EAST", "SOUTH", "NORTH"};
  const int form = p->alpha_flag ? 1 : 0;
  for (int s = 0; s < 4; ++s) {
    const bool present = (s < 2) ? nx > 1 : ny > 1;
    SflowBC* b = bcs[s][0];
    SflowBC* ba = bcs[s][1];
    if (!present) {
      for (int i = 0; i < SFLOW_MAX_VARS; ++i) {
        p->bc[s][i].flag = 1;
        p->bc[s][i].value = 0.0;
      }
      continue;
    }
    const std::string sn = side_name[s];
    if (b[0].flag == -1) return fail(SFLOW_EINVAL, sn + "_BOUNDARY_CONDITIONS: B.C. for h not set properly");
    if (nx > 1) {
      if (b[1].flag == -1) return fail(SFLOW_EINVAL, sn + "_BOUNDARY_CONDITIONS: B.C. for hu not set properly");
    } else {
      b[1].flag = 1;
      b[1].value = 0.0;
    }
    if (ny > 1) {
      if (b[2].flag == -1) return fail(SFLOW_EINVAL, sn + "_BOUNDARY_CONDITIONS: B.C. for hv not set properly");
      if (s == 0) {
        b[2].flag = 1;
        b[2].value = 0.0;
      }
    } else {
      b[2].flag = 1;
      b[2].value = 0.0;
    }
    const SflowBC* sol = form ? ba : b;
    for (int i = 0; i < ns; ++i)
      if (sol[4 + i].flag == -1)
        return fail(SFLOW_EINVAL, sn + "_BOUNDARY_CONDITIONS: B.C. for sediment concentration not set properly");
    if (b[3].flag == -1) return fail(SFLOW_EINVAL, sn + "_BOUNDARY_CONDITIONS: B.C. for temperature not set properly");
    for (int i = 0; i < 4; ++i) p->bc[s][i] = b[i];
    for (int i = 0; i < ns; ++i) p->bc[s][4 + i] = sol[4 + i];
    for (int i = nv; i < SFLOW_MAX_VARS; ++i) {
      p->bc[s][i].flag = 1;
      p->bc[s][i].value = 0.0;
    }
  }
  p->precision = SFLOW_PREC_FP64;
  g_io_err.clear();
  return SFLOW_OK;
}

}  // namespace io
}  // namespace sflow

namespace sflow {
namespace io {

// ---------------------------------------------------------------------------
// Fortran formatted output
// ---------------------------------------------------------------------------
// Ew.d: [-]0.d1..dd E+xx (|exponent| <= 99) or [-]0.d1..dd+xxx (<= 999),
// right-justified in w characters (asterisks when it does not fit)
static void fmt_E(std::string& out, double v, int w, int d) {
  char m[64];
  std::string s;
  if (std::isnan(v)) {
    s = "NaN";
  } else if (std::isinf(v)) {
    s = v < 0 ? "-Infinity" : "Infinity";
  } else {
    const bool neg = std::signbit(v);
    std::string digits;
    int e10 = 0;
    if (v == 0.0) {
      digits.assign(d, '0');
      e10 = 0;
    } else {
      std::snprintf(m, sizeof(m), "%.*e", d - 1, std::fabs(v));   // d significant digits
      const char* pe = std::strchr(m, 'e');
      for (const char* c = m; c < pe; ++c)
        if (std::isdigit((unsigned char)*c)) digits += *c;
      e10 = std::atoi(pe + 1) + 1;   // 0.ddd form
    }
    s = neg ? "-0." : "0.";
    s += digits;
    char ex[16];
    const int ae = e10 < 0 ? -e10 : e10;
    if (ae <= 99) std::snprintf(ex, sizeof(ex), "E%c%02d", e10 < 0 ? '-' : '+', ae);
    else if (ae <= 999) std::snprintf(ex, sizeof(ex), "%c%03d", e10 < 0 ? '-' : '+', ae);
    else { out.append(w, '*'); return; }
    s += ex;
    if ((int)s.size() > w && s[neg ? 1 : 0] == '0') s.erase(neg ? 1 : 0, 1);   // drop the optional zero
  }
  if ((int)s.size() > w) { out.append(w, '*'); return; }
  out.append(w - s.size(), ' ');
  out += s;
}

// ESw.dE2: [-]d.d1..dd E+xx, right-justified; an exponent beyond two digits
// does not fit E2 and prints w asterisks
static void fmt_ES(std::string& out, double v, int w, int d) {
  char m[64];
  std::string s;
  if (std::isnan(v)) {
    s = "NaN";
  } else if (std::isinf(v)) {
    s = v < 0 ? "-Infinity" : "Infinity";
  } else {
    std::snprintf(m, sizeof(m), "%.*e", d, v);
    char* pe = std::strchr(m, 'e');
    const int e10 = std::atoi(pe + 1);
    const int ae = e10 < 0 ? -e10 : e10;
    if (ae > 99) { out.append(w, '*'); return; }
    *pe = '\0';
    char ex[8];
    std::snprintf(ex, sizeof(ex), "E%c%02d", e10 < 0 ? '-' : '+', ae);
    s = std::string(m) + ex;
  }
  if ((int)s.size() > w) { out.append(w, '*'); return; }
  out.append(w - s.size(), ' ');
  out += s;
}

// a list-directed WRITE (unit, *) ' ' record: a leading blank, then the blank
static const char* kBlankRecord = "  \n";

// x_comp / y_comp (geometry_2d.f90:312-327)
static void cell_centres(const SflowParams* p, std::vector<double>& xc, std::vector<double>& yc) {
  const int nx = p->comp_cells_x, ny = p->comp_cells_y;
  const double dx = nx > 1 ? p->cell_size : 1.0, dy = ny > 1 ? p->cell_size : 1.0;
  xc.resize(nx);
  yc.resize(ny);
  for (int j = 0; j < nx; ++j) xc[j] = 0.5 * ((p->x0 + (double)j * dx) + (p->x0 + (double)(j + 1) * dx));
  for (int k = 0; k < ny; ++k) yc[k] = 0.5 * ((p->y0 + (double)k * dy) + (p->y0 + (double)(k + 1) * dy));
}

// lettera (inpout_2d.f90:6893-6912): four characters, digits for k < 10000
static std::string lettera(int k) {
  const int ithou = k / 1000, ihund = (k - ithou * 1000) / 100, iten = (k - ithou * 1000 - ihund * 100) / 10;
  const int ione = k - ithou * 1000 - ihund * 100 - iten * 10;
  std::string s;
  s += (char)(ithou + 48);
  s += (char)(ihund + 48);
  s += (char)(iten + 48);
  s += (char)(ione + 48);
  return s;
}

static int write_file(const char* path, const std::string& text) {
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(SFLOW_EINVAL, std::string("cannot open for writing: ") + path);
  const size_t n = std::fwrite(text.data(), 1, text.size(), f);
  const int rc = std::fclose(f);
  if (n != text.size() || rc != 0) return fail(SFLOW_EINVAL, std::string("write failed: ") + path);
  return SFLOW_OK;
}

// .q_2d (inpout_2d.f90:6000-6110): per cell x, y, q(1:n_vars) as
// '(2e20.12,100(e20.12))', rows of constant y separated by a blank record,
// two blank records at the end.  Values below 1e-20 in magnitude are set to
// zero in q itself first, as the reference does with its state.
int write_q2d(const char* path, const SflowParams* p, double* q) {
  if (!path || !p || !q) return fail(SFLOW_EINVAL, "NULL argument");
  const int nx = p->comp_cells_x, ny = p->comp_cells_y, nv = 4 + p->n_solid;
  std::vector<double> xc, yc;
  cell_centres(p, xc, yc);
  std::string out;
  out.reserve((size_t)nx * ny * 20 * (nv + 2) + 64 * ny);
  for (int k = 0; k < ny; ++k) {
    for (int j = 0; j < nx; ++j) {
      double* qc = q + ((size_t)k * nx + j) * nv;
      for (int i = 0; i < nv; ++i)
        if (std::fabs(qc[i]) < 1.0e-20) qc[i] = 0.0;
      fmt_E(out, xc[j], 20, 12);
      fmt_E(out, yc[k], 20, 12);
      for (int i = 0; i < nv; ++i) fmt_E(out, qc[i], 20, 12);
      out += '\n';
    }
    out += kBlankRecord;
  }
  out += kBlankRecord;
  out += kBlankRecord;
  return write_file(path, out);
}

// Ew.d formatted input field (blanks ignored, an all-blank field is zero,
// no decimal point: the last d digits are the fraction, exponent letter E or
// D or a signed exponent alone)
static bool read_E_field(const char* f, int w, int d, double& out) {
  std::string t;
  for (int i = 0; i < w && f[i] && f[i] != '\n' && f[i] != '\r'; ++i)
    if (f[i] != ' ' && f[i] != '\t') t += f[i];
  if (t.empty()) { out = 0.0; return true; }
  size_t i = 0;
  std::string mant;
  if (t[i] == '+' || t[i] == '-') mant += t[i++];
  bool point = false;
  std::string digs;
  while (i < t.size() && (std::isdigit((unsigned char)t[i]) || t[i] == '.')) {
    if (t[i] == '.') {
      if (point) return false;
      point = true;
    }
    digs += t[i++];
  }
  long ex = 0;
  if (i < t.size()) {
    if (t[i] == 'E' || t[i] == 'e' || t[i] == 'D' || t[i] == 'd') ++i;
    if (i >= t.size()) return false;
    char* end = nullptr;
    ex = std::strtol(t.c_str() + i, &end, 10);
    if (!end || *end != '\0') return false;
  }
  if (digs.empty() || digs == ".") return false;
  if (!point) ex -= d;
  std::string num = mant + digs + "e" + std::to_string(ex);
  char* end = nullptr;
  out = std::strtod(num.c_str(), &end);
  return end && *end == '\0';
}

// .q_2d restart (inpout_2d.f90:5674-5722): the reference's READ with
// '(2e20.12,100(e20.12))' per cell and one skipped record per row; cells with
// q(1) <= 0 are zeroed, negative solid masses are set to zero; the output
// index is the number in the four characters before the last '.'
int read_q2d(const char* path, const SflowParams* p, double* q, int32_t* output_idx) {
  if (!path || !p || !q) return fail(SFLOW_EINVAL, "NULL argument");
  std::ifstream in(path, std::ios::binary);
  if (!in) return fail(SFLOW_EINVAL, std::string("restart file not found: ") + path);
  const int nx = p->comp_cells_x, ny = p->comp_cells_y, ns = p->n_solid, nv = 4 + ns;
  std::string line;
  int lineno = 0;
  for (int k = 0; k < ny; ++k) {
    for (int j = 0; j < nx; ++j) {
      if (!std::getline(in, line)) return fail(SFLOW_EINVAL, std::string(path) + ": end of file in the cell records");
      ++lineno;
      line.resize(std::max<size_t>(line.size(), (size_t)20 * (nv + 2)), ' ');   // PAD = 'YES'
      double* qc = q + ((size_t)k * nx + j) * nv;
      for (int i = 0; i < nv; ++i) {
        double v;
        if (!read_E_field(line.c_str() + 20 * (2 + i), 20, 12, v))
          return fail(SFLOW_EINVAL, std::string(path) + ": bad number on line " + std::to_string(lineno));
        qc[i] = v;
      }
      if (qc[0] <= 0.0)
        for (int i = 0; i < nv; ++i) qc[i] = 0.0;
      for (int i = 4; i < 4 + ns; ++i)
        if (qc[i] <= 0.0) qc[i] = 0.0;
    }
    if (!std::getline(in, line)) {
      if (k != ny - 1) return fail(SFLOW_EINVAL, std::string(path) + ": missing record after a row");
    }
    ++lineno;
  }
  if (output_idx) {
    std::string s(path);
    const size_t slash = s.find_last_of("/\\");
    if (slash != std::string::npos) s = s.substr(slash + 1);   // the name, as in the input file
    const size_t dot = s.rfind('.');
    int idx = 0;
    if (dot == std::string::npos || dot < 4) return fail(SFLOW_EINVAL, std::string(path) + ": no output index before the extension");
    {
      const std::string four = s.substr(dot - 4, 4);
      char* end = nullptr;
      long v = std::strtol(four.c_str(), &end, 10);
      if (!end || *end != '\0') return fail(SFLOW_EINVAL, std::string(path) + ": no output index before the extension");
      idx = (int)v;
    }
    *output_idx = idx;
  }
  return SFLOW_OK;
}

// ---------------------------------------------------------------------------
// ESRI ASCII DEM (inpout_2d.f90:3684-3760) and its interpolation to the cell
// centres (geometry_2d.f90:337-350, interp_2d_scalar, interp_2d_nodata)
// ---------------------------------------------------------------------------
int read_dem(const char* path, const SflowParams* p, double* B_cent, uint8_t* nodata) {
  if (!path || !p || !B_cent) return fail(SFLOW_EINVAL, "NULL argument");
  std::ifstream in(path, std::ios::binary);
  if (!in) return fail(SFLOW_EINVAL, std::string("no dem file: ") + path);
  std::string key;
  double hv[6];
  for (int h = 0; h < 6; ++h) {
    if (!(in >> key >> hv[h])) return fail(SFLOW_EINVAL, std::string(path) + ": bad ESRI header");
  }
  const int ncols = (int)hv[0], nrows = (int)hv[1];
  const double xll = hv[2], yll = hv[3], cs = hv[4], nodata_topo = hv[5];
  if (ncols < 1 || nrows < 1 || !(cs > 0.0)) return fail(SFLOW_EINVAL, std::string(path) + ": bad ESRI header values");
  const int nx = p->comp_cells_x, ny = p->comp_cells_y;
  // domain checks of read_param (STOP in the reference)
  if (p->x0 - (xll + 0.5 * cs) < -1.0e-10) return fail(SFLOW_EINVAL, "Computational domain problem: x0 < xllcorner+0.5*cellsize");
  if (p->x0 + nx * p->cell_size > xll + (0.5 + ncols) * cs)
    return fail(SFLOW_EINVAL, "Computational domain problem: right edge > xllcorner+ncols*cellsize");
  if (p->y0 - (yll + 0.5 * cs) < -1.0e-10) return fail(SFLOW_EINVAL, "Computational domain problem: y0 < yllcorner+0.5*cellsize");
  if (std::fabs((p->y0 + ny * p->cell_size) - (yll + 0.5 + nrows * cs)) < 1.0e-10)
    return fail(SFLOW_EINVAL, "Computational domain problem: top edge > yllcorner+nrows*cellsize");
  // values row by row from the north edge
  std::vector<double> z((size_t)ncols * nrows), xs(ncols), ys(nrows);
  for (int r = 0; r < nrows; ++r) {
    const int row = nrows - 1 - r;
    for (int c = 0; c < ncols; ++c) {
      std::string tok;
      if (!(in >> tok)) return fail(SFLOW_EINVAL, std::string(path) + ": fewer values than ncols*nrows");
      for (auto& ch : tok)
        if (ch == 'd' || ch == 'D') ch = 'E';
      char* end = nullptr;
      double v = std::strtod(tok.c_str(), &end);
      if (!end || *end != '\0') return fail(SFLOW_EINVAL, std::string(path) + ": bad value '" + tok + "'");
      z[(size_t)row * ncols + c] = v;
    }
  }
  for (int c = 0; c < ncols; ++c) xs[c] = xll + ((double)(c + 1) - 0.5) * cs;
  for (int r = 0; r < nrows; ++r) ys[r] = yll + ((double)(r + 1) - 0.5) * cs;
  std::vector<double> xc, yc;
  cell_centres(p, xc, yc);
  auto locate = [](const std::vector<double>& g, double x, int& i, double& alfa) {
    const int n = (int)g.size();
    if (n > 1) {
      i = (int)std::floor((x - g[0]) / (g[1] - g[0])) + 1;
      if (i > n - 1) i = n - 1;
      if (i < 1) i = 1;   // the domain checks keep x inside the pixel centres
      alfa = (g[i] - x) / (g[i] - g[i - 1]);
    } else {
      i = 1;
      alfa = 0.0;
    }
  };
  auto Z = [&](const std::vector<double>& zz, int i, int r) { return zz[(size_t)(r - 1) * ncols + (i - 1)]; };
  // B_nodata before the clipping, B_cent after MAX(0, z)
  std::vector<double> zc(z);
  for (auto& v : zc) v = std::max(0.0, v);
  for (int k = 0; k < ny; ++k) {
    for (int j = 0; j < nx; ++j) {
      int ix, iy;
      double ax, ay;
      locate(xs, xc[j], ix, ax);
      locate(ys, yc[k], iy, ay);
      double f2;
      bool nd;
      if (ncols == 1) {
        f2 = ay * Z(zc, ix, iy) + (1.0 - ay) * Z(zc, ix, iy + 1);
        nd = Z(z, ix, iy) == nodata_topo || Z(z, ix, iy + 1) == nodata_topo;
      } else if (nrows == 1) {
        f2 = ax * Z(zc, ix, iy) + (1.0 - ax) * Z(zc, ix + 1, iy);
        nd = Z(z, ix, iy) == nodata_topo || Z(z, ix + 1, iy) == nodata_topo;
      } else {
        f2 = ax * (ay * Z(zc, ix, iy) + (1.0 - ay) * Z(zc, ix, iy + 1)) +
             (1.0 - ax) * (ay * Z(zc, ix + 1, iy) + (1.0 - ay) * Z(zc, ix + 1, iy + 1));
        nd = Z(z, ix, iy) == nodata_topo || Z(z, ix, iy + 1) == nodata_topo || Z(z, ix + 1, iy) == nodata_topo ||
             Z(z, ix + 1, iy + 1) == nodata_topo;
      }
      B_cent[(size_t)k * nx + j] = f2;
      if (nodata) nodata[(size_t)k * nx + j] = nd ? 1 : 0;
    }
  }
  return SFLOW_OK;
}

// ---------------------------------------------------------------------------
// .p_2d (inpout_2d.f90:6124-6400), format 1010 FORMAT(100ES15.7E2).  phys
// holds per cell h, u, v, T, alphas(1:n_solid), rho_m, red_grav, Ri (the
// values of qc_to_qp and mixt_var, sflow_download_phys); the columns are
//   x y h u v B h+B alphas T rho_m red_grav deposit erosion erodible alphal
//   shear_vel Ri Rouse mu_eff hmax pdynmax mod_vel_max inertial_number
// For the rheologies on the GPU path (1 and 6, no pore pressure): erosion,
// erodible, alphal, shear_vel, Rouse and the inertial number are 0; mu_eff
// is MU for rheology 1 and 0 otherwise.
// ---------------------------------------------------------------------------
int write_p2d(const char* path, const SflowParams* p, const double* phys, const double* B_cent,
              const double* deposit, const double* hmax, const double* pdynmax, const double* mvmax) {
  if (!path || !p || !phys || !B_cent || !hmax || !pdynmax || !mvmax) return fail(SFLOW_EINVAL, "NULL argument");
  const int nx = p->comp_cells_x, ny = p->comp_cells_y, ns = p->n_solid, nf = 7 + ns;
  const size_t N = (size_t)nx * ny;
  std::vector<double> xc, yc;
  cell_centres(p, xc, yc);
  auto z20 = [](double v) { return std::fabs(v) < 1.0e-20 ? 0.0 : v; };
  std::string out;
  out.reserve(N * 15 * (16 + 3 * ns) + 64 * ny);
  for (int k = 0; k < ny; ++k) {
    for (int j = 0; j < nx; ++j) {
      const size_t c = (size_t)k * nx + j;
      const double* f = phys + c * nf;
      const double r_h = z20(f[0]), r_u = z20(f[1]), r_v = z20(f[2]);
      const double B_out = z20(B_cent[c]);
      double mu_eff = 0.0;
      if (p->rheology_flag && p->rheology_model == 1 && f[0] > 0.0) mu_eff = p->mu;
      mu_eff = z20(mu_eff);
      fmt_ES(out, xc[j], 15, 7);
      fmt_ES(out, yc[k], 15, 7);
      fmt_ES(out, r_h, 15, 7);
      fmt_ES(out, r_u, 15, 7);
      fmt_ES(out, r_v, 15, 7);
      fmt_ES(out, B_out, 15, 7);
      fmt_ES(out, r_h + B_out, 15, 7);
      for (int i = 0; i < ns; ++i) fmt_ES(out, z20(f[4 + i]), 15, 7);
      fmt_ES(out, z20(f[3]), 15, 7);           // T
      fmt_ES(out, z20(f[4 + ns]), 15, 7);      // rho_m
      fmt_ES(out, z20(f[5 + ns]), 15, 7);      // red_grav
      for (int i = 0; i < ns; ++i) fmt_ES(out, deposit ? z20(deposit[(size_t)i * N + c]) : 0.0, 15, 7);
      for (int i = 0; i < ns; ++i) fmt_ES(out, 0.0, 15, 7);   // erosion
      fmt_ES(out, 0.0, 15, 7);                 // erodible / (1 - porosity)
      fmt_ES(out, 0.0, 15, 7);                 // alphal
      fmt_ES(out, 0.0, 15, 7);                 // shear_vel
      fmt_ES(out, f[6 + ns], 15, 7);           // Ri
      for (int i = 0; i < ns; ++i) fmt_ES(out, 0.0, 15, 7);   // Rouse numbers
      fmt_ES(out, mu_eff, 15, 7);
      fmt_ES(out, hmax[c], 15, 7);
      fmt_ES(out, pdynmax[c], 15, 7);
      fmt_ES(out, mvmax[c], 15, 7);
      fmt_ES(out, 0.0, 15, 7);                 // inertial number
      out += '\n';
    }
    out += kBlankRecord;
  }
  out += kBlankRecord;
  out += kBlankRecord;
  return write_file(path, out);
}

// ---------------------------------------------------------------------------
// restart.bin (inpout_2d.f90:8037-8179): Fortran unformatted sequential
// records, each framed by its byte length as a 4-byte integer before and
// after (records up to 2^31 - 1 bytes; larger ones would need sub-records)
// ---------------------------------------------------------------------------
static bool put_record(FILE* f, const void* data, size_t bytes) {
  if (bytes > 0x7fffffffu) return false;
  const int32_t m = (int32_t)bytes;
  return std::fwrite(&m, 4, 1, f) == 1 && (bytes == 0 || std::fwrite(data, 1, bytes, f) == bytes) &&
         std::fwrite(&m, 4, 1, f) == 1;
}
static bool get_record(FILE* f, void* data, size_t bytes) {
  int32_t m1 = 0, m2 = 0;
  if (std::fread(&m1, 4, 1, f) != 1 || (size_t)m1 != bytes) return false;
  if (bytes && std::fread(data, 1, bytes, f) != bytes) return false;
  return std::fread(&m2, 4, 1, f) == 1 && m2 == m1;
}

int write_restart(const char* path, const SflowParams* p, double t, double dt, const double* q, const double* B_cent,
                  const double* deposit, const double* hmax, const double* pdynmax, const double* mvmax) {
  if (!path || !p || !q || !B_cent || !hmax || !pdynmax || !mvmax) return fail(SFLOW_EINVAL, "NULL argument");
  const int nx = p->comp_cells_x, ny = p->comp_cells_y, ns = p->n_solid, nv = 4 + ns;
  const size_t N = (size_t)nx * ny;
  if ((double)N * nv * 8 > 2147483647.0) return fail(SFLOW_ERANGE, "q record above 2 GiB: sub-records are not written");
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(SFLOW_EINVAL, std::string("Unable to create restart file: ") + path);
  const int32_t dims[4] = {nx, ny, nv, ns};
  const double tdt[2] = {t, dt};
  std::vector<double> zeros((size_t)N * ns, 0.0);
  bool ok = put_record(f, dims, sizeof(dims)) && put_record(f, tdt, sizeof(tdt)) &&
            put_record(f, q, sizeof(double) * N * nv) && put_record(f, B_cent, sizeof(double) * N) &&
            put_record(f, zeros.data(), sizeof(double) * N * ns) &&                       // erodible
            put_record(f, deposit ? deposit : zeros.data(), sizeof(double) * N * ns) &&    // deposit
            put_record(f, zeros.data(), sizeof(double) * N * ns) &&                       // erosion
            put_record(f, hmax, sizeof(double) * N) && put_record(f, pdynmax, sizeof(double) * N) &&
            put_record(f, mvmax, sizeof(double) * N);
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return fail(SFLOW_EINVAL, std::string("write failed: ") + path);
  return SFLOW_OK;
}

int read_restart(const char* path, const SflowParams* p, double* t, double* dt, double* q, double* B_cent,
                 double* deposit, double* hmax, double* pdynmax, double* mvmax) {
  if (!path || !p || !t || !dt || !q || !B_cent) return fail(SFLOW_EINVAL, "NULL argument");
  const int nx = p->comp_cells_x, ny = p->comp_cells_y, ns = p->n_solid, nv = 4 + ns;
  const size_t N = (size_t)nx * ny;
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(SFLOW_EINVAL, std::string("Restart file not found: ") + path);
  int32_t dims[4];
  double tdt[2];
  std::vector<double> scratch(N * ns);
  bool ok = get_record(f, dims, sizeof(dims));
  if (ok && (dims[0] != nx || dims[1] != ny)) {
    std::fclose(f);
    return fail(SFLOW_EINVAL, "Grid dimensions in restart file do not match");
  }
  if (ok && (dims[2] != nv || dims[3] != ns)) {
    std::fclose(f);
    return fail(SFLOW_EINVAL, "n_vars / n_solid in restart file do not match");
  }
  ok = ok && get_record(f, tdt, sizeof(tdt)) && get_record(f, q, sizeof(double) * N * nv) &&
       get_record(f, B_cent, sizeof(double) * N) && get_record(f, scratch.data(), sizeof(double) * N * ns) &&
       get_record(f, deposit ? deposit : scratch.data(), sizeof(double) * N * ns) &&
       get_record(f, scratch.data(), sizeof(double) * N * ns);
  std::vector<double> m(N);
  ok = ok && get_record(f, hmax ? hmax : m.data(), sizeof(double) * N) &&
       get_record(f, pdynmax ? pdynmax : m.data(), sizeof(double) * N) &&
       get_record(f, mvmax ? mvmax : m.data(), sizeof(double) * N);
  std::fclose(f);
  if (!ok) return fail(SFLOW_EINVAL, std::string(path) + ": truncated or not a restart file of this grid");
  *t = tdt[0];
  *dt = tdt[1];
  return SFLOW_OK;
}

}  // namespace io
}  // namespace sflow

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

const char* sflow_io_error(void) { return sflow::io::g_io_err.c_str(); }

int sflow_read_input(const char* path, SflowParams* p, SflowRunInfo* run) {
  return sflow::io::read_input(path, p, run);
}
int sflow_read_dem(const char* path, const SflowParams* p, double* B_cent, uint8_t* nodata) {
  return sflow::io::read_dem(path, p, B_cent, nodata);
}
int sflow_read_q2d(const char* path, const SflowParams* p, double* q_aos, int32_t* output_idx) {
  return sflow::io::read_q2d(path, p, q_aos, output_idx);
}
int sflow_write_q2d(const char* path, const SflowParams* p, double* q_aos) {
  return sflow::io::write_q2d(path, p, q_aos);
}
int sflow_write_p2d(const char* path, const SflowParams* p, const double* phys, const double* B_cent,
                    const double* deposit, const double* hmax, const double* pdynmax, const double* mod_vel_max) {
  return sflow::io::write_p2d(path, p, phys, B_cent, deposit, hmax, pdynmax, mod_vel_max);
}
int sflow_write_restart(const char* path, const SflowParams* p, double t, double dt, const double* q_aos,
                        const double* B_cent, const double* deposit, const double* hmax, const double* pdynmax,
                        const double* mod_vel_max) {
  return sflow::io::write_restart(path, p, t, dt, q_aos, B_cent, deposit, hmax, pdynmax, mod_vel_max);
}
int sflow_read_restart(const char* path, const SflowParams* p, double* t, double* dt, double* q_aos, double* B_cent,
                       double* deposit, double* hmax, double* pdynmax, double* mod_vel_max) {
  return sflow::io::read_restart(path, p, t, dt, q_aos, B_cent, deposit, hmax, pdynmax, mod_vel_max);
}
int sflow_output_name(const char* run_name, int32_t index, const char* ext, char* out, int32_t out_len) {
  if (!run_name || !ext || !out || out_len < 1) return sflow::io::fail(SFLOW_EINVAL, "NULL argument");
  std::string s = std::string(run_name) + "_" + sflow::io::lettera(index) + "." + ext;
  if ((int)s.size() >= out_len) return sflow::io::fail(SFLOW_ERANGE, "output name buffer too small");
  std::memcpy(out, s.c_str(), s.size() + 1);
  return SFLOW_OK;
}

}  // extern "C"

// sflow_physics.cuh -- per-cell and per-face physics of the IMEX_SfloW2D
// time step as device functions, templated on the bulk arithmetic type.
//
//   Real = double : plain FP64 form.  Operation order follows the reference
//                   routine by routine; the translation unit is compiled with
//                   --fmad=false so no FMA changes the rounding.
//   Real = float  : FP32 bulk form.  State, reconstruction, fluxes and
//                   explicit sources in FP32; the implicit Newton solve, the
//                   wet/dry thresholds and the mass sums stay FP64.
//
// Each function cites the reference routine (path:line inside the reference
// project) it restates.
#pragma once
#include <cfloat>
#include <cstdint>

#include "sflow_math.h"
#include "sflow_types.cuh"

namespace sflow {

constexpr double kEps = DBL_EPSILON;  // EPSILON(1.0_wp)

template <class R>
__device__ __forceinline__ R cst(double x) { return static_cast<R>(x); }

template <class R>
__device__ __forceinline__ R rmin(R a, R b) { return a < b ? a : b; }
template <class R>
__device__ __forceinline__ R rmax(R a, R b) { return a > b ? a : b; }
template <class R>
__device__ __forceinline__ R sq(R a) { return a * a; }
// x^y and log x: in the FP64 form the library's own functions (sflow_math.h),
// which give the oracle's bits; in the FP32 form CUDA's powf and logf.
template <class R>
__device__ __forceinline__ R rpow(R x, R y) {
  if constexpr (sizeof(R) == 8) return sfm_pow(x, y);
  else return powf(x, y);
}
template <class R>
__device__ __forceinline__ R rlog(R x) {
  if constexpr (sizeof(R) == 8) return sfm_log(x);
  else return logf(x);
}
// Division of the FP32 form's per-face and per-cell closures: approximate
// (2 ulp for divisors of magnitude 2^-126 .. 2^126, far outside the
// densities, depths, temperatures and speeds divided by here); the FP64
// form divides exactly.
template <class R>
__device__ __forceinline__ R fdiv(R a, R b) {
  if constexpr (sizeof(R) == 4) return __fdividef(a, b);
  else return a / b;
}

// ---------------------------------------------------------------------------
// float <-> double conversions on the integer pipe.  GB300 executes FP64
// instructions, conversions to and from FP64 included, at 1/64 of the FP32
// rate; the FP32 form's FP64 Newton step and FP64 sums use these instead, so
// the FP64 pipe only does FP64 arithmetic.  Both follow IEEE 754 with the
// FP32 form's flush-to-zero: f2d_exact is exact (subnormal floats, which the
// FP32 form flushes, give +-0); d2f_rn rounds to nearest even and flushes
// results below the float normal range to +-0.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double f2d_exact(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu;
  const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
  unsigned long long bits = sign;
  if (e == 0xffu) bits |= 0x7ff0000000000000ull | ((unsigned long long)(u & 0x7fffffu) << 29);
  else if (e != 0u) bits |= ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)bits);
}
__device__ __forceinline__ float d2f_rn(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const int ed = (int)((b >> 52) & 0x7ffull);
  const unsigned long long frac = b & 0xfffffffffffffull;
  if (ed == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (frac ? 0x400000u : 0u));
  int e = ed - 896;                                      // biased float exponent
  unsigned long long m = (frac | 0x10000000000000ull) >> 29;   // 24 significant bits
  const unsigned long long rest = frac & 0x1fffffffull;        // 29 dropped bits
  if (rest > 0x10000000ull || (rest == 0x10000000ull && (m & 1ull))) ++m;
  if (m == 0x1000000ull) { m >>= 1; ++e; }              // carry into the exponent
  if (ed == 0 || e <= 0) return __uint_as_float(sign);
  if (e >= 255) return __uint_as_float(sign | 0x7f800000u);
  return __uint_as_float(sign | ((unsigned)e << 23) | ((unsigned)m & 0x7fffffu));
}
// (R)x of a double for either form
template <class R>
__device__ __forceinline__ R from_double(double x) {
  if constexpr (sizeof(R) == 4) return d2f_rn(x);
  else return x;
}

// ---------------------------------------------------------------------------
// geometry_2d.f90:1855-1876 minmod, 1878-1897 maxmod, 1776-1841 limit
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ R minmod(R a, R b) {
  R aa = fabs(a), ab = fabs(b);
  if (rmin(aa, ab) <= R(0)) return R(0);
  R sa = a / aa, sb = b / ab;
  return cst<R>(0.5) * (sa + sb) * rmin(aa, ab);
}
template <class R>
__device__ __forceinline__ R maxmod(R a, R b) {
  if (fabs(a * b) <= R(0)) return R(0);
  R sa = a / fabs(a), sb = b / fabs(b);
  return cst<R>(0.5) * (sa + sb) * rmax(fabs(a), fabs(b));
}
// LIM >= 0: the limiter of every variable, known at compile time; -1: lim
template <class R, int LIM = -1>
__device__ __forceinline__ R limit(R v0, R v1, R v2, R z0, R z1, R z2, int lim, R theta) {
  R a = (v2 - v1) / (z2 - z1);
  R b = (v1 - v0) / (z1 - z0);
  if constexpr (LIM >= 0) lim = LIM;
  switch (lim) {
    case 0: return R(0);
    case 1: return minmod(a, b);
    case 2: return maxmod(minmod(a, cst<R>(2.0) * b), minmod(cst<R>(2.0) * a, b));
    case 3: { R c = (v2 - v0) / (z2 - z0); return minmod(c, theta * minmod(a, b)); }
    case 4: { R c = (v2 - v0) / (z2 - z0); return minmod(c, cst<R>(2.0) * minmod(a, b)); }
    case 5: return (v2 - v0) / (z2 - z0);
    case 6: return a;
    case 7: return b;
  }
  return R(0);
}

// ---------------------------------------------------------------------------
// constitutive_2d.f90:550-976 r_phys_var + 1637-1690 qc_to_qp
// qp = (h, hu, hv, T, alphas or h*alphas ..., u, v); returns p_dyn
// ---------------------------------------------------------------------------
template <class R, int NS>
__device__ __forceinline__ R qc_to_qp(const Phys<R>& P, const R* q, R* qp) {
  constexpr int ns = NS, nv = 4 + NS;
  R xs[kMaxSolid];
  R inv_qj1;
  if (q[0] > P.thr_eps) {
    inv_qj1 = fdiv(R(1), q[0]);
    R sq_ = R(0);
    for (int i = 0; i < ns; ++i) { xs[i] = q[4 + i] * inv_qj1; sq_ += q[4 + i]; }
    if (sq_ == q[0]) {
      R s = R(0);
      for (int i = 0; i < ns; ++i) s += xs[i];
      for (int i = 0; i < ns; ++i) xs[i] = xs[i] / s;
    }
  } else {
    for (int i = 0; i < nv + 2; ++i) qp[i] = R(0);
    qp[3] = P.T_ambient;
    return R(0);
  }
  R xs_tot = R(0);
  for (int i = 0; i < ns; ++i) xs_tot += xs[i];
  R xc = R(1) - xs_tot;
  R cbyxc = P.gas ? ((xc - R(0)) * P.sp_heat_a + R(0)) : P.sp_heat_l * xc;
  R dcp = R(0);
  for (int i = 0; i < ns; ++i) dcp += xs[i] * P.sp_heat_s[i];
  R cmix = dcp + cbyxc;
  R T;
  if (q[0] > P.thr_eps_sing) {
    if (P.energy) T = fdiv(q[3] - cst<R>(0.5) * (sq(q[1]) + sq(q[2])) * inv_qj1, q[0] * cmix);
    else T = fdiv(q[3], q[0] * cmix);
    if (T <= R(0)) T = P.T_ambient;
  } else {
    T = P.T_ambient;
  }
  R inv_rho_c;
  if (P.gas) {
    // carrier of air alone: (x_c R_a) / x_c is R_a (the FP32 form uses it
    // as such; the FP64 form keeps the reference's operations)
    R Rc;
    if constexpr (sizeof(R) == 4) Rc = P.sp_gas_const_a;
    else Rc = (xc > P.thr_eps) ? ((xc - R(0)) * P.sp_gas_const_a + R(0)) / xc : P.sp_gas_const_a;
    inv_rho_c = Rc * T * P.inv_pres;
  } else {
    inv_rho_c = P.inv_rho_l;
  }
  R dinv = R(0);
  for (int i = 0; i < ns; ++i) dinv += xs[i] * P.inv_rho_s[i];
  R inv_rhom = dinv + xc * inv_rho_c;
  R rho_m = fdiv(R(1), inv_rhom);
  R h = q[0] * inv_rhom;
  R u, v;
  if (q[0] > P.thr_eps_sing) {
    u = q[1] * inv_qj1;
    v = q[2] * inv_qj1;
  } else {
    if constexpr (sizeof(R) == 8) {
      R q12 = q[0] * q[0];
      R den = sqrt(q12 * q12 + P.eps_sing4);
      u = P.sqrt2 * q[0] * q[1] / den;
      v = P.sqrt2 * q[0] * q[2] / den;
    } else {
      // same expression scaled by eps_sing: q1^4 and eps_sing^4 (1e-40)
      // are below the float range, (q1/eps)^4 is not
      R s = q[0] * P.inv_eps_sing;
      R f = P.sqrt2 * s * P.inv_eps_sing / sqrt(R(1) + (s * s) * (s * s));
      u = f * q[1];
      v = f * q[2];
    }
  }
  qp[0] = h;
  qp[1] = h * u;
  qp[2] = h * v;
  qp[3] = T;
  for (int i = 0; i < ns; ++i) {
    R al = xs[i] * rho_m * P.inv_rho_s[i];
    qp[4 + i] = P.alpha ? al : al * h;
  }
  qp[nv] = u;
  qp[nv + 1] = v;
  return cst<R>(0.5) * rho_m * (sq(u) + sq(v));
}

// constitutive_2d.f90:1718-2149 qp_to_qc (vertical profiles off)
template <class R, int NS>
__device__ __forceinline__ void qp_to_qc(const Phys<R>& P, const R* qp, R* qc) {
  constexpr int ns = NS, nv = 4 + NS;
  R r_h = qp[0];
  if (!(r_h > P.thr_eps)) {
    for (int i = 0; i < nv; ++i) qc[i] = R(0);
    return;
  }
  R r_hu = qp[1], r_hv = qp[2], r_u = qp[nv], r_v = qp[nv + 1], r_T = qp[3];
  R arhos[kMaxSolid];
  R at = R(0);
  for (int i = 0; i < ns; ++i) {
    R al = P.alpha ? qp[4 + i] : fdiv(qp[4 + i], qp[0]);
    at += al;
    arhos[i] = al * P.rho_s[i];
  }
  R rho_c;
  if (P.gas) {
    R rho_a = fdiv(P.pres, P.sp_gas_const_a * r_T);
    // carrier of air alone: ((1 - at) rho_a) / (1 - at) is rho_a
    if constexpr (sizeof(R) == 4) rho_c = rho_a;
    else rho_c = ((R(1) - R(0) - at - R(0)) * rho_a + R(0)) / (R(1) - R(0) - at);
  } else {
    rho_c = P.rho_l;
  }
  R alphac = R(1) - at;
  R sa = R(0);
  for (int i = 0; i < ns; ++i) sa += arhos[i];
  R rho_m = alphac * rho_c + sa;
  R inv_rhom = fdiv(R(1), rho_m);
  R xc = alphac * rho_c * inv_rhom;
  R cp_c;
  if (P.gas) {
    if constexpr (sizeof(R) == 4) cp_c = P.sp_heat_a;   // (x_c c_a) / x_c
    else cp_c = (xc > P.thr_eps) ? ((xc - R(0)) * P.sp_heat_a + R(0)) / xc : P.sp_heat_a;
  } else {
    cp_c = P.sp_heat_l;
  }
  R dcp = R(0);
  for (int i = 0; i < ns; ++i) dcp += (arhos[i] * inv_rhom) * P.sp_heat_s[i];
  R cmix = dcp + xc * cp_c;
  qc[0] = rho_m * r_h;
  qc[1] = rho_m * r_hu;
  qc[2] = rho_m * r_hv;
  if (P.energy) {
    qc[3] = (r_h > R(0)) ? r_h * rho_m * (cmix * r_T + cst<R>(0.5) * (sq(r_u) + sq(r_v))) : R(0);
  } else {
    qc[3] = r_h * rho_m * cmix * r_T;
  }
  for (int i = 0; i < ns; ++i) qc[4 + i] = (arhos[i] * inv_rhom) * qc[0];
}

// constitutive_2d.f90:1342-1492 mixt_var (+1513-1607 eval_sp_heat)
template <class R>
struct Mixt {
  R Ri, rho_m, rho_c, red_grav, cp_c, cp_mix;
};

template <class R, int NS>
__device__ __forceinline__ Mixt<R> mixt_var(const Phys<R>& P, const R* qpj, bool sp_heat_flag) {
  constexpr int ns = NS, nv = 4 + NS;
  Mixt<R> m;
  R r_h = qpj[0];
  if (!(qpj[0] > P.thr_eps)) {
    m.red_grav = R(0); m.rho_m = P.rho_a_amb; m.rho_c = P.rho_a_amb;
    m.cp_c = P.liquid ? P.sp_heat_l : P.sp_heat_a;
    m.cp_mix = m.cp_c;
    m.Ri = R(0);
    return m;
  }
  R r_u = qpj[nv], r_v = qpj[nv + 1], r_T = qpj[3];
  R al[kMaxSolid];
  R at = R(0);
  for (int i = 0; i < ns; ++i) { al[i] = P.alpha ? qpj[4 + i] : fdiv(qpj[4 + i], qpj[0]); at += al[i]; }
  R rho_c;
  if (P.gas) {
    R rho_a = fdiv(P.pres, P.sp_gas_const_a * r_T);
    // carrier of air alone: ((1 - at) rho_a) / (1 - at) is rho_a
    if constexpr (sizeof(R) == 4) rho_c = rho_a;
    else rho_c = ((R(1) - R(0) - at - R(0)) * rho_a + R(0)) / (R(1) - R(0) - at);
  } else {
    rho_c = P.rho_l;
  }
  R d = R(0);
  for (int i = 0; i < ns; ++i) d += al[i] * P.rho_s[i];
  R rho_m = (R(1) - at) * rho_c + d;
  R inv_rhom = fdiv(R(1), rho_m);
  R red_grav;
  if constexpr (sizeof(R) == 4) red_grav = (rho_m - P.rho_a_amb) * inv_rhom * P.grav;
  else red_grav = (rho_m - P.rho_a_amb) / rho_m * P.grav;
  R u2 = sq(r_u) + sq(r_v);
  m.Ri = (u2 > R(0)) ? rmin(cst<R>(1.0e15), fdiv(red_grav * r_h, u2)) : R(0);
  m.rho_m = rho_m;
  m.rho_c = rho_c;
  m.red_grav = red_grav;
  m.cp_c = R(0);
  m.cp_mix = R(0);
  if (sp_heat_flag) {
    R xs[kMaxSolid];
    R sxs = R(0);
    for (int i = 0; i < ns; ++i) { xs[i] = al[i] * P.rho_s[i] * inv_rhom; sxs += xs[i]; }
    R xc = R(1) - sxs;
    R cp_c;
    if (P.gas) {
      if constexpr (sizeof(R) == 4) cp_c = P.sp_heat_a;   // (x_c c_a) / x_c
      else cp_c = (xc > P.thr_eps) ? ((xc - R(0)) * P.sp_heat_a + R(0)) / xc : P.sp_heat_a;
    } else {
      cp_c = P.sp_heat_l;
    }
    R dcp = R(0);
    for (int i = 0; i < ns; ++i) dcp += xs[i] * P.sp_heat_s[i];
    m.cp_c = cp_c;
    m.cp_mix = dcp + xc * cp_c;
  }
  return m;
}

// qp_to_qc together with the densities and the reduced gravity of mixt_var
// (no Richardson number, no specific heats) for a face state: the carrier
// and mixture densities are formed once, with exactly the operations both
// routines use, so qc, rho_m and red_grav equal those of the two calls.
template <class R, int NS>
__device__ __forceinline__ Mixt<R> qp_to_qc_mixt(const Phys<R>& P, const R* qp, R* qc) {
  constexpr int ns = NS, nv = 4 + NS;
  Mixt<R> m;
  m.Ri = R(0);
  m.cp_c = R(0);
  m.cp_mix = R(0);
  R r_h = qp[0];
  if (!(r_h > P.thr_eps)) {
    for (int i = 0; i < nv; ++i) qc[i] = R(0);
    m.red_grav = R(0); m.rho_m = P.rho_a_amb; m.rho_c = P.rho_a_amb;
    return m;
  }
  R r_hu = qp[1], r_hv = qp[2], r_u = qp[nv], r_v = qp[nv + 1], r_T = qp[3];
  R arhos[kMaxSolid];
  R at = R(0);
  for (int i = 0; i < ns; ++i) {
    R al = P.alpha ? qp[4 + i] : fdiv(qp[4 + i], qp[0]);
    at += al;
    arhos[i] = al * P.rho_s[i];
  }
  R rho_c;
  if (P.gas) {
    R rho_a = fdiv(P.pres, P.sp_gas_const_a * r_T);
    // carrier of air alone: ((1 - at) rho_a) / (1 - at) is rho_a
    if constexpr (sizeof(R) == 4) rho_c = rho_a;
    else rho_c = ((R(1) - R(0) - at - R(0)) * rho_a + R(0)) / (R(1) - R(0) - at);
  } else {
    rho_c = P.rho_l;
  }
  R alphac = R(1) - at;
  R sa = R(0);
  for (int i = 0; i < ns; ++i) sa += arhos[i];
  R rho_m = alphac * rho_c + sa;
  R inv_rhom = fdiv(R(1), rho_m);
  R xc = alphac * rho_c * inv_rhom;
  R cp_c;
  if (P.gas) {
    if constexpr (sizeof(R) == 4) cp_c = P.sp_heat_a;   // (x_c c_a) / x_c
    else cp_c = (xc > P.thr_eps) ? ((xc - R(0)) * P.sp_heat_a + R(0)) / xc : P.sp_heat_a;
  } else {
    cp_c = P.sp_heat_l;
  }
  R dcp = R(0);
  for (int i = 0; i < ns; ++i) dcp += (arhos[i] * inv_rhom) * P.sp_heat_s[i];
  R cmix = dcp + xc * cp_c;
  qc[0] = rho_m * r_h;
  qc[1] = rho_m * r_hu;
  qc[2] = rho_m * r_hv;
  if (P.energy) {
    qc[3] = (r_h > R(0)) ? r_h * rho_m * (cmix * r_T + cst<R>(0.5) * (sq(r_u) + sq(r_v))) : R(0);
  } else {
    qc[3] = r_h * rho_m * cmix * r_T;
  }
  for (int i = 0; i < ns; ++i) qc[4 + i] = (arhos[i] * inv_rhom) * qc[0];
  m.rho_m = rho_m;
  m.rho_c = rho_c;
  if constexpr (sizeof(R) == 4) m.red_grav = (rho_m - P.rho_a_amb) * inv_rhom * P.grav;
  else m.red_grav = (rho_m - P.rho_a_amb) / rho_m * P.grav;
  return m;
}

// constitutive_2d.f90:2203-2307 eval_local_speeds_x / _y.  dir 1 = x, 2 = y.
template <class R, int NS>
__device__ __forceinline__ void local_speeds(const Phys<R>& P, const R* qpj, R red_grav, R gc,
                                             int dir, R& vmin, R& vmax) {
  constexpr int nv = 4 + NS;
  R r_h = qpj[0];
  R vel = (dir == 1) ? qpj[nv] : qpj[nv + 1];
  if (red_grav * r_h < R(0)) {
    vmin = vel; vmax = vel;
  } else {
    R c = (dir == 1) ? sqrt(red_grav * r_h * gc) : sqrt(gc * red_grav * r_h);
    vmin = vel - c; vmax = vel + c;
  }
}

// constitutive_2d.f90:2325-2518 eval_fluxes (vertical profiles off); the
// mixture state m is the mixt_var of qpj (only evaluated when h > eps).
template <class R, int NS>
__device__ __forceinline__ void eval_fluxes(const Phys<R>& P, const R* qcj, const R* qpj,
                                            const Mixt<R>& m, R gc, int dir, R* flux) {
  constexpr int ns = NS, nv = 4 + NS;
  if (qpj[0] > P.thr_eps) {
    R r_h = qpj[0];
    R vel = (dir == 1) ? qpj[nv] : qpj[nv + 1];
    R pterm = cst<R>(0.5) * m.rho_m * gc * m.red_grav * sq(r_h);
    flux[0] = vel * qcj[0] * R(1);
    if (dir == 1) {
      flux[1] = vel * qcj[1] * R(1) + pterm;
      flux[2] = vel * qcj[2] * R(1);
    } else {
      flux[1] = vel * qcj[1] * R(1);
      flux[2] = vel * qcj[2] * R(1) + pterm;
    }
    flux[3] = P.energy ? vel * (qcj[3] * R(1) + pterm) : vel * qcj[3] * R(1);
    for (int i = 0; i < ns; ++i) flux[4 + i] = vel * qcj[4 + i] * R(1);
    if (ns > 0 && flux[0] > R(0)) {
      R s = R(0);
      for (int i = 0; i < ns; ++i) s += flux[4 + i];
      // flux[0] > 0 here: the FP32 form compares without the division
      if (sizeof(R) == 4 ? s > flux[0] : s / flux[0] > R(1))
        for (int i = 0; i < ns; ++i) flux[4 + i] = flux[4 + i] / s * flux[0];
    }
  } else {
    for (int i = 0; i < nv; ++i) flux[i] = R(0);
  }
}

// ---------------------------------------------------------------------------
// constitutive_2d.f90:3024-3431 eval_expl_terms: gravity/slope terms, the
// bottom radial source (cell fraction bf inside the source, time factor
// b_coeff, inflow velocity b_vel) and the lateral ring inlet
// ---------------------------------------------------------------------------
template <class R, int NS>
__device__ __forceinline__ void expl_terms(const Phys<R>& P, const Geo<R>& g, const R* qpj,
                                           R t_coeff_src, R arc_perim, R arc_nx, R arc_ny,
                                           R bf, R b_coeff, R b_vel, R* e) {
  constexpr int ns = NS, nv = 4 + NS;
  for (int i = 0; i < nv; ++i) e[i] = R(0);
  if (!(qpj[0] > P.thr_eps) && bf == R(0) && arc_perim == R(0)) return;
  if (qpj[0] > P.thr_eps) {
    R r_h = qpj[0], r_u = qpj[nv], r_v = qpj[nv + 1];
    Mixt<R> m = mixt_var<R, NS>(P, qpj, true);
    R centr = P.curv ? (g.Bxx * sq(r_u) + cst<R>(2.0) * g.Bxy * r_u * r_v + g.Byy * sq(r_v)) : R(0);
    R tg = m.red_grav + centr;
    e[1] = -g.gc * m.rho_m * tg * r_h * g.Bx + cst<R>(0.5) * m.rho_m * m.red_grav * sq(r_h) * g.dgcx;
    e[2] = -g.gc * m.rho_m * tg * r_h * g.By + cst<R>(0.5) * m.rho_m * m.red_grav * sq(r_h) * g.dgcy;
    e[3] = P.energy ? (e[1] * r_u + e[2] * r_v) : R(0);
  }
  if (P.bottom_source && bf > R(0)) {
    // inflow state: h = 1, T = T_source, alphas_source (its mixt_var is
    // src_rho_m, src_cp_mix); the momentum terms add zero
    const R h_dot = bf * b_vel;
    e[0] = e[0] + b_coeff * h_dot * P.src_rho_m;
    e[1] = e[1] + R(0);
    e[2] = e[2] + R(0);
    e[3] = e[3] + b_coeff * h_dot * P.src_rho_m * P.src_cp_mix * P.T_source;
    for (int i = 0; i < ns; ++i) e[4 + i] = e[4 + i] + b_coeff * h_dot * P.alphas_source[i] * P.rho_s[i];
  }
  if (P.radial_source && arc_perim > R(0) && P.h_source > R(0)) {
    R t_coeff = t_coeff_src;
    if (t_coeff > R(0)) {
      R h_dot = P.h_source * P.vel_source * arc_perim / P.cell_area;
      e[0] = e[0] + t_coeff * h_dot * P.src_rho_m;
      e[1] = e[1] + t_coeff * h_dot * P.src_rho_m * P.vel_source * arc_nx;
      e[2] = e[2] + t_coeff * h_dot * P.src_rho_m * P.vel_source * arc_ny;
      e[3] = e[3] + t_coeff * h_dot * P.src_rho_m * P.src_cp_mix * P.T_source;
      for (int i = 0; i < ns; ++i)
        e[4 + i] = e[4 + i] + t_coeff * h_dot * P.alphas_source[i] * P.rho_s[i];
    }
  }
}

// time factor of the ring inlet (constitutive_2d.f90:3320-3349), FP64; the
// cosine is the library's own (sflow_math.h), the same bits as the oracle's
__device__ __forceinline__ double source_time_coeff(const double* tp, double pi_g, double time) {
  double t_coeff;
  if (time >= tp[3]) {
    if (tp[2] > 0.0 && time < tp[3] + tp[2]) t_coeff = 0.5 * (1.0 + sfm_cos(pi_g * (time - tp[3]) / tp[2]));
    else t_coeff = 0.0;
  } else {
    double t_rem = fmod(time, tp[0]);
    t_coeff = 0.0;
    if (tp[2] == 0.0) {
      if (t_rem <= tp[1]) t_coeff = 1.0;
    } else {
      if (t_rem < tp[2]) t_coeff = 0.5 * (1.0 - sfm_cos(pi_g * t_rem / tp[2]));
      else if (t_rem <= tp[1] - tp[2]) t_coeff = 1.0;
      else if (t_rem <= tp[1]) t_coeff = 0.5 * (1.0 + sfm_cos(pi_g * ((t_rem - tp[1]) / tp[2] + 1.0)));
    }
  }
  return t_coeff;
}

// ---------------------------------------------------------------------------
// constitutive_2d.f90:4027-4547 eval_nh_semi_impl_terms: the Coulomb term of
// rheology 1 and the mu(I) rheology 11 (4384-4458)
// ---------------------------------------------------------------------------
template <class R, int NS>
__device__ __forceinline__ void semi_impl_terms(const Phys<R>& P, const Geo<R>& g, const R* qpj,
                                                R* si) {
  constexpr int nv = 4 + NS;
  for (int i = 0; i < nv; ++i) si[i] = R(0);
  if (!P.rheo) return;
  R r_h = qpj[0], r_u = qpj[nv], r_v = qpj[nv + 1];
  Mixt<R> m = mixt_var<R, NS>(P, qpj, false);
  R r_w = P.slope_corr ? (r_u * g.Bx + r_v * g.By) : R(0);
  R mod_vel = sqrt(sq(r_u) + sq(r_v) + sq(r_w));
  if (P.rheo_model == 1 && mod_vel > R(0)) {
    R centr = P.curv ? (g.Bxx * sq(r_u) + cst<R>(2.0) * g.Bxy * r_u * r_v + g.Byy * sq(r_v)) : R(0);
    R tt = P.mu * m.rho_m * (m.red_grav + centr) * r_h * sqrt(g.gc);
    tt = rmax(R(0), tt);
    si[1] = si[1] - tt * r_u / mod_vel;
    si[2] = si[2] - tt * r_v / mod_vel;
  } else if (P.rheo_model == 11 && mod_vel > R(0)) {
    // grain diameter and density: Sauter mean and volume-weighted mean
    // (sauter_diameter, average_density_solids, constitutive_2d.f90:387-416)
    constexpr int ns = NS;
    R diam, rho_p;
    if (ns > 1) {
      R al[kMaxSolid], sa = R(0);
      for (int i = 0; i < ns; ++i) { al[i] = P.alpha ? qpj[4 + i] : qpj[4 + i] / qpj[0]; sa += al[i]; }
      if (sa < P.thr_eps) {
        R sd = R(0), sr = R(0);
        for (int i = 0; i < ns; ++i) { sd += P.diam_s[i]; sr += P.rho_s[i]; }
        diam = sd / R(ns);
        rho_p = sr / R(ns);
      } else {
        R sdi = R(0), sar = R(0);
        for (int i = 0; i < ns; ++i) { sdi += al[i] / P.diam_s[i]; sar += al[i] * P.rho_s[i]; }
        diam = sa / sdi;
        rho_p = sar / sa;
      }
    } else {
      diam = P.diam_s[0];
      rho_p = P.rho_s[0];
    }
    const R hh = (r_h < P.thr_eps) ? P.thr_eps : r_h;   // EPSILON(1.0_wp), exact in both forms
    R centr = P.curv ? (g.Bxx * sq(r_u) + cst<R>(2.0) * g.Bxy * r_u * r_v + g.Byy * sq(r_v)) : R(0);
    R vert = m.rho_m * (m.red_grav + centr) * hh;
    vert = rmax(vert, R(0));
    R eff = rmax(R(0), vert * sqrt(g.gc));
    if (eff < P.thr_eps) eff = P.thr_eps;
    const R shear = cst<R>(2.5) * mod_vel / (hh * sqrt(g.gc));
    const R I = diam * shear / sqrt(eff / rho_p);
    const R mu_I = (P.mu_s * P.I_0 + P.mu_2 * I + P.muI_inf * (I * I)) / (P.I_0 + I);
    const R tt = mu_I * eff;
    si[1] = si[1] - tt * (r_u / mod_vel);
    si[2] = si[2] - tt * (r_v / mod_vel);
  }
}

// ---------------------------------------------------------------------------
// Implicit friction (constitutive_2d.f90:3513-4009, rheology 1 and 6) with
// the gas-density / temperature closure of c_phys_var (1154-1322), written
// once over a number type N: double for the residual, Cplx for the
// complex-step Jacobian of the plain FP64 form (solver_2d.f90:2302-2367,
// the derivative the reference takes).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dsqrt(double a) { return sqrt(a); }
__device__ __forceinline__ double val(double a) { return a; }

// Complex numbers of the complex-step Jacobian with the arithmetic written
// out: textbook product, Smith's quotient (R. L. Smith, CACM 5(8), 1962),
// principal square root sqrt((|z| + |x|)/2).  The oracle spells the same
// formulas in C; compiled without contraction (--fmad=false), the two give
// the same Jacobian bits, and so the same Newton iterates.  A real operand
// is a complex number with zero imaginary part, for which each operation
// returns the real result exactly.
struct Cplx {
  double re, im;
  __device__ Cplx() {}
  __device__ Cplx(double r) : re(r), im(0.0) {}
  __device__ Cplx(double r, double i) : re(r), im(i) {}
};
__device__ __forceinline__ Cplx operator+(Cplx a, Cplx b) { return Cplx(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ Cplx operator-(Cplx a, Cplx b) { return Cplx(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ Cplx operator*(Cplx a, Cplx b) {
  return Cplx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__device__ __forceinline__ Cplx operator/(Cplx a, Cplx b) {
  if (fabs(b.re) >= fabs(b.im)) {
    const double r = b.im / b.re, den = b.re + b.im * r;
    return Cplx((a.re + a.im * r) / den, (a.im - a.re * r) / den);
  }
  const double r = b.re / b.im, den = b.re * r + b.im;
  return Cplx((a.re * r + a.im) / den, (a.im * r - a.re) / den);
}
__device__ __forceinline__ Cplx dsqrt(Cplx z) {
  const double ar = fabs(z.re), ai = fabs(z.im);
  if (ar == 0.0 && ai == 0.0) return Cplx(0.0, z.im);
  double m;
  if (ai == 0.0) m = ar;
  else if (ar == 0.0) m = ai;
  else if (ar >= ai) { const double t = ai / ar; m = ar * sqrt(1.0 + t * t); }
  else { const double t = ar / ai; m = ai * sqrt(1.0 + t * t); }
  const double t = sqrt((ar + m) * 0.5);
  if (z.re >= 0.0) return Cplx(t, z.im / (2.0 * t));
  return Cplx(ai / (2.0 * t), copysign(t, z.im));
}
__device__ __forceinline__ double val(Cplx a) { return a.re; }

template <class N, int NS>
__device__ __forceinline__ void implicit_terms(const Phys<double>& P, double Bx, double By,
                                               const N* q, N& nh1, N& nh2) {
  nh1 = N(0.0);
  nh2 = N(0.0);
  if (!P.rheo) return;
  constexpr int ns = NS;
  // c_phys_var
  N h, u, v, T, rho_m;
  if (val(q[0]) > kEps) {
    N inv_cqj1 = N(1.0) / q[0];
    N xs_tot = N(0.0), dcp = N(0.0), dinv = N(0.0);
    for (int i = 0; i < ns; ++i) {
      N xs = q[4 + i] * inv_cqj1;
      xs_tot = xs_tot + xs;
    }
    for (int i = 0; i < ns; ++i) {
      N xs = q[4 + i] * inv_cqj1;
      dcp = dcp + xs * N(P.sp_heat_s[i]);
      dinv = dinv + xs * N(P.inv_rho_s[i]);
    }
    N xc = N(1.0) - xs_tot;
    N cp_c = P.gas ? ((xc - N(0.0)) * N(P.sp_heat_a) + N(0.0)) / xc : N(P.sp_heat_l);
    N cmix = dcp + xc * cp_c;
    if (val(q[0]) > P.eps_sing_d) {
      if (P.energy) T = (q[3] - N(0.5) * (q[1] * q[1] + q[2] * q[2]) * inv_cqj1) / (q[0] * cmix);
      else T = q[3] / (q[0] * cmix);
      if (val(T) <= 0.0) T = N(P.T_ambient);
    } else {
      T = N(P.T_ambient);
    }
    N inv_rho_c;
    if (P.gas) {
      N Rc = ((xc - N(0.0)) * N(P.sp_gas_const_a) + N(0.0)) / xc;
      inv_rho_c = Rc * T * N(P.inv_pres);
    } else {
      inv_rho_c = N(P.inv_rho_l);
    }
    N inv_rhom = dinv + xc * inv_rho_c;
    rho_m = N(1.0) / inv_rhom;
    h = q[0] * inv_rhom;
    if (val(q[0]) > P.eps_sing_d) {
      u = q[1] * inv_cqj1;
      v = q[2] * inv_cqj1;
    } else {
      N q4 = q[0] * q[0];
      q4 = q4 * q4;
      N den = dsqrt(q4 + N(P.eps_sing4));
      u = N(P.sqrt2) * q[0] * q[1] / den;
      v = N(P.sqrt2) * q[0] * q[2] / den;
    }
  } else {
    return;  // h = u = v = 0: mod_vel = 0, no friction
  }
  N red_grav = (rho_m - N(P.rho_a_amb)) / rho_m * N(P.grav);
  N w = P.slope_corr ? (u * N(Bx) + v * N(By)) : N(0.0);
  N mod_vel2 = u * u + v * v + w * w;
  N mod_vel = dsqrt(mod_vel2);
  if (val(mod_vel) != 0.0) {
    if (P.rheo_model == 1) {
      N turb = rho_m * red_grav / N(P.xi) * mod_vel2;
      nh1 = nh1 - turb * (u / mod_vel);
      nh2 = nh2 - turb * (v / mod_vel);
    } else if (P.rheo_model == 6) {
      N mod_vel_hor = dsqrt(u * u + v * v);
      nh1 = nh1 - rho_m * (u / mod_vel_hor) * N(P.friction_factor) * mod_vel2;
      nh2 = nh2 - rho_m * (v / mod_vel_hor) * N(P.friction_factor) * mod_vel2;
    }
  }
}

// ---------------------------------------------------------------------------
// solver_2d.f90:1662-1996 solve_rk_step, 2021-2226 lnsrch, 2245-2284 eval_f
// (normalize_q = T, normalize_f = F, opt_search_NL = T; implicit set {hu,hv})
// ---------------------------------------------------------------------------
struct NewtonCtx {
  const Phys<double>* P;
  double dt, a_diag, Bx, By;
  const double* q_old;
  const double* Rj;
};

template <int NS>
__device__ __forceinline__ void newton_eval_f(const NewtonCtx& c, const double* qj, double* f,
                                              double& scal_f) {
  constexpr int nv = 4 + NS;
  double nh1, nh2;
  implicit_terms<double, NS>(*c.P, c.Bx, c.By, qj, nh1, nh2);
  double s = 0.0;
  for (int i = 0; i < nv; ++i) {
    double nh = (i == 1) ? nh1 : (i == 2) ? nh2 : 0.0;
    double Rj = c.Rj[i] - c.a_diag * nh;
    f[i] = qj[i] - c.q_old[i] + c.dt * Rj;
  }
  for (int i = 0; i < nv; ++i) s += f[i] * f[i];
  scal_f = 0.5 * s;
}

// Jacobian of f with respect to qj_rel for the implicit columns 1, 2
// (solver_2d.f90:2302-2367): J(k,i) = qj_org_i delta_ki - dt a_diag
// Im(NH_k(qj_rel qj_org + i h e_i qj_org)) / h with h = n_vars EPSILON, the
// complex step of the reference, evaluated at qj_rel * qj_org.
template <int NS>
__device__ __forceinline__ void newton_jacobian(const NewtonCtx& c, const double* qj_rel,
                                                const double* qj_org, double& s11, double& s12,
                                                double& s21, double& s22) {
  constexpr int nv = 4 + NS;
  const double h = nv * kEps, one_by_h = 1.0 / h;
  double jc[2][2];
  for (int col = 1; col <= 2; ++col) {
    Cplx qc[kMaxVars];
    for (int k = 0; k < nv; ++k) qc[k] = Cplx(qj_rel[k] * qj_org[k]);
    qc[col] = Cplx(qj_rel[col], h) * Cplx(qj_org[col]);
    Cplx n1, n2;
    implicit_terms<Cplx, NS>(*c.P, c.Bx, c.By, qc, n1, n2);
    jc[0][col - 1] = 1.0 * n1.im * one_by_h;
    jc[1][col - 1] = 1.0 * n2.im * one_by_h;
  }
  s11 = 1.0 * qj_org[1] - c.dt * c.a_diag * jc[0][0];
  s12 = 0.0 - c.dt * c.a_diag * jc[0][1];
  s21 = 0.0 - c.dt * c.a_diag * jc[1][0];
  s22 = 1.0 * qj_org[2] - c.dt * c.a_diag * jc[1][1];
}

// returns iterations used (kMaxNewton+1 when the limit was reached)
template <int NS>
__device__ int solve_rk_step(const NewtonCtx& c, double* qj) {
  constexpr int nv = 4 + NS;
  const double STPMX = 100.0, TOLF = 1.0e-10, TOLMIN = 1.0e-6, TOLX = kEps;
  double qj_org[kMaxVars], qj_rel[kMaxVars], f[kMaxVars], p[kMaxVars], g[kMaxVars],
      x_old[kMaxVars], qt[kMaxVars];
  double scal_f, scal_f_old;
  bool check = false;
  for (int i = 0; i < nv; ++i) {
    g[i] = 0.0;
    qj_org[i] = rmax(fabs(qj[i]), 1.0e-3);
    qj_rel[i] = qj[i] / qj_org[i];
  }
  for (int it = 1; it <= kMaxNewton; ++it) {
    newton_eval_f<NS>(c, qj, f, scal_f);
    double mf = 0.0;
    for (int i = 0; i < nv; ++i) mf = rmax(mf, fabs(f[i]));
    if (mf < TOLF) return it;
    if (!isfinite(scal_f)) return kMaxNewton + 1;   // NaN/Inf state: give up at once
    double s11, s12, s21, s22;
    newton_jacobian<NS>(c, qj_rel, qj_org, s11, s12, s21, s22);
    // explicit rows: diagonal qj_org (mask11); coupling mask21 is zero
    for (int i = 0; i < nv; ++i) p[i] = (i == 1 || i == 2) ? 0.0 : -(f[i] / qj_org[i]) + 0.0;
    double d2a = f[1], d2b = f[2];
    for (int i = 0; i < nv; ++i) {
      if (i == 1 || i == 2) continue;
      d2a = d2a - (f[i] / qj_org[i]) * 0.0;
      d2b = d2b - (f[i] / qj_org[i]) * 0.0;
    }
    double inv_det = 1.0 / (s11 * s22 - s21 * s12);
    p[1] = -((d2a * s22 - d2b * s12) * inv_det) + 0.0;
    p[2] = -((s11 * d2b - s21 * d2a) * inv_det) + 0.0;
    for (int i = 0; i < nv; ++i) x_old[i] = qj_rel[i];
    scal_f_old = scal_f;
    if (it > 1) {
      double nr = 0.0;
      for (int i = 0; i < nv; ++i) nr += qj_rel[i] * qj_rel[i];
      double stpmax = STPMX * rmax(sqrt(nr), double(nv));
      // grad_f = right_term . left_matrix: explicit columns diag qj_org
      for (int i = 0; i < nv; ++i) g[i] = (i == 1 || i == 2) ? 0.0 : f[i] * qj_org[i];
      g[1] = f[1] * s11 + f[2] * s21;
      g[2] = f[1] * s12 + f[2] * s22;
      // lnsrch
      check = false;
      double nrm = 0.0;
      for (int i = 0; i < nv; ++i) nrm += p[i] * p[i];
      nrm = sqrt(nrm);
      if (nrm > stpmax)
        for (int i = 0; i < nv; ++i) p[i] = p[i] * stpmax / nrm;
      double slope = 0.0;
      for (int i = 0; i < nv; ++i) slope += g[i] * p[i];
      double mx = 0.0;
      for (int i = 0; i < nv; ++i) {
        double t = fabs(p[i]) / rmax(fabs(x_old[i]), 1.0);
        if (i == 0 || t > mx) mx = t;
      }
      double alamin = TOLX / mx;
      if (alamin == 0.0) {
        for (int i = 0; i < nv; ++i) qj_rel[i] = x_old[i];
      } else {
        double alam = 1.0, alam2 = 0.0, f2 = 0.0, tmplam = 0.0;
        for (int ls = 0; ls < 4096; ++ls) {
          for (int i = 0; i < nv; ++i) {
            qj_rel[i] = x_old[i] + alam * p[i];
            qt[i] = qj_rel[i] * qj_org[i];
          }
          newton_eval_f<NS>(c, qt, f, scal_f);
          if (scal_f <= 0.9 * scal_f_old) break;
          if (alam < alamin) {
            for (int i = 0; i < nv; ++i) qj_rel[i] = x_old[i];
            scal_f = scal_f_old;
            check = true;
            break;
          }
          if (alam == 1.0) {
            tmplam = -slope / (2.0 * (scal_f - scal_f_old - slope));
          } else {
            double rhs1 = scal_f - scal_f_old - alam * slope;
            double rhs2 = f2 - scal_f_old - alam2 * slope;
            double a = (rhs1 / sq(alam) - rhs2 / sq(alam2)) / (alam - alam2);
            double b = (-alam2 * rhs1 / sq(alam) + alam * rhs2 / sq(alam2)) / (alam - alam2);
            if (a == 0.0) {
              tmplam = -slope / (2.0 * b);
            } else {
              double disc = b * b - 3.0 * a * slope;
              if (disc < 0.0) tmplam = 0.5 * alam;
              else if (b <= 0.0) tmplam = (-b + sqrt(disc)) / (3.0 * a);
              else tmplam = -slope / (b + sqrt(disc));
            }
            if (tmplam > 0.5 * alam) tmplam = 0.5 * alam;
          }
          alam2 = alam;
          f2 = scal_f;
          alam = rmax(tmplam, 0.5 * alam);
        }
      }
    } else {
      for (int i = 0; i < nv; ++i) {
        qj_rel[i] = x_old[i] + p[i];
        qj[i] = qj_rel[i] * qj_org[i];
      }
      newton_eval_f<NS>(c, qj, f, scal_f);
    }
    for (int i = 0; i < nv; ++i) qj[i] = qj_rel[i] * qj_org[i];
    mf = 0.0;
    for (int i = 0; i < nv; ++i) mf = rmax(mf, fabs(f[i]));
    if (mf < TOLF) return it;
    if (check) {
      double mc = 0.0;
      for (int i = 0; i < nv; ++i)
        mc = rmax(mc, fabs(g[i]) * rmax(fabs(qj_rel[i]), 1.0) / rmax(scal_f, 0.5 * nv));
      check = mc < TOLMIN;
    }
    double mx = 0.0;
    for (int i = 0; i < nv; ++i) mx = rmax(mx, fabs(qj_rel[i] - x_old[i]) / rmax(fabs(qj_rel[i]), 1.0));
    if (mx < TOLX) return it;
  }
  return kMaxNewton + 1;
}

// ---------------------------------------------------------------------------
// constitutive_2d.f90:5326-5404 settling_velocity and 4574-5153
// eval_mass_exchange_terms (settling, erosion of the erodible layer, air
// entrainment; no pore pressure / vaporisation)
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ R settling_velocity(const Phys<R>& P, R diam, R rhos, R rhoc,
                                               R inv_kin_visc) {
  R inv_sqrt_C_D = R(1);
  if (rhos <= rhoc) return R(0);
  R const_part = sqrt((cst<R>(4.0) / cst<R>(3.0)) * (rhos / rhoc - R(1)) * diam * P.grav);
  R sv = const_part * inv_sqrt_C_D;
  R Rey = diam * sv * inv_kin_visc;
  if (Rey <= cst<R>(1000.0)) {
    for (int i = 1; i <= 20; ++i) {
      R sv_old = sv;
      if (P.collective)
        inv_sqrt_C_D = sqrt(R(1) / (cst<R>(24.0) * (R(1) + cst<R>(0.15) * rpow<R>(Rey, cst<R>(0.687))) / Rey +
                                    P.A_drag * (rlog<R>(Rey) - P.B_drag)));
      else
        inv_sqrt_C_D = sqrt(Rey / (cst<R>(24.0) * (R(1) + cst<R>(0.15) * rpow<R>(Rey, cst<R>(0.687)))));
      sv = const_part * inv_sqrt_C_D;
      if (fabs(sv_old - sv) / sv_old < cst<R>(1.0e-6)) return sv;
      Rey = diam * sv * inv_kin_visc;
    }
  }
  return sv;
}

// erodible: the cell's erodible solid thicknesses (null: none, as with
// EROSION_COEFF = 0).  Returns the deposition and erosion rates (dep, ers),
// the equation terms and the topography rate topo.  As in the reference the
// erosion rates are set before the ALPHASTOT_MIN return, which leaves the
// equation terms at zero.  With ERODIBLE_DEPOSIT_FLAG the erodible layer
// takes the cell's temperature (the reference sets its module-wide
// T_erodible to the cell's T just before this use).
template <class R, int NS>
__device__ __forceinline__ void mass_exchange(const Phys<R>& P, const R* qpj, R Bx, R By, R dt,
                                              const R* erodible, R* dep, R* ers, R* eqn, R& topo,
                                              unsigned* dep_limited = nullptr) {
  constexpr int ns = NS, nv = 4 + NS;
  for (int i = 0; i < ns; ++i) { dep[i] = R(0); ers[i] = R(0); }
  for (int i = 0; i < nv; ++i) eqn[i] = R(0);
  topo = R(0);
  if (!(qpj[0] > P.thr_eps)) return;
  const R alpha_max = cst<R>(0.6), hind_exp = cst<R>(4.65);
  R r_h = qpj[0], r_u = qpj[nv], r_v = qpj[nv + 1];
  R al[kMaxSolid];
  R at = R(0);
  for (int i = 0; i < ns; ++i) { al[i] = P.alpha ? qpj[4 + i] : qpj[4 + i] / qpj[0]; at += al[i]; }
  R r_w = P.slope_corr ? (r_u * Bx + r_v * By) : R(0);
  R mod_vel2 = sq(r_u) + sq(r_v) + sq(r_w);
  if (P.erosion_coeff > R(0)) {
    // Fagents & Baloga (2006) eq. 5 with the solid volume fraction
    const R mod_vel = sqrt(mod_vel2);
    const R tot = P.erosion_coeff * mod_vel * r_h * (R(1) - at);
    const R tot_solid = tot * (R(1) - P.erodible_porosity);
    for (int i = 0; i < ns; ++i) ers[i] = P.erodible_fract[i] * tot_solid;
  }
  for (int i = 0; i < ns; ++i) ers[i] = rmax(R(0), rmin(ers[i], (erodible ? erodible[i] : R(0)) / dt));
  R tot_solid_erosion = R(0);
  for (int i = 0; i < ns; ++i) tot_solid_erosion += ers[i];
  R tot_erosion = tot_solid_erosion / (R(1) - P.erodible_porosity);
  R cont_erosion = tot_erosion * P.erodible_porosity;
  if (at <= P.alphastot_min) return;
  R r_T = qpj[3];
  Mixt<R> m = mixt_var<R, NS>(P, qpj, true);
  R inv_kin_visc = R(1) / P.kin_visc_c;
  R sdep = R(0);
  for (int i = 0; i < ns; ++i) {
    if (al[i] > R(0) && P.settling) {
      R sv = settling_velocity<R>(P, P.diam_s[i], P.rho_s[i], m.rho_c, inv_kin_visc);
      dep[i] = al[i] * sv * R(1);
      dep[i] = dep[i] * rpow<R>(R(1) - rmin(R(1), at / alpha_max), hind_exp);
      const R cap = r_h * al[i] / dt;
      if (dep_limited && !(dep[i] < cap)) *dep_limited |= 1u << i;   // the whole class settles out
      dep[i] = rmin(dep[i], cap);
    }
  }
  for (int i = 0; i < ns; ++i) sdep += dep[i];
  R sal = R(0);
  for (int i = 0; i < ns; ++i) sal += al[i];
  R cpl = P.liquid ? P.loss_rate : R(0);
  cpl = cpl + P.coeff_porosity * sdep;
  cpl = rmin(cpl, r_h * rmax(R(0), P.max_packing - sal) / dt);
  cpl = rmin(cpl, (r_h * (R(1) - sal) - P.coeff_porosity * (r_h * sal - dt * sdep)) / dt);
  R air_entr = R(0);
  if (P.entrain && r_h > R(0) && m.Ri > R(0)) {
    R entr_coeff = cst<R>(0.075) / sqrt(R(1) + cst<R>(718.0) * rpow<R>(m.Ri, cst<R>(2.4)));
    air_entr = entr_coeff * sqrt(mod_vel2);
  }
  const R T_ers = P.erodible_deposit ? r_T : P.T_erodible;
  R rho_dep_tot = R(0), rho_ers_tot = R(0), s_dep = R(0), s_ers = R(0), dep_tot = R(0), ers_tot = R(0);
  for (int i = 0; i < ns; ++i) dep_tot += dep[i];
  for (int i = 0; i < ns; ++i) ers_tot += ers[i];
  for (int i = 0; i < ns; ++i) rho_dep_tot += P.rho_s[i] * dep[i];
  for (int i = 0; i < ns; ++i) rho_ers_tot += P.rho_s[i] * ers[i];
  for (int i = 0; i < ns; ++i) s_dep += P.rho_s[i] * P.sp_heat_s[i] * dep[i];
  for (int i = 0; i < ns; ++i) s_ers += P.rho_s[i] * P.sp_heat_s[i] * ers[i];
  eqn[0] = P.rho_a_amb * air_entr + rho_ers_tot - rho_dep_tot + P.rho_c_sub * cont_erosion -
           m.rho_c * cpl;
  eqn[1] = -r_u * (rho_dep_tot + m.rho_c * cpl);
  eqn[2] = -r_v * (rho_dep_tot + m.rho_c * cpl);
  if (P.energy)
    eqn[3] = -r_T * (s_dep + m.rho_c * m.cp_c * cpl) - cst<R>(0.5) * mod_vel2 * (rho_dep_tot + m.rho_c * cpl) +
             T_ers * (s_ers + P.rho_c_sub * m.cp_c * cont_erosion) +
             P.T_ambient * P.sp_heat_a * P.rho_a_amb * air_entr;
  else
    eqn[3] = -r_T * (s_dep + m.rho_c * m.cp_c * cpl) +
             T_ers * (s_ers + P.rho_c_sub * m.cp_c * cont_erosion) +
             P.T_ambient * P.sp_heat_a * P.rho_a_amb * air_entr;
  for (int i = 0; i < ns; ++i) eqn[4 + i] = P.rho_s[i] * (ers[i] - dep[i]);
  topo = (dep_tot - ers_tot) / (R(1) - P.erodible_porosity);
}

// ---------------------------------------------------------------------------
// FP32 form: the implicit friction step solved as a scalar FP64 Newton.
// With the non-momentum components fixed, q_h = q_si_h + dt*a*NH_h(q) and
// NH_h is antiparallel to q_h (rheologies 1 and 6), so the solution is s*e
// with e = q_si_h/|q_si_h| and s >= 0 the root of
//     g(s) = s + dt*a*K(s)*s^2 - S,   S = |q_si_h|,
// K = (rho_m - rho_a) g kappa phi^2 / xi (Voellmy) or rho_m ff kappa^2
// phi^2 (rheology 6), kappa = sqrt(1 + (e.grad B)^2) with slope correction,
// phi = u/hu.  K depends on s only through T (the energy equation subtracts
// the kinetic energy) and through the gas density.  This is the fixed point
// of the reference's 2x2 Newton (solver_2d.f90:1662-1996).  The
// coefficients come from the FP32 state; an FP32 Newton gives the start and
// one FP64 Newton step with the analytic derivative finishes it.
// ---------------------------------------------------------------------------

// 1/x to ~1 ulp: float estimate + two Newton-Raphson refinements in FP64
__device__ __forceinline__ double rcp64(double x) {
  double r = (double)__frcp_rn((float)x);
  r = r * (2.0 - x * r);
  r = r * (2.0 - x * r);
  return r;
}

// The same root with every coefficient formed in FP64 from the FP32 state
// (entering through f2d_exact) and Newton iterated in FP64 with its FP64
// derivative to a relative step of 4 ulp (the reference's TOLX is the
// FP64 epsilon, solver_2d.f90:1826, 1984-1990), started from the explicit
// quadratic root; the result is rounded to float once.
template <int NS>
__device__ __noinline__ float reduced_friction_solve_fp64(const Phys<float>& P, const Phys<double>& PD,
                                                           float Bx, float By, const float* q, double dta,
                                                           float Sf, float e1, float e2, int& iters) {
  constexpr int ns = NS;
  const double q1 = f2d_exact(q[0]), inv_q1 = 1.0 / q1;
  double xs_tot = 0.0, dcp = 0.0, dinv = 0.0;
#pragma unroll
  for (int i = 0; i < ns; ++i) {
    const double xs = f2d_exact(q[4 + i]) * inv_q1;
    xs_tot += xs;
    dcp += xs * PD.sp_heat_s[i];
    dinv += xs * PD.inv_rho_s[i];
  }
  const double xc = 1.0 - xs_tot;
  const double cmix = dcp + xc * (PD.gas ? PD.sp_heat_a : PD.sp_heat_l);
  double phi;
  if (q1 > PD.eps_sing_d) {
    phi = inv_q1;
  } else {
    const double sc = q1 * PD.inv_eps_sing;
    phi = PD.sqrt2 * sc * PD.inv_eps_sing / sqrt(1.0 + (sc * sc) * (sc * sc));
  }
  double kappa2 = 1.0;
  if (PD.slope_corr) {
    const double w = f2d_exact(e1) * f2d_exact(Bx) + f2d_exact(e2) * f2d_exact(By);
    kappa2 = 1.0 + w * w;
  }
  const double cgeo = (PD.rheo_model == 1) ? PD.grav * sqrt(kappa2) * phi * phi / PD.xi
                                           : PD.friction_factor * kappa2 * phi * phi;
  const bool gas = PD.gas;
  const bool varT = gas && PD.energy && (q1 > PD.eps_sing_d);
  const double icm = 1.0 / (q1 * cmix);
  const double a_T = (q1 > PD.eps_sing_d) ? f2d_exact(q[3]) * icm : PD.T_ambient;
  const double b_T = varT ? 0.5 * inv_q1 * icm : 0.0;
  const double c_inv = gas ? xc * PD.sp_gas_const_a * PD.inv_pres : 0.0;
  const double base_inv = gas ? dinv : dinv + xc * PD.inv_rho_l;
  const double rho_a = (PD.rheo_model == 1) ? PD.rho_a_amb : 0.0;
  const double S = f2d_exact(Sf);
  auto Kd = [&](double sv, double& dK) -> double {
    double T = a_T - b_T * sv * sv, dT = -2.0 * b_T * sv;
    if (T <= 0.0) { T = PD.T_ambient; dT = 0.0; }
    const double rho_m = 1.0 / (base_inv + c_inv * T);
    dK = cgeo * (-rho_m * rho_m * c_inv * dT);
    return cgeo * (rho_m - rho_a);
  };
  double dK;
  double K = Kd(S, dK);
  const double disc = 1.0 + 4.0 * dta * K * S;
  if (!(disc >= 0.0)) { iters = 0; return Sf; }   // no real root (see reduced_friction_solve)
  double sd = 2.0 * S / (1.0 + sqrt(disc));
  int it = 0;
  for (; it < 12; ++it) {
    K = Kd(sd, dK);
    const double g = sd + dta * K * sd * sd - S;
    const double gd = 1.0 + dta * (dK * sd * sd + 2.0 * K * sd);
    const double ds = g / gd;
    sd -= ds;
    if (!(fabs(ds) > 4.0 * kEps * sd)) { ++it; break; }
  }
  iters = it;
  const long long sb = __double_as_longlong(sd);
  return (sb > 0 && sb <= 0x7ff0000000000000ll) ? d2f_rn(sd) : 0.0f;
}

template <int NS>
__device__ __forceinline__ float reduced_friction_solve(const Phys<float>& P, const Phys<double>& PD,
                                                        float Bx, float By,
                                                        const float* q, double dta, float& e1,
                                                        float& e2, int& iters) {
  constexpr int ns = NS;
  iters = 0;
  const float S = sqrtf(q[1] * q[1] + q[2] * q[2]);
  if (S == 0.0f) { e1 = 0.0f; e2 = 0.0f; return 0.0f; }
  const float iS = 1.0f / S;
  e1 = q[1] * iS;
  e2 = q[2] * iS;
  if (!P.rheo || P.rheo_model == 11 || !(q[0] > P.thr_eps)) return S;   // model 11: no implicit friction
  const float q1 = q[0], inv_q1 = 1.0f / q1;
  float xs_tot = 0.0f, dcp = 0.0f, dinv = 0.0f;
#pragma unroll
  for (int i = 0; i < ns; ++i) {
    const float xs = q[4 + i] * inv_q1;
    xs_tot += xs;
    dcp += xs * P.sp_heat_s[i];
    dinv += xs * P.inv_rho_s[i];
  }
  const float xc = 1.0f - xs_tot;
  const float cmix = dcp + xc * (P.gas ? P.sp_heat_a : P.sp_heat_l);
  float phi;
  if (q1 > P.thr_eps_sing) phi = inv_q1;
  else {
    const float sc = q1 * P.inv_eps_sing;
    phi = P.sqrt2 * sc * P.inv_eps_sing / sqrtf(1.0f + (sc * sc) * (sc * sc));
  }
  float kappa2 = 1.0f;
  if (P.slope_corr) { const float w = e1 * Bx + e2 * By; kappa2 = 1.0f + w * w; }
  const float cgeo = (P.rheo_model == 1) ? P.grav * sqrtf(kappa2) * phi * phi / P.xi
                                         : P.friction_factor * kappa2 * phi * phi;
  const bool gas = P.gas;
  const bool varT = gas && P.energy && (q1 > P.thr_eps_sing);
  const float icm = 1.0f / (q1 * cmix);
  const float a_T = (q1 > P.thr_eps_sing) ? q[3] * icm : P.T_ambient;
  const float b_T = varT ? 0.5f * inv_q1 * icm : 0.0f;
  const float c_inv = gas ? xc * P.sp_gas_const_a * P.inv_pres : 0.0f;
  const float base_inv = gas ? dinv : dinv + xc * P.inv_rho_l;
  const float rho_a = (P.rheo_model == 1) ? P.rho_a_amb : 0.0f;
  // K(s) and dK/ds in float
  auto Kf = [&](float sv, float& dK) -> float {
    float T = a_T - b_T * sv * sv, dT = -2.0f * b_T * sv;
    if (T <= 0.0f) { T = P.T_ambient; dT = 0.0f; }
    const float inv_rhom = base_inv + c_inv * T;
    const float rho_m = 1.0f / inv_rhom;
    dK = cgeo * (-rho_m * rho_m * c_inv * dT);
    return cgeo * (rho_m - rho_a);
  };
  if (PD.newton64) return reduced_friction_solve_fp64<NS>(P, PD, Bx, By, q, dta, S, e1, e2, iters);
  const float dtaf = d2f_rn(dta);
  float dKf;
  float K = Kf(S, dKf);
  // K < 0 (a mixture lighter than the ambient: the buoyancy-reduced
  // friction changes sign) with 1 + 4 dt a K S < 0 leaves g without a real
  // root: the friction step keeps the predictor's momentum (taking the
  // clamped quadratic instead doubled a film's momentum every step)
  const float disc = 1.0f + 4.0f * dtaf * K * S;
  if (!(disc >= 0.0f)) return S;
  float s = 2.0f * S / (1.0f + sqrtf(disc));
  float gdf = 1.0f + 2.0f * dtaf * K * s;
  if (varT) {
    const float s0 = s, gd0 = gdf;
    for (int it = 0; it < 8; ++it) {
      K = Kf(s, dKf);
      const float gv = s + dtaf * K * s * s - S;
      gdf = 1.0f + dtaf * (dKf * s * s + 2.0f * K * s);
      const float ds = gv / gdf;
      s -= ds;
      if (!(fabsf(ds) > 1.0e-7f * s)) break;
    }
    // the root lies in (0, 2S] (K > 0: below S; K < 0: at most 2S)
    if (!(s > 0.0f && s <= 2.0f * S)) { s = s0; gdf = gd0; }
  }
  // One FP64 Newton step from the FP32 root: the residual g(s) in FP64
  // (rho_m to ~1e-14 by one refinement of the float reciprocal), the
  // derivative from the last FP32 iteration.  The FP32 root is within ~1e-7
  // relative of the solution and g' is known to ~1e-7, so the step leaves an
  // error of order 1e-14, far below the float the result is stored in.
  // FP32 values enter through f2d_exact and leave through d2f_rn, and the
  // sign tests read the sign bit, so the FP64 pipe only does the FP64
  // arithmetic (FP64 constants come from the FP64 parameter block).
  double sd = f2d_exact(s);
  {
    const double sd2 = sd * sd;
    double T = f2d_exact(a_T) - f2d_exact(b_T) * sd2;
    if (__double_as_longlong(T) <= 0) T = PD.T_ambient;   // T <= 0 (sign bit or zero)
    const double x = f2d_exact(base_inv) + f2d_exact(c_inv) * T;
    double rho_m = f2d_exact(__frcp_rn(d2f_rn(x)));
    rho_m = rho_m * (2.0 - x * rho_m);
    const double Kd = f2d_exact(cgeo) * (rho_m - ((P.rheo_model == 1) ? PD.rho_a_amb : 0.0));
    const double gv = (sd - f2d_exact(S)) + dta * Kd * sd2;
    sd -= gv * f2d_exact(__frcp_rn(gdf));
    iters = 1;
  }
  // sd > 0 (finite or +inf): positive sign and not a NaN
  const long long sb = __double_as_longlong(sd);
  return (sb > 0 && sb <= 0x7ff0000000000000ll) ? d2f_rn(sd) : 0.0f;
}

}  // namespace sflow

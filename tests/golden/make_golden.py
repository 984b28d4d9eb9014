"""Generate the known-answer fixtures in tests/golden/golden.json.

The reference's own tests (TESTS/run_tests.sh) only check that an output
file appears, so there are no reference golden vectors for this path and
the reference (Fortran, no compiler available) cannot be run to make any.
The values here are derived independently of the oracle, from the
formulas of the reference routines written out by hand with numpy, and
from closed-form solutions:

  limiter      geometry_2d.f90:1776-1897 on a fixed 3-point stencil
  mixture      constitutive_2d.f90:1342-1492 (mixt_var) for a hot
               gas-particle state, evaluated term by term
  friction     the backward-Euler Voellmy step of a liquid-carrier cell
               (rho_m and g' independent of momentum): the 2x2 Newton of
               solver_2d.f90:1662-1996 converges to the positive root of
               dt*K*s^2 + s - S = 0, K = (rho_m - rho_a) g kappa / (xi q1^2)
  stoker       wet-bed dam break (h_L = 1 m, h_R = 0.1 m) of the shallow
               water equations with the reduced gravity of a water carrier
               in ambient air; depth profile at t = 5 s

Run: python tests/golden/make_golden.py   (rewrites golden.json)
"""
import json
import math
import os

import numpy as np
from scipy.optimize import brentq

HERE = os.path.dirname(os.path.abspath(__file__))


def limiter_table():
    v = [1.0, 2.0, 4.0]
    z = [0.0, 1.0, 2.0]
    # a = (v3-v2)/(z3-z2) = 2, b = (v2-v1)/(z2-z1) = 1, c = (v3-v1)/(z3-z1) = 1.5
    return {"v": v, "z": z, "theta": 1.0,
            "slopes": {"0": 0.0, "1": 1.0, "2": 2.0, "3": 1.0, "4": 1.5, "5": 1.5, "6": 2.0,
                       "7": 1.0},
            "minmod_pairs": [[1.0, 2.0, 1.0], [-1.0, 2.0, 0.0], [0.0, 5.0, 0.0],
                             [-3.0, -2.0, -2.0], [2.5, 2.5, 2.5]]}


def gas_constants():
    return {"pres": 101300.0, "sp_gas_const_a": 287.051, "T_ambient": 300.0, "grav": 9.81,
            "sp_heat_a": 998.0, "rho_s": [2500.0, 1500.0], "sp_heat_s": [1100.0, 1100.0]}


def mixture_case():
    c = gas_constants()
    h, u, v, T = 3.0, 12.0, -5.0, 1000.0
    alphas = [0.01, 0.02]
    rho_a_amb = c["pres"] / (c["sp_gas_const_a"] * c["T_ambient"])
    rho_a = c["pres"] / (c["sp_gas_const_a"] * T)
    at = sum(alphas)
    rho_c = rho_a                     # single gas component
    rho_m = (1 - at) * rho_c + sum(a * r for a, r in zip(alphas, c["rho_s"]))
    red_grav = (rho_m - rho_a_amb) / rho_m * c["grav"]
    Ri = red_grav * h / (u * u + v * v)
    xs = [a * r / rho_m for a, r in zip(alphas, c["rho_s"])]
    xc = 1 - sum(xs)
    cp_mix = sum(x * cp for x, cp in zip(xs, c["sp_heat_s"])) + xc * c["sp_heat_a"]
    qp = [h, h * u, h * v, T, alphas[0] * h, alphas[1] * h, u, v]
    # conservative state with total energy (energy_flag = T)
    qc = [rho_m * h, rho_m * h * u, rho_m * h * v,
          h * rho_m * (cp_mix * T + 0.5 * (u * u + v * v)),
          xs[0] * rho_m * h, xs[1] * rho_m * h]
    return {"constants": c, "qp": qp, "qc": qc,
            "expect": {"rho_m": rho_m, "rho_c": rho_c, "red_grav": red_grav, "Ri": Ri,
                       "cp_mix": cp_mix}}


def friction_case():
    """One liquid-carrier cell: implicit Voellmy step with slope correction."""
    rho_l, rho_s, alpha = 1000.0, 2500.0, 0.05
    pres, R_a, T_amb, g = 101300.0, 287.051, 300.0, 9.81
    xi, dt, a_diag = 500.0, 0.05, 1.0
    Bx, By = 0.2, -0.1
    h = 2.0
    rho_m = (1 - alpha) * rho_l + alpha * rho_s
    q1 = rho_m * h
    q_si = [q1, 0.8 * q1 * 6.0, 0.6 * q1 * 6.0]     # |u| = 6 m/s along (0.8, 0.6)
    S = math.hypot(q_si[1], q_si[2])
    e = (q_si[1] / S, q_si[2] / S)
    kappa = math.sqrt(1.0 + (e[0] * Bx + e[1] * By) ** 2)
    rho_a = pres / (R_a * T_amb)
    K = (rho_m - rho_a) * g * kappa / (xi * q1 * q1)
    s = 2.0 * S / (1.0 + math.sqrt(1.0 + 4.0 * dt * a_diag * K * S))
    return {"rho_l": rho_l, "rho_s": rho_s, "alpha": alpha, "h": h, "xi": xi, "dt": dt,
            "a_diag": a_diag, "Bx": Bx, "By": By, "q_si_mom": q_si[1:], "q1": q1,
            "solution_mom": [s * e[0], s * e[1]]}


def stoker_profile():
    """Wet-bed dam break: h_L, h_R, gravity g' of water in air."""
    hL, hR = 1.0, 0.1
    g = 9.81 * (1000.0 - 101300.0 / (287.051 * 300.0)) / 1000.0
    cL, cR = math.sqrt(g * hL), math.sqrt(g * hR)

    def f(hm):
        um_raref = 2.0 * (cL - math.sqrt(g * hm))
        um_shock = (hm - hR) * math.sqrt(0.5 * g * (hm + hR) / (hm * hR))
        return um_raref - um_shock

    hm = brentq(f, hR * 1.0000001, hL * 0.9999999, xtol=1e-15)
    cm = math.sqrt(g * hm)
    um = 2.0 * (cL - cm)
    s_shock = hm * um / (hm - hR)
    t = 5.0
    x0 = 100.0
    x = np.arange(200) + 0.5
    hx = np.empty_like(x)
    for i, xx in enumerate(x):
        xi = (xx - x0) / t
        if xi <= -cL:
            hx[i] = hL
        elif xi <= um - cm:
            hx[i] = (2.0 * cL - xi) ** 2 / (9.0 * g)
        elif xi <= s_shock:
            hx[i] = hm
        else:
            hx[i] = hR
    return {"g_reduced": g, "h_m": hm, "u_m": um, "shock_speed": s_shock, "t": t, "x0": x0,
            "dx": 1.0, "h": hx.tolist()}


def main():
    data = {"limiter": limiter_table(), "mixture": mixture_case(),
            "friction": friction_case(), "stoker": stoker_profile()}
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump(data, fh, indent=1)
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()

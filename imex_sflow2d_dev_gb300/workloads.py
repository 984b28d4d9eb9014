"""Seeded synthetic inputs for the benchmark and parity workloads.

The reference measures nothing on a public dataset; its real DEMs (Etna,
Taal, CF) are not part of the source tree.  The workloads below are seeded
synthetic stand-ins with the shapes and parameter ranges of the benchmark
configurations:

  dam_break       200x200, dx=1 m, flat bed, liquid carrier, h=1 / 0.1 m
  pyroclastic     1024x1024, dx=10 m, Gaussian cone + fBm DEM, radial
                  (ring) source 1e6 kg/s, 2 particle classes, hot gas,
                  Voellmy friction, slope correction, settling
  ensemble_member one run of the 256-run ensemble (side log-uniform in
                  [128,1024], dx U[5,20], per-run mu, xi, source radius and
                  temperature, particle fractions)
  large_domain    8192x8192, dx=2 m, diamond-square DEM, 3 classes,
                  entrainment on, one radial source

Random numbers come from splitmix64 (a counter-based generator with a fixed
published recurrence) so the same seed gives the same inputs on every
machine and numpy version.
"""
import math

import numpy as np

from .params import (MAX_SOLID, PREC_FP32, PREC_FP64, SCHEME_KT, default_params)

_M64 = (1 << 64) - 1


def splitmix64(seed, n):
    """n uint64 values of the splitmix64 sequence started at `seed`."""
    out = np.empty(n, dtype=np.uint64)
    x = seed & _M64
    for i in range(n):
        x = (x + 0x9E3779B97F4A7C15) & _M64
        z = x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        out[i] = z ^ (z >> 31)
    return out


def splitmix64_np(seed, n):
    """Vectorised splitmix64: element i is the (i+1)-th output after `seed`."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed, n):
    """n doubles in [0,1) from the top 53 bits of splitmix64."""
    return (splitmix64_np(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


# ---------------------------------------------------------------------------
# DEMs
# ---------------------------------------------------------------------------

def fbm_surface(nx, ny, dx, hurst, rms, seed):
    """Fractional Brownian surface by spectral synthesis: amplitude
    |k|^-(H+1), phases from splitmix64, scaled to the given RMS."""
    kx = np.fft.fftfreq(nx, d=dx)
    ky = np.fft.fftfreq(ny, d=dx)
    k = np.sqrt(kx[None, :] ** 2 + ky[:, None] ** 2)
    k[0, 0] = 1.0
    amp = k ** (-(hurst + 1.0))
    amp[0, 0] = 0.0
    u = uniform01(seed, 2 * nx * ny).reshape(2, ny, nx)
    # Box-Muller gives Gaussian coefficients (real and imaginary parts)
    r = np.sqrt(-2.0 * np.log(np.maximum(u[0], 1e-300)))
    g = r * np.cos(2.0 * np.pi * u[1]) + 1j * r * np.sin(2.0 * np.pi * u[1])
    z = np.fft.ifft2(amp * g).real
    z -= z.mean()
    s = np.sqrt(np.mean(z * z))
    return z * (rms / s) if s > 0 else z


def cone_fbm_dem(nx, ny, dx, height=1500.0, sigma=2000.0, hurst=0.8, rms=20.0, seed=1):
    """Gaussian cone centred in the domain plus fBm noise; cell-centred
    values B_cent(j,k), returned as an (ny, nx) array (row k, column j)."""
    x = (np.arange(nx) + 0.5) * dx
    y = (np.arange(ny) + 0.5) * dx
    xc, yc = 0.5 * nx * dx, 0.5 * ny * dx
    r2 = (x[None, :] - xc) ** 2 + (y[:, None] - yc) ** 2
    B = height * np.exp(-r2 / (2.0 * sigma * sigma)) + fbm_surface(nx, ny, dx, hurst, rms, seed)
    # the reference clamps the DEM at zero (geometry_2d.f90:350)
    return np.maximum(B, 0.0)


def diamond_square_dem(n_pow2, relief, hurst, seed):
    """Diamond-square surface on a (2^p+1)^2 node grid scaled to `relief`."""
    n = (1 << n_pow2) + 1
    z = np.zeros((n, n))
    u = uniform01(seed, 4)
    z[0, 0], z[0, -1], z[-1, 0], z[-1, -1] = (u - 0.5)
    step = n - 1
    scale = 1.0
    level = 0
    while step > 1:
        half = step // 2
        level += 1
        # diamond step: centres of squares
        c = z[0:n - 1:step, 0:n - 1:step] + z[0:n - 1:step, step::step] \
            + z[step::step, 0:n - 1:step] + z[step::step, step::step]
        m = c.shape[0] * c.shape[1]
        r = uniform01(seed * 7919 + 2 * level, m).reshape(c.shape) - 0.5
        z[half::step, half::step] = 0.25 * c + scale * r
        # square step: edge midpoints
        for (i0, j0) in ((0, half), (half, 0)):
            ii = np.arange(i0, n, step)
            jj = np.arange(j0, n, step)
            I, J = np.meshgrid(ii, jj, indexing="ij")
            acc = np.zeros(I.shape)
            cnt = np.zeros(I.shape)
            for di, dj in ((-half, 0), (half, 0), (0, -half), (0, half)):
                I2, J2 = I + di, J + dj
                ok = (I2 >= 0) & (I2 < n) & (J2 >= 0) & (J2 < n)
                acc[ok] += z[I2[ok], J2[ok]]
                cnt[ok] += 1
            r = uniform01(seed * 7919 + 2 * level + 1 + i0, I.size).reshape(I.shape) - 0.5
            z[I, J] = acc / cnt + scale * r
        step = half
        scale *= 0.5 ** hurst
    z -= z.min()
    z *= relief / max(z.max(), 1e-300)
    return z


# ---------------------------------------------------------------------------
# conversions for initial states (reference constitutive_2d.f90:1718-2149
# qp_to_qc, restricted to u = v = 0 which is all the initial states need)
# ---------------------------------------------------------------------------

def rest_state_q(p, h, T, alphas):
    """Conservative state (n_vars, ny, nx) for thickness h (ny,nx), uniform
    temperature T and solid volume fractions alphas (list), at rest."""
    ns = p.n_solid
    nv = 4 + ns
    ny, nx = h.shape
    q = np.zeros((nv, ny, nx))
    at = float(sum(alphas[:ns]))
    if p.gas_flag:
        rho_a = p.pres / (p.sp_gas_const_a * T)
        rho_c = ((1.0 - 0.0 - at - 0.0) * rho_a + 0.0) / (1.0 - 0.0 - at)
    else:
        rho_c = p.rho_l
    arhos = [alphas[i] * p.rho_s[i] for i in range(ns)]
    alphac = 1.0 - at
    rho_m = alphac * rho_c + sum(arhos)
    inv_rhom = 1.0 / rho_m
    xs = [a * inv_rhom for a in arhos]
    xc = alphac * rho_c * inv_rhom
    if p.gas_flag:
        cp_c = ((xc - 0.0) * p.sp_heat_a + 0.0) / xc if xc > np.finfo(float).eps else p.sp_heat_a
    else:
        cp_c = p.sp_heat_l
    cmix = sum(xs[i] * p.sp_heat_s[i] for i in range(ns)) + xc * cp_c
    wet = h > np.finfo(float).eps
    q0 = np.where(wet, rho_m * h, 0.0)
    q[0] = q0
    if p.energy_flag:
        q[3] = np.where(wet, h * rho_m * (cmix * T + 0.5 * 0.0), 0.0)
    else:
        q[3] = np.where(wet, h * rho_m * cmix * T, 0.0)
    for i in range(ns):
        q[4 + i] = xs[i] * q0
    return q


def to_aos(q_sna):
    """(n_vars, ny, nx) -> reference layout q(1:n_vars,1:nx,1:ny) flattened
    Fortran order == C array [ny][nx][n_vars]."""
    return np.ascontiguousarray(np.transpose(q_sna, (1, 2, 0))).reshape(-1)


def from_aos(q_flat, nv, nx, ny):
    return np.transpose(q_flat.reshape(ny, nx, nv), (2, 0, 1))


def _gas_common(p):
    p.pres = 101300.0
    p.sp_heat_a = 998.0
    p.sp_gas_const_a = 287.051
    p.kin_visc_a = 1.48e-5
    p.T_ambient = 300.0


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------

def dam_break(nx=200, ny=200, dx=1.0, n_rk=2, precision=PREC_FP64, t_end=10.0, n_solid=1):
    """Plain-method dam break on a flat bed with a liquid carrier (a gas-only
    carrier at T_ambient has zero reduced gravity in the reference physics
    and does not move, constitutive_2d.f90:1470); particle classes at zero
    concentration."""
    p = default_params()
    p.precision = precision
    p.comp_cells_x, p.comp_cells_y, p.cell_size = nx, ny, dx
    p.x0 = p.y0 = 0.0
    p.n_solid = n_solid
    p.gas_flag, p.liquid_flag, p.energy_flag = 0, 1, 0
    p.rheology_flag = 0
    _gas_common(p)
    p.rho_l, p.sp_heat_l, p.kin_visc_l, p.loss_rate = 1000.0, 4186.0, 1.0e-6, 0.0
    for i in range(n_solid):
        p.rho_s[i], p.diam_s[i], p.sp_heat_s[i] = 2500.0, 1.0e-4 * 10 ** i, 1100.0
    p.n_rk = n_rk
    p.cfl, p.dt0, p.max_dt = 0.24, 1.0e-3, 1.0
    p.set_bc_all(1, 0.0)
    p.t_start, p.t_end = 0.0, t_end
    p.dt_output = 2.0 * (p.t_end - p.t_start)
    B = np.zeros((ny, nx))
    x = (np.arange(nx) + 0.5) * dx
    h = np.where(x[None, :] < 0.5 * nx * dx, 1.0, 0.1) * np.ones((ny, 1))
    q = rest_state_q(p, h, 300.0, [0.0] * n_solid)
    return p, B, q


def pyroclastic(nx=1024, ny=1024, dx=10.0, precision=PREC_FP64, t_end=600.0, seed=1,
                n_rk=2, settling=True, entrainment=False, n_solid=2):
    """Single pyroclastic-style current from a ring source at the summit of
    a Gaussian cone (height 1500 m, sigma 2 km) with fBm noise."""
    p = default_params()
    p.precision = precision
    p.comp_cells_x, p.comp_cells_y, p.cell_size = nx, ny, dx
    p.x0 = p.y0 = 0.0
    p.n_solid = n_solid
    p.gas_flag, p.liquid_flag, p.energy_flag = 1, 0, 1
    p.rheology_flag, p.rheology_model = 1, 1
    p.mu, p.xi = 0.1, 1000.0
    p.slope_correction_flag = 1
    _gas_common(p)
    diam = [1.0e-4, 1.0e-3, 1.0e-5][:n_solid]
    rho = [2500.0, 1500.0, 2500.0][:n_solid]
    alph = [0.01, 0.02, 0.01][:n_solid]
    for i in range(n_solid):
        p.rho_s[i], p.diam_s[i], p.sp_heat_s[i] = rho[i], diam[i], 1100.0
        p.alphas_source[i] = alph[i]
    p.settling_flag = 1 if settling else 0
    p.entrainment_flag = 1 if entrainment else 0
    p.radial_source_flag = 1
    p.x_source, p.y_source, p.r_source = 0.5 * nx * dx, 0.5 * ny * dx, 50.0
    p.mfr_source, p.vel_source, p.T_source = 1.0e6, 20.0, 1000.0
    p.n_rk = n_rk
    p.cfl, p.dt0, p.max_dt = 0.24, 1.0e-2, 10.0
    p.set_bc_all(1, 0.0)
    p.t_start, p.t_end = 0.0, t_end
    p.dt_output = 2.0 * (p.t_end - p.t_start)
    B = cone_fbm_dem(nx, ny, dx, seed=seed)
    q = np.zeros((p.n_vars, ny, nx))
    return p, B, q


def bottom_source_flow(nx=96, ny=80, dx=10.0, precision=PREC_FP64, t_end=60.0, intervals=False,
                       angle=30.0, erosion=False, topo_change=False, vuln=False, seed=3):
    """Hot particle-laden gas rising from a bottom radial source (an
    ellipse of semi-axes 60 m x 40 m turned by `angle` degrees, vertical
    inflow 4 m/s ramped by time_param, or piecewise-constant intervals) on
    a cone + fBm DEM, with Voellmy friction, slope correction, settling and
    optionally erosion of a 0.5 m erodible layer with topography change and
    a vulnerability table."""
    p = default_params()
    p.precision = precision
    p.comp_cells_x, p.comp_cells_y, p.cell_size = nx, ny, dx
    p.x0 = p.y0 = 0.0
    p.n_solid = 2
    p.gas_flag, p.liquid_flag, p.energy_flag = 1, 0, 1
    p.rheology_flag, p.rheology_model = 1, 1
    p.mu, p.xi = 0.15, 800.0
    p.slope_correction_flag = 1
    _gas_common(p)
    for i, (rho, d, a) in enumerate([(2500.0, 2.0e-4, 0.04), (1500.0, 1.0e-3, 0.02)]):
        p.rho_s[i], p.diam_s[i], p.sp_heat_s[i] = rho, d, 1100.0
        p.alphas_source[i] = a
    p.settling_flag = 1
    p.bottom_radial_source_flag = 1
    p.x_source, p.y_source = 0.45 * nx * dx, 0.5 * ny * dx
    p.r_source, p.r2_source, p.angle_source = 60.0, 40.0, angle
    p.vel_source, p.T_source = 4.0, 900.0
    p.h_source = p.mfr_source = -1.0
    if intervals:
        p.n_intervals = 3
        for i, (t, v) in enumerate([(0.0, 4.0), (8.0, 0.0), (14.0, 6.0)]):
            p.t_intervals[i], p.vel_intervals[i] = t, v
    else:
        p.time_param[0], p.time_param[1], p.time_param[2], p.time_param[3] = 40.0, 30.0, 5.0, 0.0
    if erosion:
        p.erosion_coeff = 2.0e-4
        p.erodible_porosity = 0.35
        p.T_erodible = 320.0
        p.initial_erodible_thickness = 0.5
        p.erodible_fract[0], p.erodible_fract[1] = 0.75, 0.5    # normalised to 0.6 / 0.4
        p.topo_change_flag = 1 if topo_change else 0
    if vuln:
        for i, v in enumerate([0.05, 0.5, 2.0]):
            p.thickness_levels[i] = v
        for i, v in enumerate([10.0, 500.0]):
            p.dyn_pres_levels[i] = v
    p.n_rk = 2
    p.cfl, p.dt0, p.max_dt = 0.24, 1.0e-2, 10.0
    p.set_bc_all(1, 0.0)
    p.t_start, p.t_end = 0.0, t_end
    p.dt_output = 2.0 * (p.t_end - p.t_start)
    B = cone_fbm_dem(nx, ny, dx, height=120.0, sigma=600.0, rms=2.0, seed=seed)
    q = np.zeros((p.n_vars, ny, nx))
    return p, B, q


def eroding_dam_break(nx=120, ny=60, dx=2.0, precision=PREC_FP64, t_end=12.0, deposit_flag=False,
                      topo_change=True):
    """A 2 m high column of sediment-laden water released on a 6 % slope
    over a 0.3 m erodible bed (liquid carrier, two particle classes,
    settling, erosion, topography change)."""
    p = default_params()
    p.precision = precision
    p.comp_cells_x, p.comp_cells_y, p.cell_size = nx, ny, dx
    p.x0 = p.y0 = 0.0
    p.n_solid = 2
    p.gas_flag, p.liquid_flag, p.energy_flag = 0, 1, 0
    p.rheology_flag, p.rheology_model = 1, 1
    p.mu, p.xi = 0.05, 500.0
    p.slope_correction_flag = 1
    _gas_common(p)
    p.rho_l, p.sp_heat_l, p.kin_visc_l, p.loss_rate = 1000.0, 4186.0, 1.0e-6, 0.0
    for i, (rho, d) in enumerate([(2600.0, 3.0e-4), (2000.0, 1.0e-4)]):
        p.rho_s[i], p.diam_s[i], p.sp_heat_s[i] = rho, d, 900.0
    p.settling_flag = 1
    p.erosion_coeff = 1.0e-3
    p.erodible_porosity = 0.4
    p.T_erodible = 290.0
    p.initial_erodible_thickness = 0.3
    p.erodible_fract[0], p.erodible_fract[1] = 0.5, 0.5
    p.erodible_deposit_flag = 1 if deposit_flag else 0
    p.topo_change_flag = 1 if topo_change else 0
    p.n_rk = 2
    p.cfl, p.dt0, p.max_dt = 0.24, 1.0e-3, 1.0
    p.set_bc_all(1, 0.0)
    p.t_start, p.t_end = 0.0, t_end
    p.dt_output = 2.0 * (p.t_end - p.t_start)
    x = (np.arange(nx) + 0.5) * dx
    y = (np.arange(ny) + 0.5) * dx
    B = np.broadcast_to(0.06 * (nx * dx - x)[None, :], (ny, nx)).copy()
    r2 = (x[None, :] - 0.2 * nx * dx) ** 2 + (y[:, None] - 0.5 * ny * dx) ** 2
    h = np.where(r2 <= (0.15 * ny * dx) ** 2, 2.0, 0.0)
    q = rest_state_q(p, h, 290.0, [0.15, 0.1])
    return p, B, q


def granular_slide(nx=120, ny=64, dx=2.0, precision=PREC_FP64, t_end=20.0, n_solid=1):
    """A dense granular column (solid fraction 0.5, 1 mm grains) released
    on a 35-degree slope into a run-out flat, with the mu(I) rheology 11
    (mu_s 0.48, mu_2 0.73, I_0 0.279, muI_inf 0.005) and slope correction;
    air carrier at ambient temperature."""
    p = default_params()
    p.precision = precision
    p.comp_cells_x, p.comp_cells_y, p.cell_size = nx, ny, dx
    p.x0 = p.y0 = 0.0
    p.n_solid = n_solid
    p.gas_flag, p.liquid_flag, p.energy_flag = 1, 0, 1
    p.rheology_flag, p.rheology_model = 1, 11
    p.mu_s, p.mu_2, p.I_0, p.muI_inf = 0.48, 0.73, 0.279, 0.005
    p.slope_correction_flag = 1
    _gas_common(p)
    for i, (rho, d) in enumerate([(2500.0, 1.0e-3), (1800.0, 4.0e-3), (2700.0, 5.0e-4)][:n_solid]):
        p.rho_s[i], p.diam_s[i], p.sp_heat_s[i] = rho, d, 1100.0
    p.n_rk = 2
    p.cfl, p.dt0, p.max_dt = 0.24, 1.0e-3, 1.0
    p.set_bc_all(1, 0.0)
    p.t_start, p.t_end = 0.0, t_end
    p.dt_output = 2.0 * (p.t_end - p.t_start)
    x = (np.arange(nx) + 0.5) * dx
    y = (np.arange(ny) + 0.5) * dx
    xb = 0.6 * nx * dx
    z = np.where(x < xb, np.tan(np.radians(35.0)) * (xb - x), 0.0)
    B = np.broadcast_to(z[None, :], (ny, nx)).copy()
    r2 = (x[None, :] - 0.15 * nx * dx) ** 2 + (y[:, None] - 0.5 * ny * dx) ** 2
    h = np.where(r2 <= (0.2 * ny * dx) ** 2, 2.0, 0.0)
    alphas = [0.5 / n_solid] * n_solid
    q = rest_state_q(p, h, 300.0, alphas)
    return p, B, q


def developed_current_state(p, B, radius=3500.0, h_max=3.0, u_max=15.0, T=950.0, seed=11):
    """A spread gas-particle current over the cone, as a seeded stand-in for
    the state of the pyroclastic run a few minutes after the inlet opened:
    thickness 1 - (r/R)^2 profile (max h_max), radial velocity growing as
    sqrt(r/R) up to u_max, uniform temperature T, the inlet's particle volume
    fractions, and a 5 % seeded perturbation of h.  Returns q (n_vars, ny, nx)."""
    nx, ny, dx = p.comp_cells_x, p.comp_cells_y, p.cell_size
    x = p.x0 + (np.arange(nx) + 0.5) * dx
    y = p.y0 + (np.arange(ny) + 0.5) * dx
    X, Y = np.meshgrid(x, y)
    dxs, dys = X - p.x_source, Y - p.y_source
    r = np.sqrt(dxs * dxs + dys * dys)
    rr = np.minimum(r / radius, 1.0)
    pert = 1.0 + 0.05 * (uniform01(seed, nx * ny).reshape(ny, nx) - 0.5)
    # the ring interior stays dry: the reference never updates those cells
    h = np.where((r < radius) & (r > p.r_source), h_max * (1.0 - rr * rr) * pert, 0.0)
    ur = u_max * np.sqrt(rr)
    with np.errstate(invalid="ignore", divide="ignore"):
        ex = np.where(r > 0, dxs / r, 0.0)
        ey = np.where(r > 0, dys / r, 0.0)
    alphas = [p.alphas_source[i] for i in range(p.n_solid)]
    q = rest_state_q(p, h, T, alphas)
    # add momentum and, with the energy equation, its kinetic energy
    q[1] = q[0] * ur * ex
    q[2] = q[0] * ur * ey
    if p.energy_flag:
        q[3] = q[3] + 0.5 * q[0] * ur * ur
    return q


def ensemble_params(index, precision=PREC_FP32, steps=2000):
    """Member `index` of the 256-run ensemble; its draws use seed = index."""
    u = uniform01(0x5EED0000 + index, 8)
    side = int(round(math.exp(math.log(128) + u[0] * (math.log(1024) - math.log(128)))))
    side = max(16, side)
    dx = 5.0 + 15.0 * u[1]
    p, B, q = pyroclastic(nx=side, ny=side, dx=dx, precision=precision, seed=index + 1,
                          t_end=1.0e9)
    p.mu = 0.05 + 0.25 * u[2]
    p.xi = 200.0 + 1800.0 * u[3]
    p.r_source = 20.0 + 180.0 * u[4]
    # keep the ring well inside the domain
    p.r_source = min(p.r_source, 0.2 * side * dx)
    p.T_source = 600.0 + 600.0 * u[5]
    p.alphas_source[0] = 0.005 + 0.045 * u[6]
    p.alphas_source[1] = 0.005 + 0.045 * u[7]
    return p, B, q, steps


def large_domain(n=8192, dx=2.0, precision=PREC_FP32, seed=5, t_end=1.0e9):
    """8192^2 diamond-square DEM, 3 classes, entrainment, one ring source."""
    p, _, _ = pyroclastic(nx=8, ny=8, dx=dx, precision=precision, entrainment=True,
                          n_solid=3, t_end=t_end)
    p.comp_cells_x = p.comp_cells_y = n
    p.x_source = p.y_source = 0.5 * n * dx
    pw = int(math.ceil(math.log2(n)))
    Z = diamond_square_dem(pw, 2000.0, 0.8, seed)
    B = Z[:n, :n].copy()
    q = np.zeros((p.n_vars, n, n))
    return p, B, q


def served_job(index, precision=PREC_FP32):
    """Job `index` of the served request stream (draws use seed = index):
    a dam break (liquid carrier) or a ring-inlet current with equal odds,
    grid side log-uniform in [64, 2048], 1-3 particle classes, step count
    uniform in [500, 5000].  Returns (params, B_cent, q, steps, kind)."""
    u = uniform01(0x5E4E0000 + index, 4)
    side = int(round(math.exp(math.log(64) + u[0] * (math.log(2048) - math.log(64)))))
    ns = 1 + min(int(u[1] * 3), 2)
    steps = 500 + min(int(u[2] * 4501), 4500)
    if u[3] < 0.5:
        p, B, q = dam_break(nx=side, ny=side, dx=1.0, precision=precision, t_end=1.0e9, n_solid=ns)
        kind = "dam_break"
    else:
        dx = 10.0
        p, B, q = pyroclastic(nx=side, ny=side, dx=dx, precision=precision, t_end=1.0e9,
                              seed=index + 1, settling=False, n_solid=ns)
        p.r_source = min(50.0, 0.2 * side * dx)
        kind = "ring_inlet"
    return p, B, q, steps, kind


def poisson_arrivals(n, rate, seed=0x5E4E):
    """n arrival times (s) of a Poisson process with the given mean rate."""
    u = uniform01(seed, n)
    gaps = -np.log(np.maximum(1.0 - u, 1e-300)) / rate
    return np.cumsum(gaps) - gaps[0]

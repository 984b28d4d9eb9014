// sflow_kernels.cuh -- the GB300 kernels of one IMEX_SfloW2D time step.
//
// One driver iteration (IMEX_SfloW2D.f90:395-505) with N_RK = 2 runs as
//   k_mask    check_solve: active-cell mask, per-tile activity, cell count
//   k_flux    reconstruction + KT speeds/fluxes + divergence + explicit
//             sources at q0 (stage 1 == timestep state) and the CFL minimum
//   k_dt      dt from the CFL minimum and the driver's clamps; t += dt
//   k_stage2  stage 2 pointwise: semi-implicit friction, implicit Newton,
//             assembly + positivity fixes, erosion/deposition epilogue,
//             post-step maxima
// Other tableaux (N_RK = 1, 3, 4) use k_flux per explicit stage, k_stage for
// each stage and k_assemble.
//
// Layout in HBM: structure of arrays, one plane per conservative variable,
// rows of `pitch` elements (pitch a multiple of 32), plane stride
// pitch*ny.  Per-cell static data: topography terms (5 planes, 8 with the
// curvature term), a flag byte (source ring membership), the ring inlet
// perimeter/normal (read only for ring cells), the active mask byte.
#pragma once
#include <cuda_runtime.h>

#include "sflow_physics.cuh"

namespace sflow {

constexpr int TX = 32;   // tile width  (cells)
constexpr int TY = 8;    // tile height (cells)
constexpr int HALO = 2;  // reconstruction stencil reach for a cell's faces
constexpr int RX = TX + 2 * HALO;
constexpr int RY = TY + 2 * HALO;
constexpr int FLUX_THREADS = 288;  // 9 warps: covers (TX+1)*TY and TX*(TY+1) faces

// flag byte bits
constexpr uint8_t F_SC_MASK = 0x3;  // source_cell (0, 1 ring interior, 2 ring boundary)
constexpr uint8_t F_E = 0x4, F_W = 0x8, F_N = 0x10, F_S = 0x20;
constexpr uint8_t F_ACTIVE = 0x80;  // set in shared memory only

template <class R>
struct KArgs {
  Grid<R> g;
  Phys<R> pr;        // bulk arithmetic constants
  Phys<double> pd;   // FP64 constants (Newton, thresholds)
  BC<R> bc;
  R* q;              // state planes (n_vars)
  R* rd;             // stage residual planes: divFlux - expl (n_vars per stage)
  R* rn;             // stage implicit planes: NH + SI (n_vars per stage)
  R* qs;             // stage state planes (n_vars per stage) / q0 copy
  const R* geo[8];   // Bx, By, Bxx, Bxy, Byy, gc, dgcx, dgcy (Bxx.. may be null)
  const uint8_t* cflags;
  const R* arc;      // 3 planes: perimeter, n_x, n_y
  uint8_t* mask;
  uint8_t* tile_active;
  R* hmax;
  R* pdynmax;
  R* mvmax;
  RunState* st;
  double tableau_at[16], tableau_ad[16], omega_t[4], omega[4];
  int take_last;
};

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ int64_t cidx(const Grid<R>& g, int j, int k) {
  return (int64_t)k * g.pitch + j;
}

__device__ __forceinline__ bool running(const RunState* st) {
  return st->t < st->t_stop && st->steps < st->step_limit;
}

__device__ __forceinline__ unsigned long long dbits(double x) {
  return (unsigned long long)__double_as_longlong(x);
}

// x_stag(j) = x0 + j*dx, x_comp(j) = 0.5*(x_stag(j)+x_stag(j+1))
// (geometry_2d.f90:312-327); in FP32 form the same values rounded to float.
template <class R>
__device__ __forceinline__ R xstag(const Grid<R>& g, int j) {
  if constexpr (sizeof(R) == 8) return g.x0 + (double)j * g.dx;
  else return (R)g.x0 + (R)j * g.rdx;
}
template <class R>
__device__ __forceinline__ R xcomp(const Grid<R>& g, int j) {
  if constexpr (sizeof(R) == 8) return 0.5 * ((g.x0 + (double)j * g.dx) + (g.x0 + (double)(j + 1) * g.dx));
  else return (R)g.x0 + ((R)j + 0.5f) * g.rdx;
}
template <class R>
__device__ __forceinline__ R ystag(const Grid<R>& g, int k) {
  if constexpr (sizeof(R) == 8) return g.y0 + (double)k * g.dy;
  else return (R)g.y0 + (R)k * g.rdy;
}
template <class R>
__device__ __forceinline__ R ycomp(const Grid<R>& g, int k) {
  if constexpr (sizeof(R) == 8) return 0.5 * ((g.y0 + (double)k * g.dy) + (g.y0 + (double)(k + 1) * g.dy));
  else return (R)g.y0 + ((R)k + 0.5f) * g.rdy;
}

template <class R>
__device__ __forceinline__ Geo<R> load_geo(const KArgs<R>& a, int64_t c) {
  Geo<R> g;
  g.Bx = __ldg(a.geo[0] + c);
  g.By = __ldg(a.geo[1] + c);
  g.Bxx = a.geo[2] ? __ldg(a.geo[2] + c) : R(0);
  g.Bxy = a.geo[3] ? __ldg(a.geo[3] + c) : R(0);
  g.Byy = a.geo[4] ? __ldg(a.geo[4] + c) : R(0);
  g.gc = __ldg(a.geo[5] + c);
  g.dgcx = __ldg(a.geo[6] + c);
  g.dgcy = __ldg(a.geo[7] + c);
  return g;
}

// ---------------------------------------------------------------------------
// k_mask: check_solve (solver_2d.f90:667-858).  A cell is active when it is
// within Manhattan distance n_RK of a seed (border cell, wet interior cell,
// ring-boundary cell) and is not a ring-interior cell.
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(TX* TY) k_mask(KArgs<R> a, int solve_all) {
  RunState* st = a.st;
  const double t = st->t;
  if (!running(st)) return;
  const Grid<R>& g = a.g;
  const int j = blockIdx.x * TX + threadIdx.x % TX;
  const int k = blockIdx.y * TY + threadIdx.x / TX;
  const int nrk = a.pd.nrk;
  int act = 0;
  if (j < g.nx && k < g.ny) {
    const int64_t c = cidx(g, j, k);
    const uint8_t fl = a.cflags[c];
    if (solve_all) {
      act = 1;
    } else {
      for (int dk = -nrk; dk <= nrk && !act; ++dk) {
        int kk = k + dk;
        if (kk < 0 || kk >= g.ny) continue;
        int rem = nrk - (dk < 0 ? -dk : dk);
        for (int dj = -rem; dj <= rem; ++dj) {
          int jj = j + dj;
          if (jj < 0 || jj >= g.nx) continue;
          bool border = (jj == 0 || jj == g.nx - 1 || kk == 0 || kk == g.ny - 1);
          if (border) { act = 1; break; }
          int64_t cc = cidx(g, jj, kk);
          if (a.q[cc] > R(0)) { act = 1; break; }
          if (a.pd.radial_source && (a.cflags[cc] & F_SC_MASK) == 2) { act = 1; break; }
        }
      }
    }
    if (a.pd.radial_source && (fl & F_SC_MASK) == 1) act = 0;
    a.mask[c] = (uint8_t)act;
  }
  int cnt = __syncthreads_count(act);
  if (threadIdx.x == 0) {
    a.tile_active[blockIdx.y * gridDim.x + blockIdx.x] = cnt > 0;
    if (cnt) atomicAdd((unsigned long long*)&st->cells_acc[st->steps & 1], (unsigned long long)cnt);
  }
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) {
    st->src_t_coeff = source_time_coeff(st->tp, st->pi_g, t);
  }
}

// ---------------------------------------------------------------------------
// Reconstruction of one side of one face (solver_2d.f90:3095-3924).
// The cell is at region coordinates (rx, ry) of the shared tile, global
// (j, k).  dir 1: x faces, plus = 1 east side, 0 west side; dir 2: y faces,
// plus = 1 north side, 0 south side.  Writes the physical face state qp
// (n_vars+2).  Only the stencil along `dir` enters, apart from the
// reference's use of y_stag in the x slope of v at some ring cells
// (solver_2d.f90:3605, kept as is).
// ---------------------------------------------------------------------------
template <class R, int NS>
__device__ __forceinline__ void recon_side(const KArgs<R>& a, const R* sqp, const uint8_t* sfl,
                                           int rx, int ry, int j, int k, int dir, int plus, R* out) {
  constexpr int nv = 4 + NS, np = nv + 2;
  const Grid<R>& g = a.g;
  const Phys<R>& P = a.pr;
  const int plane = RX * RY;
  auto QP = [&](int i, int ox, int oy) -> R { return sqp[i * plane + (ry + oy) * RX + (rx + ox)]; };
  const uint8_t fl = sfl[ry * RX + rx];
  const int sc = fl & F_SC_MASK;
  const bool radial = P.radial_source;
  const bool src2 = radial && sc == 2;
  R cell[np];
#pragma unroll
  for (int i = 0; i < np; ++i) cell[i] = QP(i, 0, 0);
  R qm[np];   // the reconstructed side (W/S for plus=0, E/N for plus=1)
  if (dir == 1) {
    const int nx = g.nx;
    const bool jb0 = (j == 0), jb1 = (j == nx - 1);
    const bool interior = !jb0 && !jb1;
    const bool sE = fl & F_E, sW = fl & F_W;
    R z0, z1 = xcomp(g, j), z2;
    if (jb0) { z0 = xstag(g, 0); z2 = xcomp(g, 1); }
    else if (jb1) { z0 = xcomp(g, nx - 2); z2 = xstag(g, nx); }
    else {
      z0 = xcomp(g, j - 1); z2 = xcomp(g, j + 1);
      if (src2) { if (sE) z2 = xstag(g, j + 1); else if (sW) z0 = xstag(g, j); }
    }
    // conservative-index variables (vars_loop)
    R wv[nv], ev[nv];
#pragma unroll
    for (int i = 0; i < nv; ++i) {
      R slope;
      const R v1 = cell[i];
      if (jb0) {
        if (sc == 2) slope = limit(cell[i], v1, QP(i, 1, 0), z0, z1, z2, g.limiter[i], g.theta);
        else if (a.bc.flag[SFLOW_W][i] == 0) slope = limit(a.bc.value[SFLOW_W][i], v1, QP(i, 1, 0), z0, z1, z2, g.limiter[i], g.theta);
        else if (a.bc.flag[SFLOW_W][i] == 1) slope = a.bc.value[SFLOW_W][i];
        else slope = (QP(i, 1, 0) - QP(i, 0, 0)) * g.one_by_dx;
      } else if (jb1) {
        if (sc == 2) slope = limit(QP(i, -1, 0), v1, cell[i], z0, z1, z2, g.limiter[i], g.theta);
        else if (a.bc.flag[SFLOW_E][i] == 0) slope = limit(QP(i, -1, 0), v1, a.bc.value[SFLOW_E][i], z0, z1, z2, g.limiter[i], g.theta);
        else if (a.bc.flag[SFLOW_E][i] == 1) slope = a.bc.value[SFLOW_E][i];
        else slope = (QP(i, 0, 0) - QP(i, -1, 0)) * g.one_by_dx;
      } else {
        R v0 = QP(i, -1, 0), v2 = QP(i, 1, 0);
        if (src2) { if (sE) v2 = cell[i]; else if (sW) v0 = cell[i]; }
        slope = limit(v0, v1, v2, z0, z1, z2, g.limiter[i], g.theta);
      }
      const R dq = g.rc * g.dx2 * slope;
      R w = v1 - dq, e = v1 + dq;
      if (jb0) {
        if (sc == 2) w = cell[i];
        else if (a.bc.flag[SFLOW_W][i] == 0) w = a.bc.value[SFLOW_W][i];
        else if (i == 1) w = rmin(w, R(0));
      }
      if (jb1) {
        if (sc == 2) e = cell[i];
        else if (a.bc.flag[SFLOW_E][i] == 0) e = a.bc.value[SFLOW_E][i];
        else if (i == 1) e = rmax(e, R(0));
      }
      wv[i] = w;
      ev[i] = e;
      qm[i] = plus ? e : w;
    }
    // velocities (add_vars_loop); qp_to_qp2 (constitutive_2d.f90:2164-2188)
    // gives u = hu/h, v = hv/h of the west/east state at the domain edges
    const bool kint = (k > 0 && k < g.ny - 1);
    const bool sN = fl & F_N, sS = fl & F_S;
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      const int i = nv + m;
      const R v1 = cell[i];
      const R uw = (wv[0] <= R(0)) ? R(0) : wv[1 + m] / wv[0];
      const R ue = (ev[0] <= R(0)) ? R(0) : ev[1 + m] / ev[0];
      R v0, v2, zz0 = z0, zz2 = z2;
      if (jb0) {
        v0 = uw;
        v2 = QP(i, 1, 0);
      } else if (jb1) {
        v0 = QP(i, -1, 0);
        v2 = ue;
      } else {
        v0 = QP(i, -1, 0);
        v2 = QP(i, 1, 0);
        if (m == 1 && src2 && kint && !sS && sN) zz2 = ystag(g, k + 1);
        if (src2) {
          if (sE) { zz2 = xstag(g, j + 1); v2 = cell[i]; }
          else if (sW) { zz0 = xstag(g, j); v0 = cell[i]; }
        }
      }
      const R slope = limit(v0, v1, v2, zz0, z1, zz2, g.limiter[i], g.theta);
      const R dq = g.rc * g.dx2 * slope;
      R val = plus ? v1 + dq : v1 - dq;
      if (jb0 && !plus) val = uw;
      if (jb1 && plus) val = ue;
      qm[i] = val;
    }
    if (interior && src2) {
      if (plus && sE) {
#pragma unroll
        for (int i = 0; i < np; ++i) qm[i] = cell[i];
      } else if (!plus && sW && !sE) {
#pragma unroll
        for (int i = 0; i < np; ++i) qm[i] = cell[i];
      }
    }
  } else {
    const int ny = g.ny;
    const bool kb0 = (k == 0), kb1 = (k == ny - 1);
    const bool interior = !kb0 && !kb1;
    const bool sN = fl & F_N, sS = fl & F_S;
    R z0, z1 = ycomp(g, k), z2;
    if (kb0) { z0 = ystag(g, 0); z2 = ycomp(g, 1); }
    else if (kb1) { z0 = ycomp(g, ny - 2); z2 = ystag(g, ny); }
    else {
      z0 = ycomp(g, k - 1); z2 = ycomp(g, k + 1);
      if (src2) { if (sS) z0 = ystag(g, k); else if (sN) z2 = ystag(g, k + 1); }
    }
    R sv[nv], nvv[nv];
#pragma unroll
    for (int i = 0; i < nv; ++i) {
      R slope;
      const R v1 = cell[i];
      if (kb0) {
        if (a.bc.flag[SFLOW_S][i] == 0) slope = limit(a.bc.value[SFLOW_S][i], v1, QP(i, 0, 1), z0, z1, z2, g.limiter[i], g.theta);
        else if (a.bc.flag[SFLOW_S][i] == 1) slope = a.bc.value[SFLOW_S][i];
        else slope = (QP(i, 0, 1) - QP(i, 0, 0)) * g.one_by_dy;
      } else if (kb1) {
        if (a.bc.flag[SFLOW_N][i] == 0) slope = limit(QP(i, 0, -1), v1, a.bc.value[SFLOW_N][i], z0, z1, z2, g.limiter[i], g.theta);
        else if (a.bc.flag[SFLOW_N][i] == 1) slope = a.bc.value[SFLOW_N][i];
        else slope = (QP(i, 0, 0) - QP(i, 0, -1)) * g.one_by_dy;
      } else {
        R v0 = QP(i, 0, -1), v2 = QP(i, 0, 1);
        if (src2) { if (sS) v0 = cell[i]; else if (sN) v2 = cell[i]; }
        slope = limit(v0, v1, v2, z0, z1, z2, g.limiter[i], g.theta);
      }
      const R dq = g.rc * g.dy2 * slope;
      R s_ = v1 - dq, n_ = v1 + dq;
      if (kb0) {
        if (a.bc.flag[SFLOW_S][i] == 0) s_ = a.bc.value[SFLOW_S][i];
        else if (i == 2) s_ = rmin(s_, R(0));
      }
      if (kb1) {
        if (a.bc.flag[SFLOW_N][i] == 0) n_ = a.bc.value[SFLOW_N][i];
        else if (i == 2) n_ = rmax(n_, R(0));
      }
      sv[i] = s_;
      nvv[i] = n_;
      qm[i] = plus ? n_ : s_;
    }
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      const int i = nv + m;
      const R v1 = cell[i];
      const R us = (sv[0] <= R(0)) ? R(0) : sv[1 + m] / sv[0];
      const R un = (nvv[0] <= R(0)) ? R(0) : nvv[1 + m] / nvv[0];
      R v0, v2, zz0 = z0;
      if (kb0) {
        v0 = us;
        v2 = QP(i, 0, 1);
      } else if (kb1) {
        v0 = QP(i, 0, -1);
        v2 = un;
      } else {
        v0 = QP(i, 0, -1);
        v2 = QP(i, 0, 1);
        if (src2) {
          if (sS) { zz0 = ystag(g, k); v0 = cell[i]; }
          else if (sN) { v2 = cell[i]; }
        }
      }
      const R slope = limit(v0, v1, v2, zz0, z1, z2, g.limiter[i], g.theta);
      const R dq = g.rc * g.dy2 * slope;
      R val = plus ? v1 + dq : v1 - dq;
      if (kb0 && !plus) val = us;
      if (kb1 && plus) val = un;
      qm[i] = val;
    }
    if (interior && src2) {
      if (!plus && sS) {
#pragma unroll
        for (int i = 0; i < np; ++i) qm[i] = cell[i];
      } else if (plus && sN && !sS) {
#pragma unroll
        for (int i = 0; i < np; ++i) qm[i] = cell[i];
      }
    }
  }
#pragma unroll
  for (int i = 0; i < np; ++i) out[i] = qm[i];
}

// One side of a face reduced to what the KT flux needs.
template <class R, int NS>
struct Side {
  R q[4 + NS];
  R f[4 + NS];
  R vmin, vmax;
  R hu_p;   // qp(2): x zero-velocity test
};

template <class R, int NS>
__device__ __forceinline__ void side_from_qp(const KArgs<R>& a, const R* qp, R gcs, int dir,
                                             Side<R, NS>& s, int negate = -1) {
  const Phys<R>& P = a.pr;
  qp_to_qc<R, NS>(P, qp, s.q);
  if (negate >= 0) s.q[negate] = -s.q[negate];
  Mixt<R> m = mixt_var<R, NS>(P, qp, false);
  local_speeds<R, NS>(P, qp, m.red_grav, gcs, dir, s.vmin, s.vmax);
  eval_fluxes<R, NS>(P, s.q, qp, m, gcs, dir, s.f);
  s.hu_p = qp[1];
}

template <class R, int NS>
__device__ __forceinline__ void side_zero(Side<R, NS>& s) {
#pragma unroll
  for (int i = 0; i < 4 + NS; ++i) { s.q[i] = R(0); s.f[i] = R(0); }
  s.vmin = R(0); s.vmax = R(0); s.hu_p = R(0);
}

// KT flux across one face (solver_2d.f90:2834-3049).  H has n_vars entries.
template <class R, int NS>
__device__ __forceinline__ R kt_flux(const Side<R, NS>& L, const Side<R, NS>& Rt, int dir, R* H) {
  constexpr int nv = 4 + NS, ns = NS;
  R a1 = rmin(rmin(L.vmin, Rt.vmin), R(0));
  R a2 = rmax(rmax(L.vmax, Rt.vmax), R(0));
  if (a1 == a2) {
#pragma unroll
    for (int i = 0; i < nv; ++i) H[i] = R(0);
  } else {
    const R den = a2 - a1;
    const R fac = (a2 * a1) / den;
#pragma unroll
    for (int i = 0; i < nv; ++i) {
      R avg = (a2 * L.f[i] - a1 * Rt.f[i]) / den;
      H[i] = avg + fac * (Rt.q[i] - L.q[i]);
    }
  }
  if (ns > 0) {
    if (dir == 1) {
      R s = R(0), s2 = R(0);
#pragma unroll
      for (int i = 0; i < ns; ++i) { s += H[4 + i] / H[0]; s2 += H[4 + i]; }
      if (s2 / H[0] >= R(1)) {
#pragma unroll
        for (int i = 0; i < ns; ++i) H[4 + i] = H[4 + i] / s;
      }
    } else {
      R s = R(0);
#pragma unroll
      for (int i = 0; i < ns; ++i) s += H[4 + i];
      if (s / H[0] > R(1)) {
        const R r = s / H[0];
#pragma unroll
        for (int i = 0; i < ns; ++i) H[4 + i] = H[4 + i] / r;
      }
    }
  }
  const bool zero_vel = (dir == 1) ? (L.hu_p == R(0) && Rt.hu_p == R(0))
                                   : (L.q[2] == R(0) && Rt.q[2] == R(0));
  if (zero_vel) {
    H[0] = R(0);
#pragma unroll
    for (int i = 3; i < nv; ++i) H[i] = R(0);
  }
  return rmax(a2, -a1);
}

// ---------------------------------------------------------------------------
// k_flux: divFlux - expl_terms of one explicit stage for every active cell
// of a 32x8 tile (eval_hyperbolic_terms, solver_2d.f90:2616-2693, and
// eval_expl_terms), plus the CFL minimum of timestep (solver_2d.f90:873-1006)
// when want_dt.  The tile's qp (with a 2-cell halo) is computed once into
// shared memory; each thread then evaluates one face (both reconstructed
// sides, speeds, physical fluxes, KT flux) and finally one cell.
// ---------------------------------------------------------------------------
template <class R, int NS>
__global__ void __launch_bounds__(FLUX_THREADS) k_flux(KArgs<R> a, const R* __restrict__ qin,
                                                       R* __restrict__ rout, int want_dt) {
  constexpr int nv = 4 + NS, np = nv + 2;
  const RunState* st = a.st;
  if (!running(st)) return;
  if (!a.tile_active[blockIdx.y * gridDim.x + blockIdx.x]) return;
  const Grid<R>& g = a.g;
  const Phys<R>& P = a.pr;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  R* sqp = reinterpret_cast<R*>(smem_raw);                       // np * RX*RY
  R* sHx = sqp + np * RX * RY;                                   // nv * TY*(TX+1)
  R* sHy = sHx + nv * TY * (TX + 1);                             // nv * (TY+1)*TX
  R* sAx = sHy + nv * (TY + 1) * TX;                             // TY*(TX+1)
  R* sAy = sAx + TY * (TX + 1);                                  // (TY+1)*TX
  uint8_t* sfl = reinterpret_cast<uint8_t*>(sAy + (TY + 1) * TX);  // RX*RY
  const int j0 = blockIdx.x * TX, k0 = blockIdx.y * TY;
  const int tid = threadIdx.x;

  // 1. physical variables of the tile + halo (qc_to_qp; inactive = dry)
  for (int idx = tid; idx < RX * RY; idx += FLUX_THREADS) {
    const int rx = idx % RX, ry = idx / RX;
    const int j = j0 + rx - HALO, k = k0 + ry - HALO;
    R qp[np];
    uint8_t fl = 0;
    bool wet = false;
    if (j >= 0 && j < g.nx && k >= 0 && k < g.ny) {
      const int64_t c = cidx(g, j, k);
      fl = a.cflags[c];
      if (a.mask[c]) {
        fl |= F_ACTIVE;
        R q[nv];
#pragma unroll
        for (int i = 0; i < nv; ++i) q[i] = qin[i * g.plane + c];
        if (q[0] > R(0)) { qc_to_qp<R, NS>(P, q, qp); wet = true; }
      }
    }
    if (!wet) {
#pragma unroll
      for (int i = 0; i < np; ++i) qp[i] = R(0);
      qp[3] = P.T_ambient;
    }
#pragma unroll
    for (int i = 0; i < np; ++i) sqp[i * RX * RY + idx] = qp[i];
    sfl[idx] = fl;
  }
  __syncthreads();

  // 2. x faces: face f = j0+fx between cells f-1 and f
  for (int fi = tid; fi < (TX + 1) * TY; fi += FLUX_THREADS) {
    const int fx = fi % (TX + 1), fy = fi / (TX + 1);
    const int f = j0 + fx, k = k0 + fy;
    R H[nv];
    R amax = R(0);
    bool done = false;
    if (k < g.ny && f <= g.nx) {
      const int rxl = fx - 1 + HALO, rxr = fx + HALO, ry = fy + HALO;
      const bool actl = (f - 1 >= 0) && (sfl[ry * RX + rxl] & F_ACTIVE);
      const bool actr = (f < g.nx) && (sfl[ry * RX + rxr] & F_ACTIVE);
      if (actl || actr) {
        const int64_t cl = cidx(g, f > 0 ? f - 1 : 0, k), cr = cidx(g, f < g.nx ? f : g.nx - 1, k);
        R gcs;
        if (f == 0) gcs = __ldg(a.geo[5] + cr);
        else if (f == g.nx) gcs = __ldg(a.geo[5] + cl);
        else gcs = cst<R>(0.5) * (__ldg(a.geo[5] + cl) + __ldg(a.geo[5] + cr));
        Side<R, NS> L, Rt;
        R qp[np];
        if (f == 0) {
          recon_side<R, NS>(a, sqp, sfl, rxr, ry, f, k, 1, 0, qp);
          side_from_qp<R, NS>(a, qp, gcs, 1, Rt);
          L = Rt;
        } else if (f == g.nx) {
          recon_side<R, NS>(a, sqp, sfl, rxl, ry, f - 1, k, 1, 1, qp);
          side_from_qp<R, NS>(a, qp, gcs, 1, L);
          Rt = L;
        } else {
          const uint8_t fll = sfl[ry * RX + rxl], flr = sfl[ry * RX + rxr];
          const bool mirror_r = actl && P.radial_source && (fll & F_SC_MASK) == 2 && (fll & F_E) &&
                                f - 1 > 0 && f - 1 < g.nx - 1;
          const bool mirror_l = !mirror_r && actr && P.radial_source && (flr & F_SC_MASK) == 2 &&
                                (flr & F_W) && !(flr & F_E) && f > 0 && f < g.nx - 1;
          if (actl) {
            recon_side<R, NS>(a, sqp, sfl, rxl, ry, f - 1, k, 1, 1, qp);
            side_from_qp<R, NS>(a, qp, gcs, 1, L);
            if (mirror_r) {
              // wall mirror: only hu (q) and u (qp) change sign
              // (solver_2d.f90:3735-3738); qp(2) keeps its sign
              qp[nv] = -qp[nv];
              side_from_qp<R, NS>(a, qp, gcs, 1, Rt, 1);
            }
          } else {
            side_zero(L);
          }
          if (!mirror_r) {
            if (actr) {
              recon_side<R, NS>(a, sqp, sfl, rxr, ry, f, k, 1, 0, qp);
              side_from_qp<R, NS>(a, qp, gcs, 1, Rt);
              if (mirror_l) {
                qp[nv] = -qp[nv];
                side_from_qp<R, NS>(a, qp, gcs, 1, L, 1);
              }
            } else {
              side_zero(Rt);
            }
          }
        }
        amax = kt_flux<R, NS>(L, Rt, 1, H);
        done = true;
      }
    }
    if (!done) {
#pragma unroll
      for (int i = 0; i < nv; ++i) H[i] = R(0);
    }
#pragma unroll
    for (int i = 0; i < nv; ++i) sHx[i * TY * (TX + 1) + fi] = H[i];
    sAx[fi] = amax;
  }

  // 3. y faces: face f = k0+fy between cells f-1 and f
  for (int fi = tid; fi < TX * (TY + 1); fi += FLUX_THREADS) {
    const int fx = fi % TX, fy = fi / TX;
    const int j = j0 + fx, f = k0 + fy;
    R H[nv];
    R amax = R(0);
    bool done = false;
    if (j < g.nx && f <= g.ny) {
      const int rx = fx + HALO, ryb = fy - 1 + HALO, ryt = fy + HALO;
      const bool actb = (f - 1 >= 0) && (sfl[ryb * RX + rx] & F_ACTIVE);
      const bool actt = (f < g.ny) && (sfl[ryt * RX + rx] & F_ACTIVE);
      if (actb || actt) {
        const int64_t cb = cidx(g, j, f > 0 ? f - 1 : 0), ct = cidx(g, j, f < g.ny ? f : g.ny - 1);
        R gcs;
        if (f == 0) gcs = __ldg(a.geo[5] + ct);
        else if (f == g.ny) gcs = __ldg(a.geo[5] + cb);
        else gcs = cst<R>(0.5) * (__ldg(a.geo[5] + cb) + __ldg(a.geo[5] + ct));
        Side<R, NS> B, T;
        R qp[np];
        if (f == 0) {
          recon_side<R, NS>(a, sqp, sfl, rx, ryt, j, f, 2, 0, qp);
          side_from_qp<R, NS>(a, qp, gcs, 2, T);
          B = T;
        } else if (f == g.ny) {
          recon_side<R, NS>(a, sqp, sfl, rx, ryb, j, f - 1, 2, 1, qp);
          side_from_qp<R, NS>(a, qp, gcs, 2, B);
          T = B;
        } else {
          const uint8_t flb = sfl[ryb * RX + rx], flt = sfl[ryt * RX + rx];
          // cell below with ring to its north mirrors onto the top side
          const bool mirror_t = actb && P.radial_source && (flb & F_SC_MASK) == 2 && (flb & F_N) &&
                                !(flb & F_S) && f - 1 > 0 && f - 1 < g.ny - 1;
          const bool mirror_b = !mirror_t && actt && P.radial_source && (flt & F_SC_MASK) == 2 &&
                                (flt & F_S) && f > 0 && f < g.ny - 1;
          if (actb) {
            recon_side<R, NS>(a, sqp, sfl, rx, ryb, j, f - 1, 2, 1, qp);
            side_from_qp<R, NS>(a, qp, gcs, 2, B);
            if (mirror_t) {
              qp[nv + 1] = -qp[nv + 1];
              side_from_qp<R, NS>(a, qp, gcs, 2, T, 2);
            }
          } else {
            side_zero(B);
          }
          if (!mirror_t) {
            if (actt) {
              recon_side<R, NS>(a, sqp, sfl, rx, ryt, j, f, 2, 0, qp);
              side_from_qp<R, NS>(a, qp, gcs, 2, T);
              if (mirror_b) {
                qp[nv + 1] = -qp[nv + 1];
                side_from_qp<R, NS>(a, qp, gcs, 2, B, 2);
              }
            } else {
              side_zero(T);
            }
          }
        }
        amax = kt_flux<R, NS>(B, T, 2, H);
        done = true;
      }
    }
    if (!done) {
#pragma unroll
      for (int i = 0; i < nv; ++i) H[i] = R(0);
    }
#pragma unroll
    for (int i = 0; i < nv; ++i) sHy[i * (TY + 1) * TX + fi] = H[i];
    sAy[fi] = amax;
  }
  __syncthreads();

  // 4. cells: divergence, explicit terms, CFL step
  double dtloc = 1.0e300;
  if (tid < TX * TY) {
    const int cx = tid % TX, cy = tid / TX;
    const int j = j0 + cx, k = k0 + cy;
    const int rx = cx + HALO, ry = cy + HALO;
    if (j < g.nx && k < g.ny && (sfl[ry * RX + rx] & F_ACTIVE)) {
      const int64_t c = cidx(g, j, k);
      R qp[np];
#pragma unroll
      for (int i = 0; i < np; ++i) qp[i] = sqp[i * RX * RY + ry * RX + rx];
      R e[nv];
      const Geo<R> geo = load_geo(a, c);
      const uint8_t fl = sfl[ry * RX + rx];
      R ap = R(0), anx = R(0), any_ = R(0);
      if (P.radial_source && (fl & F_SC_MASK) == 2) {
        ap = __ldg(a.arc + c);
        anx = __ldg(a.arc + g.plane + c);
        any_ = __ldg(a.arc + 2 * g.plane + c);
      }
      expl_terms<R, NS>(P, geo, qp, (R)st->src_t_coeff, ap, anx, any_, e);
#pragma unroll
      for (int i = 0; i < nv; ++i) {
        R d = R(0);
        d = d + (sHx[i * TY * (TX + 1) + cy * (TX + 1) + cx + 1] - sHx[i * TY * (TX + 1) + cy * (TX + 1) + cx]) * g.one_by_dx;
        d = d + (sHy[i * (TY + 1) * TX + (cy + 1) * TX + cx] - sHy[i * (TY + 1) * TX + cy * TX + cx]) * g.one_by_dy;
        rout[i * g.plane + c] = d - e[i];
      }
      if (want_dt) {
        R ax = rmax(sAx[cy * (TX + 1) + cx], sAx[cy * (TX + 1) + cx + 1]);
        R ay = rmax(sAy[cy * TX + cx], sAy[(cy + 1) * TX + cx]);
        if constexpr (sizeof(R) == 8) {
          double dtx = (ax > 0.0) ? g.cfl * g.dx / ax : 1.0e300;
          double dty = (ay > 0.0) ? g.cfl * g.dy / ay : 1.0e300;
          dtloc = rmin(dtx, dty);
        } else {
          // FP32 form: the CFL bound in float, widened once per block
          float dtx = (ax > 0.0f) ? g.cfl_dx / ax : 3.0e38f;
          float dty = (ay > 0.0f) ? g.cfl_dy / ay : 3.0e38f;
          float m = fminf(dtx, dty);
          dtloc = (m < 3.0e38f) ? (double)m : 1.0e300;
        }
      }
    }
  }
  if (want_dt) {
    // block minimum: warp shuffle then shared memory
    unsigned long long b = dbits(dtloc);
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long ob = __shfl_xor_sync(0xffffffffu, b, o);
      b = ob < b ? ob : b;
    }
    __shared__ unsigned long long wmin[FLUX_THREADS / 32];
    if ((tid & 31) == 0) wmin[tid >> 5] = b;
    __syncthreads();
    if (tid == 0) {
      unsigned long long m = wmin[0];
      for (int w = 1; w < FLUX_THREADS / 32; ++w) m = wmin[w] < m ? wmin[w] : m;
      if (m < dbits(1.0e300)) atomicMin(&a.st->dtmin_bits, m);
    }
  }
}

// ---------------------------------------------------------------------------
// k_dt: dt of this step (timestep + IMEX_SfloW2D.f90:417-439), one thread.
// ---------------------------------------------------------------------------
static __global__ void k_dt(RunState* st, double max_dt) {
  if (!running(st)) { st->run_step = 0; return; }
  double dtmin = __longlong_as_double((long long)st->dtmin_bits);
  double dt = max_dt;
  if (dtmin < dt) dt = dtmin;
  if (st->t_end - st->t_output < 1.0e-7) st->t_output = st->t_end;
  if (st->t + dt > st->t_end) dt = st->t_end - st->t;
  if (st->t + dt > st->t_output) dt = st->t_output - st->t;
  double lim = 1.1 * 0.5 * (st->dt_old + st->dt_old_old);
  if (lim < dt) dt = lim;
  st->dt_old_old = st->dt_old;
  st->dt_old = dt;
  st->dt = dt;
  st->t_prev = st->t;
  st->t = st->t + dt;
  st->run_step = 1;
  const int p = (int)(st->steps & 1);
  st->last_cells = (long long)st->cells_acc[p];
  st->cells_total += (long long)st->cells_acc[p];
  st->cells_acc[p] = 0ull;
  st->steps += 1;
  st->dtmin_bits = dbits(1.0e300);
}

// ---------------------------------------------------------------------------
// Positivity fixes of assemble_sol (solver_2d.f90:1381-1628) on an FP64 or
// FP32 state; returns status bits.
// ---------------------------------------------------------------------------
template <class R, int NS>
__device__ __forceinline__ unsigned assemble_fixes(const Phys<R>& P, R* q) {
  constexpr int nv = 4 + NS, ns = NS;
  unsigned st = 0;
#pragma unroll
  for (int i = 0; i < nv; ++i)
    if (isnan(q[i])) st |= SFLOW_S_NAN;
  if (q[0] < P.thr_eps) {   // EPSILON(1.0_wp) is a power of two, exact in float
    if (q[0] > P.thr_neg1e7) {
#pragma unroll
      for (int i = 0; i < nv; ++i) q[i] = R(0);
    } else {
      st |= SFLOW_S_NEG_H;
    }
  }
  bool anyneg = false, anybad = false;
#pragma unroll
  for (int i = 0; i < ns; ++i) {
    if (q[4 + i] < R(0)) anyneg = true;
    if (!(q[4 + i] > P.thr_neg1e7)) anybad = true;
  }
  if (anyneg) {
    if (anybad) st |= SFLOW_S_NEG_ALPHA;
    else {
#pragma unroll
      for (int i = 0; i < ns; ++i)
        if (q[4 + i] > P.thr_neg1e7) q[4 + i] = R(0);
    }
  }
  R qp[nv + 2];
  qc_to_qp<R, NS>(P, q, qp);
  if (qp[3] < P.thr_273) st |= SFLOW_S_LOW_T;
  if (ns > 0) {
    R ssum = R(0);
#pragma unroll
    for (int i = 0; i < ns; ++i) ssum += q[4 + i];
    if (ssum > q[0]) {
      bool small;
      if constexpr (sizeof(R) == 8) small = ((ssum - q[0]) / q[0] < 1.0e-10) || (q[0] < P.thr_eps);
      else small = !((ssum - q[0]) / q[0] > P.thr_1em10) || (q[0] < P.thr_eps);
      if (!small) st |= SFLOW_S_SOLID_GT_MASS;
      R s = R(0);
#pragma unroll
      for (int i = 0; i < ns; ++i) s += q[4 + i];
#pragma unroll
      for (int i = 0; i < ns; ++i) q[4 + i] = q[4 + i] / s * q[0];
    }
  }
  return st;
}

// update_erosion_deposition_cell (solver_2d.f90:2382-2597) for one cell
template <class R, int NS>
__device__ __forceinline__ unsigned erosion_deposition(const Phys<R>& P, const Geo<R>& geo, R dt,
                                                       R* q) {
  constexpr int nv = 4 + NS, ns = NS;
  unsigned st = 0;
  R qp[nv + 2], dep[kMaxSolid], eqn[nv];
  if (q[0] > R(0)) qc_to_qp<R, NS>(P, q, qp);
  else {
#pragma unroll
    for (int i = 0; i < nv + 2; ++i) qp[i] = R(0);
    qp[3] = P.T_ambient;
  }
  mass_exchange<R, NS>(P, qp, geo.Bx, geo.By, dt, dep, eqn);
#pragma unroll
  for (int i = 0; i < nv; ++i) q[i] = q[i] + dt * eqn[i];
#pragma unroll
  for (int i = 0; i < ns; ++i) q[4 + i] = rmax(R(0), q[4 + i]);
  if (!(q[0] > R(0))) {
    if (q[0] > P.thr_neg1e10) {
#pragma unroll
      for (int i = 0; i < nv; ++i) q[i] = R(0);
    } else {
      st |= SFLOW_S_EROSION;
    }
  }
  if (ns > 0) {
    R ssum = R(0);
#pragma unroll
    for (int i = 0; i < ns; ++i) ssum += q[4 + i];
    if (ssum > q[0]) {
      bool small;
      if constexpr (sizeof(R) == 8) small = q[0] < 1.0e-10;
      else small = !(q[0] > P.thr_1em10);
      if (small) {
        R s = R(0);
#pragma unroll
        for (int i = 0; i < ns; ++i) s += q[4 + i];
#pragma unroll
        for (int i = 0; i < ns; ++i) q[4 + i] = q[4 + i] / s * q[0];
      } else {
        st |= SFLOW_S_EROSION;
      }
    }
  }
  R red_grav = R(0);
  if (q[0] > R(0)) {
    qc_to_qp<R, NS>(P, q, qp);
    Mixt<R> m = mixt_var<R, NS>(P, qp, false);
    red_grav = m.red_grav;
  }
  if (red_grav <= R(0)) {
#pragma unroll
    for (int i = 0; i < nv; ++i) q[i] = R(0);
  }
  return st;
}

// post-step maxima (IMEX_SfloW2D.f90:449-505)
template <class R, int NS>
__device__ __forceinline__ void post_step_maps(const KArgs<R>& a, int64_t c, const R* q) {
  constexpr int nv = 4 + NS;
  if (q[0] > R(0)) {
    R qp[nv + 2];
    R p_dyn = qc_to_qp<R, NS>(a.pr, q, qp);
    R hm = a.hmax[c];
    a.hmax[c] = rmax(hm, qp[0]);
    if (qp[0] > a.pr.thr_1em3) {
      R mv = sqrt(sq(qp[nv]) + sq(qp[nv + 1]));
      a.pdynmax[c] = rmax(a.pdynmax[c], p_dyn);
      a.mvmax[c] = rmax(a.mvmax[c], mv);
    }
  }
}

// ---------------------------------------------------------------------------
// k_stage2: the pointwise part of an N_RK = 2 step after the flux stage:
// imex_RK_solver stage 2 (solver_2d.f90:1103-1328), assemble_sol
// (1342-1630), update_erosion_deposition_cell, post-step maxima.
// ---------------------------------------------------------------------------
// mode -1: stage + assembly + erosion/deposition + maxima (fused step);
// 0: stage + assembly (imex_RK_solver); 1: erosion/deposition only;
// 2: maxima only.
template <class R, int NS>
__global__ void __launch_bounds__(TX* TY) k_stage2(KArgs<R> a, int mode) {
  constexpr int nv = 4 + NS;
  RunState* st = a.st;
  if (!st->run_step) return;
  if (!a.tile_active[blockIdx.y * gridDim.x + blockIdx.x]) return;
  const Grid<R>& g = a.g;
  const int j = blockIdx.x * TX + threadIdx.x % TX;
  const int k = blockIdx.y * TY + threadIdx.x / TX;
  unsigned status = 0;
  int nit = 0;
  if (j < g.nx && k < g.ny) {
    const int64_t c = cidx(g, j, k);
    if (a.mask[c] && mode > 0) {
      const double dt = st->dt;
      R q[nv];
#pragma unroll
      for (int i = 0; i < nv; ++i) q[i] = a.q[i * g.plane + c];
      if (mode == 1) {
        const Geo<R> geo = load_geo(a, c);
        status |= erosion_deposition<R, NS>(a.pr, geo, (R)dt, q);
#pragma unroll
        for (int i = 0; i < nv; ++i) a.q[i * g.plane + c] = q[i];
      } else {
        post_step_maps<R, NS>(a, c, q);
      }
    } else if (a.mask[c]) {
      const double dt = st->dt;
      const Geo<R> geo = load_geo(a, c);
      R q[nv];
      if constexpr (sizeof(R) == 8) {
        // ---- plain FP64 form: the reference's Newton, step by step ----
        const Phys<double>& P = a.pd;
        double q0[nv], r1[nv], qfv[nv], qp[nv + 2], si[nv], qsi[nv], qg[nv], Rj[nv];
#pragma unroll
        for (int i = 0; i < nv; ++i) { q0[i] = a.q[i * g.plane + c]; r1[i] = a.rd[i * g.plane + c]; }
#pragma unroll
        for (int i = 0; i < nv; ++i) qfv[i] = q0[i] - dt * (r1[i] * 1.0 - 0.0);
        qc_to_qp<double, NS>(P, qfv, qp);
        const double a_diag = 1.0;
        if (qfv[0] > 0.0) {
          semi_impl_terms<double, NS>(P, geo, qp, si);
#pragma unroll
          for (int i = 0; i < nv; ++i) qsi[i] = qfv[i] + dt * a_diag * si[i];
          if (sq(qfv[1]) + sq(qfv[2]) == 0.0) {
            qsi[1] = 0.0; qsi[2] = 0.0;
          } else if (qsi[1] * qfv[1] < 0.0 || qsi[2] * qfv[2] < 0.0) {
            qsi[1] = 0.0; qsi[2] = 0.0;
          } else {
            double m1 = sqrt(sq(qsi[1]) + sq(qsi[2])), m0 = sqrt(sq(qfv[1]) + sq(qfv[2]));
            qsi[1] = m1 * qfv[1] / m0;
            qsi[2] = m1 * qfv[2] / m0;
          }
#pragma unroll
          for (int i = 0; i < nv; ++i) { si[i] = (qsi[i] - qfv[i]) / (dt * a_diag); qg[i] = qsi[i]; }
#pragma unroll
          for (int i = 0; i < nv; ++i) Rj[i] = (r1[i] * 1.0 - 0.0) - a_diag * si[i];
          NewtonCtx nc{&P, dt, a_diag, geo.Bx, geo.By, q0, Rj};
          nit = solve_rk_step<NS>(nc, qg);
          if (nit > kMaxNewton) status |= SFLOW_S_NEWTON_MAXIT;
          if (g.ny == 1) qg[2] = 0.0;
          if (sq(qsi[1]) + sq(qsi[2]) == 0.0) {
            qg[1] = 0.0; qg[2] = 0.0;
          } else if (qg[1] * qsi[1] <= 0.0 && qg[2] * qsi[2] <= 0.0) {
            qg[1] = 0.0; qg[2] = 0.0;
          } else {
            double m1 = sqrt(sq(qg[1]) + sq(qg[2])), m0 = sqrt(sq(qsi[1]) + sq(qsi[2]));
            qg[1] = m1 * qsi[1] / m0;
            qg[2] = m1 * qsi[2] / m0;
          }
        } else {
#pragma unroll
          for (int i = 0; i < nv; ++i) qg[i] = qfv[i];
        }
#pragma unroll
        for (int i = 0; i < nv; ++i) q[i] = qg[i];
      } else {
        // ---- FP32 bulk form: FP32 explicit part, FP64 scalar Newton ----
        const Phys<R>& P = a.pr;
        const R dtr = (R)dt;
        R qfv[nv], qp[nv + 2], si[nv], qsi[nv];
#pragma unroll
        for (int i = 0; i < nv; ++i) qfv[i] = a.q[i * g.plane + c] - dtr * a.rd[i * g.plane + c];
        qc_to_qp<R, NS>(P, qfv, qp);
        if (qfv[0] > R(0)) {
          semi_impl_terms<R, NS>(P, geo, qp, si);
#pragma unroll
          for (int i = 0; i < nv; ++i) qsi[i] = qfv[i] + dtr * si[i];
          if (sq(qfv[1]) + sq(qfv[2]) == R(0)) {
            qsi[1] = R(0); qsi[2] = R(0);
          } else if (qsi[1] * qfv[1] < R(0) || qsi[2] * qfv[2] < R(0)) {
            qsi[1] = R(0); qsi[2] = R(0);
          } else {
            R m1 = sqrt(sq(qsi[1]) + sq(qsi[2])), m0 = sqrt(sq(qfv[1]) + sq(qfv[2]));
            qsi[1] = m1 * qfv[1] / m0;
            qsi[2] = m1 * qfv[2] / m0;
          }
          double qd[nv];
#pragma unroll
          for (int i = 0; i < nv; ++i) qd[i] = (double)qsi[i];
          double e1, e2;
          double s = reduced_friction_solve<NS>(a.pd, (double)geo.Bx, (double)geo.By, qd, dt, e1, e2, nit);
#pragma unroll
          for (int i = 0; i < nv; ++i) q[i] = qsi[i];
          q[1] = (R)(s * e1);
          q[2] = (R)(s * e2);
          if (g.ny == 1) q[2] = R(0);
        } else {
#pragma unroll
          for (int i = 0; i < nv; ++i) q[i] = qfv[i];
        }
      }
      status |= assemble_fixes<R, NS>(a.pr, q);
      if (mode < 0 && (a.pd.settling || a.pd.entrain))
        status |= erosion_deposition<R, NS>(a.pr, geo, (R)dt, q);
#pragma unroll
      for (int i = 0; i < nv; ++i) a.q[i * g.plane + c] = q[i];
      if (mode < 0) post_step_maps<R, NS>(a, c, q);
    }
  }
  if (status) atomicOr(&st->status, status);
  // Newton iteration statistics (one atomic per warp)
  int wsum = nit;
  for (int o = 16; o > 0; o >>= 1) wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
  int wmax = nit;
  for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
  if ((threadIdx.x & 31) == 0 && wsum > 0) {
    atomicAdd((unsigned long long*)&st->newton_iters, (unsigned long long)wsum);
    atomicMax(&st->newton_max, wmax);
  }
}

}  // namespace sflow

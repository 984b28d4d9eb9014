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
#include "sflow_sum.cuh"

namespace sflow {

constexpr int TX = 32;   // tile width (cells): one warp per tile row
constexpr int HALO = 2;  // reconstruction stencil reach for a cell's faces
constexpr int RX = TX + 2 * HALO;

// A tile is TX x TH cells; the tile height TH is a template parameter of
// every tiled kernel (the tile-shape autotuner picks it per run or batch).
// The results of a step do not depend on TH: every face and cell is
// computed from the same stencil whatever tile it falls in.
template <int TH>
struct TileShape {
  static constexpr int TY = TH;
  static constexpr int RY = TH + 2 * HALO;
  // whole warps covering the (TX+1)*TH x-faces and the TX*(TH+1) y-faces
  static constexpr int FLUX_THREADS = (TX * (TH + 1) + 31) / 32 * 32;
  // resident blocks per SM the persistent flux kernel is compiled for
  static constexpr int FLUX_MIN_BLOCKS = (TH >= 16) ? 2 : (TH >= 8 ? 4 : 6);
  // pointwise kernels: 32 x 8 threads, one cell each (a single run's
  // blocks cover 32 x 8 cells; a batched block walks a tile 8 rows at a time)
  static constexpr int STAGE_THREADS = TX * 8;
  static constexpr int STAGE_MIN_BLOCKS = 5;
  static constexpr int MASK_THREADS = TX * TH;
};
constexpr int kTileHDefault = 8;

// flag byte bits
constexpr uint8_t F_SC_MASK = 0x3;  // source_cell (0, 1 ring interior, 2 ring boundary)
constexpr uint8_t F_E = 0x4, F_W = 0x8, F_N = 0x10, F_S = 0x20;
constexpr uint8_t F_STATIC = 0x3f;  // the bits above: copied to the flux kernel's shared flags
// in the flag plane only
constexpr uint8_t F_NODATA = 0x40;  // B_nodata: the assembly empties the cell (solver_2d.f90:1626)
constexpr uint8_t F_BSRC = 0x80;    // inside the bottom radial source (cell fraction > 0)
// in the flux kernel's shared flags only
constexpr uint8_t F_WET = 0x40;     // active and q1 > 0
constexpr uint8_t F_ACTIVE = 0x80;

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
  uint8_t* tile_wet;   // a cell of the tile holds mass after the step (stage kernel)
  // single runs: the same per step parity (2 x tiles; written by the
  // N_RK = 2 stage kernel) and the tiles within n_RK cells of a static seed
  // (border or ring-boundary cell); check_solve skips the other tiles
  uint8_t* tile_wet_step;
  const uint8_t* tile_static;
  uint16_t* tile_count;   // active cells of a tile of code 3 (dry border)
  R* hmax;
  R* pdynmax;
  R* mvmax;
  double* deposit;   // n_solid planes (settling only): accumulated dt * deposition
  double* erosion;   // n_solid planes (erosion only): accumulated dt * erosion
  double* erodible;  // n_solid planes (erosion only): erodible solid thickness
  double* Bc;        // topography (topography change only), FP64
  const R* bfrac;    // bottom radial source: cell fraction inside the source
  const double* bsrc_tab;   // bottom radial source: n_intervals, t_intervals, vel_intervals
  uint32_t* vuln;    // vulnerability table: words planes of 32 entries
  int vuln_words;
  RunState* st;
  double tableau_at[16], tableau_ad[16], omega_t[4], omega[4];
  int take_last;
};

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
// Launch with programmatic stream serialisation (see step_kernel_entry);
// pdl = 0 gives an ordinary launch.
template <typename... KParams, typename... Args>
static cudaError_t launch_step_kernel(void (*kern)(KParams...), dim3 grid, dim3 block, size_t smem,
                                      cudaStream_t s, int pdl, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, args...);
}
template <class R>
__device__ __forceinline__ int64_t cidx(const Grid<R>& g, int j, int k) {
  return (int64_t)k * g.pitch + j;
}

// Programmatic dependent launch: the kernels of a step are launched with
// programmatic stream serialisation, so a kernel's blocks may be scheduled
// while the previous kernel still runs.  Every kernel first waits for the
// previous grid to complete and its memory to be visible (a no-op when the
// launch had no programmatic dependency), then lets the next kernel's
// launch begin.
__device__ __forceinline__ void step_kernel_entry() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Order-preserving integer key of a double (for non-NaN values: a < b iff
// key(a) < key(b); -0 maps to +0).  Every thread of the step kernels tests
// the run clock, and a double comparison runs on GB300's FP64 pipe at 1/64
// of the FP32 rate; the key comparison runs on the integer pipe.
__device__ __forceinline__ long long order_key(double x) {
  long long b = __double_as_longlong(x);
  if (b == (long long)0x8000000000000000ull) b = 0;
  return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}

__device__ __forceinline__ bool running(const RunState* st) {
  return order_key(st->t) < order_key(st->t_stop) && st->steps < st->step_limit && !(st->status & SFLOW_S_FATAL);
}

__device__ __forceinline__ unsigned long long dbits(double x) {
  return (unsigned long long)__double_as_longlong(x);
}

// x_stag(j) = x0 + j*dx, x_comp(j) = 0.5*(x_stag(j)+x_stag(j+1))
// (geometry_2d.f90:312-327); in FP32 form the same values rounded to float.
template <class R>
__device__ __forceinline__ R xstag(const Grid<R>& g, int j) {
  if constexpr (sizeof(R) == 8) return g.x0 + (double)j * g.dx;
  else return g.x0r + (R)j * g.rdx;
}
template <class R>
__device__ __forceinline__ R xcomp(const Grid<R>& g, int j) {
  if constexpr (sizeof(R) == 8) return 0.5 * ((g.x0 + (double)j * g.dx) + (g.x0 + (double)(j + 1) * g.dx));
  else return g.x0r + ((R)j + 0.5f) * g.rdx;
}
template <class R>
__device__ __forceinline__ R ystag(const Grid<R>& g, int k) {
  k += g.k_off;
  if constexpr (sizeof(R) == 8) return g.y0 + (double)k * g.dy;
  else return g.y0r + (R)k * g.rdy;
}
template <class R>
__device__ __forceinline__ R ycomp(const Grid<R>& g, int k) {
  k += g.k_off;
  if constexpr (sizeof(R) == 8) return 0.5 * ((g.y0 + (double)k * g.dy) + (g.y0 + (double)(k + 1) * g.dy));
  else return g.y0r + ((R)k + 0.5f) * g.rdy;
}
// the row is one this domain owns (row slabs; always true for a whole domain)
template <class R>
__device__ __forceinline__ bool owned_row(const Grid<R>& g, int k) {
  return g.whole || (k >= g.own_lo && k < g.own_hi);
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
// Seeds of check_solve (solver_2d.f90:667-858): border cells, wet cells and
// ring-boundary cells; a cell is active when a seed lies within Manhattan
// distance n_RK (<= 4) and it is not a ring-interior cell.  The seeds of
// the tile and a 4-cell frame (40 columns) become one 64-bit mask per frame
// row (warp ballots); the distance test of a cell is then one shifted mask
// test per row within n_RK, and a tile with no seed in its frame is
// inactive without scanning its cells.
constexpr int MASK_HALO = 4;
constexpr int MRX = TX + 2 * MASK_HALO;
static_assert(MRX <= 64, "a frame row must fit one 64-bit mask");

// Tile codes of tile_active: 0 inactive; 1 active; 2 active, dry and
// without ring cells (found by the flux kernel: the stage kernel leaves it
// unchanged); 3 active through border seeds only (found by check_solve with
// mark_dry: no cell of its 4-cell frame holds mass or belongs to the ring
// inlet, and its ghosts are dry or it lies 2 cells inside the domain) --
// the flux and stage kernels would compute zero fluxes and no change, and
// skip it.
constexpr uint8_t TILE_DRY_BORDER = 3;

// One warp evaluates one tile: lane x owns frame columns x and 32 + x
// (x < 8) of every frame row, the seeds of a row become one 64-bit mask by
// two ballots, and lane x then tests the cells of tile column x row by
// row.  A tile needs no barrier and no other warp, so a block of 8 warps
// keeps 8 tiles (their load latencies) in flight.  Returns the tile code
// (warp-uniform).  srow: the warp's MRY masks in shared memory.
// Returns the tile code (block-uniform).
template <class R, int TH>
__device__ __forceinline__ int mask_tile(const KArgs<R>& a, int solve_all, int tx, int ty, int tiles_x,
                                         bool mark_dry = false, int* act_out = nullptr) {
  constexpr int TY = TH, MRY = TH + 2 * MASK_HALO;
  constexpr int RPW = (MRY + TH - 1) / TH;   // frame rows per warp (TH warps)
  __shared__ unsigned long long srow[MRY];   // bit x: seed at frame column x
  __shared__ unsigned s_spec[TH];            // per warp: a frame cell with mass or a ring cell
  RunState* st = a.st;
  const Grid<R>& g = a.g;
  const int j0 = tx * TX, k0 = ty * TY;
  const int nrk = a.pd.nrk;
  const int lane = threadIdx.x % TX, warp = threadIdx.x / TX;
  int any = 0;
  unsigned wspec = 0u;
  if (!solve_all) {
    // frame row y = warp + r*TH; columns lane and 32 + lane (lane < 8); all
    // loads of a thread are issued before any is used
    R qv[RPW][2];
    uint8_t fv[RPW][2];
#pragma unroll
    for (int r = 0; r < RPW; ++r)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int y = warp + r * TH, x = lane + TX * h;
        const int jj = j0 + x - MASK_HALO, kk = k0 + y - MASK_HALO;
        qv[r][h] = R(0);
        fv[r][h] = 0;
        if (y < MRY && x < MRX && jj >= 0 && jj < g.nx && kk >= 0 && kk < g.ny) {
          const int64_t cc = cidx(g, jj, kk);
          qv[r][h] = a.q[cc];
          fv[r][h] = a.cflags[cc];
        }
      }
#pragma unroll
    for (int r = 0; r < RPW; ++r) {
      const int y = warp + r * TH;
      if (y >= MRY) break;   // warp-uniform
      unsigned bits[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int x = lane + TX * h;
        const int jj = j0 + x - MASK_HALO, kk = k0 + y - MASK_HALO;
        int sd = 0, sp = 0;
        if (x < MRX && jj >= 0 && jj < g.nx && kk >= 0 && kk < g.ny) {
          if (jj == 0 || jj == g.nx - 1 || kk == 0 || kk == g.ny - 1) sd = 1;
          else if (qv[r][h] > R(0)) sd = 1;
          else if (a.pd.radial_source && (fv[r][h] & F_SC_MASK) == 2) sd = 1;
          else if (a.pd.bottom_source && (fv[r][h] & F_BSRC)) sd = 1;
          sp = (qv[r][h] > R(0)) || (a.pd.radial_source && (fv[r][h] & F_SC_MASK) != 0) ||
               (a.pd.bottom_source && (fv[r][h] & F_BSRC));
        }
        bits[h] = __ballot_sync(0xffffffffu, sd);
        wspec |= __ballot_sync(0xffffffffu, sp);
      }
      if (lane == 0) srow[y] = (unsigned long long)bits[0] | ((unsigned long long)bits[1] << 32);
      any |= (bits[0] | bits[1]) != 0u;
    }
    if (lane == 0) s_spec[warp] = wspec;
    any = __syncthreads_or(any);
  }
  const int j = j0 + lane;
  const int k = k0 + warp;
  int act = 0;
  if (j < g.nx && k < g.ny) {
    const int64_t c = cidx(g, j, k);
    if (solve_all) {
      act = 1;
    } else if (any) {
      // seeds within Manhattan distance n_RK: in frame row cy + dk, the
      // columns cx - r .. cx + r with r = n_RK - |dk|
      const int cx = lane + MASK_HALO, cy = warp + MASK_HALO;
      if ((srow[cy] >> cx) & 1ull) {
        act = 1;                       // the cell is a seed itself
      } else if (nrk == 2) {
        act = (((srow[cy - 2] >> cx) & 1ull) | ((srow[cy + 2] >> cx) & 1ull) |
               ((srow[cy - 1] >> (cx - 1)) & 7ull) | ((srow[cy + 1] >> (cx - 1)) & 7ull) |
               ((srow[cy] >> (cx - 2)) & 31ull)) != 0ull;
      } else {
        for (int dk = -nrk; dk <= nrk; ++dk) {
          const int r = nrk - (dk < 0 ? -dk : dk);
          if ((srow[cy + dk] >> (cx - r)) & ((2ull << (2 * r)) - 1ull)) act = 1;
        }
      }
    }
    if (act && a.pd.radial_source && (a.cflags[c] & F_SC_MASK) == 1) act = 0;
    a.mask[c] = (uint8_t)act;
  }
  if (act_out) *act_out = act;
  int cnt, code;
  if (g.whole) {
    cnt = __syncthreads_count(act);
    code = cnt > 0 ? 1 : 0;
  } else {
    cnt = __syncthreads_count(act && owned_row(g, k));
    code = __syncthreads_or(act) ? 1 : 0;
  }
  if (code && mark_dry && !solve_all) {
    unsigned spec = 0u;
#pragma unroll
    for (int w = 0; w < TH; ++w) spec |= s_spec[w];
    const bool inside = j0 - HALO >= 0 && k0 - HALO >= 0 && j0 + TX + HALO <= g.nx && k0 + TY + HALO <= g.ny;
    if (!spec && (g.dry_bc || inside)) code = TILE_DRY_BORDER;
  }
  if (threadIdx.x == 0) {
    a.tile_active[ty * tiles_x + tx] = (uint8_t)code;
    if (code == TILE_DRY_BORDER) {
      a.tile_count[ty * tiles_x + tx] = (uint16_t)cnt;
      atomicAdd(&st->border_acc[st->steps & 1], (unsigned long long)cnt);
    }
    if (cnt) atomicAdd((unsigned long long*)&st->cells_acc[st->steps & 1], (unsigned long long)cnt);
  }
  return code;
}

// A tile without a static seed within n_RK cells, with no tile of its 3 x 3
// neighbourhood holding mass after the last step and inactive in the last
// step cannot have an active cell (a seed within n_RK <= 4 cells of it lies
// in that neighbourhood) and already has an all-zero mask: check_solve
// skips it.  The tile also clears its wet flag of the buffer that this
// step's stage kernel sets.
//
// A tile of code 3 (active through border seeds only, dry frame) keeps its
// code, mask and active count while no tile of its 3 x 3 neighbourhood
// holds mass: its 4-cell frame then stays dry, and its seeds are static.
// Only its count is added.
// Threads 0-8 read the nine wet flags together; one barrier shares the
// result (block-uniform).
template <class R>
__device__ __forceinline__ bool mask_tile_skippable(const KArgs<R>& a, int tx, int ty, int tiles_x, int tiles_y) {
  const int nt = tiles_x * tiles_y, t = ty * tiles_x + tx;
  const unsigned par = (unsigned)(a.st->steps & 1);
  int wet = 0;
  if (threadIdx.x < 9) {
    const int x = tx + (int)threadIdx.x % 3 - 1, y = ty + (int)threadIdx.x / 3 - 1;
    if (x >= 0 && x < tiles_x && y >= 0 && y < tiles_y) wet = a.tile_wet_step[par * nt + y * tiles_x + x] != 0;
  }
  const uint8_t ta = a.tile_active[t];
  const bool any_wet = __syncthreads_or(wet) != 0;
  if (threadIdx.x == 0) a.tile_wet_step[(par ^ 1u) * nt + t] = 0;
  const bool skip = (ta == TILE_DRY_BORDER || (ta == 0 && !a.tile_static[t])) && !any_wet;
  if (skip && ta == TILE_DRY_BORDER && threadIdx.x == 0) {
    atomicAdd((unsigned long long*)&a.st->cells_acc[a.st->steps & 1], (unsigned long long)a.tile_count[t]);
    atomicAdd(&a.st->border_acc[a.st->steps & 1], (unsigned long long)a.tile_count[t]);
  }
  return skip;
}

// Time factor and inflow velocity of the bottom radial source at `time`
// (constitutive_2d.f90:3151-3187): the piecewise-constant velocity of the
// last interval started (factor 1 while it is positive), or vel_source
// with the linear ramps of time_param.
__device__ __forceinline__ void bottom_source_coeff(const double* tab, const double* tp, double vel_source,
                                                    double time, double& t_coeff, double& vel) {
  const int n = tab ? (int)tab[0] : 0;
  if (n > 0) {
    vel = 0.0;
    for (int i = n - 1; i >= 0; --i)
      if (time >= tab[1 + i]) { vel = tab[1 + n + i]; break; }
    t_coeff = (vel > 0.0) ? 1.0 : 0.0;
    return;
  }
  vel = vel_source;
  const double t_rem = fmod(time + tp[3], tp[0]);
  if (tp[2] == 0.0) {
    t_coeff = (t_rem <= tp[1]) ? 1.0 : 0.0;
  } else if (t_rem <= tp[2]) {
    t_coeff = t_rem / tp[2];
  } else if (t_rem <= tp[1] - tp[2]) {
    t_coeff = 1.0;
  } else if (t_rem <= tp[1]) {
    t_coeff = 1.0 - (t_rem - tp[1] + tp[2]) / tp[2];
  } else {
    t_coeff = 0.0;
  }
}

// start-of-step source factors of a run (ring inlet, bottom source)
template <class R>
__device__ __forceinline__ void source_factors(const KArgs<R>& a, RunState* st, double t) {
  st->src_t_coeff = source_time_coeff(st->tp, st->pi_g, t);
  st->src_t_coeff_f = (float)st->src_t_coeff;
  if (a.pd.bottom_source) {
    double tc, vel;
    bottom_source_coeff(a.bsrc_tab, st->tp, a.pd.vel_source, t, tc, vel);
    st->bsrc_t_coeff = tc;
    st->bsrc_vel = vel;
    st->bsrc_t_coeff_f = (float)tc;
    st->bsrc_vel_f = (float)vel;
  }
}

// mode 0: check_solve(.FALSE.); 1: check_solve(.TRUE.) (solve_all); 2: as 0
// with the tile skip of mask_tile_skippable (the N_RK = 2 step, whose stage
// kernel keeps the wet flags)
template <class R, int TH>
__global__ void __launch_bounds__(TileShape<TH>::MASK_THREADS) k_mask(KArgs<R> a, int mode) {
  step_kernel_entry();
  RunState* st = a.st;
  const double t = st->t;
  if (!running(st)) return;
  if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0) source_factors(a, st, t);
  if (mode == 2 && mask_tile_skippable(a, blockIdx.x, blockIdx.y, gridDim.x, gridDim.y)) return;
  mask_tile<R, TH>(a, mode == 1, blockIdx.x, blockIdx.y, gridDim.x, mode == 2);
}

// ---------------------------------------------------------------------------
// Limited slopes (geometry_2d.f90:1776-1897).  The plain FP64 form divides by
// the stencil spacings exactly as the reference; the FP32 form multiplies by
// reciprocals (1/dx for the uniform interior stencil) and takes signs with
// copysign instead of a/|a|.
// ---------------------------------------------------------------------------
template <class R>
struct Spacing {
  R z0, z1, z2;
  R r01, r12, r02;   // FP32 form only
};

template <class R>
__device__ __forceinline__ Spacing<R> spacing(R z0, R z1, R z2, bool uniform, R inv_d) {
  Spacing<R> s;
  s.z0 = z0; s.z1 = z1; s.z2 = z2;
  if constexpr (sizeof(R) == 4) {
    if (uniform) { s.r01 = inv_d; s.r12 = inv_d; s.r02 = 0.5f * inv_d; }
    else { s.r01 = 1.0f / (z1 - z0); s.r12 = 1.0f / (z2 - z1); s.r02 = 1.0f / (z2 - z0); }
  } else {
    s.r01 = s.r12 = s.r02 = R(0);
  }
  return s;
}

__device__ __forceinline__ float minmod_f(float a, float b) {
  float m = fminf(fabsf(a), fabsf(b));
  if (m <= 0.0f) return 0.0f;
  return 0.5f * (copysignf(1.0f, a) + copysignf(1.0f, b)) * m;
}
// minmod of two differences by their sign bits: min(|a|, |b|) with a's
// sign when the signs agree, else 0 (a zero gives a zero of either sign)
__device__ __forceinline__ float minmod_sign_f(float a, float b) {
  const float m = fminf(fabsf(a), fabsf(b));
  return ((__float_as_uint(a) ^ __float_as_uint(b)) & 0x80000000u) ? 0.0f : copysignf(m, a);
}
__device__ __forceinline__ float maxmod_f(float a, float b) {
  if (fabsf(a * b) <= 0.0f) return 0.0f;
  return 0.5f * (copysignf(1.0f, a) + copysignf(1.0f, b)) * fmaxf(fabsf(a), fabsf(b));
}

template <class R, int LIM>
__device__ __forceinline__ R slope(R v0, R v1, R v2, const Spacing<R>& s, int lim, R theta) {
  if constexpr (sizeof(R) == 8) {
    return limit<R, LIM>(v0, v1, v2, s.z0, s.z1, s.z2, lim, theta);
  } else {
    const float a = (v2 - v1) * s.r12, b = (v1 - v0) * s.r01;
    if constexpr (LIM >= 0) lim = LIM;
    switch (lim) {
      case 0: return 0.0f;
      case 1: return minmod_f(a, b);
      case 2: return maxmod_f(minmod_f(a, 2.0f * b), minmod_f(2.0f * a, b));
      case 3: return minmod_f((v2 - v0) * s.r02, theta * minmod_f(a, b));
      case 4: return minmod_f((v2 - v0) * s.r02, 2.0f * minmod_f(a, b));
      case 5: return (v2 - v0) * s.r02;
      case 6: return a;
      case 7: return b;
    }
    return 0.0f;
  }
}

// ---------------------------------------------------------------------------
// Reconstruction of one side of one face (solver_2d.f90:3095-3924).
// The cell is at region coordinates (rx, ry) of the shared tile, global
// (j, k).  DIR 1: x faces, plus = 1 east side, 0 west side; DIR 2: y faces,
// plus = 1 north side, 0 south side.  Writes the physical face state qp
// (n_vars+2).  Only the stencil along DIR enters, apart from the
// reference's use of y_stag in the x slope of v at ring cells with a ring
// face to the north only (solver_2d.f90:3605, kept as is).
// ---------------------------------------------------------------------------
template <class R, int NS, int DIR, int LIM, int TH>
__device__ __noinline__ void recon_side_edge(const KArgs<R>& a, const R* sqp, const uint8_t* sfl,
                                           int rx, int ry, int j, int k, int plus, R* out) {
  constexpr int nv = 4 + NS, np = nv + 2;
  const Grid<R>& g = a.g;
  constexpr int plane = RX * TileShape<TH>::RY;
  constexpr int side_lo = (DIR == 1) ? SFLOW_W : SFLOW_S;
  constexpr int side_hi = (DIR == 1) ? SFLOW_E : SFLOW_N;
  constexpr int mom = DIR;   // hu (x) or hv (y) in the conservative/physical index
  auto QP = [&](int i, int o) -> R {
    return (DIR == 1) ? sqp[i * plane + ry * RX + (rx + o)] : sqp[i * plane + (ry + o) * RX + rx];
  };
  const uint8_t fl = sfl[ry * RX + rx];
  const int sc = fl & F_SC_MASK;
  const bool src2 = a.pr.radial_source && sc == 2;
  const int n = (DIR == 1) ? g.nx : g.ny;
  const int c = (DIR == 1) ? j : k;
  const bool b0 = (c == 0), b1 = (c == n - 1);
  const bool interior = !b0 && !b1;
  // ring faces of the cell along DIR: "hi" = E or N, "lo" = W or S
  const bool s_hi = (DIR == 1) ? (fl & F_E) : (fl & F_N);
  const bool s_lo = (DIR == 1) ? (fl & F_W) : (fl & F_S);
  // x: IF sourceE ... ELSEIF sourceW;  y: IF sourceS ... ELSEIF sourceN
  const bool use_hi = (DIR == 1) ? s_hi : (s_hi && !s_lo);
  const bool use_lo = (DIR == 1) ? (s_lo && !s_hi) : s_lo;
  auto stag = [&](int m) -> R { return (DIR == 1) ? xstag(g, m) : ystag(g, m); };
  auto comp = [&](int m) -> R { return (DIR == 1) ? xcomp(g, m) : ycomp(g, m); };
  const R inv_d = (DIR == 1) ? g.one_by_dx : g.one_by_dy;
  const R d2 = (DIR == 1) ? g.dx2 : g.dy2;
  R cell[np];
#pragma unroll
  for (int i = 0; i < np; ++i) cell[i] = QP(i, 0);
  R z0, z1 = comp(c), z2;
  bool uniform = false;
  if (b0) { z0 = stag(0); z2 = comp(1); }
  else if (b1) { z0 = comp(n - 2); z2 = stag(n); }
  else {
    z0 = comp(c - 1); z2 = comp(c + 1);
    uniform = true;
    if (src2) {
      if (use_hi) { z2 = stag(c + 1); uniform = false; }
      else if (use_lo) { z0 = stag(c); uniform = false; }
    }
  }
  const Spacing<R> sp = spacing<R>(z0, z1, z2, uniform, inv_d);
  R qm[np];
  R lo[nv], hi[nv];
  // conservative-index variables (vars_loop)
#pragma unroll
  for (int i = 0; i < nv; ++i) {
    const R v1 = cell[i];
    const int bl = a.bc.flag[side_lo][i], bh = a.bc.flag[side_hi][i];
    R sl;
    if (b0) {
      if (DIR == 1 && sc == 2) sl = slope<R, LIM>(cell[i], v1, QP(i, 1), sp, g.limiter[i], g.theta);
      else if (bl == 0) sl = slope<R, LIM>(a.bc.value[side_lo][i], v1, QP(i, 1), sp, g.limiter[i], g.theta);
      else if (bl == 1) sl = a.bc.value[side_lo][i];
      else sl = (QP(i, 1) - QP(i, 0)) * inv_d;
    } else if (b1) {
      if (DIR == 1 && sc == 2) sl = slope<R, LIM>(QP(i, -1), v1, cell[i], sp, g.limiter[i], g.theta);
      else if (bh == 0) sl = slope<R, LIM>(QP(i, -1), v1, a.bc.value[side_hi][i], sp, g.limiter[i], g.theta);
      else if (bh == 1) sl = a.bc.value[side_hi][i];
      else sl = (QP(i, 0) - QP(i, -1)) * inv_d;
    } else {
      R v0 = QP(i, -1), v2 = QP(i, 1);
      if (src2) { if (use_hi) v2 = cell[i]; else if (use_lo) v0 = cell[i]; }
      sl = slope<R, LIM>(v0, v1, v2, sp, g.limiter[i], g.theta);
    }
    const R dq = g.rc * d2 * sl;
    R l_ = v1 - dq, h_ = v1 + dq;
    if (b0) {
      if (DIR == 1 && sc == 2) l_ = cell[i];
      else if (bl == 0) l_ = a.bc.value[side_lo][i];
      else if (i == mom) l_ = rmin(l_, R(0));
    }
    if (b1) {
      if (DIR == 1 && sc == 2) h_ = cell[i];
      else if (bh == 0) h_ = a.bc.value[side_hi][i];
      else if (i == mom) h_ = rmax(h_, R(0));
    }
    lo[i] = l_;
    hi[i] = h_;
    qm[i] = plus ? h_ : l_;
  }
  // velocities u, v (add_vars_loop); qp_to_qp2 (constitutive_2d.f90:2164-2188)
  // gives u = hu/h, v = hv/h of the low / high state at the domain edges
  Spacing<R> spv = sp;
  if (DIR == 1 && interior && src2 && !s_hi) {
    const bool kint = (k > 0 && k < g.ny - 1);
    const bool sN = fl & F_N, sS = fl & F_S;
    if (kint && sN && !sS) spv = spacing<R>(sp.z0, sp.z1, ystag(g, k + 1), false, inv_d);
  }
#pragma unroll
  for (int m = 0; m < 2; ++m) {
    const int i = nv + m;
    const R v1 = cell[i];
    const R ul = (lo[0] <= R(0)) ? R(0) : lo[1 + m] / lo[0];
    const R uh = (hi[0] <= R(0)) ? R(0) : hi[1 + m] / hi[0];
    R v0, v2;
    if (b0) { v0 = ul; v2 = QP(i, 1); }
    else if (b1) { v0 = QP(i, -1); v2 = uh; }
    else {
      v0 = QP(i, -1);
      v2 = QP(i, 1);
      if (src2) { if (use_hi) v2 = cell[i]; else if (use_lo) v0 = cell[i]; }
    }
    const R sl = slope<R, LIM>(v0, v1, v2, (m == 1) ? spv : sp, g.limiter[i], g.theta);
    const R dq = g.rc * d2 * sl;
    R val = plus ? v1 + dq : v1 - dq;
    if (b0 && !plus) val = ul;
    if (b1 && plus) val = uh;
    qm[i] = val;
  }
  if (interior && src2 && ((plus && use_hi) || (!plus && use_lo))) {
#pragma unroll
    for (int i = 0; i < np; ++i) qm[i] = cell[i];
  }
#pragma unroll
  for (int i = 0; i < np; ++i) out[i] = qm[i];
}

// Interior cells without a ring face (almost every cell): three-point
// slopes on the uniform grid, no boundary or wall rule.  The same operations
// as recon_side_edge takes for such a cell, so both give identical values;
// the edge version is a separate (not inlined) function so that the face
// code every thread runs stays small.
template <class R, int NS, int DIR, int LIM, int TH>
__device__ __forceinline__ void recon_side(const KArgs<R>& a, const R* sqp, const uint8_t* sfl,
                                           int rx, int ry, int j, int k, int plus, R* out) {
  constexpr int nv = 4 + NS, np = nv + 2;
  const Grid<R>& g = a.g;
  constexpr int plane = RX * TileShape<TH>::RY;
  const int n = (DIR == 1) ? g.nx : g.ny;
  const int c = (DIR == 1) ? j : k;
  const uint8_t fl = sfl[ry * RX + rx];
  const bool src2 = a.pr.radial_source && (fl & F_SC_MASK) == 2;
  if (c == 0 || c == n - 1 || src2) {
    recon_side_edge<R, NS, DIR, LIM, TH>(a, sqp, sfl, rx, ry, j, k, plus, out);
    return;
  }
  auto QP = [&](int i, int o) -> R {
    return (DIR == 1) ? sqp[i * plane + ry * RX + (rx + o)] : sqp[i * plane + (ry + o) * RX + rx];
  };
  auto comp = [&](int m) -> R { return (DIR == 1) ? xcomp(g, m) : ycomp(g, m); };
  const R inv_d = (DIR == 1) ? g.one_by_dx : g.one_by_dy;
  const R d2 = (DIR == 1) ? g.dx2 : g.dy2;
  if constexpr (sizeof(R) == 4 && LIM == 1) {
    // FP32 form, minmod on every variable, uniform spacing: the limited
    // slope times rc dx/2 is (rc dx/2)(1/dx) minmod of the two differences
    const R kd = g.rc * d2 * inv_d;
#pragma unroll
    for (int i = 0; i < np; ++i) {
      const R v1 = QP(i, 0);
      const R dq = kd * minmod_sign_f(QP(i, 1) - v1, v1 - QP(i, -1));
      out[i] = plus ? v1 + dq : v1 - dq;
    }
    return;
  }
  const Spacing<R> sp = spacing<R>(comp(c - 1), comp(c), comp(c + 1), true, inv_d);
#pragma unroll
  for (int i = 0; i < np; ++i) {
    const R v1 = QP(i, 0);
    const R sl = slope<R, LIM>(QP(i, -1), v1, QP(i, 1), sp, g.limiter[i], g.theta);
    const R dq = g.rc * d2 * sl;
    out[i] = plus ? v1 + dq : v1 - dq;
  }
}

// One side of a face reduced to what the KT flux needs.
template <class R, int NS>
struct Side {
  R q[4 + NS];
  R f[4 + NS];
  R vmin, vmax;
  R hu_p;   // qp(2): x zero-velocity test
  R un;     // upwind test of eval_flux_UP: qp u (x faces) or q hv (y faces)
};

template <class R, int NS, int DIR>
__device__ __forceinline__ void side_from_qp(const KArgs<R>& a, const R* qp, R gcs, Side<R, NS>& s,
                                             bool mirrored) {
  const Phys<R>& P = a.pr;
  Mixt<R> m = qp_to_qc_mixt<R, NS>(P, qp, s.q);
  if (mirrored) s.q[DIR] = -s.q[DIR];   // hu (x) / hv (y) of the wall mirror
  local_speeds<R, NS>(P, qp, m.red_grav, gcs, DIR, s.vmin, s.vmax);
  eval_fluxes<R, NS>(P, s.q, qp, m, gcs, DIR, s.f);
  s.hu_p = qp[1];
  s.un = (DIR == 1) ? qp[4 + NS] : s.q[2];
}

template <class R, int NS>
__device__ __forceinline__ void side_zero(Side<R, NS>& s) {
#pragma unroll
  for (int i = 0; i < 4 + NS; ++i) { s.q[i] = R(0); s.f[i] = R(0); }
  s.vmin = R(0); s.vmax = R(0); s.hu_p = R(0); s.un = R(0);
}

// Upwind flux (solver_2d.f90:2705-2821, SOLVER_SCHEME = 'UP'): the side the
// normal velocity comes from, or the mean; on y faces with zero hv on both
// sides the mass, energy and solid fluxes are zero.  (The x counterpart of
// that test reads q_interfaceL(n_vars+1), past the conservative vector, and
// is not reproduced.)  The local speeds still give the CFL bound.
template <class R, int NS, int DIR>
__device__ __forceinline__ R up_flux(const Side<R, NS>& L, const Side<R, NS>& Rt, R* H) {
  constexpr int nv = 4 + NS;
  const R ul = L.un, ur = Rt.un;
#pragma unroll
  for (int i = 0; i < nv; ++i) {
    if (ul > R(0) && ur >= R(0)) H[i] = L.f[i];
    else if (ul <= R(0) && ur < R(0)) H[i] = Rt.f[i];
    else H[i] = cst<R>(0.5) * (L.f[i] + Rt.f[i]);
  }
  if (DIR == 2 && ul == R(0) && ur == R(0)) {
    H[0] = R(0);
#pragma unroll
    for (int i = 3; i < nv; ++i) H[i] = R(0);
  }
  const R a1 = rmin(rmin(L.vmin, Rt.vmin), R(0));
  const R a2 = rmax(rmax(L.vmax, Rt.vmax), R(0));
  return rmax(a2, -a1);
}

// KT flux across one face (solver_2d.f90:2834-3049).  H has n_vars entries.
template <class R, int NS, int DIR>
__device__ __forceinline__ R kt_flux(const Side<R, NS>& L, const Side<R, NS>& Rt, R* H) {
  constexpr int nv = 4 + NS, ns = NS;
  R a1 = rmin(rmin(L.vmin, Rt.vmin), R(0));
  R a2 = rmax(rmax(L.vmax, Rt.vmax), R(0));
  if (a1 == a2) {
#pragma unroll
    for (int i = 0; i < nv; ++i) H[i] = R(0);
  } else {
    const R den = a2 - a1;
    if constexpr (sizeof(R) == 8) {
      const R fac = (a2 * a1) / den;
#pragma unroll
      for (int i = 0; i < nv; ++i) H[i] = (a2 * L.f[i] - a1 * Rt.f[i]) / den + fac * (Rt.q[i] - L.q[i]);
    } else {
      const R inv_den = fdiv(R(1), den);
      const R fac = (a2 * a1) * inv_den;
#pragma unroll
      for (int i = 0; i < nv; ++i) H[i] = (a2 * L.f[i] - a1 * Rt.f[i]) * inv_den + fac * (Rt.q[i] - L.q[i]);
    }
  }
  if (ns > 0) {
    if (DIR == 1) {
      R s = R(0), s2 = R(0);
      if constexpr (sizeof(R) == 4) {
        // one reciprocal of the mass flux for the FP32 form
        const R inv0 = fdiv(R(1), H[0]);
#pragma unroll
        for (int i = 0; i < ns; ++i) { s += H[4 + i] * inv0; s2 += H[4 + i]; }
        s2 = s2 * inv0;
      } else {
#pragma unroll
        for (int i = 0; i < ns; ++i) { s += H[4 + i] / H[0]; s2 += H[4 + i]; }
        s2 = s2 / H[0];
      }
      if (s2 >= R(1)) {
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
  const bool zero_vel = (DIR == 1) ? (L.hu_p == R(0) && Rt.hu_p == R(0))
                                   : (L.q[2] == R(0) && Rt.q[2] == R(0));
  if (zero_vel) {
    H[0] = R(0);
#pragma unroll
    for (int i = 3; i < nv; ++i) H[i] = R(0);
  }
  return rmax(a2, -a1);
}

// One face along DIR between the low cell (f-1) and the high cell (f):
// reconstruction of both sides, the domain-edge copies and the wall mirror
// at ring-inlet faces (solver_2d.f90:3716-3920), KT flux.  Returns the
// largest |speed| at the face (a_interface_*_max).
template <class R, int NS, int DIR, int LIM, int TH>
__device__ __forceinline__ R face_flux(const KArgs<R>& a, const R* sqp, const uint8_t* sfl, int f,
                                       int o, int rxl, int ryl, int rxh, int ryh, R gcs, R* H) {
  constexpr int nv = 4 + NS, np = nv + 2;
  constexpr int vel = (DIR == 1) ? nv : nv + 1;
  const int n = (DIR == 1) ? a.g.nx : a.g.ny;
  const uint8_t fll = (f > 0) ? sfl[ryl * RX + rxl] : 0;
  const uint8_t flh = (f < n) ? sfl[ryh * RX + rxh] : 0;
  const bool actl = fll & F_ACTIVE, acth = flh & F_ACTIVE;
  const bool radial = a.pr.radial_source;
  const bool ring_l = radial && (fll & F_SC_MASK) == 2 && f - 1 > 0 && f - 1 < n - 1;
  const bool ring_h = radial && (flh & F_SC_MASK) == 2 && f > 0 && f < n - 1;
  const bool mirror_h = actl && ring_l && ((DIR == 1) ? (fll & F_E) : ((fll & F_N) && !(fll & F_S)));
  const bool mirror_l = !mirror_h && acth && ring_h && ((DIR == 1) ? ((flh & F_W) && !(flh & F_E)) : (flh & F_S));
  R qpl[np], qph[np];
  bool hl = false, hh = false;
  const int jl = (DIR == 1) ? f - 1 : o, kl = (DIR == 1) ? o : f - 1;
  const int jh = (DIR == 1) ? f : o, kh = (DIR == 1) ? o : f;
  if (f > 0 && actl) { recon_side<R, NS, DIR, LIM, TH>(a, sqp, sfl, rxl, ryl, jl, kl, 1, qpl); hl = true; }
  if (f < n && acth && !mirror_h) { recon_side<R, NS, DIR, LIM, TH>(a, sqp, sfl, rxh, ryh, jh, kh, 0, qph); hh = true; }
  if (f == 0) {
#pragma unroll
    for (int i = 0; i < np; ++i) qpl[i] = qph[i];
    hl = hh;
  }
  if (f == n) {
#pragma unroll
    for (int i = 0; i < np; ++i) qph[i] = qpl[i];
    hh = hl;
  }
  if (mirror_h) {
#pragma unroll
    for (int i = 0; i < np; ++i) qph[i] = qpl[i];
    qph[vel] = -qph[vel];
    hh = true;
  }
  if (mirror_l) {
#pragma unroll
    for (int i = 0; i < np; ++i) qpl[i] = qph[i];
    qpl[vel] = -qpl[vel];
    hl = true;
  }
  Side<R, NS> L, Hs;
  if (hl) side_from_qp<R, NS, DIR>(a, qpl, gcs, L, mirror_l);
  else side_zero(L);
  if (hh) side_from_qp<R, NS, DIR>(a, qph, gcs, Hs, mirror_h);
  else side_zero(Hs);
  if (a.pr.scheme == SFLOW_SCHEME_UP) return up_flux<R, NS, DIR>(L, Hs, H);
  return kt_flux<R, NS, DIR>(L, Hs, H);
}

// ---------------------------------------------------------------------------
// k_flux: divFlux - expl_terms of one explicit stage for every active cell
// of a 32 x TH tile (eval_hyperbolic_terms, solver_2d.f90:2616-2693, and
// eval_expl_terms), plus the CFL minimum of timestep (solver_2d.f90:873-1006)
// when want_dt.  The tile's qp (with a 2-cell halo) is computed once into
// shared memory; each thread then evaluates one face (both reconstructed
// sides, speeds, physical fluxes, KT flux) and finally one cell.
// ---------------------------------------------------------------------------
template <class R, int NS, int LIM, int TH>
__device__ __forceinline__ void flux_tile(const KArgs<R>& a, const R* __restrict__ qin,
                                          R* __restrict__ rout, int want_dt, int tx, int ty,
                                          unsigned char* smem_raw) {
  constexpr int TY = TH, RY = TileShape<TH>::RY, FLUX_THREADS = TileShape<TH>::FLUX_THREADS;
  constexpr int nv = 4 + NS, np = nv + 2;
  const RunState* st = a.st;
  const Grid<R>& g = a.g;
  const Phys<R>& P = a.pr;
  R* sqp = reinterpret_cast<R*>(smem_raw);                       // np * RX*RY
  R* sHx = sqp + np * RX * RY;                                   // nv * TY*(TX+1)
  R* sHy = sHx + nv * TY * (TX + 1);                             // nv * (TY+1)*TX
  R* sAx = sHy + nv * (TY + 1) * TX;                             // TY*(TX+1)
  R* sAy = sAx + TY * (TX + 1);                                  // (TY+1)*TX
  R* sgeo = sAy + (TY + 1) * TX;                                 // 5 * TX*TY
  uint8_t* sfl = reinterpret_cast<uint8_t*>(sgeo + 5 * TX * TY);  // RX*RY
  const int j0 = tx * TX, k0 = ty * TY;
  const int tid = threadIdx.x;

  __syncthreads();   // shared memory of the previous tile of a persistent block is free
  // 0. the topography terms of the cell this thread finishes in step 4
  // (B'x, B'y, g_c, dg_c/dx, dg_c/dy) start on their way to shared memory
  // now (asynchronous copies); the thread waits for its own copies in step 4
  if (tid < TX * TY) {
    const int j = j0 + tid % TX, k = k0 + tid / TX;
    if (j < g.nx && k < g.ny) {
      const int64_t c = cidx(g, j, k);
      const R* src[5] = {a.geo[0] + c, a.geo[1] + c, a.geo[5] + c, a.geo[6] + c, a.geo[7] + c};
#pragma unroll
      for (int p = 0; p < 5; ++p) {
        const unsigned dst = (unsigned)__cvta_generic_to_shared(sgeo + p * TX * TY + tid);
        if constexpr (sizeof(R) == 4)
          asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src[p]) : "memory");
        else
          asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src[p]) : "memory");
      }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  // 1. physical variables of the tile + halo (qc_to_qp; inactive = dry).
  // Each thread covers two region cells; all their loads (flags, mask,
  // state) are issued before any is used.
  int any_wet = 0, all_wet = 1;
  constexpr int NIT = (RX * RY + FLUX_THREADS - 1) / FLUX_THREADS;
  R qv[NIT][nv];
  uint8_t flv[NIT], mv[NIT];
#pragma unroll
  for (int it = 0; it < NIT; ++it) {
    const int idx = tid + it * FLUX_THREADS;
    const int rx = idx % RX, ry = idx / RX;
    const int j = j0 + rx - HALO, k = k0 + ry - HALO;
    flv[it] = 0;
    mv[it] = 0;
#pragma unroll
    for (int i = 0; i < nv; ++i) qv[it][i] = R(0);
    if (idx < RX * RY && j >= 0 && j < g.nx && k >= 0 && k < g.ny) {
      const int64_t c = cidx(g, j, k);
      flv[it] = a.cflags[c];
      mv[it] = a.mask[c];
#pragma unroll
      for (int i = 0; i < nv; ++i) qv[it][i] = qin[i * g.plane + c];
    }
  }
  int any_bsrc = 0;
#pragma unroll
  for (int it = 0; it < NIT; ++it) {
    const int idx = tid + it * FLUX_THREADS;
    if (idx >= RX * RY) break;
    R qp[np];
    any_bsrc |= (flv[it] & F_BSRC) != 0;
    uint8_t fl = flv[it] & F_STATIC;
    bool wet = false;
    if (mv[it]) {
      fl |= F_ACTIVE;
      if (qv[it][0] > R(0)) { qc_to_qp<R, NS>(P, qv[it], qp); wet = true; fl |= F_WET; }
    }
    if (!wet) {
#pragma unroll
      for (int i = 0; i < np; ++i) qp[i] = R(0);
      qp[3] = P.T_ambient;
    }
#pragma unroll
    for (int i = 0; i < np; ++i) sqp[i * RX * RY + idx] = qp[i];
    sfl[idx] = fl;
    any_wet |= wet;
    all_wet &= wet;
  }
  // A face whose reconstruction stencil (two cells each side) is dry has
  // dry states on both sides: zero fluxes, zero speeds, and the KT flux is
  // exactly 0 (solver_2d.f90 eval_flux_KT with a+ = a- = 0).  Ghost states
  // beyond the domain edge are dry too when every boundary condition is
  // (Neumann, 0).  A tile with no wet cell in its halo skips the faces.
  const bool some_wet = __syncthreads_or(any_wet);
  const bool any_bsrc_tile = P.bottom_source ? __syncthreads_or(any_bsrc) != 0 : false;
  const bool inside = j0 - HALO >= 0 && k0 - HALO >= 0 && j0 + TX + HALO <= g.nx && k0 + TY + HALO <= g.ny;
  const bool tile_dry = !some_wet && (g.dry_bc || inside);
  // every halo cell wet: no face can have a dry stencil
  const bool face_checks = !__syncthreads_and(all_wet);
  if (tile_dry) {
    // a dry tile without ring or bottom-source cells is left unchanged by
    // the stage kernel (q stays 0, divFlux - expl = 0, the maxima keep
    // their values)
    int ring = any_bsrc;
    for (int idx = tid; idx < TX * TY; idx += FLUX_THREADS) {
      const int rx = idx % TX + HALO, ry = idx / TX + HALO;
      ring |= (sfl[ry * RX + rx] & F_SC_MASK) != 0;
    }
    if (!__syncthreads_or(ring) && tid == 0) a.tile_active[ty * g.tiles_x + tx] = 2;
  }

  // 2. x faces: face f = j0+fx between cells f-1 and f
  for (int fi = tid; fi < (TX + 1) * TY && !tile_dry; fi += FLUX_THREADS) {
    const int fx = fi % (TX + 1), fy = fi / (TX + 1);
    const int f = j0 + fx, k = k0 + fy;
    R H[nv];
    R amax = R(0);
    const int ry = fy + HALO, rxl = fx - 1 + HALO, rxh = fx + HALO;
    const bool stencil_dry =
        face_checks &&
        !((sfl[ry * RX + rxl - 1] | sfl[ry * RX + rxl] | sfl[ry * RX + rxh] | sfl[ry * RX + rxh + 1]) & F_WET) &&
        (g.dry_bc || (f >= 2 && f + 1 <= g.nx - 1));
    const bool any = (k < g.ny && f <= g.nx) && !stencil_dry &&
                     (((f > 0) && (sfl[ry * RX + rxl] & F_ACTIVE)) || ((f < g.nx) && (sfl[ry * RX + rxh] & F_ACTIVE)));
    if (any) {
      const int64_t cl = cidx(g, f > 0 ? f - 1 : 0, k), ch = cidx(g, f < g.nx ? f : g.nx - 1, k);
      R gcs;
      if (f == 0) gcs = __ldg(a.geo[5] + ch);
      else if (f == g.nx) gcs = __ldg(a.geo[5] + cl);
      else gcs = cst<R>(0.5) * (__ldg(a.geo[5] + cl) + __ldg(a.geo[5] + ch));
      amax = face_flux<R, NS, 1, LIM, TH>(a, sqp, sfl, f, k, rxl, ry, rxh, ry, gcs, H);
    } else {
#pragma unroll
      for (int i = 0; i < nv; ++i) H[i] = R(0);
    }
#pragma unroll
    for (int i = 0; i < nv; ++i) sHx[i * TY * (TX + 1) + fi] = H[i];
    sAx[fi] = amax;
  }

  // 3. y faces: face f = k0+fy between cells f-1 and f
  // (one-row domains have no y fluxes: solver_2d.f90 eval_hyperbolic_terms
  // skips the y direction when comp_cells_y = 1)
  for (int fi = tid; fi < TX * (TY + 1) && !tile_dry && g.ny > 1; fi += FLUX_THREADS) {
    const int fx = fi % TX, fy = fi / TX;
    const int j = j0 + fx, f = k0 + fy;
    R H[nv];
    R amax = R(0);
    const int rx = fx + HALO, ryl = fy - 1 + HALO, ryh = fy + HALO;
    const bool stencil_dry =
        face_checks &&
        !((sfl[(ryl - 1) * RX + rx] | sfl[ryl * RX + rx] | sfl[ryh * RX + rx] | sfl[(ryh + 1) * RX + rx]) & F_WET) &&
        (g.dry_bc || (f >= 2 && f + 1 <= g.ny - 1));
    const bool any = (j < g.nx && f <= g.ny) && !stencil_dry &&
                     (((f > 0) && (sfl[ryl * RX + rx] & F_ACTIVE)) || ((f < g.ny) && (sfl[ryh * RX + rx] & F_ACTIVE)));
    if (any) {
      const int64_t cl = cidx(g, j, f > 0 ? f - 1 : 0), ch = cidx(g, j, f < g.ny ? f : g.ny - 1);
      R gcs;
      if (f == 0) gcs = __ldg(a.geo[5] + ch);
      else if (f == g.ny) gcs = __ldg(a.geo[5] + cl);
      else gcs = cst<R>(0.5) * (__ldg(a.geo[5] + cl) + __ldg(a.geo[5] + ch));
      amax = face_flux<R, NS, 2, LIM, TH>(a, sqp, sfl, f, j, rx, ryl, rx, ryh, gcs, H);
    } else {
#pragma unroll
      for (int i = 0; i < nv; ++i) H[i] = R(0);
    }
#pragma unroll
    for (int i = 0; i < nv; ++i) sHy[i * (TY + 1) * TX + fi] = H[i];
    sAy[fi] = amax;
  }
  __syncthreads();

  // 4. cells: divergence, explicit terms, CFL step.  Every thread first
  // waits for its own copies of step 0 (also those of cells it does not
  // finish: none may land after the tile is left)
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  R dtloc = R(3.0e38);
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
      Geo<R> geo;   // this thread's copies of step 0
      geo.Bx = sgeo[tid];
      geo.By = sgeo[TX * TY + tid];
      geo.gc = sgeo[2 * TX * TY + tid];
      geo.dgcx = sgeo[3 * TX * TY + tid];
      geo.dgcy = sgeo[4 * TX * TY + tid];
      geo.Bxx = a.geo[2] ? __ldg(a.geo[2] + c) : R(0);
      geo.Bxy = a.geo[3] ? __ldg(a.geo[3] + c) : R(0);
      geo.Byy = a.geo[4] ? __ldg(a.geo[4] + c) : R(0);
      const uint8_t fl = sfl[ry * RX + rx];
      R ap = R(0), anx = R(0), any_ = R(0);
      R tcoef = R(0);   // read at ring cells only (arc perimeter > 0)
      if (P.radial_source && (fl & F_SC_MASK) == 2) {
        ap = __ldg(a.arc + c);
        anx = __ldg(a.arc + g.plane + c);
        any_ = __ldg(a.arc + 2 * g.plane + c);
        if constexpr (sizeof(R) == 8) tcoef = st->src_t_coeff;
        else tcoef = st->src_t_coeff_f;
      }
      R bf = R(0), btc = R(0), bvel = R(0);   // bottom source cells only
      if (P.bottom_source && any_bsrc_tile && (__ldg(a.cflags + c) & F_BSRC)) {
        bf = __ldg(a.bfrac + c);
        if constexpr (sizeof(R) == 8) { btc = st->bsrc_t_coeff; bvel = st->bsrc_vel; }
        else { btc = st->bsrc_t_coeff_f; bvel = st->bsrc_vel_f; }
      }
      expl_terms<R, NS>(P, geo, qp, tcoef, ap, anx, any_, bf, btc, bvel, e);
#pragma unroll
      for (int i = 0; i < nv; ++i) {
        R d = R(0);
        if (!tile_dry) {
          d = d + (sHx[i * TY * (TX + 1) + cy * (TX + 1) + cx + 1] - sHx[i * TY * (TX + 1) + cy * (TX + 1) + cx]) * g.one_by_dx;
          if (g.ny > 1)
            d = d + (sHy[i * (TY + 1) * TX + (cy + 1) * TX + cx] - sHy[i * (TY + 1) * TX + cy * TX + cx]) * g.one_by_dy;
        }
        if (rout) rout[i * g.plane + c] = d - e[i];
      }
      if (want_dt && !tile_dry && owned_row(g, k)) {
        R ax = rmax(sAx[cy * (TX + 1) + cx], sAx[cy * (TX + 1) + cx + 1]);
        R ay = (g.ny > 1) ? rmax(sAy[cy * TX + cx], sAy[(cy + 1) * TX + cx]) : R(0);
        if constexpr (sizeof(R) == 8) {
          double dtx = (ax > 0.0) ? g.cfl * g.dx / ax : 1.0e300;
          double dty = (ay > 0.0) ? g.cfl * g.dy / ay : 1.0e300;
          dtloc = rmin(dtx, dty);
        } else {
          float dtx = (ax > 0.0f) ? fdiv(g.cfl_dx, ax) : 3.0e38f;
          float dty = (ay > 0.0f) ? fdiv(g.cfl_dy, ay) : 3.0e38f;
          dtloc = fminf(dtx, dty);
        }
      }
    }
  }
  if (want_dt) {
    // block minimum (warp shuffle, then shared memory), one atomic per block
    R m = dtloc;
    for (int o = 16; o > 0; o >>= 1) m = rmin(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ R wmin[FLUX_THREADS / 32];
    if ((tid & 31) == 0) wmin[tid >> 5] = m;
    __syncthreads();
    if (tid == 0) {
      R b = wmin[0];
      for (int w = 1; w < FLUX_THREADS / 32; ++w) b = rmin(b, wmin[w]);
      const double bd = (double)b;
      if (bd < (sizeof(R) == 8 ? 1.0e300 : 3.0e38)) atomicMin(&a.st->dtmin_bits, dbits(bd));
    }
  }
}

// ---------------------------------------------------------------------------
// k_dt: dt of this step (timestep + IMEX_SfloW2D.f90:417-439), one thread.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void dt_update(RunState* st, double max_dt) {
  if (!running(st)) { st->run_step = 0; return; }
  // the CFL minimum and the active count were accumulated with atomics by
  // the blocks of the kernels before: read and reset them with atomics
  double dtmin = __longlong_as_double((long long)atomicExch(&st->dtmin_bits, dbits(1.0e300)));
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
  const unsigned long long cells = atomicExch(&st->cells_acc[p], 0ull);
  st->last_cells = (long long)cells;
  st->cells_total += (long long)cells;
  st->border_total += (long long)atomicExch(&st->border_acc[p], 0ull);
  st->steps += 1;
}

static __global__ void k_dt(RunState* st, double max_dt) {
  step_kernel_entry();
  dt_update(st, max_dt);
}

template <class R, int NS, int LIM, int TH>
__global__ void __launch_bounds__(TileShape<TH>::FLUX_THREADS) k_flux(KArgs<R> a, const R* __restrict__ qin,
                                                       R* __restrict__ rout, int want_dt) {
  step_kernel_entry();
  const RunState* st = a.st;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // the timestep pass runs before k_dt advances the clock; the later stage
  // fluxes of a step run after it and follow its run_step decision
  if (want_dt ? !running(st) : !st->run_step) return;
  const uint8_t ta = a.tile_active[blockIdx.y * gridDim.x + blockIdx.x];
  if (ta == 0 || ta == TILE_DRY_BORDER) return;
  flux_tile<R, NS, LIM, TH>(a, qin, rout, want_dt, blockIdx.x, blockIdx.y, smem_raw);
}

// ---------------------------------------------------------------------------
// topography_reconstruction (geometry_2d.f90:555-895): 5-point centred
// slopes and curvatures of B on cells 3 .. n-2, the two-cell frame copied
// from the nearest computed row / column (a clamped index), then the slope
// factor and its derivatives.  FP64 with every product and sum rounded on
// its own (the host's order, sflow_setup.cpp), written to the topography
// planes in R; B is a pitched FP64 plane.  One thread per cell.
// ---------------------------------------------------------------------------
template <class R>
__device__ __forceinline__ void topography_cell(const double* __restrict__ B, int nx, int ny, int64_t pitch,
                                                double dx, double dy, bool slope_corr, R* const* geo,
                                                int j, int k, int64_t c) {
  const int jj = j < 2 ? 2 : (j > nx - 3 ? nx - 3 : j);
  const int kk = ny == 1 ? 0 : (k < 2 ? 2 : (k > ny - 3 ? ny - 3 : k));
  const double c1[5] = {-2.0, -1.0, 0.0, 1.0, 2.0};
  const double c2[5] = {2.0, -1.0, -2.0, -1.0, 2.0};
  auto Bat = [&](int x, int y) { return B[(int64_t)y * pitch + x]; };
  double px = 0.0, py = 0.0, sxx = 0.0, syy = 0.0, ws = 0.0;
  for (int m = 0; m < 5; ++m) {
    px = __dadd_rn(px, __dmul_rn(c1[m], Bat(jj + m - 2, kk)));
    sxx = __dadd_rn(sxx, __dmul_rn(c2[m], Bat(jj + m - 2, kk)));
  }
  double bx, by, bxx, byy, bxy;
  bx = __ddiv_rn(px, __dmul_rn(10.0, dx));
  bxx = __ddiv_rn(sxx, __dmul_rn(7.0, __dmul_rn(dx, dx)));
  if (ny == 1) {
    by = __ddiv_rn(0.0, __dmul_rn(10.0, dy));
    byy = __ddiv_rn(0.0, __dmul_rn(7.0, __dmul_rn(dy, dy)));
    bxy = 0.0;
  } else {
    for (int m = 0; m < 5; ++m) {
      py = __dadd_rn(py, __dmul_rn(c1[m], Bat(jj, kk + m - 2)));
      syy = __dadd_rn(syy, __dmul_rn(c2[m], Bat(jj, kk + m - 2)));
    }
    for (int mm = 0; mm < 5; ++mm)
      for (int m = 0; m < 5; ++m) ws = __dadd_rn(ws, __dmul_rn(__dmul_rn(c1[m], c1[mm]), Bat(jj + m - 2, kk + mm - 2)));
    by = __ddiv_rn(py, __dmul_rn(10.0, dy));
    byy = __ddiv_rn(syy, __dmul_rn(7.0, __dmul_rn(dy, dy)));
    bxy = __ddiv_rn(ws, __dmul_rn(__dmul_rn(10.0, dx), __dmul_rn(10.0, dy)));
  }
  geo[0][c] = (R)bx;
  geo[1][c] = (R)by;
  if (geo[2]) { geo[2][c] = (R)bxx; geo[3][c] = (R)bxy; geo[4][c] = (R)byy; }
  if (slope_corr) {
    const double gc = __ddiv_rn(1.0, __dadd_rn(__dadd_rn(1.0, __dmul_rn(bx, bx)), __dmul_rn(by, by)));
    const double gc2 = __dmul_rn(-2.0, __dmul_rn(gc, gc));
    geo[5][c] = (R)gc;
    geo[6][c] = (R)__dmul_rn(gc2, __dadd_rn(__dmul_rn(bx, bxx), __dmul_rn(by, bxy)));
    geo[7][c] = (R)__dmul_rn(gc2, __dadd_rn(__dmul_rn(bx, bxy), __dmul_rn(by, byy)));
  }
}

// after the topography changed (TOPO_CHANGE_FLAG, IMEX_SfloW2D.f90:445)
template <class R>
__global__ void __launch_bounds__(256) k_topography(KArgs<R> a) {
  step_kernel_entry();
  const Grid<R>& g = a.g;
  if (!a.st->run_step) return;
  const int64_t n = (int64_t)g.nx * g.ny;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j = (int)(i % g.nx), k = (int)(i / g.nx);
  topography_cell<R>(a.Bc, g.nx, g.ny, g.pitch, (double)g.dx, (double)g.dy, a.pd.slope_corr,
                     const_cast<R* const*>(a.geo), j, k, cidx(g, j, k));
}

// the eight topography planes (Bx, By, Bxx, Bxy, Byy, gc, dgcx, dgcy; the
// curvature ones null without the curvature term) as a kernel argument
template <class R>
struct TopoPlanes {
  R* p[8];
};

// at creation, from B in a pitched FP64 plane: the slope factor is 1 and its
// derivatives 0 without the slope correction (the host's initial values)
template <class R>
__global__ void __launch_bounds__(256) k_topography_setup(const double* __restrict__ B, int nx, int ny,
                                                          int64_t pitch, double dx, double dy, int slope_corr,
                                                          TopoPlanes<R> geo) {
  const int64_t n = (int64_t)nx * ny;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int j = (int)(i % nx), k = (int)(i / nx);
  const int64_t c = (int64_t)k * pitch + j;
  topography_cell<R>(B, nx, ny, pitch, dx, dy, slope_corr != 0, geo.p, j, k, c);
  if (!slope_corr) {
    geo.p[5][c] = R(1);
    geo.p[6][c] = R(0);
    geo.p[7][c] = R(0);
  }
}

// ---------------------------------------------------------------------------
// The physical variables of a cell's current state, kept between the
// assembly fixes, the erosion/deposition step and the post-step maxima of
// one step so that qc_to_qp of an unchanged state is not evaluated again
// (the same function of the same state: the same values).
template <class R, int NS>
struct CellQp {
  R qp[4 + NS + 2];
  R pdyn;
  bool valid;
};

// ---------------------------------------------------------------------------
// Positivity fixes of assemble_sol (solver_2d.f90:1381-1628) on an FP64 or
// FP32 state; returns status bits.  cq (may be null) receives qc_to_qp of
// the state when the fixes leave it unchanged after that evaluation.
// ---------------------------------------------------------------------------
template <class R, int NS>
__device__ __forceinline__ unsigned assemble_fixes(const Phys<R>& P, R* q, CellQp<R, NS>* cq = nullptr) {
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
  R qp_local[nv + 2];
  R* qp = cq ? cq->qp : qp_local;
  const R pdyn = qc_to_qp<R, NS>(P, q, qp);
  if (cq) { cq->pdyn = pdyn; cq->valid = true; }
  if (qp[3] < P.thr_273) st |= SFLOW_S_LOW_T;
  if (ns > 0) {
    R ssum = R(0);
#pragma unroll
    for (int i = 0; i < ns; ++i) ssum += q[4 + i];
    if (ssum > q[0]) {
      if (cq) cq->valid = false;
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

// Per-cell inputs and results of the mass exchange.
template <class R, int NS>
struct CellExch {
  R erodible[NS];   // erodible solid thicknesses (erosion only, else 0)
  R bf;             // bottom radial source: cell fraction inside the source
  R dep[NS], ers[NS], topo;   // deposition / erosion rates, topography rate
};

// update_erosion_deposition_cell (solver_2d.f90:2382-2597) for one cell: the
// state part.  cq (may be null): on entry the qc_to_qp of q if valid, on
// return that of the final state (invalid when the cell was emptied).
template <class R, int NS>
__device__ __forceinline__ unsigned erosion_deposition(const Phys<R>& P, const Geo<R>& geo, R dt,
                                                       R* q, CellExch<R, NS>& ex, CellQp<R, NS>* cq = nullptr) {
  constexpr int nv = 4 + NS, ns = NS;
  unsigned st = 0;
  R qp[nv + 2], eqn[nv];
  R* dep = ex.dep;
  if (cq && cq->valid) {
    // qc_to_qp of a state with q(1) <= eps is the dry state, as below
#pragma unroll
    for (int i = 0; i < nv + 2; ++i) qp[i] = cq->qp[i];
  } else if (q[0] > R(0)) {
    qc_to_qp<R, NS>(P, q, qp);
  } else {
#pragma unroll
    for (int i = 0; i < nv + 2; ++i) qp[i] = R(0);
    qp[3] = P.T_ambient;
  }
  if (cq) cq->valid = false;
  unsigned dep_limited = 0u;
  mass_exchange<R, NS>(P, qp, geo.Bx, geo.By, dt, P.erosion_coeff > R(0) ? ex.erodible : nullptr, dep, ex.ers,
                       eqn, ex.topo, sizeof(R) == 4 ? &dep_limited : nullptr);
  if (P.bottom_source && ex.bf > R(0)) {
    // the part of the cell inside the bottom source exchanges nothing
    const R out_frac = R(1) - ex.bf;
#pragma unroll
    for (int i = 0; i < ns; ++i) { dep[i] = dep[i] * out_frac; ex.ers[i] = ex.ers[i] * out_frac; }
#pragma unroll
    for (int i = 0; i < nv; ++i) eqn[i] = eqn[i] * out_frac;
    ex.topo = ex.topo * out_frac;
  }
  const R q0_before = q[0];
#pragma unroll
  for (int i = 0; i < nv; ++i) q[i] = q[i] + dt * eqn[i];
#pragma unroll
  for (int i = 0; i < ns; ++i) q[4 + i] = rmax(R(0), q[4 + i]);
  if constexpr (sizeof(R) == 4) {
    // FP32 form: a class whose deposition took the limiter r_h alpha/dt
    // settles out entirely -- zero in exact arithmetic; the FP32 sum leaves
    // a few ulp of its old mass (an alpha of ~1e-9 where the FP64 form
    // keeps ~1e-18), which is cleared
    if (!(P.bottom_source && ex.bf > R(0))) {
#pragma unroll
      for (int i = 0; i < ns; ++i)
        if (((dep_limited >> i) & 1u) && ex.ers[i] == R(0)) q[4 + i] = R(0);
    }
    // FP32 form: when the limited deposition and carrier loss remove the
    // whole mass (exactly zero in exact arithmetic), the sum leaves a
    // rounding residual of a few ulp of the old mass, with a momentum
    // residual of its own: a film with an arbitrary velocity.  A cell left
    // with less than 2^-16 of its mass is emptied (the FP64 form empties
    // residuals down to -1e-10 and keeps positive ones, which are 2^-52
    // relative there).
    if (fabsf(q[0]) <= q0_before * 0x1p-16f) {
#pragma unroll
      for (int i = 0; i < nv; ++i) q[i] = R(0);
    }
  }
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
    const R pdyn = qc_to_qp<R, NS>(P, q, qp);
    Mixt<R> m = mixt_var<R, NS>(P, qp, false);
    red_grav = m.red_grav;
    // FP32 form: a cell of particle-free gas at T_ambient -- also a film
    // just filled from a neighbour whose energy came out below its kinetic
    // energy, for which qc_to_qp takes T = T_ambient as the reference's
    // r_phys_var does -- is ambient air, whose reduced gravity the FP64 form
    // computes as exactly 0 and lifts off.  In FP32, rho_c = 1/(R T/p) can
    // land an ulp above rho_a_amb and keep the film, with an arbitrary
    // velocity (measured on the 1024^2 current with settling: a 5e-5 kg/m^2
    // film at 2e4 m/s).  Such a cell is lifted off here too.
    if constexpr (sizeof(R) == 4) {
      if (P.gas && qp[3] == P.T_ambient) {
        R ssum = R(0);
#pragma unroll
        for (int i = 0; i < ns; ++i) ssum += q[4 + i];
        if (ssum == R(0)) red_grav = R(0);
      }
    }
    if (cq && red_grav > R(0)) {
#pragma unroll
      for (int i = 0; i < nv + 2; ++i) cq->qp[i] = qp[i];
      cq->pdyn = pdyn;
      cq->valid = true;
    }
  }
  if (red_grav <= R(0)) {
#pragma unroll
    for (int i = 0; i < nv; ++i) q[i] = R(0);
  }
  return st;
}

template <class R>
__device__ __forceinline__ double to_d(R x) {
  if constexpr (sizeof(R) == 4) return f2d_exact(x);
  else return x;
}

// The accumulated fields of update_erosion_deposition_cell
// (solver_2d.f90:2476-2494), in FP64: deposit += dt*deposition, erosion +=
// dt*erosion, erodible -= dt*erosion (+ dt*deposition with
// ERODIBLE_DEPOSIT_FLAG), B += dt*topo_term with TOPO_CHANGE_FLAG.
template <class R, int NS>
__device__ __forceinline__ void add_deposit(const KArgs<R>& a, int64_t c, double dt, const CellExch<R, NS>& ex) {
  const int64_t pl = a.g.plane;
  if (a.deposit) {
#pragma unroll
    for (int i = 0; i < NS; ++i) a.deposit[i * pl + c] += dt * to_d(ex.dep[i]);
  }
  if (a.erosion) {
#pragma unroll
    for (int i = 0; i < NS; ++i) a.erosion[i * pl + c] += dt * to_d(ex.ers[i]);
#pragma unroll
    for (int i = 0; i < NS; ++i) a.erodible[i * pl + c] = a.erodible[i * pl + c] - dt * to_d(ex.ers[i]);
    if (a.pd.erodible_deposit) {
#pragma unroll
      for (int i = 0; i < NS; ++i) a.erodible[i * pl + c] = a.erodible[i * pl + c] + dt * to_d(ex.dep[i]);
    }
  }
  if (a.Bc) a.Bc[c] = a.Bc[c] + dt * to_d(ex.topo);
}

// nodata emptying of assemble_sol (solver_2d.f90:1626) and
// update_erosion_deposition_cell for one cell after the assembly
template <class R, int NS>
__device__ __forceinline__ unsigned cell_exchange(const KArgs<R>& a, int64_t c, double dt, R* q,
                                                  CellQp<R, NS>* cq) {
  constexpr int nv = 4 + NS;
  if (a.pd.nodata && (__ldg(a.cflags + c) & F_NODATA)) {
#pragma unroll
    for (int i = 0; i < nv; ++i) q[i] = R(0);
    if (cq) cq->valid = false;
  }
  if (!a.pd.exchange) return 0;
  const Geo<R> geo = load_geo(a, c);
  CellExch<R, NS> ex;
#pragma unroll
  for (int i = 0; i < NS; ++i) ex.erodible[i] = a.erodible ? (R)a.erodible[i * a.g.plane + c] : R(0);
  ex.bf = (a.pd.bottom_source && (__ldg(a.cflags + c) & F_BSRC)) ? __ldg(a.bfrac + c) : R(0);
  const unsigned st = erosion_deposition<R, NS>(a.pr, geo, from_double<R>(dt), q, ex, cq);
  add_deposit<R, NS>(a, c, dt, ex);
  return st;
}

// vulnerability table (IMEX_SfloW2D.f90:339-353, 477-491): entry
// i_thk * n_dyn + i_dyn of a cell holding mass is h >= thickness level i_thk
// and p_dyn >= dynamic-pressure level i_dyn; OR-ed over the steps (set at
// the start).  Entry e is bit e % 32 of the cell's word plane e / 32.
template <class R>
__device__ __forceinline__ void vuln_update(const KArgs<R>& a, int64_t c, R h, R p_dyn, bool accumulate) {
  const Phys<R>& P = a.pr;
  unsigned w[(SFLOW_MAX_LEVELS * SFLOW_MAX_LEVELS + 31) / 32];
  for (int i = 0; i < a.vuln_words; ++i) w[i] = 0u;
  int e = 0;
  for (int it = 0; it < P.n_thk; ++it) {
    const bool th = h >= P.thk_levels[it];
    for (int id = 0; id < P.n_dyn; ++id, ++e)
      if (th && p_dyn >= P.dyn_levels[id]) w[e >> 5] |= 1u << (e & 31);
  }
  for (int i = 0; i < a.vuln_words; ++i) {
    uint32_t* p = a.vuln + (int64_t)i * a.g.plane + c;
    *p = accumulate ? (*p | w[i]) : w[i];
  }
}

// post-step maxima (IMEX_SfloW2D.f90:449-505)
template <class R, int NS>
__device__ __forceinline__ void post_step_maps(const KArgs<R>& a, int64_t c, const R* q,
                                               const CellQp<R, NS>* cq = nullptr) {
  constexpr int nv = 4 + NS;
  if (q[0] > R(0)) {
    R qp[nv + 2];
    R p_dyn;
    if (cq && cq->valid) {
#pragma unroll
      for (int i = 0; i < nv + 2; ++i) qp[i] = cq->qp[i];
      p_dyn = cq->pdyn;
    } else {
      p_dyn = qc_to_qp<R, NS>(a.pr, q, qp);
    }
    R hm = a.hmax[c];
    a.hmax[c] = rmax(hm, qp[0]);
    if (qp[0] > a.pr.thr_1em3) {
      R mv = sqrt(sq(qp[nv]) + sq(qp[nv + 1]));
      a.pdynmax[c] = rmax(a.pdynmax[c], p_dyn);
      a.mvmax[c] = rmax(a.mvmax[c], mv);
    }
    if (a.vuln) vuln_update<R>(a, c, qp[0], p_dyn, true);
  }
}

// ---------------------------------------------------------------------------
// One stage of imex_RK_solver for one cell (solver_2d.f90:1103-1281):
//   q_fv = q0 - dt*(s1 - s2),  s1 = sum a_tilde*(divFlux - expl),
//                              s2 = sum a_dirk*(NH + SI) over earlier stages,
// then for an implicit stage (a_diag /= 0) and q_fv(1) > 0 the semi-implicit
// Coulomb term with its velocity fixes, the implicit Newton, the fixes after
// it, and NH = (q_guess - q_si)/(dt a_diag).  Writes q_guess (the stage
// state q_rk) and NH + SI of the stage.
// ---------------------------------------------------------------------------
template <class R, int NS>
__device__ __forceinline__ unsigned stage_cell(const KArgs<R>& a, const Geo<R>& geo, const R* q0,
                                               const R* s1, const R* s2, double dt, double a_diag,
                                               R* qg_out, R* rn_out, int& nit) {
  constexpr int nv = 4 + NS;
  unsigned status = 0;
  nit = 0;
  if constexpr (sizeof(R) == 8) {
    // ---- plain FP64 form: the reference's Newton, step by step ----
    const Phys<double>& P = a.pd;
    double qfv[nv], qp[nv + 2], si[nv], qsi[nv], qg[nv], Rj[nv];
#pragma unroll
    for (int i = 0; i < nv; ++i) qfv[i] = q0[i] - dt * (s1[i] - s2[i]);
#pragma unroll
    for (int i = 0; i < nv; ++i) { si[i] = 0.0; qsi[i] = qfv[i]; qg[i] = qfv[i]; }
    if (a_diag != 0.0) {
      if (qfv[0] > 0.0) {
        qc_to_qp<double, NS>(P, qfv, qp);
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
        for (int i = 0; i < nv; ++i) Rj[i] = (s1[i] - s2[i]) - a_diag * si[i];
        NewtonCtx nc{&P, dt, a_diag, geo.Bx, geo.By, q0, Rj};
        nit = solve_rk_step<NS>(nc, qg);
        if (nit > kMaxNewton) status |= SFLOW_S_NEWTON_MAXIT;
        if (a.g.ny == 1) qg[2] = 0.0;
        if (sq(qsi[1]) + sq(qsi[2]) == 0.0) {
          qg[1] = 0.0; qg[2] = 0.0;
        } else if (qg[1] * qsi[1] <= 0.0 && qg[2] * qsi[2] <= 0.0) {
          qg[1] = 0.0; qg[2] = 0.0;
        } else {
          double m1 = sqrt(sq(qg[1]) + sq(qg[2])), m0 = sqrt(sq(qsi[1]) + sq(qsi[2]));
          qg[1] = m1 * qsi[1] / m0;
          qg[2] = m1 * qsi[2] / m0;
        }
      }
#pragma unroll
      for (int i = 0; i < nv; ++i) rn_out[i] = (qg[i] - qsi[i]) / (dt * a_diag) + si[i];
    } else {
#pragma unroll
      for (int i = 0; i < nv; ++i) rn_out[i] = 0.0;
    }
#pragma unroll
    for (int i = 0; i < nv; ++i) qg_out[i] = qg[i];
  } else {
    // ---- FP32 bulk form: FP32 explicit part, FP64 scalar Newton ----
    const Phys<R>& P = a.pr;
    const R dtr = from_double<R>(dt);
    const R dta = from_double<R>(dt * a_diag);
    R qfv[nv], qp[nv + 2], si[nv], qsi[nv], qg[nv];
#pragma unroll
    for (int i = 0; i < nv; ++i) qfv[i] = q0[i] - dtr * (s1[i] - s2[i]);
#pragma unroll
    for (int i = 0; i < nv; ++i) { si[i] = R(0); qsi[i] = qfv[i]; qg[i] = qfv[i]; }
    if (a_diag != 0.0) {
      if (qfv[0] > R(0)) {
        qc_to_qp<R, NS>(P, qfv, qp);
        semi_impl_terms<R, NS>(P, geo, qp, si);
#pragma unroll
        for (int i = 0; i < nv; ++i) qsi[i] = qfv[i] + dta * si[i];
        if (sq(qfv[1]) + sq(qfv[2]) == R(0)) {
          qsi[1] = R(0); qsi[2] = R(0);
        } else if (qsi[1] * qfv[1] < R(0) || qsi[2] * qfv[2] < R(0)) {
          qsi[1] = R(0); qsi[2] = R(0);
        } else {
          R m1 = sqrt(sq(qsi[1]) + sq(qsi[2])), m0 = sqrt(sq(qfv[1]) + sq(qfv[2]));
          qsi[1] = m1 * qfv[1] / m0;
          qsi[2] = m1 * qfv[2] / m0;
        }
        const R idta = R(1) / dta;
#pragma unroll
        for (int i = 0; i < nv; ++i) { si[i] = (qsi[i] - qfv[i]) * idta; qg[i] = qsi[i]; }
        float e1, e2;
        const float sv = reduced_friction_solve<NS>(P, a.pd, geo.Bx, geo.By, qsi, dt * a_diag, e1, e2, nit);
        qg[1] = sv * e1;
        qg[2] = sv * e2;
        if (a.g.ny == 1) qg[2] = R(0);
      }
      const R idta = R(1) / dta;
#pragma unroll
      for (int i = 0; i < nv; ++i) rn_out[i] = (qg[i] - qsi[i]) * idta + si[i];
    } else {
#pragma unroll
      for (int i = 0; i < nv; ++i) rn_out[i] = R(0);
    }
#pragma unroll
    for (int i = 0; i < nv; ++i) qg_out[i] = qg[i];
  }
  return status;
}

template <class R>
__device__ __forceinline__ void newton_stats(RunState* st, unsigned status, int nit_sum, int nit_max) {
  if (status) atomicOr(&st->status, status);
  int wsum = nit_sum;
  for (int o = 16; o > 0; o >>= 1) wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
  int wmax = nit_max;
  for (int o = 16; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, o));
  if ((threadIdx.x & 31) == 0 && wsum > 0) {
    atomicAdd((unsigned long long*)&st->newton_iters, (unsigned long long)wsum);
    atomicMax(&st->newton_max, wmax);
  }
}

// ---------------------------------------------------------------------------
// k_stage2: the pointwise part of an N_RK = 2 step after the flux stage:
// imex_RK_solver stage 2 (a_tilde(2,1) = 1, a_dirk(2,2) = 1), assemble_sol
// (1342-1630; the last tableau row equals omega, so q = q_rk(2)),
// update_erosion_deposition_cell, post-step maxima.
// mode -1: stage + assembly + erosion/deposition + maxima (fused step);
// 0: stage + assembly (imex_RK_solver); 1: erosion/deposition only;
// 2: maxima only.
// ---------------------------------------------------------------------------
// One cell (j, k) of the pointwise step; returns 1 when the cell is active
// and holds mass afterwards.  One cell per thread in every caller, so the
// cell's arithmetic is the same code whatever the tile height.
template <class R, int NS>
__device__ __forceinline__ int stage2_cell(const KArgs<R>& a, int mode, int j, int k, unsigned& status,
                                           int& nit) {
  constexpr int nv = 4 + NS;
  RunState* st = a.st;
  const Grid<R>& g = a.g;
  nit = 0;
  if (j >= g.nx || k >= g.ny) return 0;
  const int64_t c = cidx(g, j, k);
  if (!a.mask[c]) return 0;
  const double dt = st->dt;
  R q[nv];
#pragma unroll
  for (int i = 0; i < nv; ++i) q[i] = a.q[i * g.plane + c];
  if (mode > 0) {
    if (mode == 1) {
      status |= cell_exchange<R, NS>(a, c, dt, q, nullptr);
#pragma unroll
      for (int i = 0; i < nv; ++i) a.q[i * g.plane + c] = q[i];
    } else {
      post_step_maps<R, NS>(a, c, q);
    }
  } else {
    const Geo<R> geo = load_geo(a, c);
    R s1[nv], s2[nv], rn[nv];
#pragma unroll
    for (int i = 0; i < nv; ++i) {
      s1[i] = R(0) + a.rd[i * g.plane + c] * R(1);
      s2[i] = R(0);
    }
    status |= stage_cell<R, NS>(a, geo, q, s1, s2, dt, 1.0, q, rn, nit);
    CellQp<R, NS> cq;
    status |= assemble_fixes<R, NS>(a.pr, q, &cq);
    if (mode < 0) status |= cell_exchange<R, NS>(a, c, dt, q, &cq);
    else if (a.pd.nodata && (__ldg(a.cflags + c) & F_NODATA)) {
#pragma unroll
      for (int i = 0; i < nv; ++i) q[i] = R(0);
    }
#pragma unroll
    for (int i = 0; i < nv; ++i) a.q[i * g.plane + c] = q[i];
    if (mode < 0) post_step_maps<R, NS>(a, c, q, &cq);
  }
  return q[0] > R(0);
}

// Wet byte of a batched run's tile after the step (read by the candidate
// rule): bit 0 a cell holds mass; bits 1-4 a cell holding mass lies within
// n_RK = 2 cells of the west / east / south / north tile edge, so only the
// neighbours across those edges can gain active cells.  0xff: unknown.
constexpr uint8_t TW_ANY = 1, TW_W = 2, TW_E = 4, TW_S = 8, TW_N = 16;

// single run: one block per 32 x 8 cells (grid tiles_x x ceil(ny/8)); the
// activity byte is the one of the 32 x TH tile holding the block.  The FP32
// form is compiled for 6 resident blocks per SM (40 registers): the kernel
// waits on memory, and more warps hide more of it.
template <class R, int NS, int TH>
__global__ void __launch_bounds__(TileShape<TH>::STAGE_THREADS, sizeof(R) == 4 ? 6 : 1)
    k_stage2(KArgs<R> a, int mode) {
  step_kernel_entry();
  if (!a.st->run_step) return;
  const int kk = blockIdx.y * 8 + threadIdx.x / TX;
  // inactive, or left unchanged (k_flux's dry tiles, k_mask's dry border)
  auto skipped = [](uint8_t ta) { return ta == 0 || ta == 2 || ta == TILE_DRY_BORDER; };
  int tile;
  bool run = true;
  if constexpr (TH >= 8) {
    tile = (blockIdx.y * 8 / TH) * gridDim.x + blockIdx.x;
    if (skipped(a.tile_active[tile])) return;
  } else {
    // 32 x 4 tiles: the block's two halves belong to two tiles
    tile = (kk / TH) * gridDim.x + blockIdx.x;
    run = kk < a.g.ny && !skipped(a.tile_active[tile]);
  }
  unsigned status = 0;
  int nit = 0;
  int wet = run ? stage2_cell<R, NS>(a, mode, blockIdx.x * TX + threadIdx.x % TX, kk, status, nit) : 0;
  if (!owned_row(a.g, kk)) { status = 0u; nit = 0; }   // halo rows of a row slab
  newton_stats<R>(a.st, status, nit, nit);
  if (mode < 0) {
    // wet flag of the tile for the next check_solve (buffer of the new
    // step count's parity; set only, the check_solve of this step cleared it)
    const int nt = gridDim.x * a.g.tiles_y;
    if constexpr (TH >= 8) {
      wet = __syncthreads_or(wet);
      if (wet && threadIdx.x == 0) a.tile_wet_step[(unsigned)(a.st->steps & 1) * nt + tile] = 1;
    } else {
      if (wet) a.tile_wet_step[(unsigned)(a.st->steps & 1) * nt + tile] = 1;
    }
  }
}

// ---------------------------------------------------------------------------
// General tableaux (N_RK = 1, 3, 4; solver_2d.f90:429-487): one kernel per
// stage, the flux kernel for stages with omega_tilde > 0, one assembly.
// rd holds divFlux - expl and rn holds NH + SI of every stage (n_vars planes
// per stage); qs holds the state of the running stage.
// ---------------------------------------------------------------------------
template <class R, int NS, int TH>
__global__ void __launch_bounds__(TileShape<TH>::STAGE_THREADS) k_stage(KArgs<R> a, int irk) {
  step_kernel_entry();
  constexpr int nv = 4 + NS;
  RunState* st = a.st;
  if (!st->run_step) return;
  if constexpr (TH >= 8) {
    if (!a.tile_active[(blockIdx.y * 8 / TH) * gridDim.x + blockIdx.x]) return;
  }
  const Grid<R>& g = a.g;
  const int j = blockIdx.x * TX + threadIdx.x % TX;
  const int k = blockIdx.y * 8 + threadIdx.x / TX;
  unsigned status = 0;
  int nit = 0;
  if (j < g.nx && k < g.ny && (TH >= 8 || a.tile_active[(k / TH) * gridDim.x + blockIdx.x])) {
    const int64_t c = cidx(g, j, k);
    if (a.mask[c]) {
      const double dt = st->dt;
      const Geo<R> geo = load_geo(a, c);
      const int64_t sv = (int64_t)nv * g.plane;
      R q0[nv], s1[nv], s2[nv], qg[nv], rn[nv];
#pragma unroll
      for (int i = 0; i < nv; ++i) {
        q0[i] = a.q[i * g.plane + c];
        s1[i] = R(0);
        s2[i] = R(0);
      }
      for (int r = 0; r < irk; ++r) {
        const R at = (R)a.tableau_at[irk * 4 + r], ad = (R)a.tableau_ad[irk * 4 + r];
#pragma unroll
        for (int i = 0; i < nv; ++i) {
          s1[i] = s1[i] + a.rd[r * sv + i * g.plane + c] * at;
          s2[i] = s2[i] + a.rn[r * sv + i * g.plane + c] * ad;
        }
      }
      status |= stage_cell<R, NS>(a, geo, q0, s1, s2, dt, a.tableau_ad[irk * 4 + irk], qg, rn, nit);
      if (!owned_row(g, k)) { status = 0u; nit = 0; }   // halo rows of a row slab
#pragma unroll
      for (int i = 0; i < nv; ++i) {
        a.qs[i * g.plane + c] = qg[i];
        a.rn[irk * sv + i * g.plane + c] = rn[i];
      }
    }
  }
  newton_stats<R>(st, status, nit, nit);
}

// assemble_sol (solver_2d.f90:1342-1630) + erosion/deposition + maxima
template <class R, int NS, int TH>
__global__ void __launch_bounds__(TileShape<TH>::STAGE_THREADS) k_assemble(KArgs<R> a) {
  step_kernel_entry();
  constexpr int nv = 4 + NS;
  RunState* st = a.st;
  if (!st->run_step) return;
  if constexpr (TH >= 8) {
    if (!a.tile_active[(blockIdx.y * 8 / TH) * gridDim.x + blockIdx.x]) return;
  }
  const Grid<R>& g = a.g;
  const int j = blockIdx.x * TX + threadIdx.x % TX;
  const int k = blockIdx.y * 8 + threadIdx.x / TX;
  unsigned status = 0;
  if (j < g.nx && k < g.ny && (TH >= 8 || a.tile_active[(k / TH) * gridDim.x + blockIdx.x])) {
    const int64_t c = cidx(g, j, k);
    if (a.mask[c]) {
      const double dt = st->dt;
      const int64_t sv = (int64_t)nv * g.plane;
      const int nrk = a.pd.nrk;
      R q[nv];
      if (a.take_last) {
#pragma unroll
        for (int i = 0; i < nv; ++i) q[i] = a.qs[i * g.plane + c];
      } else {
        R s1[nv], s2[nv];
#pragma unroll
        for (int i = 0; i < nv; ++i) { s1[i] = R(0); s2[i] = R(0); }
        for (int r = 0; r < nrk; ++r) {
          const R ot = (R)a.omega_t[r], om = (R)a.omega[r];
#pragma unroll
          for (int i = 0; i < nv; ++i) {
            s1[i] = s1[i] + a.rd[r * sv + i * g.plane + c] * ot;
            s2[i] = s2[i] + a.rn[r * sv + i * g.plane + c] * om;
          }
        }
        const R dtr = from_double<R>(dt);
#pragma unroll
        for (int i = 0; i < nv; ++i) q[i] = a.q[i * g.plane + c] - dtr * (s1[i] - s2[i]);
      }
      CellQp<R, NS> cq;
      status |= assemble_fixes<R, NS>(a.pr, q, &cq);
      status |= cell_exchange<R, NS>(a, c, dt, q, &cq);
      if (!owned_row(g, k)) status = 0u;   // halo rows of a row slab
#pragma unroll
      for (int i = 0; i < nv; ++i) a.q[i * g.plane + c] = q[i];
      post_step_maps<R, NS>(a, c, q, &cq);
    }
  }
  if (status) atomicOr(&st->status, status);
}

}  // namespace sflow

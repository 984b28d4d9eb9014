// sflow_batch_kernels.cuh -- many independent runs advanced together.
//
// Every run keeps its own state, geometry, RunState and kernel arguments
// (KArgs) in device memory.  One batch step is five launches for all runs
// of a solid-class count together:
//
//   k_b_cand    from the active tiles of the previous step (list L[pp]):
//               every tile within one tile of an active tile becomes a
//               candidate (deduplicated by a per-tile flag) -> list C;
//               also the per-run start-of-step work of k_mask (ring inlet
//               time factor)
//   k_b_mask    check_solve on the candidate tiles; tiles with an active
//               cell -> list L[pp^1]
//   k_b_flux    k_flux on L[pp^1] (persistent blocks, dynamic tile fetch)
//   k_b_dt      k_dt of every live run (one thread per run); pp ^= 1
//   k_b_stage2  k_stage2 on the active cells of L[pp]: k_b_mask lists
//               them (entry = slot | tile | cell in the tile), so
//               the warps of the pointwise stage carry active cells only
//               instead of the mostly idle lanes of sparse tiles
//
// Why candidates suffice: a cell outside the active set is not updated, so
// a wet cell (a check_solve seed) was active in the previous step; active
// cells lie within n_RK = 2 cells of a seed, and tiles are 32 x TH cells
// with TH >= 4, so they lie in the 3 x 3 tile neighbourhood of a previously
// active tile that held mass within n_RK cells of the edge (or corner) they
// share (tile_wet, written by the stage kernel: one bit per edge).  Border
// and ring cells
// are seeds of every step, so their tiles stay in the lists; a border seed
// reaches into the neighbouring tile only when the edge tile is narrower
// than n_RK + 1 cells, and ring seeds may reach any neighbour, so those
// tiles are dilated too (tile_seed).  A newly admitted run puts all its tiles in L[pp] (full scan for
// its first step).  Tiles outside the candidate set keep an all-zero mask
// (they were processed when they last stopped being active), so the flux
// halo reads them as inactive, as the single-run kernels do.
//
// List entries are 64-bit: slot (16 bits) | generation (16 bits) | tile (32
// bits).  k_b_cand drops entries whose slot is free or holds a newer run,
// so a slot can be reused at once after its run is collected.
//
// The per-cell arithmetic is the single-run code (mask_tile, flux_tile,
// stage2_cell) on the run's own arguments, so a run gives bit-identical
// results alone, with the single-run solver, and in any mix.
#pragma once
#include <cuda_runtime.h>

#include "sflow_kernels.cuh"

namespace sflow {

struct BatchRun {
  RunState* st;      // the run's device state
  uint32_t* cand;    // per-tile candidate flag
  const uint8_t* tile_wet;    // wet byte of the tile after the last step (TW_*; 0xff: unknown)
  const uint8_t* tile_seed;   // tile holds ring-boundary cells, or is a narrow edge tile
  const uint16_t* tile_count; // active cells of a tile of code 3
  int tiles_x, tiles_y;
  unsigned gen;      // generation of the run in this slot
  int live;          // slot holds a run
  double max_dt;
};

struct BatchCtl {
  unsigned count[2];   // entries in tile list 0 / 1
  unsigned dcount[2];  // entries in dry-border list 0 / 1
  unsigned ncand;      // entries in the candidate list
  unsigned pp;         // list read by k_b_cand
  unsigned work[3];    // dynamic tile counters of k_b_mask, k_b_flux, k_b_stage2
  unsigned steps;      // batch steps done
  unsigned ncells;     // entries in the active-cell list (k_b_mask -> k_b_stage2)
  unsigned overflow;   // set when the active-cell list was too short (never expected)
};

// per-slot summary copied to the host after a batch advance
struct BatchSummary {
  long long steps;
  long long cells_total;
  double t;
  unsigned status;
  int running;
};

template <class R>
struct BatchArgs {
  const KArgs<R>* args;      // [max_runs]
  BatchRun* runs;            // [max_runs]
  BatchCtl* ctl;
  unsigned long long* list0;
  unsigned long long* list1;
  // active tiles whose only seeds are border cells (tile code 3): check_solve
  // keeps evaluating them (candidates of the next step), flux and stage skip
  unsigned long long* dlist0;
  unsigned long long* dlist1;
  unsigned long long* cand;
  unsigned long long* cells; // active cells: slot (16 bits) | tile (39) | cell in the tile (9)
  unsigned cells_cap;        // entries the cell list holds
  BatchSummary* summary;     // [max_runs]
  int max_runs;
};

constexpr int kBatchCandThreads = 256;
// 128-thread stage blocks (4 per SM at least): the bound then leaves the
// per-cell Newton its registers without spills; measured 5 % faster than
// 256-thread blocks held to 64 registers
constexpr int kBatchStageThreads = 128;

__device__ __forceinline__ int entry_slot(unsigned long long e) { return (int)(e >> 48); }
__device__ __forceinline__ unsigned entry_gen(unsigned long long e) { return (unsigned)(e >> 32) & 0xffffu; }
__device__ __forceinline__ unsigned entry_tile(unsigned long long e) { return (unsigned)(e & 0xffffffffull); }

// copy one run's kernel arguments into shared memory (all threads)
template <class R>
__device__ __forceinline__ void load_args(KArgs<R>* dst, const KArgs<R>* src) {
  static_assert(sizeof(KArgs<R>) % 8 == 0, "KArgs size");
  const unsigned long long* s = reinterpret_cast<const unsigned long long*>(src);
  unsigned long long* d = reinterpret_cast<unsigned long long*>(dst);
  for (int i = threadIdx.x; i < (int)(sizeof(KArgs<R>) / 8); i += blockDim.x) d[i] = s[i];
}

// Tiles of a persistent kernel come from a counter in global memory.
// Thread 0 claims the next index as soon as the block starts on a tile, so
// the atomic's latency overlaps the tile's work, and one barrier per tile
// hands the claimed index to the block (which also frees the block's shared
// memory for the next tile).
struct TileQueue {
  unsigned* counter;
  unsigned* s_idx;   // shared, 2 entries
  unsigned par = 0;
  unsigned claim = 0;
  __device__ __forceinline__ unsigned first() {
    if (threadIdx.x == 0) s_idx[0] = atomicAdd(counter, 1u);
    __syncthreads();
    return s_idx[0];
  }
  // first statement of the loop body, before any continue
  __device__ __forceinline__ void prefetch() {
    if (threadIdx.x == 0) claim = atomicAdd(counter, 1u);
  }
  __device__ __forceinline__ unsigned next() {
    if (threadIdx.x == 0) s_idx[par ^ 1u] = claim;
    __syncthreads();
    par ^= 1u;
    return s_idx[par];
  }
};

template <class R>
__global__ void __launch_bounds__(kBatchCandThreads) k_b_cand(BatchArgs<R> b) {
  step_kernel_entry();
  BatchCtl* ctl = b.ctl;
  const unsigned pp = ctl->pp;
  const unsigned long long* L = pp ? b.list1 : b.list0;
  const unsigned long long* Ld = pp ? b.dlist1 : b.dlist0;
  const unsigned n = ctl->count[pp], nd = ctl->dcount[pp];
  const unsigned gt = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned G = gridDim.x * blockDim.x;
  unsigned long long* Ldout = pp ? b.dlist0 : b.dlist1;   // cleared by k_b_dt
  if (gt == 0) {
    ctl->count[pp ^ 1u] = 0u;
    ctl->work[0] = 0u;
    ctl->ncells = 0u;
  }
  // Three independent loops on disjoint threads so that their latencies
  // overlap: the candidate expansion on threads 0 .. 9n-1, the dry border
  // strips on the threads after those, the per-run work (an FP64 cosine per
  // run) on the last threads of the grid.
  for (unsigned r = G - 1u - gt; r < (unsigned)b.max_runs; r += G) {
    const BatchRun br = b.runs[r];
    if (!br.live) continue;
    RunState* st = br.st;
    if (running(st)) {
      st->src_t_coeff = source_time_coeff(st->tp, st->pi_g, st->t);
      st->src_t_coeff_f = (float)st->src_t_coeff;
    }
  }
  auto add_cand = [&](const BatchRun& br, unsigned long long e, int tx, int ty) {
    if (tx < 0 || ty < 0 || tx >= br.tiles_x || ty >= br.tiles_y) return;
    const unsigned t2 = (unsigned)(ty * br.tiles_x + tx);
    if (atomicExch(&br.cand[t2], 1u) == 0u) {
      const unsigned pos = atomicAdd(&ctl->ncand, 1u);
      b.cand[pos] = (e & 0xffffffff00000000ull) | (unsigned long long)t2;
    }
  };
  // active tiles of the last step: one thread per (tile, neighbour)
  for (unsigned i = gt; i < n * 9u; i += G) {
    const unsigned long long e = L[i / 9u];
    const int slot = entry_slot(e);
    const BatchRun& br = b.runs[slot];
    if (!br.live || (br.gen & 0xffffu) != entry_gen(e) || !running(br.st)) continue;
    const unsigned tile = entry_tile(e);
    const int nb = (int)(i % 9u);
    const int dx = nb % 3 - 1, dy = nb / 3 - 1;
    // only tiles with mass near the shared edge, ring cells or a narrow
    // domain edge can activate cells of their neighbours
    if (nb != 4 && !br.tile_seed[tile]) {
      const unsigned tw = br.tile_wet[tile];
      const unsigned need = TW_ANY | (dx < 0 ? TW_W : 0u) | (dx > 0 ? TW_E : 0u) | (dy < 0 ? TW_S : 0u) |
                            (dy > 0 ? TW_N : 0u);
      if ((tw & need) != need) continue;
    }
    add_cand(br, e, (int)(tile % (unsigned)br.tiles_x) + dx, (int)(tile / (unsigned)br.tiles_x) + dy);
  }
  // dry border strips (code 3) of the last step: one thread per tile.  With
  // no mass in its 3 x 3 neighbourhood the tile keeps its code, mask and
  // count (see mask_tile_skippable) and is carried to the next dry-border
  // list -- not when a neighbour dilates to every neighbour (tile_seed): it
  // is a candidate of this step then and must not be listed twice.  Else it
  // is its own candidate (it holds no mass, so it dilates only as a
  // tile_seed tile).
  const unsigned base = (n * 9u < G) ? n * 9u : 0u;
  for (unsigned k = (gt >= base) ? gt - base : gt + (G - base); k < nd; k += G) {
    const unsigned long long e = Ld[k];
    const int slot = entry_slot(e);
    const BatchRun& br = b.runs[slot];
    if (!br.live || (br.gen & 0xffffu) != entry_gen(e) || !running(br.st)) continue;
    const unsigned tile = entry_tile(e);
    const int tx0 = (int)(tile % (unsigned)br.tiles_x), ty0 = (int)(tile / (unsigned)br.tiles_x);
    bool keep = true;
    for (int yy = ty0 - 1; yy <= ty0 + 1 && keep; ++yy)
      for (int xx = tx0 - 1; xx <= tx0 + 1; ++xx) {
        if (xx < 0 || yy < 0 || xx >= br.tiles_x || yy >= br.tiles_y) continue;
        const int t3 = yy * br.tiles_x + xx;
        if ((br.tile_wet[t3] & TW_ANY) || (t3 != (int)tile && br.tile_seed[t3])) {
          keep = false;
          break;
        }
      }
    if (keep) {
      const unsigned pos = atomicAdd(&ctl->dcount[pp ^ 1u], 1u);
      Ldout[pos] = e;
      atomicAdd((unsigned long long*)&br.st->cells_acc[br.st->steps & 1], (unsigned long long)br.tile_count[tile]);
      atomicAdd(&br.st->border_acc[br.st->steps & 1], (unsigned long long)br.tile_count[tile]);
      continue;
    }
    if (br.tile_seed[tile]) {
      for (int nb = 0; nb < 9; ++nb) add_cand(br, e, tx0 + nb % 3 - 1, ty0 + nb / 3 - 1);
    } else {
      add_cand(br, e, tx0, ty0);
    }
  }
}

// check_solve reads a handful of the run's arguments (grid sizes, n_RK,
// the ring flag, four pointers), so they come straight from the argument
// table in global memory (L1-cached) instead of a shared-memory copy of the
// whole KArgs per run change: candidate lists interleave the runs' tiles.
// Compiled for 8 resident blocks per SM (32 x 8 tiles: 64 warps, the
// SM's limit): more candidate tiles' frame loads in flight; measured 9 %
// faster than the 6 blocks the registers allowed unbounded.
template <class R, int TH>
__global__ void __launch_bounds__(TileShape<TH>::MASK_THREADS, 2048 / TileShape<TH>::MASK_THREADS) k_b_mask(BatchArgs<R> b) {
  __shared__ unsigned s_idx[2];
  step_kernel_entry();
  BatchCtl* ctl = b.ctl;
  const unsigned pp = ctl->pp;
  unsigned long long* out = pp ? b.list0 : b.list1;
  unsigned long long* dout = pp ? b.dlist0 : b.dlist1;
  const unsigned n = ctl->ncand;
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->work[1] = 0u;
  TileQueue tq{&ctl->work[0], s_idx};
  for (unsigned i = tq.first(); i < n; i = tq.next()) {
    tq.prefetch();
    const unsigned long long e = b.cand[i];
    const int slot = entry_slot(e);
    const unsigned tile = entry_tile(e);
    const KArgs<R>& a = b.args[slot];
    const BatchRun& br = b.runs[slot];
    if (threadIdx.x == 0) br.cand[tile] = 0u;
    // k_b_cand listed only running runs, and no run's clock moves before k_b_dt
    const int tx = (int)(tile % (unsigned)br.tiles_x), ty = (int)(tile / (unsigned)br.tiles_x);
    int act = 0;
    const int code = mask_tile<R, TH>(a, 0, tx, ty, br.tiles_x, true, &act);
    if (code == 1) {
      // the tile into the active list, its active cells into the cell list
      // (one thread per cell of the tile: thread = row * 32 + column), one
      // atomic per warp holding active cells
      if (threadIdx.x == 0) {
        const unsigned pos = atomicAdd(&ctl->count[pp ^ 1u], 1u);
        out[pos] = e;
        a.tile_wet[tile] = 0;   // the stage kernel ORs the wet bits of the step in
      }
      const int lane = threadIdx.x % TX;
      const unsigned bal = __ballot_sync(0xffffffffu, act);
      if (bal) {
        const unsigned nw = __popc(bal);
        unsigned base = 0;
        if (lane == 0) {
          base = atomicAdd(&ctl->ncells, nw);
          if (base + nw > b.cells_cap) ctl->overflow = 1u;
        }
        base = __shfl_sync(0xffffffffu, base, 0);
        const unsigned idx = base + __popc(bal & ((1u << lane) - 1u));
        if (act && idx < b.cells_cap)
          b.cells[idx] = (e & 0xffff000000000000ull) | ((unsigned long long)tile << 9) | (unsigned)threadIdx.x;
      }
    } else if (code == TILE_DRY_BORDER && threadIdx.x == 0) {
      const unsigned pos = atomicAdd(&ctl->dcount[pp ^ 1u], 1u);
      dout[pos] = e;
      a.tile_wet[tile] = 0;   // dry; the stage kernel does not visit it
    } else if (code == 0 && threadIdx.x == 0) {
      a.tile_wet[tile] = 0;   // an inactive tile holds no mass
    }
  }
}

// 32 x 8 tiles: 4 blocks per SM (36 warps, 56 registers, a few spills):
// without the bound the persistent loop keeps loop-invariant values of the
// tile body live and needs ~120 registers; 4 blocks measured 4 % faster
// than 3 on the ensemble
template <class R, int NS, int LIM, int TH>
__global__ void __launch_bounds__(TileShape<TH>::FLUX_THREADS, TileShape<TH>::FLUX_MIN_BLOCKS)
    k_b_flux(BatchArgs<R> b) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(16) unsigned char sa_raw[sizeof(KArgs<R>)];
  __shared__ unsigned s_idx[2];
  step_kernel_entry();
  KArgs<R>& a = *reinterpret_cast<KArgs<R>*>(sa_raw);
  BatchCtl* ctl = b.ctl;
  const unsigned pp = ctl->pp;
  const unsigned long long* L = pp ? b.list0 : b.list1;
  const unsigned n = ctl->count[pp ^ 1u];
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->work[2] = 0u;
  int cur = -1;
  TileQueue tq{&ctl->work[1], s_idx};
  for (unsigned i = tq.first(); i < n; i = tq.next()) {
    tq.prefetch();
    const unsigned long long e = L[i];
    const int slot = entry_slot(e);
    const unsigned tile = entry_tile(e);
    if (slot != cur) {
      load_args(&a, &b.args[slot]);
      cur = slot;
      __syncthreads();
    }
    // the list holds tiles of running runs only (k_b_cand, k_b_mask)
    const int tiles_x = (a.g.nx + TX - 1) / TX;
    flux_tile<R, NS, LIM, TH>(a, a.q, a.rd, 1, (int)(tile % (unsigned)tiles_x), (int)(tile / (unsigned)tiles_x),
                     smem_raw);
  }
}


template <class R>
__global__ void __launch_bounds__(kBatchCandThreads) k_b_dt(BatchArgs<R> b) {
  step_kernel_entry();
  const unsigned gt = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned G = gridDim.x * blockDim.x;
  for (unsigned r = gt; r < (unsigned)b.max_runs; r += G) {
    const BatchRun& br = b.runs[r];
    if (br.live) dt_update(br.st, br.max_dt);
  }
  if (gt == 0) {
    BatchCtl* ctl = b.ctl;
    ctl->pp ^= 1u;
    // the next step's k_b_cand and k_b_mask append dry-border tiles to the
    // lists this step read (k_b_cand carries tiles there while it runs, so
    // the count is cleared here, not by it)
    ctl->dcount[ctl->pp ^ 1u] = 0u;
    ctl->ncand = 0u;
    ctl->steps += 1u;
  }
}

// One active cell per thread from the cell list (grid-stride; the warps'
// lanes are all active cells, whatever the tiles' density).  The cell's
// run arguments come straight from the argument table (L1-cached).  Each
// wet cell ORs its tile's wet bits (TW_*) in with one atomic on the word
// holding the tile's byte; the Newton counters are summed per run over the
// lanes of a warp that share it.
template <class R, int NS, int TH>
__global__ void __launch_bounds__(kBatchStageThreads, sizeof(R) == 4 ? 4 : 1) k_b_stage2(BatchArgs<R> b) {
  step_kernel_entry();
  BatchCtl* ctl = b.ctl;
  const unsigned n = min(ctl->ncells, b.cells_cap);
  const unsigned stride = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  for (unsigned i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < n; i0 += stride) {
    const unsigned i = i0 + lane;
    const bool have = i < n;
    int slot = -1, nit = 0;
    unsigned status = 0;
    if (have) {
      const unsigned long long ce = b.cells[i];
      slot = entry_slot(ce);
      const unsigned tile = (unsigned)((ce >> 9) & 0x7fffffffffull);
      const unsigned c = (unsigned)(ce & 511u);
      const KArgs<R>& a = b.args[slot];
      // a tile the flux kernel found dry (code 2) is left unchanged
      if (a.st->run_step && a.tile_active[tile] != 2) {
        const int cl = (int)(c & 511u) % TX, row = (int)(c & 511u) / TX;
        const int tiles_x = (a.g.nx + TX - 1) / TX;
        const int j = (int)(tile % (unsigned)tiles_x) * TX + cl, k = (int)(tile / (unsigned)tiles_x) * TH + row;
        if (stage2_cell<R, NS>(a, -1, j, k, status, nit)) {
          const unsigned bits = TW_ANY | (cl < 2 ? TW_W : 0u) | (cl >= TX - 2 ? TW_E : 0u) |
                                (row < 2 ? TW_S : 0u) | (row >= TH - 2 ? TW_N : 0u);
          uint8_t* wb = a.tile_wet + tile;
          unsigned* word = reinterpret_cast<unsigned*>(reinterpret_cast<uintptr_t>(wb) & ~(uintptr_t)3);
          atomicOr(word, bits << (8u * (unsigned)(reinterpret_cast<uintptr_t>(wb) & 3u)));
        }
      }
    }
    // Newton counters and status per run: the lanes of one run together
    const unsigned grp = __match_any_sync(0xffffffffu, slot);
    const int leader = __ffs(grp) - 1;
    int sum = 0, mx = 0;
    unsigned st_or = 0;
    for (unsigned m = grp; m; m &= m - 1u) {
      const int src = __ffs(m) - 1;
      sum += __shfl_sync(grp, nit, src);
      mx = max(mx, __shfl_sync(grp, nit, src));
      st_or |= __shfl_sync(grp, status, src);
    }
    if (lane == leader && slot >= 0) {
      RunState* st = b.args[slot].st;
      if (st_or) atomicOr(&st->status, st_or);
      if (sum > 0) {
        atomicAdd((unsigned long long*)&st->newton_iters, (unsigned long long)sum);
        atomicMax(&st->newton_max, mx);
      }
    }
  }
}

// all tiles of a newly admitted run into the list of the next k_b_cand
template <class R>
__global__ void __launch_bounds__(256) k_b_admit(BatchArgs<R> b, int slot, unsigned gen, unsigned ntiles) {
  __shared__ unsigned base;
  BatchCtl* ctl = b.ctl;
  const unsigned pp = ctl->pp;
  unsigned long long* L = pp ? b.list1 : b.list0;
  if (threadIdx.x == 0) base = atomicAdd(&ctl->count[pp], ntiles);
  __syncthreads();
  const unsigned long long hi = ((unsigned long long)(unsigned)slot << 48) |
                                ((unsigned long long)(gen & 0xffffu) << 32);
  for (unsigned t = threadIdx.x; t < ntiles; t += blockDim.x) L[base + t] = hi | t;
}

template <class R>
__global__ void __launch_bounds__(256) k_b_summary(BatchArgs<R> b) {
  const unsigned r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= (unsigned)b.max_runs) return;
  const BatchRun& br = b.runs[r];
  BatchSummary s;
  s.steps = 0;
  s.cells_total = 0;
  s.t = 0.0;
  s.status = 0u;
  s.running = 0;
  if (br.live) {
    const RunState* st = br.st;
    s.steps = st->steps;
    s.cells_total = st->cells_total;
    s.t = st->t;
    s.status = st->status;
    s.running = running(st) ? 1 : 0;
  }
  b.summary[r] = s;
}

}  // namespace sflow

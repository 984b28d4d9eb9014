// sflow_table_impl.cuh -- launch wrappers of the class-count-templated
// kernels; included by the sflow_k_*.cu translation units only.
#pragma once
#include "sflow_batch_kernels.cuh"
#include "sflow_kernels.cuh"
#include "sflow_table.h"

namespace sflow {

// qp of every cell (IMEX_SfloW2D.f90:449-505 values) in host layout
template <class R, int NS>
__global__ void k_qp_to_aos(KArgs<R> a, double* __restrict__ aos) {
  constexpr int nv = 4 + NS, np = nv + 2;
  const Grid<R>& g = a.g;
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)g.nx * g.ny) return;
  int j = (int)(c % g.nx), k = (int)(c / g.nx);
  int64_t d = cidx(g, j, k);
  R q[nv], qp[np];
  for (int i = 0; i < nv; ++i) q[i] = a.q[i * g.plane + d];
  if (q[0] > R(0)) qc_to_qp<R, NS>(a.pr, q, qp);
  else {
    for (int i = 0; i < np; ++i) qp[i] = R(0);
    qp[3] = a.pr.T_ambient;
  }
  for (int i = 0; i < np; ++i) aos[c * np + i] = (double)qp[i];
}

// per-cell physical fields of the .p_2d output (inpout_2d.f90:6150-6200):
// h, u, v, T, alphas (NS), rho_m, red_grav, Ri -- qc_to_qp and mixt_var of
// every cell, in host layout
template <class R, int NS>
__global__ void k_phys_to_aos(KArgs<R> a, double* __restrict__ aos) {
  constexpr int nv = 4 + NS, np = nv + 2, nf = 7 + NS;
  const Grid<R>& g = a.g;
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)g.nx * g.ny) return;
  int j = (int)(c % g.nx), k = (int)(c / g.nx);
  int64_t d = cidx(g, j, k);
  R q[nv], qp[np];
  for (int i = 0; i < nv; ++i) q[i] = a.q[i * g.plane + d];
  if (q[0] > R(0)) qc_to_qp<R, NS>(a.pr, q, qp);
  else {
    for (int i = 0; i < np; ++i) qp[i] = R(0);
    qp[3] = a.pr.T_ambient;
  }
  const Mixt<R> m = mixt_var<R, NS>(a.pr, qp, false);
  double* o = aos + c * nf;
  const R h = qp[0];
  o[0] = (double)h;
  o[1] = (double)qp[nv];
  o[2] = (double)qp[nv + 1];
  o[3] = (double)qp[3];
  for (int i = 0; i < NS; ++i) o[4 + i] = (h > R(0)) ? (double)(a.pr.alpha ? qp[4 + i] : qp[4 + i] / h) : 0.0;
  o[4 + NS] = (double)m.rho_m;
  o[5 + NS] = (double)m.red_grav;
  o[6 + NS] = (double)m.Ri;
}

// initial maxima after the initial check_solve(.TRUE.) (IMEX_SfloW2D.f90:307-368)
template <class R, int NS>
__global__ void k_init_maps(KArgs<R> a) {
  constexpr int nv = 4 + NS, np = nv + 2;
  const Grid<R>& g = a.g;
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)g.nx * g.ny) return;
  int j = (int)(c % g.nx), k = (int)(c / g.nx);
  int64_t d = cidx(g, j, k);
  R q[nv], qp[np];
  for (int i = 0; i < nv; ++i) q[i] = a.q[i * g.plane + d];
  R h = R(0), pd = R(0), mv = R(0);
  if (q[0] > R(0)) {
    R p_dyn = qc_to_qp<R, NS>(a.pr, q, qp);
    h = qp[0];
    if (qp[0] > a.pr.thr_1em3) {
      pd = p_dyn;
      mv = sqrt(sq(qp[nv]) + sq(qp[nv + 1]));
    }
  }
  a.hmax[d] = h;
  a.pdynmax[d] = pd;
  a.mvmax[d] = mv;
  if (a.vuln) {
    if (q[0] > R(0)) {
      const R p_dyn = qc_to_qp<R, NS>(a.pr, q, qp);
      vuln_update<R>(a, d, qp[0], p_dyn, false);
    } else {
      for (int w = 0; w < a.vuln_words; ++w) a.vuln[(int64_t)w * g.plane + d] = 0u;
    }
  }
}

// log-line sums over all cells (IMEX_SfloW2D.f90:535-542) in FP64 with a
// fixed reduction order: 4 values per block, then one block over blocks.
template <class R, int NS>
__global__ void k_stats_partial(KArgs<R> a, double* __restrict__ part) {
  constexpr int nv = 4 + NS, np = nv + 2;
  const Grid<R>& g = a.g;
  double v[4] = {0, 0, 0, 0}, cv[4] = {0, 0, 0, 0};
  const int64_t N = (int64_t)g.nx * g.ny;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < N;
       c += (int64_t)gridDim.x * blockDim.x) {
    int j = (int)(c % g.nx), k = (int)(c / g.nx);
    if (!owned_row(g, k)) continue;   // halo rows of a row slab
    int64_t d = cidx(g, j, k);
    R q[nv];
    for (int i = 0; i < nv; ++i) q[i] = a.q[i * g.plane + d];
    csum_add(v[0], cv[0], (double)q[0]);
    if (q[0] > R(0)) {
      R qp[np];
      qc_to_qp<R, NS>(a.pr, q, qp);
      csum_add(v[1], cv[1], (double)qp[0]);
    }
    if ((double)q[0] > 1.0e-7) v[2] += 1.0;
    for (int i = 0; i < NS; ++i) csum_add(v[3], cv[3], (double)q[4 + i]);
  }
  __shared__ double sh_s[4 * 256], sh_c[4 * 256];
  csum_block<4, 256>(v, cv, sh_s, sh_c, part + blockIdx.x * 4);
}


// ---- tile-height dependent entries (one translation unit per height) ----
// pointwise kernels of a single run: one block per 32 x 8 cells
static inline dim3 stage_grid(dim3 tiles, int ny) { return dim3(tiles.x, (unsigned)((ny + 7) / 8)); }

template <class R, int NS, int TH>
static cudaError_t tab_mask(const KArgs<R>& a, dim3 grid, cudaStream_t s, int solve_all) {
  return launch_step_kernel(k_mask<R, TH>, grid, dim3(TileShape<TH>::MASK_THREADS), 0, s, a.g.pdl, a, solve_all);
}
template <class R, int NS, int TH>
static cudaError_t tab_flux(const KArgs<R>& a, dim3 grid, size_t smem, cudaStream_t s, const R* qin,
                            R* rout, int want_dt) {
  // minmod everywhere (the reference default) has its own instantiation:
  // one limiter case instead of eight per variable keeps the code small
  const dim3 T(TileShape<TH>::FLUX_THREADS);
  if (a.g.lim_all == 1) return launch_step_kernel(k_flux<R, NS, 1, TH>, grid, T, smem, s, a.g.pdl, a, qin, rout, want_dt);
  return launch_step_kernel(k_flux<R, NS, -1, TH>, grid, T, smem, s, a.g.pdl, a, qin, rout, want_dt);
}
template <class R, int NS, int TH>
static cudaError_t tab_stage2(const KArgs<R>& a, dim3 grid, cudaStream_t s, int mode) {
  return launch_step_kernel(k_stage2<R, NS, TH>, stage_grid(grid, a.g.ny), dim3(TileShape<TH>::STAGE_THREADS), 0, s,
                            a.g.pdl, a, mode);
}
template <class R, int NS, int TH>
static cudaError_t tab_stage(const KArgs<R>& a, dim3 grid, cudaStream_t s, int irk) {
  return launch_step_kernel(k_stage<R, NS, TH>, stage_grid(grid, a.g.ny), dim3(TileShape<TH>::STAGE_THREADS), 0, s,
                            a.g.pdl, a, irk);
}
template <class R, int NS, int TH>
static cudaError_t tab_assemble(const KArgs<R>& a, dim3 grid, cudaStream_t s) {
  return launch_step_kernel(k_assemble<R, NS, TH>, stage_grid(grid, a.g.ny), dim3(TileShape<TH>::STAGE_THREADS), 0,
                            s, a.g.pdl, a);
}
template <class R, int NS, int TH>
static cudaError_t tab_smem(size_t bytes) {
  cudaError_t e = cudaFuncSetAttribute(k_flux<R, NS, 1, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_flux<R, NS, -1, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}
template <class R, int NS, int TH>
static cudaError_t tab_b_setup(size_t smem_flux, int* grids) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_b_flux<R, NS, 1, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_flux);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_b_flux<R, NS, -1, TH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_flux);
  if (e != cudaSuccess) return e;
  int occ[3] = {0, 0, 0};
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[0], k_b_mask<R, TH>, TileShape<TH>::MASK_THREADS, 0);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[1], k_b_flux<R, NS, -1, TH>, TileShape<TH>::FLUX_THREADS,
                                                    smem_flux);
  if (e != cudaSuccess) return e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ[2], k_b_stage2<R, NS, TH>, kBatchStageThreads, 0);
  if (e != cudaSuccess) return e;
  grids[0] = sms * 4;
  grids[1] = sms * (occ[0] > 0 ? occ[0] : 1);
  grids[2] = sms * (occ[1] > 0 ? occ[1] : 1);
  grids[3] = sms * (occ[2] > 0 ? occ[2] : 1);
  return cudaSuccess;
}
template <class R, int NS, int TH>
static cudaError_t tab_b_step(const BatchArgs<R>& b, cudaStream_t s, const int* grids, size_t smem_flux, int lim,
                              int pdl, cudaEvent_t* ev) {
  const dim3 T(TileShape<TH>::FLUX_THREADS);
  auto rec = [&](int i) -> cudaError_t { return ev ? cudaEventRecord(ev[i], s) : cudaSuccess; };
  cudaError_t e = rec(0);
  if (e == cudaSuccess) e = launch_step_kernel(k_b_cand<R>, dim3(grids[0]), dim3(kBatchCandThreads), 0, s, pdl, b);
  if (e == cudaSuccess) e = rec(1);
  if (e == cudaSuccess)
    e = launch_step_kernel(k_b_mask<R, TH>, dim3(grids[1]), dim3(TileShape<TH>::MASK_THREADS), 0, s, pdl, b);
  if (e == cudaSuccess) e = rec(2);
  if (e == cudaSuccess) {
    if (lim == 1) e = launch_step_kernel(k_b_flux<R, NS, 1, TH>, dim3(grids[2]), T, smem_flux, s, pdl, b);
    else e = launch_step_kernel(k_b_flux<R, NS, -1, TH>, dim3(grids[2]), T, smem_flux, s, pdl, b);
  }
  if (e == cudaSuccess) e = rec(3);
  if (e == cudaSuccess) e = launch_step_kernel(k_b_dt<R>, dim3(1), dim3(kBatchCandThreads), 0, s, pdl, b);
  if (e == cudaSuccess) e = rec(4);
  if (e == cudaSuccess)
    e = launch_step_kernel(k_b_stage2<R, NS, TH>, dim3(grids[3]), dim3(kBatchStageThreads), 0, s, pdl, b);
  if (e == cudaSuccess) e = rec(5);
  return e;
}

template <class R, int NS, int TH>
void fill_tile_entries(KernelTable<R>& t) {
  t.tile_h = TH;
  t.mask = &tab_mask<R, NS, TH>;
  t.flux = &tab_flux<R, NS, TH>;
  t.stage2 = &tab_stage2<R, NS, TH>;
  t.stage = &tab_stage<R, NS, TH>;
  t.assemble = &tab_assemble<R, NS, TH>;
  t.set_smem = &tab_smem<R, NS, TH>;
  t.b_setup = &tab_b_setup<R, NS, TH>;
  t.b_step = &tab_b_step<R, NS, TH>;
}

// ---- entries that do not depend on the tile height ----
template <class R, int NS>
static cudaError_t tab_init_maps(const KArgs<R>& a, unsigned blocks, cudaStream_t s) {
  k_init_maps<R, NS><<<blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}
template <class R, int NS>
static cudaError_t tab_qp(const KArgs<R>& a, unsigned blocks, cudaStream_t s, double* out) {
  k_qp_to_aos<R, NS><<<blocks, 256, 0, s>>>(a, out);
  return cudaGetLastError();
}
template <class R, int NS>
static cudaError_t tab_phys(const KArgs<R>& a, unsigned blocks, cudaStream_t s, double* out) {
  k_phys_to_aos<R, NS><<<blocks, 256, 0, s>>>(a, out);
  return cudaGetLastError();
}
template <class R, int NS>
static cudaError_t tab_stats(const KArgs<R>& a, int blocks, cudaStream_t s, double* part) {
  k_stats_partial<R, NS><<<blocks, 256, 0, s>>>(a, part);
  return cudaGetLastError();
}
template <class R, int NS>
static cudaError_t tab_b_admit(const BatchArgs<R>& b, cudaStream_t s, int slot, unsigned gen, unsigned ntiles) {
  k_b_admit<R><<<1, 256, 0, s>>>(b, slot, gen, ntiles);
  return cudaGetLastError();
}
template <class R, int NS>
static cudaError_t tab_b_summary(const BatchArgs<R>& b, cudaStream_t s) {
  k_b_summary<R><<<(b.max_runs + 255) / 256, 256, 0, s>>>(b);
  return cudaGetLastError();
}

template <class R, int NS>
KernelTable<R> make_table() {
  KernelTable<R> t;
  t.init_maps = &tab_init_maps<R, NS>;
  t.qp = &tab_qp<R, NS>;
  t.phys = &tab_phys<R, NS>;
  t.stats = &tab_stats<R, NS>;
  t.b_admit = &tab_b_admit<R, NS>;
  t.b_summary = &tab_b_summary<R, NS>;
  return t;
}

}  // namespace sflow

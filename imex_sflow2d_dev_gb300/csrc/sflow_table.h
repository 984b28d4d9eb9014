// sflow_table.h -- per-(precision, solid-class count, tile height) kernel
// entry points.  The class count is a compile-time parameter of the heavy
// kernels so their per-variable arrays stay in registers, and the tile
// height (cells per tile column) one of every tiled kernel; each
// (precision, count, height) triple is its own translation unit
// (sflow_k_*.cu) so the build parallelises.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

#include "sflow_types.cuh"

namespace sflow {

template <class R>
struct KArgs;
template <class R>
struct BatchArgs;

template <class R>
struct KernelTable {
  int tile_h = 0;   // tile height of the tiled entries
  cudaError_t (*mask)(const KArgs<R>&, dim3, cudaStream_t, int) = nullptr;
  cudaError_t (*flux)(const KArgs<R>&, dim3, size_t, cudaStream_t, const R*, R*, int) = nullptr;
  cudaError_t (*stage2)(const KArgs<R>&, dim3, cudaStream_t, int) = nullptr;
  cudaError_t (*stage)(const KArgs<R>&, dim3, cudaStream_t, int) = nullptr;
  cudaError_t (*assemble)(const KArgs<R>&, dim3, cudaStream_t) = nullptr;
  cudaError_t (*init_maps)(const KArgs<R>&, unsigned, cudaStream_t) = nullptr;
  cudaError_t (*qp)(const KArgs<R>&, unsigned, cudaStream_t, double*) = nullptr;
  cudaError_t (*phys)(const KArgs<R>&, unsigned, cudaStream_t, double*) = nullptr;
  cudaError_t (*stats)(const KArgs<R>&, int, cudaStream_t, double*) = nullptr;
  cudaError_t (*set_smem)(size_t) = nullptr;
  // batched runs (sflow_batch_kernels.cuh): grids[4] = persistent grid sizes
  // of k_b_cand / k_b_mask / k_b_flux / k_b_stage2 for this device
  cudaError_t (*b_setup)(size_t smem_flux, int* grids) = nullptr;
  // lim = 1: every run of the group uses minmod for every variable
  // pdl: launch with programmatic dependent launch; ev: NULL, or 6 events
  // recorded before, between and after the five kernels
  cudaError_t (*b_step)(const BatchArgs<R>&, cudaStream_t, const int* grids, size_t smem_flux, int lim,
                        int pdl, cudaEvent_t* ev) = nullptr;
  cudaError_t (*b_admit)(const BatchArgs<R>&, cudaStream_t, int slot, unsigned gen, unsigned ntiles) = nullptr;
  cudaError_t (*b_summary)(const BatchArgs<R>&, cudaStream_t) = nullptr;
};

template <class R, int NS>
KernelTable<R> make_table();
template <class R, int NS, int TH>
void fill_tile_entries(KernelTable<R>& t);

// solid-class counts with compiled kernels
constexpr int kMinSolidBuilt = 1;
constexpr int kMaxSolidBuilt = 3;

// tile heights the autotuner tries, and those with compiled kernels: 8, 16
// and 4 for the FP32 bulk form, 8 for the FP64 plain form
constexpr int kTileCandidates = 3;
constexpr int kTileCandidate[kTileCandidates] = {8, 16, 4};
template <class R>
inline bool tile_h_built(int th) {
  return th == 8 || (std::is_same<R, float>::value && (th == 16 || th == 4));
}

template <class R, int NS>
inline void fill_tiles(KernelTable<R>& t, int th) {
  if (th == 8) fill_tile_entries<R, NS, 8>(t);
  if constexpr (std::is_same<R, float>::value) {
    if (th == 16) fill_tile_entries<R, NS, 16>(t);
    if (th == 4) fill_tile_entries<R, NS, 4>(t);
  }
}

// the table of (ns, th); entries are null when either has no kernels
template <class R>
inline KernelTable<R> kernel_table(int ns, int th) {
  KernelTable<R> t;
  if (!tile_h_built<R>(th)) return t;
  switch (ns) {
    case 1: t = make_table<R, 1>(); fill_tiles<R, 1>(t, th); break;
    case 2: t = make_table<R, 2>(); fill_tiles<R, 2>(t, th); break;
    case 3: t = make_table<R, 3>(); fill_tiles<R, 3>(t, th); break;
  }
  return t;
}

}  // namespace sflow

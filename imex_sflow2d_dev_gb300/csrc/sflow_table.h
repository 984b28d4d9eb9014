// sflow_table.h -- per-(precision, solid-class count) kernel entry points.
// The class count is a compile-time parameter of the heavy kernels so their
// per-variable arrays stay in registers; each (precision, count) pair is its
// own translation unit (sflow_k_*.cu) so the build parallelises.
#pragma once
#include <cuda_runtime.h>

#include "sflow_types.cuh"

namespace sflow {

template <class R>
struct KArgs;
template <class R>
struct BatchArgs;

template <class R>
struct KernelTable {
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
  cudaError_t (*b_step)(const BatchArgs<R>&, cudaStream_t, const int* grids, size_t smem_flux, int lim) = nullptr;
  cudaError_t (*b_admit)(const BatchArgs<R>&, cudaStream_t, int slot, unsigned gen, unsigned ntiles) = nullptr;
  cudaError_t (*b_summary)(const BatchArgs<R>&, cudaStream_t) = nullptr;
};

template <class R, int NS>
KernelTable<R> make_table();

// solid-class counts with compiled kernels
constexpr int kMinSolidBuilt = 1;
constexpr int kMaxSolidBuilt = 3;

template <class R>
inline KernelTable<R> kernel_table(int ns) {
  switch (ns) {
    case 1: return make_table<R, 1>();
    case 2: return make_table<R, 2>();
    case 3: return make_table<R, 3>();
  }
  return KernelTable<R>();
}

}  // namespace sflow

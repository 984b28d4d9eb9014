// sflow_noalloc.cu -- the driver's log-line sums (mass, volume, wet area,
// solid mass) of a state that already sits in device memory, computed
// without allocating anything.
//
// Who needs it: a host that cannot call cudaMalloc at the point where it
// wants the sums -- code running while a CUDA graph is being captured (an
// allocation is not a capturable operation), code that runs inside a
// stream callback or a host node (no CUDA API calls allowed there), or a
// host framework that owns all device memory through its own pool and
// forbids raw allocations.  Such a caller hands over a device pointer to its
// own copy of q and a device pointer for the 4 results.
//
// The per-block partial sums that sflow_get_stats keeps in memory it
// allocates live here in one file-scope device array of fixed size.  That
// array is part of the library image: every GPU that loads the library
// holds its 128 KiB until the process exits.  All calls share it; it keeps
// the last call's contents (every entry a call reads is first written by
// the same call).  Two calls whose kernels overlap on the GPU (different
// streams, no ordering between them) race on the array and may return wrong
// sums; calls on one stream are ordered and safe.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/sflow.h"
#include "sflow_physics.cuh"

namespace sflow {
namespace {

constexpr int kThreads = 256;
constexpr int64_t kCellsPerBlock = 16384;          // 64 cells per thread
constexpr int kMaxBlocks = 4096;
constexpr int64_t kMaxCells = kCellsPerBlock * kMaxBlocks;   // 67,108,864 = 8192^2

// the scratch: 4 partial sums per block, FP64
static __device__ __align__(256) double g_partials[kMaxBlocks * 4];

template <int NS>
__global__ void __launch_bounds__(kThreads) k_sums_partial(Phys<double> P,
                                                           const double* __restrict__ q,
                                                           int64_t ncells, double* __restrict__ part) {
  constexpr int nv = 4 + NS;
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  const int64_t c0 = (int64_t)blockIdx.x * kCellsPerBlock;
  const int64_t c1 = (c0 + kCellsPerBlock < ncells) ? c0 + kCellsPerBlock : ncells;
  for (int64_t c = c0 + threadIdx.x; c < c1; c += kThreads) {
    double qc[nv], qp[nv + 2];
#pragma unroll
    for (int i = 0; i < nv; ++i) qc[i] = q[c * nv + i];
    v[0] += qc[0];
    if (qc[0] > 0.0) {
      qc_to_qp<double, NS>(P, qc, qp);
      v[1] += qp[0];
    }
    if (qc[0] > 1.0e-7) v[2] += 1.0;
#pragma unroll
    for (int i = 0; i < NS; ++i) v[3] += qc[4 + i];
  }
  __shared__ double sh[4][kThreads];
  for (int m = 0; m < 4; ++m) sh[m][threadIdx.x] = v[m];
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int m = 0; m < 4; ++m) sh[m][threadIdx.x] += sh[m][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int m = 0; m < 4; ++m) part[blockIdx.x * 4 + m] = sh[m][0];
}

__global__ void __launch_bounds__(kThreads) k_sums_final(const double* __restrict__ part, int nblk,
                                                         double area, double* __restrict__ out) {
  const int m = blockIdx.x;
  double s = 0.0, cmp = 0.0;
  for (int b = threadIdx.x; b < nblk; b += kThreads) {
    const double x = part[b * 4 + m];
    const double t = s + x;
    if (fabs(s) >= fabs(x)) cmp += (s - t) + x;
    else cmp += (x - t) + s;
    s = t;
  }
  __shared__ double sh[kThreads];
  sh[threadIdx.x] = s + cmp;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[m] = area * sh[0];
}

// device address of g_partials, looked up once per device
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_partials_addr[kMaxDevices] = {nullptr};

thread_local char g_na_err[256] = "";

int na_fail(int code, const char* msg) {
  std::snprintf(g_na_err, sizeof(g_na_err), "%s", msg);
  return code;
}

}  // namespace
}  // namespace sflow

extern "C" const char* sflow_log_sums_noalloc_error(void) { return sflow::g_na_err; }

extern "C" int sflow_log_sums_noalloc(const SflowParams* p, const double* q_dev, double* sums_dev,
                                      void* stream) {
  using namespace sflow;
  if (!p || !q_dev || !sums_dev) return na_fail(SFLOW_EINVAL, "NULL argument");
  if (p->abi_version != SFLOW_ABI_VERSION) return na_fail(SFLOW_EINVAL, "abi_version mismatch");
  if (p->n_solid < 1 || p->n_solid > 3)
    return na_fail(SFLOW_EINVAL, "n_solid must be 1, 2 or 3");
  if (p->comp_cells_x < 1 || p->comp_cells_y < 1) return na_fail(SFLOW_EINVAL, "empty domain");
  if (p->gas_flag == p->liquid_flag) return na_fail(SFLOW_EINVAL, "exactly one of gas_flag / liquid_flag");
  const int64_t ncells = (int64_t)p->comp_cells_x * p->comp_cells_y;
  if (ncells > kMaxCells)
    return na_fail(SFLOW_ERANGE,
                   "domain larger than the fixed scratch allows (at most 67,108,864 cells, 8192 x 8192)");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return na_fail(SFLOW_ECUDA, "no current CUDA device");
  double* part = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partials_addr[dev]) {
      void* ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&ptr, g_partials);
      if (e != cudaSuccess || !ptr) return na_fail(SFLOW_ECUDA, cudaGetErrorString(e));
      g_partials_addr[dev] = static_cast<double*>(ptr);
    }
    part = g_partials_addr[dev];
  }
  // FP64 constants of qc_to_qp (constitutive_2d.f90:550-976, 1637-1690)
  Phys<double> P;
  std::memset(&P, 0, sizeof(P));
  const int ns = p->n_solid;
  P.ns = ns;
  P.nv = 4 + ns;
  P.gas = p->gas_flag;
  P.liquid = p->liquid_flag;
  P.energy = p->energy_flag;
  P.alpha = p->alpha_flag;
  const double dx = p->comp_cells_x > 1 ? p->cell_size : 1.0;
  const double dy = p->comp_cells_y > 1 ? p->cell_size : 1.0;
  const double eps_sing = std::fmin(std::fmin(std::pow(dx, 4.0), std::pow(dy, 4.0)), 1.0e-10);
  P.eps_sing_d = eps_sing;
  P.thr_eps = DBL_EPSILON;
  P.thr_eps_sing = eps_sing;
  P.eps_sing4 = (eps_sing * eps_sing) * (eps_sing * eps_sing);
  P.inv_eps_sing = 1.0 / eps_sing;
  P.sqrt2 = std::sqrt(2.0);
  P.T_ambient = p->T_ambient;
  P.sp_heat_a = p->sp_heat_a;
  P.sp_heat_l = p->sp_heat_l;
  P.sp_gas_const_a = p->sp_gas_const_a;
  P.inv_pres = p->pres > 0.0 ? 1.0 / p->pres : 0.0;
  P.inv_rho_l = p->rho_l > 0.0 ? 1.0 / p->rho_l : 0.0;
  for (int i = 0; i < ns; ++i) {
    P.sp_heat_s[i] = p->sp_heat_s[i];
    P.inv_rho_s[i] = p->rho_s[i] > 0.0 ? 1.0 / p->rho_s[i] : 0.0;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nblk = (int)((ncells + kCellsPerBlock - 1) / kCellsPerBlock);
  switch (ns) {
    case 1: k_sums_partial<1><<<nblk, kThreads, 0, s>>>(P, q_dev, ncells, part); break;
    case 2: k_sums_partial<2><<<nblk, kThreads, 0, s>>>(P, q_dev, ncells, part); break;
    default: k_sums_partial<3><<<nblk, kThreads, 0, s>>>(P, q_dev, ncells, part); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return na_fail(SFLOW_ECUDA, cudaGetErrorString(e));
  k_sums_final<<<4, kThreads, 0, s>>>(part, nblk, dx * dy, sums_dev);
  e = cudaGetLastError();
  if (e != cudaSuccess) return na_fail(SFLOW_ECUDA, cudaGetErrorString(e));
  return SFLOW_OK;
}

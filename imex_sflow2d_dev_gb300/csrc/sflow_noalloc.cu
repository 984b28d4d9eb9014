// sflow_noalloc.cu -- the driver's log-line sums (mass, volume, wet area,
// solid mass) of a state that already sits in device memory, computed
// without allocating anything.
//
// Who needs it: a host that cannot call cudaMalloc where it wants the sums,
// typically a host framework that owns all device memory through its own
// pool or a fixed arena and forbids raw allocations by the libraries it
// loads (an allocation there would also synchronise the device).  Such a
// caller hands over a device pointer to its own copy of q and a device
// pointer for the 4 results, and calls from ordinary host code.
//
// The per-block partial sums that sflow_get_stats keeps in memory it
// allocates live here in one file-scope device array of fixed size.  That
// array is part of the library image: every GPU that loads the library
// holds its 128 KiB until the process exits.  Host code cannot pass the
// array's name to a kernel (on the host it names a host-side stand-in, not
// device memory): its device address is looked up once per device with
// cudaGetSymbolAddress, with that device current, on the first call there.
// All calls share the array; it keeps the last call's contents, and every
// entry a call reads is first written by the same call.  Two calls whose
// kernels overlap on the GPU (different streams, no ordering between them)
// race on the array and may return wrong sums; calls on one stream are
// ordered and safe.
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/sflow.h"
#include "sflow_physics.cuh"
#include "sflow_sum.cuh"

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
  double v[4] = {0.0, 0.0, 0.0, 0.0}, cv[4] = {0.0, 0.0, 0.0, 0.0};
  const int64_t c0 = (int64_t)blockIdx.x * kCellsPerBlock;
  const int64_t c1 = (c0 + kCellsPerBlock < ncells) ? c0 + kCellsPerBlock : ncells;
  for (int64_t c = c0 + threadIdx.x; c < c1; c += kThreads) {
    double qc[nv], qp[nv + 2];
#pragma unroll
    for (int i = 0; i < nv; ++i) qc[i] = q[c * nv + i];
    csum_add(v[0], cv[0], qc[0]);
    if (qc[0] > 0.0) {
      qc_to_qp<double, NS>(P, qc, qp);
      csum_add(v[1], cv[1], qp[0]);
    }
    if (qc[0] > 1.0e-7) v[2] += 1.0;
#pragma unroll
    for (int i = 0; i < NS; ++i) csum_add(v[3], cv[3], qc[4 + i]);
  }
  __shared__ double sh_s[4 * kThreads], sh_c[4 * kThreads];
  csum_block<4, kThreads>(v, cv, sh_s, sh_c, part + blockIdx.x * 4);
}

__global__ void __launch_bounds__(kThreads) k_sums_final(const double* __restrict__ part, int nblk,
                                                         double area, double* __restrict__ out) {
  const int m = blockIdx.x;
  double s[1] = {0.0}, cmp[1] = {0.0}, r[1];
  for (int b = threadIdx.x; b < nblk; b += kThreads) csum_add(s[0], cmp[0], part[b * 4 + m]);
  __shared__ double sh_s[kThreads], sh_c[kThreads];
  csum_block<1, kThreads>(s, cmp, sh_s, sh_c, r);
  if (threadIdx.x == 0) out[m] = area * r[0];
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
  g_na_err[0] = '\0';
  if (!p || !q_dev || !sums_dev) return na_fail(SFLOW_EINVAL, "NULL argument");
  if (p->abi_version != SFLOW_ABI_VERSION) return na_fail(SFLOW_EINVAL, "abi_version mismatch");
  if (p->n_solid < 1 || p->n_solid > 3)
    return na_fail(SFLOW_EINVAL, "n_solid must be 1, 2 or 3");
  // the domain and closure constants sflow_create accepts (sflow_setup.cpp)
  if (p->comp_cells_x < 5 || (p->comp_cells_y < 5 && p->comp_cells_y != 1))
    return na_fail(SFLOW_EINVAL, "comp_cells_x must be >= 5 and comp_cells_y 1 or >= 5");
  if (p->gas_flag && p->liquid_flag) return na_fail(SFLOW_EINVAL, "gas carrier with a liquid phase is not supported");
  if (!p->gas_flag && !p->liquid_flag) return na_fail(SFLOW_EINVAL, "one of gas_flag / liquid_flag must be set");
  if (!(p->cell_size > 0.0)) return na_fail(SFLOW_EINVAL, "cell_size must be > 0");
  if (!(p->pres > 0.0) || !(p->sp_gas_const_a > 0.0) || !(p->T_ambient > 0.0))
    return na_fail(SFLOW_EINVAL, "pres, sp_gas_const_a, T_ambient must be > 0");
  if (p->liquid_flag && !(p->rho_l > 0.0)) return na_fail(SFLOW_EINVAL, "rho_l must be > 0");
  for (int i = 0; i < p->n_solid; ++i)
    if (!(p->rho_s[i] > 0.0)) return na_fail(SFLOW_EINVAL, "rho_s must be > 0");
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
  P.inv_pres = 1.0 / p->pres;
  P.inv_rho_l = p->liquid_flag ? 1.0 / p->rho_l : 0.0;
  for (int i = 0; i < ns; ++i) {
    P.sp_heat_s[i] = p->sp_heat_s[i];
    P.inv_rho_s[i] = 1.0 / p->rho_s[i];
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

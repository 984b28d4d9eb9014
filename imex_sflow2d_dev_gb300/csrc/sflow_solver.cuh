// sflow_solver.cuh -- device-resident solver of one domain, templated on the
// bulk arithmetic type (double: plain FP64 form, float: FP32 bulk form).
// Included by sflow_fp64.cu and sflow_fp32.cu only.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sflow_host.h"
#include "sflow_kernels.cuh"
#include "sflow_table.h"

namespace sflow {

// ---------------------------------------------------------------------------
// layout kernels: host layout q(1:n,1:nx,1:ny) (variable fastest) <-> planes
// ---------------------------------------------------------------------------
template <class R>
__global__ void k_aos_to_planes(const double* __restrict__ aos, R* __restrict__ q, int nv, int nx,
                                int ny, int pitch, int64_t plane) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)nx * ny) return;
  int j = (int)(c % nx), k = (int)(c / nx);
  for (int i = 0; i < nv; ++i) q[i * plane + (int64_t)k * pitch + j] = (R)aos[c * nv + i];
}

template <class R>
__global__ void k_planes_to_aos(const R* __restrict__ q, double* __restrict__ aos, int nv, int nx,
                                int ny, int pitch, int64_t plane) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)nx * ny) return;
  int j = (int)(c % nx), k = (int)(c / nx);
  for (int i = 0; i < nv; ++i) aos[c * nv + i] = (double)q[i * plane + (int64_t)k * pitch + j];
}

// The same through host memory mapped into the device address space (read
// or written over NVLink-C2C): a block moves 256 cells of the host layout
// as one contiguous run of doubles (coalesced, every cache line used once)
// through shared memory, then converts cell by cell.
constexpr int kHostChunk = 256;
template <class R>
__global__ void __launch_bounds__(kHostChunk) k_host_aos_to_planes(const double* __restrict__ aos, R* __restrict__ q,
                                                                   int nv, int nx, int ny, int pitch, int64_t plane) {
  extern __shared__ double sbuf[];
  const int64_t N = (int64_t)nx * ny;
  const int64_t c0 = (int64_t)blockIdx.x * kHostChunk;
  const int ncell = (int)((N - c0) < kHostChunk ? (N - c0) : kHostChunk);
  const int nval = ncell * nv;
  for (int i = threadIdx.x; i < nval; i += kHostChunk) sbuf[i] = aos[c0 * nv + i];
  __syncthreads();
  if (threadIdx.x < ncell) {
    const int64_t c = c0 + threadIdx.x;
    const int j = (int)(c % nx), k = (int)(c / nx);
    for (int i = 0; i < nv; ++i) q[i * plane + (int64_t)k * pitch + j] = (R)sbuf[threadIdx.x * nv + i];
  }
}
template <class R>
__global__ void __launch_bounds__(kHostChunk) k_host_planes_to_aos(const R* __restrict__ q, double* __restrict__ aos,
                                                                   int nv, int nx, int ny, int pitch, int64_t plane) {
  extern __shared__ double sbuf[];
  const int64_t N = (int64_t)nx * ny;
  const int64_t c0 = (int64_t)blockIdx.x * kHostChunk;
  const int ncell = (int)((N - c0) < kHostChunk ? (N - c0) : kHostChunk);
  if (threadIdx.x < ncell) {
    const int64_t c = c0 + threadIdx.x;
    const int j = (int)(c % nx), k = (int)(c / nx);
    for (int i = 0; i < nv; ++i) sbuf[threadIdx.x * nv + i] = (double)q[i * plane + (int64_t)k * pitch + j];
  }
  __syncthreads();
  const int nval = ncell * nv;
  for (int i = threadIdx.x; i < nval; i += kHostChunk) aos[c0 * nv + i] = sbuf[i];
}

// One FP64 plane of the host layout (nx x ny, row-major) into a pitched
// device plane of R, the pad columns zeroed; `src` is host memory the device
// reads directly (pageable memory on a system with pageable access, or
// mapped pinned memory) or a device buffer.
template <class R>
__global__ void k_plane_to_pitched(const double* __restrict__ src, R* __restrict__ dst, int nx, int ny, int pitch) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)pitch * ny) return;
  const int j = (int)(c % pitch), k = (int)(c / pitch);
  dst[c] = (j < nx) ? (R)src[(int64_t)k * nx + j] : R(0);
}

// The same for a byte plane (the cell flags).
static __global__ void k_bytes_to_pitched(const uint8_t* __restrict__ src, uint8_t* __restrict__ dst, int nx, int ny,
                                          int pitch) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)pitch * ny) return;
  const int j = (int)(c % pitch), k = (int)(c / pitch);
  dst[c] = (j < nx) ? src[(int64_t)k * nx + j] : (uint8_t)0;
}

// Whether kernels on `dev` may read and write pageable host memory (a
// Grace-Blackwell node with address translation services); queried once
// per device.  SFLOW_HOST_READS=0 in the environment turns the direct
// reads off (uploads then go through the staging buffer).
inline bool pageable_access(int dev) {
  static std::atomic<int> cached[64];   // 0 unknown, 1 no, 2 yes (any thread)
  if (dev < 0 || dev >= 64) return false;
  const char* env = std::getenv("SFLOW_HOST_READS");
  if (env && env[0] == '0') return false;
  int c = cached[dev].load(std::memory_order_relaxed);
  if (!c) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
      cudaGetLastError();
      v = 0;
    }
    c = v ? 2 : 1;
    cached[dev].store(c, std::memory_order_relaxed);
  }
  return c == 2;
}
inline bool pageable_access() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return pageable_access(dev);
}

template <class R>
__global__ void k_map_to_host(const R* __restrict__ m, double* __restrict__ out, int nx, int ny,
                              int pitch) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= (int64_t)nx * ny) return;
  int j = (int)(c % nx), k = (int)(c / nx);
  out[c] = (double)m[(int64_t)k * pitch + j];
}

static __global__ void k_stats_final(const double* __restrict__ part, int nblk, double* __restrict__ out) {
  // block m reduces value m: Neumaier-compensated strided sums per thread,
  // then a fixed-order compensated tree (deterministic)
  const int m = blockIdx.x;
  double s[1] = {0.0}, cmp[1] = {0.0};
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) csum_add(s[0], cmp[0], part[b * 4 + m]);
  __shared__ double sh_s[256], sh_c[256];
  csum_block<1, 256>(s, cmp, sh_s, sh_c, out + m);
}

// ---------------------------------------------------------------------------
// host driver of one domain
// ---------------------------------------------------------------------------
#define SFLOW_CU(call)                                                        \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) {                                                  \
      err_ = std::string(#call) + ": " + cudaGetErrorString(e_);              \
      return SFLOW_ECUDA;                                                     \
    }                                                                         \
  } while (0)

template <class R>
class Solver : public SolverBase {
 public:
  explicit Solver(const HostSetup& s, int tile_h = kTileHDefault) : hs_(s), tile_h_(tile_h) {
    tab_ = kernel_table<R>(hs_.ns, tile_h);
  }
  // takes the set-up's host arrays over instead of copying them
  explicit Solver(HostSetup&& s, int tile_h) : hs_(std::move(s)), tile_h_(tile_h) {
    tab_ = kernel_table<R>(hs_.ns, tile_h);
  }
  ~Solver() override { release(); }

  std::string err_;

  int init() {
    if (!tab_.flux) { err_ = "no kernels built for this number of solid classes and tile height"; return SFLOW_EINVAL; }
    const int nx = hs_.nx, ny = hs_.ny, nv = hs_.nv;
    pitch_ = (nx + 31) / 32 * 32;
    plane_ = (int64_t)pitch_ * ny;
    tiles_x_ = (nx + TX - 1) / TX;
    tiles_y_ = (ny + tile_h_ - 1) / tile_h_;
    SFLOW_CU(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    // one allocation for the buffers below (alloc() carves it; anything it
    // cannot hold gets its own cudaMalloc)
    arena_cap_ = init_bytes();
    if (cudaMalloc((void**)&arena_, arena_cap_) != cudaSuccess) {
      cudaGetLastError();
      arena_ = nullptr;
      arena_cap_ = 0;
    }
    arena_used_ = 0;
    SFLOW_CU(alloc((void**)&q_, sizeof(R) * plane_ * nv));
    const int nstage = (hs_.nrk == 2) ? 1 : hs_.nrk;
    SFLOW_CU(alloc((void**)&rd_, sizeof(R) * plane_ * nv * nstage));
    if (hs_.nrk != 2) {
      SFLOW_CU(alloc((void**)&rn_, sizeof(R) * plane_ * nv * nstage));
      SFLOW_CU(cudaMemset(rn_, 0, sizeof(R) * plane_ * nv * nstage));
      SFLOW_CU(alloc((void**)&qs_, sizeof(R) * plane_ * nv));
      SFLOW_CU(cudaMemset(qs_, 0, sizeof(R) * plane_ * nv));
    }
    for (int i = 0; i < 8; ++i) geo_[i] = nullptr;
    const std::vector<double>* gsrc[8] = {&hs_.Bx, &hs_.By, &hs_.Bxx, &hs_.Bxy, &hs_.Byy, &hs_.gc, &hs_.dgcx, &hs_.dgcy};
    const bool device_topo = hs_.Bx.empty();
    for (int i = 0; i < 8; ++i) {
      if ((i >= 2 && i <= 4) && !hs_.p.curvature_term_flag) continue;
      SFLOW_CU(alloc((void**)&geo_[i], sizeof(R) * plane_));
      if (!device_topo) SFLOW_CU(put_plane(geo_[i], *gsrc[i]));
    }
    if (device_topo) {
      // B (pitched FP64) in the stage-residual buffer, which is cleared
      // right after: sizeof(R) * nv >= 8 bytes per cell
      if (hs_.B.size() != (size_t)nx * ny) { err_ = "set-up without topography"; return SFLOW_EINVAL; }
      double* Bp = reinterpret_cast<double*>(rd_);
      if (pageable_access()) {
        k_plane_to_pitched<double><<<(unsigned)(((size_t)plane_ + 255) / 256), 256, 0, stream_>>>(
            hs_.B.data(), Bp, nx, ny, pitch_);
        ++launches_;
        SFLOW_CU(cudaGetLastError());
      } else {
        SFLOW_CU(cudaMemcpy2DAsync(Bp, sizeof(double) * pitch_, hs_.B.data(), sizeof(double) * nx,
                                   sizeof(double) * nx, ny, cudaMemcpyHostToDevice, stream_));
      }
      TopoPlanes<R> tp;
      for (int i = 0; i < 8; ++i) tp.p[i] = geo_[i];
      const int64_t n = (int64_t)nx * ny;
      k_topography_setup<R><<<(unsigned)((n + 255) / 256), 256, 0, stream_>>>(
          Bp, nx, ny, (int64_t)pitch_, hs_.dx, hs_.dy, hs_.p.slope_correction_flag ? 1 : 0, tp);
      ++launches_;
      SFLOW_CU(cudaGetLastError());
    }
    SFLOW_CU(cudaMemsetAsync(rd_, 0, sizeof(R) * plane_ * nv * nstage, stream_));
    SFLOW_CU(alloc((void**)&cflags_, plane_));
    SFLOW_CU(put_flags());
    SFLOW_CU(alloc((void**)&arc_, sizeof(R) * plane_ * 3));
    SFLOW_CU(put_plane(arc_, hs_.arc_perim));
    SFLOW_CU(put_plane(arc_ + plane_, hs_.arc_nx));
    SFLOW_CU(put_plane(arc_ + 2 * plane_, hs_.arc_ny));
    SFLOW_CU(alloc((void**)&mask_, plane_));
    SFLOW_CU(cudaMemset(mask_, 0, plane_));
    SFLOW_CU(alloc_tiles());
    SFLOW_CU(alloc((void**)&hmax_, sizeof(R) * plane_));
    SFLOW_CU(alloc((void**)&pdynmax_, sizeof(R) * plane_));
    SFLOW_CU(alloc((void**)&mvmax_, sizeof(R) * plane_));
    if (hs_.exchange) {
      SFLOW_CU(alloc((void**)&deposit_, sizeof(double) * plane_ * hs_.ns));
      SFLOW_CU(cudaMemset(deposit_, 0, sizeof(double) * plane_ * hs_.ns));
    }
    if (hs_.p.erosion_coeff > 0.0 || (hs_.p.erodible_deposit_flag && hs_.exchange)) {
      // erosion, or deposits that build the erodible layer
      SFLOW_CU(alloc((void**)&erosion_, sizeof(double) * plane_ * hs_.ns));
      SFLOW_CU(alloc((void**)&erodible_, sizeof(double) * plane_ * hs_.ns));
      SFLOW_CU(reset_erosion());
    }
    if (hs_.p.topo_change_flag && hs_.exchange) {
      SFLOW_CU(alloc((void**)&Bc_, sizeof(double) * plane_));
      SFLOW_CU(put_plane_d(Bc_, hs_.B));
    }
    if (hs_.p.bottom_radial_source_flag) {
      SFLOW_CU(alloc((void**)&bfrac_, sizeof(R) * plane_));
      SFLOW_CU(put_plane(bfrac_, hs_.cell_fract));
      std::vector<double> tab(1 + 2 * (size_t)SFLOW_MAX_INTERVALS, 0.0);
      tab[0] = (double)hs_.p.n_intervals;
      for (int i = 0; i < hs_.p.n_intervals; ++i) {
        tab[1 + i] = hs_.p.t_intervals[i];
        tab[1 + hs_.p.n_intervals + i] = hs_.p.vel_intervals[i];
      }
      SFLOW_CU(alloc((void**)&bsrc_tab_, sizeof(double) * tab.size()));
      SFLOW_CU(cudaMemcpy(bsrc_tab_, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice));
    }
    if (hs_.n_thk * hs_.n_dyn > 0) {
      vuln_words_ = (hs_.n_thk * hs_.n_dyn + 31) / 32;
      SFLOW_CU(alloc((void**)&vuln_, sizeof(uint32_t) * plane_ * vuln_words_));
      SFLOW_CU(cudaMemset(vuln_, 0, sizeof(uint32_t) * plane_ * vuln_words_));
    }
    SFLOW_CU(alloc((void**)&st_, sizeof(RunState)));
    nstat_blocks_ = 1024;
    SFLOW_CU(alloc((void**)&stat_part_, sizeof(double) * 4 * nstat_blocks_));
    SFLOW_CU(alloc((void**)&stat_out_, sizeof(double) * 4));
    SFLOW_CU(cudaMemset(q_, 0, sizeof(R) * plane_ * nv));
    fill_args();
    // shared memory of the flux kernel
    smem_flux_ = flux_smem_bytes(hs_.nv, tile_h_);
    SFLOW_CU(set_smem_attr());
    std::memset(&hst_, 0, sizeof(hst_));
    init_state_host();
    limits_known_ = false;
    SFLOW_CU(cudaStreamSynchronize(stream_));   // plane uploads read the set-up's host arrays
    SFLOW_CU(cudaMemcpy(st_, &hst_, sizeof(RunState), cudaMemcpyHostToDevice));
    return SFLOW_OK;
  }

  // device bytes of init()'s allocations, each rounded as alloc() rounds
  size_t init_bytes() const {
    auto A = [](size_t b) { return (b + kArenaAlign - 1) / kArenaAlign * kArenaAlign; };
    const size_t P = (size_t)plane_, nv = (size_t)hs_.nv, ns = (size_t)hs_.ns;
    const size_t nstage = (hs_.nrk == 2) ? 1 : (size_t)hs_.nrk;
    const size_t tiles = (size_t)tiles_x_ * tiles_y_;
    size_t b = A(sizeof(R) * P * nv) + A(sizeof(R) * P * nv * nstage);
    if (hs_.nrk != 2) b += A(sizeof(R) * P * nv * nstage) + A(sizeof(R) * P * nv);
    b += (size_t)(hs_.p.curvature_term_flag ? 8 : 5) * A(sizeof(R) * P);
    b += A(P) + A(sizeof(R) * P * 3) + A(P);                        // flags, arc, mask
    b += A(tiles) + A(3 * tiles) + A(tiles) + A(tiles * sizeof(uint16_t));
    b += 3 * A(sizeof(R) * P);                                      // maxima
    if (hs_.exchange) b += A(sizeof(double) * P * ns);
    if (hs_.p.erosion_coeff > 0.0 || (hs_.p.erodible_deposit_flag && hs_.exchange))
      b += 2 * A(sizeof(double) * P * ns);
    if (hs_.p.topo_change_flag && hs_.exchange) b += A(sizeof(double) * P);
    if (hs_.p.bottom_radial_source_flag)
      b += A(sizeof(R) * P) + A(sizeof(double) * (1 + 2 * (size_t)SFLOW_MAX_INTERVALS));
    if (hs_.n_thk * hs_.n_dyn > 0) b += A(sizeof(uint32_t) * P * (size_t)((hs_.n_thk * hs_.n_dyn + 31) / 32));
    b += A(sizeof(RunState)) + A(sizeof(double) * 4 * 1024) + A(sizeof(double) * 4);
    return b + extra_bytes_;
  }
  // room in the run's allocation for buffers its owner adds after init()
  // (the batch's per-tile flags): call before init(); carve() hands it out
  void reserve_extra(size_t bytes) { extra_bytes_ += (bytes + kArenaAlign - 1) / kArenaAlign * kArenaAlign; }
  void* carve(size_t bytes) {
    const size_t a = (bytes + kArenaAlign - 1) / kArenaAlign * kArenaAlign;
    if (!arena_ || arena_used_ + a > arena_cap_) return nullptr;
    void* p = arena_ + arena_used_;
    arena_used_ += a;
    bytes_ += (int64_t)bytes;
    return p;
  }

  // --- used by the batch engine ----------------------------------------------
  const KArgs<R>& kargs() const { return ka_; }
  RunState* state_dev() const { return st_; }
  int tiles_x() const { return tiles_x_; }
  int tiles_y() const { return tiles_y_; }
  size_t smem_flux() const { return smem_flux_; }
  // dynamic shared memory of flux_tile: qp of the tile + halo, x- and
  // y-face fluxes and speeds, the tile's 5 topography planes, flag bytes of
  // the tile + halo
  static size_t flux_smem_bytes(int nv, int th) {
    const int np = nv + 2;
    const size_t ry = (size_t)th + 2 * HALO;
    const size_t r = (size_t)np * RX * ry + (size_t)nv * th * (TX + 1) + (size_t)nv * (th + 1) * TX +
                     (size_t)th * (TX + 1) + (size_t)(th + 1) * TX + (size_t)5 * TX * th;
    return (r * sizeof(R) + RX * ry + 15) / 16 * 16;
  }
  cudaStream_t stream() const { return stream_; }
  const HostSetup& setup() const { return hs_; }
  int limits(double t_stop, int64_t step_limit) {
    SFLOW_CU(set_limits(t_stop, step_limit));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    return SFLOW_OK;
  }
  // frees the host-layout staging buffer (allocated again when needed)
  void trim_stage() {
    if (!stage_aos_) return;
    cudaStreamSynchronize(stream_);
    cudaFree(stage_aos_);
    bytes_ -= (int64_t)(sizeof(double) * (size_t)hs_.nx * hs_.ny * (hs_.nv + 3));
    stage_aos_ = nullptr;
  }
  // per tile: 1 when its cells can activate neighbouring tiles whatever the
  // flow (ring-boundary cells, or an edge tile narrower than n_RK + 1 cells)
  std::vector<uint8_t> tile_seed_host() const {
    std::vector<uint8_t> ts((size_t)tiles_x_ * tiles_y_, 0);
    const int nx = hs_.nx, ny = hs_.ny, nrk = hs_.nrk;
    const int TY = tile_h_;
    const int wlast = nx - (tiles_x_ - 1) * TX, hlast = ny - (tiles_y_ - 1) * TY;
    for (int ty = 0; ty < tiles_y_; ++ty)
      for (int tx = 0; tx < tiles_x_; ++tx) {
        uint8_t v = 0;
        if ((tx == tiles_x_ - 1 && wlast <= nrk) || (ty == tiles_y_ - 1 && hlast <= nrk)) v = 1;
        if (hs_.p.radial_source_flag)
          for (int k = ty * TY; k < std::min(ny, (ty + 1) * TY) && !v; ++k)
            for (int j = tx * TX; j < std::min(nx, (tx + 1) * TX); ++j)
              if ((hs_.cflags[(size_t)k * nx + j] & 3) == 2) { v = 1; break; }
        ts[(size_t)ty * tiles_x_ + tx] = v;
      }
    return ts;
  }
  uint8_t* tile_wet_dev() const { return tile_wet_; }
  const uint16_t* tile_count_dev() const { return tile_count_; }

  // device bytes a run of this set-up holds while it is in a batch
  static int64_t batch_bytes(const HostSetup& hs, int tile_h) {
    const int64_t pitch = (hs.nx + 31) / 32 * 32, plane = pitch * hs.ny;
    const int ngeo = hs.p.curvature_term_flag ? 8 : 5;
    const int64_t tiles = (int64_t)((hs.nx + TX - 1) / TX) * ((hs.ny + tile_h - 1) / tile_h);
    return plane * (int64_t)sizeof(R) * (2 * hs.nv + ngeo + 3 + 3) + 2 * plane + tiles * 7 +
           (int64_t)sizeof(double) * 4 * 1024 + 4096;
  }

  // --- SolverBase -----------------------------------------------------------
  int upload(const double* q_aos) override {
    const int nx = hs_.nx, ny = hs_.ny, nv = hs_.nv;
    const size_t N = (size_t)nx * ny;
    SFLOW_CU(layout_in(q_aos));
    ++launches_;
    SFLOW_CU(cudaGetLastError());
    init_state_host();
    limits_known_ = false;
    SFLOW_CU(cudaMemcpyAsync(st_, &hst_, sizeof(RunState), cudaMemcpyHostToDevice, stream_));
    SFLOW_CU(dispatch_init_maps((unsigned)((N + 255) / 256)));
    if (deposit_) SFLOW_CU(cudaMemsetAsync(deposit_, 0, sizeof(double) * plane_ * hs_.ns, stream_));
    if (erosion_) SFLOW_CU(reset_erosion());
    if (Bc_) SFLOW_CU(reset_topography());
    SFLOW_CU(cudaMemsetAsync(tile_wet_, 0xff, 3 * (size_t)tiles_x_ * tiles_y_, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    uploaded_ = true;
    return SFLOW_OK;
  }

  // Pinned (page-locked) host memory is mapped into the device address
  // space; on a Grace-Blackwell node the layout kernels then read or write
  // it over NVLink-C2C directly, with no staging copy.  Other host memory
  // goes through the device staging buffer and the copy engines.
  // q (host layout) into the state planes: the device reads the host array
  // itself when it can (mapped pinned memory; pageable memory on a system
  // with pageable access), else through the staging buffer
  cudaError_t layout_in(const double* q_aos) {
    const int nx = hs_.nx, ny = hs_.ny, nv = hs_.nv;
    const size_t N = (size_t)nx * ny;
    const double* src = mapped_host(q_aos);
    if (!src && pageable_access()) src = q_aos;
    if (src) {
      k_host_aos_to_planes<R><<<(unsigned)((N + kHostChunk - 1) / kHostChunk), kHostChunk,
                                sizeof(double) * kHostChunk * nv, stream_>>>(src, q_, nv, nx, ny, pitch_, plane_);
      return cudaGetLastError();
    }
    cudaError_t e = ensure_stage();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(stage_aos_, q_aos, sizeof(double) * N * nv, cudaMemcpyHostToDevice, stream_);
    if (e != cudaSuccess) return e;
    k_aos_to_planes<R><<<(unsigned)((N + 255) / 256), 256, 0, stream_>>>(stage_aos_, q_, nv, nx, ny, pitch_, plane_);
    return cudaGetLastError();
  }

  // host memory the device reads or writes through its own mapping (pinned)
  static bool is_mapped_host(const void* p) { return mapped_host(p) != nullptr; }
  static const double* mapped_host(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer) return nullptr;
    return static_cast<const double*>(at.devicePointer);
  }

  int put(const double* q_aos) override {
    if (!uploaded_) { err_ = "no state uploaded"; return SFLOW_ESTATE; }
    const int nx = hs_.nx, ny = hs_.ny, nv = hs_.nv;
    const size_t N = (size_t)nx * ny;
    (void)N;
    SFLOW_CU(layout_in(q_aos));
    SFLOW_CU(reset_wet_flags());
    ++launches_;
    SFLOW_CU(cudaGetLastError());
    SFLOW_CU(cudaStreamSynchronize(stream_));
    return SFLOW_OK;
  }

  int set_clock(double t, double dt_old, double dt_old_old) override {
    if (!uploaded_) { err_ = "no state uploaded"; return SFLOW_ESTATE; }
    SFLOW_CU(cudaMemcpyAsync(&hst_, st_, sizeof(RunState), cudaMemcpyDeviceToHost, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    hst_.t = t;
    hst_.t_prev = t;
    hst_.dt_old = dt_old;
    hst_.dt_old_old = dt_old_old;
    limits_known_ = false;
    SFLOW_CU(cudaMemcpyAsync(st_, &hst_, sizeof(RunState), cudaMemcpyHostToDevice, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    return SFLOW_OK;
  }

  int advance_timed(int64_t steps, int flush, double* ms) override {
    if (!uploaded_) { err_ = "no state uploaded"; return SFLOW_ESTATE; }
    SFLOW_CU(prepare_timing(flush));
    SFLOW_CU(set_limits(hs_.p.t_end, -1));
    if (!graph1_exec_) SFLOW_CU(build_graph1());
    double total = 0.0;
    for (int64_t i = 0; i < steps; ++i) {
      if (flush) SFLOW_CU(flush_l2());
      SFLOW_CU(cudaEventRecord(ev_[0], stream_));
      SFLOW_CU(cudaGraphLaunch(graph1_exec_, stream_));
      launches_ += steps_launches();
      SFLOW_CU(cudaEventRecord(ev_[1], stream_));
      SFLOW_CU(cudaEventSynchronize(ev_[1]));
      float m = 0.0f;
      SFLOW_CU(cudaEventElapsedTime(&m, ev_[0], ev_[1]));
      total += m;
    }
    *ms = total;
    return SFLOW_OK;
  }

  int profile_kernels(int64_t steps, int flush, double* ms4) override {
    if (!uploaded_) { err_ = "no state uploaded"; return SFLOW_ESTATE; }
    if (hs_.nrk != 2) { err_ = "kernel profile is for N_RK = 2"; return SFLOW_EINVAL; }
    SFLOW_CU(prepare_timing(flush));
    SFLOW_CU(set_limits(hs_.p.t_end, -1));
    double tot[4] = {0, 0, 0, 0};
    for (int64_t i = 0; i < steps; ++i) {
      if (flush) SFLOW_CU(flush_l2());
      SFLOW_CU(cudaEventRecord(ev_[0], stream_));
      SFLOW_CU(launch_mask(2));
      SFLOW_CU(cudaEventRecord(ev_[1], stream_));
      SFLOW_CU(launch_flux(1));
      SFLOW_CU(cudaEventRecord(ev_[2], stream_));
      SFLOW_CU(launch_step_kernel(k_dt, dim3(1), dim3(1), 0, stream_, ka_.g.pdl, st_, hs_.p.max_dt));
      ++launches_;
      SFLOW_CU(cudaGetLastError());
      SFLOW_CU(cudaEventRecord(ev_[3], stream_));
      SFLOW_CU(launch_stage2(-1));
      SFLOW_CU(cudaEventRecord(ev_[4], stream_));
      SFLOW_CU(cudaEventSynchronize(ev_[4]));
      for (int k = 0; k < 4; ++k) {
        float m = 0.0f;
        SFLOW_CU(cudaEventElapsedTime(&m, ev_[k], ev_[k + 1]));
        tot[k] += m;
      }
    }
    for (int k = 0; k < 4; ++k) ms4[k] = tot[k];
    return SFLOW_OK;
  }

  int download(double* q_aos) override {
    const int nx = hs_.nx, ny = hs_.ny, nv = hs_.nv;
    const size_t N = (size_t)nx * ny;
    double* dst = const_cast<double*>(mapped_host(q_aos));
    if (dst) {
      k_host_planes_to_aos<R><<<(unsigned)((N + kHostChunk - 1) / kHostChunk), kHostChunk,
                                sizeof(double) * kHostChunk * nv, stream_>>>(q_, dst, nv, nx, ny, pitch_, plane_);
      ++launches_;
      SFLOW_CU(cudaGetLastError());
      SFLOW_CU(cudaStreamSynchronize(stream_));
      return SFLOW_OK;
    }
    SFLOW_CU(ensure_stage());
    k_planes_to_aos<R><<<(unsigned)((N + 255) / 256), 256, 0, stream_>>>(q_, stage_aos_, nv, nx, ny, pitch_, plane_);
    ++launches_;
    SFLOW_CU(cudaGetLastError());
    SFLOW_CU(cudaMemcpyAsync(q_aos, stage_aos_, sizeof(double) * N * nv, cudaMemcpyDeviceToHost, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    return SFLOW_OK;
  }

  int download_qp(double* qp_aos) override {
    const size_t N = (size_t)hs_.nx * hs_.ny;
    SFLOW_CU(ensure_stage());
    SFLOW_CU(dispatch_qp((unsigned)((N + 255) / 256)));
    SFLOW_CU(cudaMemcpyAsync(qp_aos, stage_aos_, sizeof(double) * N * (hs_.nv + 2), cudaMemcpyDeviceToHost, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    return SFLOW_OK;
  }

  // .p_2d fields per cell: h, u, v, T, alphas, rho_m, red_grav, Ri
  int download_phys(double* out) override {
    const size_t N = (size_t)hs_.nx * hs_.ny;
    SFLOW_CU(ensure_stage());
    ++launches_;
    SFLOW_CU(tab_.phys(ka_, (unsigned)((N + 255) / 256), stream_, stage_aos_));
    SFLOW_CU(cudaMemcpyAsync(out, stage_aos_, sizeof(double) * N * (hs_.ns + 7), cudaMemcpyDeviceToHost, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    return SFLOW_OK;
  }

  int download_maps(double* h, double* p, double* v) override {
    const int nx = hs_.nx, ny = hs_.ny;
    const size_t N = (size_t)nx * ny;
    SFLOW_CU(ensure_stage());
    R* src[3] = {hmax_, pdynmax_, mvmax_};
    double* dst[3] = {h, p, v};
    for (int m = 0; m < 3; ++m) {
      if (!dst[m]) continue;
      k_map_to_host<R><<<(unsigned)((N + 255) / 256), 256, 0, stream_>>>(src[m], stage_aos_, nx, ny, pitch_);
      ++launches_;
      SFLOW_CU(cudaGetLastError());
      SFLOW_CU(cudaMemcpyAsync(dst[m], stage_aos_, sizeof(double) * N, cudaMemcpyDeviceToHost, stream_));
      SFLOW_CU(cudaStreamSynchronize(stream_));
    }
    return SFLOW_OK;
  }

  // deposit(1:nx,1:ny,1:n_solid) in the reference layout (column-major, class
  // slowest); zeros when the run has no settling
  int download_deposit(double* out) override {
    const int nx = hs_.nx, ny = hs_.ny;
    const size_t N = (size_t)nx * ny;
    if (!deposit_) {
      std::memset(out, 0, sizeof(double) * N * hs_.ns);
      return SFLOW_OK;
    }
    std::vector<double> buf((size_t)plane_);
    SFLOW_CU(cudaStreamSynchronize(stream_));
    for (int i = 0; i < hs_.ns; ++i) {
      SFLOW_CU(cudaMemcpy(buf.data(), deposit_ + (size_t)i * plane_, sizeof(double) * plane_, cudaMemcpyDeviceToHost));
      for (int k = 0; k < ny; ++k)
        for (int j = 0; j < nx; ++j) out[(size_t)i * N + (size_t)k * nx + j] = buf[(size_t)k * pitch_ + j];
    }
    return SFLOW_OK;
  }
  int upload_deposit(const double* in) override {
    if (!deposit_) { err_ = "the run has no settling: no deposit to set"; return SFLOW_EINVAL; }
    const int nx = hs_.nx, ny = hs_.ny;
    const size_t N = (size_t)nx * ny;
    std::vector<double> buf((size_t)plane_, 0.0);
    SFLOW_CU(cudaStreamSynchronize(stream_));
    for (int i = 0; i < hs_.ns; ++i) {
      for (int k = 0; k < ny; ++k)
        for (int j = 0; j < nx; ++j) buf[(size_t)k * pitch_ + j] = in[(size_t)i * N + (size_t)k * nx + j];
      SFLOW_CU(cudaMemcpy(deposit_ + (size_t)i * plane_, buf.data(), sizeof(double) * plane_, cudaMemcpyHostToDevice));
    }
    return SFLOW_OK;
  }
  // erosion (accumulated dt * erosion_term) or the erodible layer, n_solid
  // planes of nx*ny (class slowest)
  int download_erosion(int which, double* out) override {
    const double* src = which == 0 ? erosion_ : erodible_;
    if (!src) {
      std::memset(out, 0, sizeof(double) * (size_t)hs_.nx * hs_.ny * hs_.ns);
      return SFLOW_OK;
    }
    for (int i = 0; i < hs_.ns; ++i) SFLOW_CU(get_plane_d(out + (size_t)i * hs_.nx * hs_.ny, src + (size_t)i * plane_));
    return SFLOW_OK;
  }
  // B_cent (changes with TOPO_CHANGE_FLAG)
  int download_topography(double* out) override {
    if (!Bc_) {
      std::memcpy(out, hs_.B.data(), sizeof(double) * hs_.B.size());
      return SFLOW_OK;
    }
    return get_plane_d(out, Bc_) == cudaSuccess ? SFLOW_OK : SFLOW_ECUDA;
  }
  // erodible layer thickness per cell (the reference's erodible_init: each
  // class gets erodible_fract * (1 - erodible_porosity) of it)
  int set_erodible(const double* thickness) override {
    if (!erodible_) { err_ = "the run has no erodible layer (erosion_coeff = 0)"; return SFLOW_EINVAL; }
    const size_t N = (size_t)hs_.nx * hs_.ny;
    std::vector<double> pl(N);
    SFLOW_CU(cudaStreamSynchronize(stream_));
    for (int i = 0; i < hs_.ns; ++i) {
      for (size_t c = 0; c < N; ++c) pl[c] = hs_.erodible_fract[i] * (1.0 - hs_.erodible_porosity) * thickness[c];
      SFLOW_CU(put_plane_d(erodible_ + (size_t)i * plane_, pl));
    }
    erodible_user_.assign(thickness, thickness + N);
    return SFLOW_OK;
  }
  // B_nodata cells (nonzero): the assembly empties them
  int set_nodata(const uint8_t* nodata) override {
    const int nx = hs_.nx, ny = hs_.ny;
    bool any = false;
    for (int k = 0; k < ny; ++k)
      for (int j = 0; j < nx; ++j) {
        uint8_t& f = hs_.cflags[(size_t)k * nx + j];
        f = (uint8_t)((f & ~kFlagNodata) | (nodata && nodata[(size_t)k * nx + j] ? kFlagNodata : 0));
        any |= (f & kFlagNodata) != 0;
      }
    SFLOW_CU(cudaStreamSynchronize(stream_));
    SFLOW_CU(put_flags());
    ka_.pr.nodata = ka_.pd.nodata = any ? 1 : 0;
    drop_graphs();
    return SFLOW_OK;
  }
  // vulnerability table: n_thk * n_dyn planes of nx*ny bytes (0/1)
  int vuln_table(int* n_thk, int* n_dyn, uint8_t* out) override {
    if (n_thk) *n_thk = hs_.n_thk;
    if (n_dyn) *n_dyn = hs_.n_dyn;
    if (!out || !vuln_) return SFLOW_OK;
    const int nx = hs_.nx, ny = hs_.ny;
    std::vector<uint32_t> buf((size_t)plane_);
    SFLOW_CU(cudaStreamSynchronize(stream_));
    const int ne = hs_.n_thk * hs_.n_dyn;
    for (int w = 0; w < vuln_words_; ++w) {
      SFLOW_CU(cudaMemcpy(buf.data(), vuln_ + (size_t)w * plane_, sizeof(uint32_t) * plane_, cudaMemcpyDeviceToHost));
      for (int e = 32 * w; e < std::min(ne, 32 * w + 32); ++e)
        for (int k = 0; k < ny; ++k)
          for (int j = 0; j < nx; ++j)
            out[(size_t)e * nx * ny + (size_t)k * nx + j] = (uint8_t)((buf[(size_t)k * pitch_ + j] >> (e & 31)) & 1u);
    }
    return SFLOW_OK;
  }

  // rows k_lo .. k_lo+n-1 of q in the reference layout ([row][j][var])
  int get_rows(int k_lo, int n, double* out) override {
    if (k_lo < 0 || n < 0 || k_lo + n > hs_.ny) { err_ = "rows outside the domain"; return SFLOW_EINVAL; }
    const int nx = hs_.nx, nv = hs_.nv;
    std::vector<R> buf((size_t)n * nx);
    SFLOW_CU(cudaStreamSynchronize(stream_));
    for (int i = 0; i < nv; ++i) {
      SFLOW_CU(cudaMemcpy2D(buf.data(), sizeof(R) * nx, q_ + (size_t)i * plane_ + (size_t)k_lo * pitch_,
                            sizeof(R) * pitch_, sizeof(R) * nx, n, cudaMemcpyDeviceToHost));
      for (size_t c = 0; c < (size_t)n * nx; ++c) out[c * nv + i] = (double)buf[c];
    }
    return SFLOW_OK;
  }
  int put_rows(int k_lo, int n, const double* in) override {
    if (!uploaded_) { err_ = "no state uploaded"; return SFLOW_ESTATE; }
    if (k_lo < 0 || n < 0 || k_lo + n > hs_.ny) { err_ = "rows outside the domain"; return SFLOW_EINVAL; }
    const int nx = hs_.nx, nv = hs_.nv;
    std::vector<R> buf((size_t)n * nx);
    SFLOW_CU(cudaStreamSynchronize(stream_));
    for (int i = 0; i < nv; ++i) {
      for (size_t c = 0; c < (size_t)n * nx; ++c) buf[c] = (R)in[c * nv + i];
      SFLOW_CU(cudaMemcpy2D(q_ + (size_t)i * plane_ + (size_t)k_lo * pitch_, sizeof(R) * pitch_, buf.data(),
                            sizeof(R) * nx, sizeof(R) * nx, n, cudaMemcpyHostToDevice));
    }
    SFLOW_CU(reset_wet_flags());
    SFLOW_CU(cudaStreamSynchronize(stream_));
    return SFLOW_OK;
  }

  int set_output_time(double t_output) override {
    if (!uploaded_) { err_ = "no state uploaded"; return SFLOW_ESTATE; }
    SFLOW_CU(cudaMemcpyAsync(&st_->t_output, &t_output, sizeof(double), cudaMemcpyHostToDevice, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    hst_.t_output = t_output;
    return SFLOW_OK;
  }

  // maxima maps from the host (restart.bin), reference layout
  int upload_maps(const double* h, const double* p, const double* v) override {
    const int nx = hs_.nx, ny = hs_.ny;
    SFLOW_CU(cudaStreamSynchronize(stream_));
    R* dst[3] = {hmax_, pdynmax_, mvmax_};
    const double* src[3] = {h, p, v};
    std::vector<R> buf((size_t)plane_, R(0));
    for (int m = 0; m < 3; ++m) {
      if (!src[m]) continue;
      for (int k = 0; k < ny; ++k)
        for (int j = 0; j < nx; ++j) buf[(size_t)k * pitch_ + j] = (R)src[m][(size_t)k * nx + j];
      SFLOW_CU(cudaMemcpy(dst[m], buf.data(), sizeof(R) * plane_, cudaMemcpyHostToDevice));
    }
    return SFLOW_OK;
  }

  // granular entry points (one Fortran call site each) ------------------------
  int check_solve(int solve_all) override {
    if (!uploaded_) { err_ = "no state uploaded"; return SFLOW_ESTATE; }
    SFLOW_CU(launch_mask(solve_all));
    return SFLOW_OK;
  }
  int timestep(double* dt_out) override {
    if (!uploaded_) { err_ = "no state uploaded"; return SFLOW_ESTATE; }
    if (hs_.nrk != 2) { err_ = "the per-call-site entry points need N_RK = 2; use sflow_step / sflow_advance"; return SFLOW_EINVAL; }
    SFLOW_CU(launch_flux(1));
    RunState h;
    SFLOW_CU(cudaMemcpyAsync(&h, st_, sizeof(RunState), cudaMemcpyDeviceToHost, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    double dtmin;
    unsigned long long b = h.dtmin_bits;
    std::memcpy(&dtmin, &b, sizeof(double));
    double dt = hs_.p.max_dt;
    if (dtmin < dt) dt = dtmin;
    if (dt_out) *dt_out = dt;
    flux_ready_ = true;
    return SFLOW_OK;
  }
  int imex_rk(double t, double dt) override {
    SFLOW_CU(reset_wet_flags());   // stage kernel of mode 0 keeps no wet flags
    if (!flux_ready_) { err_ = "sflow_imex_rk needs sflow_timestep on the same state first"; return SFLOW_ESTATE; }
    RunState h;
    SFLOW_CU(cudaMemcpyAsync(&h, st_, sizeof(RunState), cudaMemcpyDeviceToHost, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    if (t != h.t) { err_ = "t differs from the handle's time (sflow_get_stats)"; return SFLOW_ESTATE; }
    h.dt_old_old = h.dt_old;
    h.dt_old = dt;
    h.dt = dt;
    h.t_prev = h.t;
    h.run_step = 1;
    int p = (int)(h.steps & 1);
    h.last_cells = (long long)h.cells_acc[p];
    h.cells_total += (long long)h.cells_acc[p];
    h.cells_acc[p] = 0;
    h.border_total += (long long)h.border_acc[p];
    h.border_acc[p] = 0;
    h.dtmin_bits = bits_of(1.0e300);
    limits_known_ = false;
    SFLOW_CU(cudaMemcpyAsync(st_, &h, sizeof(RunState), cudaMemcpyHostToDevice, stream_));
    SFLOW_CU(launch_stage2(0));
    flux_ready_ = false;
    pending_dt_ = dt;
    return SFLOW_OK;
  }
  int erosion_deposition(double dt) override {
    SFLOW_CU(reset_wet_flags());
    if (dt != pending_dt_) { err_ = "dt differs from the last sflow_imex_rk"; return SFLOW_ESTATE; }
    if (hs_.exchange) SFLOW_CU(launch_stage2(1));
    if (Bc_) SFLOW_CU(launch_topography());
    return SFLOW_OK;
  }
  int post_step(SflowStepStats* s) override {
    SFLOW_CU(launch_stage2(2));
    RunState h;
    SFLOW_CU(cudaMemcpyAsync(&h, st_, sizeof(RunState), cudaMemcpyDeviceToHost, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    h.t = h.t + h.dt;
    h.steps += 1;
    h.run_step = 0;
    limits_known_ = false;
    SFLOW_CU(cudaMemcpyAsync(st_, &h, sizeof(RunState), cudaMemcpyHostToDevice, stream_));
    return s ? stats(s) : SFLOW_OK;
  }

  // tile shape ----------------------------------------------------------------
  int tile_shape() const override { return tile_h_; }

  // Switch the tiled kernels to tiles of TX x th cells.  The step's results
  // do not depend on the tile height, so a run may switch between steps: the
  // per-tile arrays are re-made (wet flags unknown = 1; activity is
  // recomputed by the next check_solve) and the captured graphs dropped.
  int set_tile_shape(int th) override {
    if (th == tile_h_) return SFLOW_OK;
    KernelTable<R> t = kernel_table<R>(hs_.ns, th);
    if (!t.flux) { err_ = "no kernels built for this tile height"; return SFLOW_EINVAL; }
    SFLOW_CU(cudaStreamSynchronize(stream_));
    drop_graphs();
    const size_t n_old = (size_t)tiles_x_ * tiles_y_;
    free_tracked(tile_active_, n_old);
    free_tracked(tile_wet_, 3 * n_old);
    free_tracked(tile_static_, n_old);
    free_tracked(tile_count_, n_old * sizeof(uint16_t));
    tile_active_ = tile_wet_ = tile_static_ = nullptr;
    tile_count_ = nullptr;
    tab_ = t;
    tile_h_ = th;
    tiles_y_ = (hs_.ny + th - 1) / th;
    SFLOW_CU(alloc_tiles());
    ka_.g.tiles_y = tiles_y_;
    ka_.tile_active = tile_active_;
    ka_.tile_wet = tile_wet_;
    ka_.tile_wet_step = tile_wet_ + (size_t)tiles_x_ * tiles_y_;
    ka_.tile_static = tile_static_;
    ka_.tile_count = tile_count_;
    smem_flux_ = flux_smem_bytes(hs_.nv, th);
    SFLOW_CU(set_smem_attr());
    return SFLOW_OK;
  }

  // Tile-shape autotuner: times `steps` graph-replayed steps of this run
  // with every compiled tile height (after one untimed chunk that captures
  // the graph) and keeps the height with the least time per active-cell
  // update.  The steps are real steps of the run (the results are the same
  // with every height); ms_per_mcu[i] receives the time per 10^6 cell
  // updates of candidate i of kTileCandidates (-1 when not compiled).
  static constexpr double kTuneMargin = 0.02;
  int autotune(int64_t steps, int* best, double* ms_per_mcu) override {
    if (!uploaded_) { err_ = "no state uploaded"; return SFLOW_ESTATE; }
    if (steps < 1) { err_ = "autotune needs at least one step per tile height"; return SFLOW_EINVAL; }
    SFLOW_CU(prepare_timing(0));
    int best_th = tile_h_;
    double best_v = -1.0;
    for (int i = 0; i < kTileCandidates; ++i) {
      const int th = kTileCandidate[i];
      ms_per_mcu[i] = -1.0;
      if (!tile_h_built<R>(th)) continue;
      int rc = set_tile_shape(th);
      if (rc != SFLOW_OK) return rc;
      SFLOW_CU(set_limits(hs_.p.t_end, -1));
      if (!graph_exec_) SFLOW_CU(build_graph());
      SFLOW_CU(cudaGraphLaunch(graph_exec_, stream_));   // warm-up chunk
      launches_ += kChunk * steps_launches();
      RunState h0, h1;
      SFLOW_CU(cudaMemcpyAsync(&h0, st_, sizeof(RunState), cudaMemcpyDeviceToHost, stream_));
      SFLOW_CU(cudaEventRecord(ev_[0], stream_));
      const int64_t chunks = (steps + kChunk - 1) / kChunk;
      for (int64_t c = 0; c < chunks; ++c) {
        SFLOW_CU(cudaGraphLaunch(graph_exec_, stream_));
        launches_ += kChunk * steps_launches();
      }
      SFLOW_CU(cudaEventRecord(ev_[1], stream_));
      SFLOW_CU(cudaMemcpyAsync(&h1, st_, sizeof(RunState), cudaMemcpyDeviceToHost, stream_));
      SFLOW_CU(cudaStreamSynchronize(stream_));
      float m = 0.0f;
      SFLOW_CU(cudaEventElapsedTime(&m, ev_[0], ev_[1]));
      const long long cells = h1.cells_total - h0.cells_total;
      if (cells <= 0) continue;   // the run stopped: nothing measured
      ms_per_mcu[i] = (double)m / ((double)cells * 1.0e-6);
      // a later candidate must beat the best so far by more than 2 %: a
      // near tie is measurement noise, and the first candidate (32 x 8) is
      // the default
      if (best_v < 0.0 || ms_per_mcu[i] < best_v * (1.0 - kTuneMargin)) {
        best_v = ms_per_mcu[i];
        best_th = th;
      }
    }
    int rc = set_tile_shape(best_th);
    if (rc != SFLOW_OK) return rc;
    *best = best_th;
    return SFLOW_OK;
  }

  // fused driver iteration -----------------------------------------------------
  int step() override {
    if (!uploaded_) { err_ = "no state uploaded"; return SFLOW_ESTATE; }
    SFLOW_CU(set_limits(hs_.p.t_end, -1));
    SFLOW_CU(launch_step());
    SFLOW_CU(cudaStreamSynchronize(stream_));
    return SFLOW_OK;
  }

  int advance(double t_stop, int64_t max_steps, SflowStepStats* s) override {
    if (!uploaded_) { err_ = "no state uploaded"; return SFLOW_ESTATE; }
    if (max_steps <= 0) return s ? stats(s) : SFLOW_OK;
    SFLOW_CU(cudaMemcpyAsync(&hst_, st_, sizeof(RunState), cudaMemcpyDeviceToHost, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    const double stop = t_stop < hs_.p.t_end ? t_stop : hs_.p.t_end;
    const int64_t limit = hst_.steps + max_steps;
    SFLOW_CU(set_limits(stop, limit));
    if (!graph_exec_) SFLOW_CU(build_graph());
    // replay chunks until the device reports t >= stop or the step budget
    for (;;) {
      const int64_t left = limit - hst_.steps;
      const int64_t chunks = (left + kChunk - 1) / kChunk;
      const int64_t burst = chunks < 8 ? chunks : 8;
      for (int64_t b = 0; b < burst; ++b) {
        SFLOW_CU(cudaGraphLaunch(graph_exec_, stream_));
        launches_ += kChunk * steps_launches();
      }
      SFLOW_CU(cudaMemcpyAsync(&hst_, st_, sizeof(RunState), cudaMemcpyDeviceToHost, stream_));
      SFLOW_CU(cudaStreamSynchronize(stream_));
      if (!(hst_.t < stop) || hst_.steps >= limit || (hst_.status & SFLOW_S_FATAL)) break;
    }
    return s ? stats(s) : SFLOW_OK;
  }

  int stats(SflowStepStats* s) override {
    SFLOW_CU(dispatch_stats());
    double out[4];
    SFLOW_CU(cudaMemcpyAsync(out, stat_out_, sizeof(out), cudaMemcpyDeviceToHost, stream_));
    SFLOW_CU(cudaMemcpyAsync(&hst_, st_, sizeof(RunState), cudaMemcpyDeviceToHost, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    const double a = hs_.dx * hs_.dy;
    s->t = hst_.t;
    s->dt = hst_.dt;
    s->mass = a * out[0];
    s->volume = a * out[1];
    s->area = a * out[2];
    s->solid_mass = a * out[3];
    s->solve_cells = hst_.last_cells;
    s->steps = hst_.steps;
    s->status = hst_.status;
    s->pad = 0;
    return SFLOW_OK;
  }
  int status(uint32_t* f) override {
    RunState h;
    SFLOW_CU(cudaMemcpyAsync(&h, st_, sizeof(RunState), cudaMemcpyDeviceToHost, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    *f = h.status;
    return SFLOW_OK;
  }
  int clear_status() override {
    unsigned z = 0;
    SFLOW_CU(cudaMemcpyAsync(&st_->status, &z, sizeof(z), cudaMemcpyHostToDevice, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    return SFLOW_OK;
  }
  int64_t launches() const override { return launches_; }
  int64_t device_bytes() const override { return bytes_; }
  int newton_stats(int64_t* total, int* maxit) override {
    RunState h;
    SFLOW_CU(cudaMemcpyAsync(&h, st_, sizeof(RunState), cudaMemcpyDeviceToHost, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    *total = h.newton_iters;
    *maxit = h.newton_max;
    return SFLOW_OK;
  }
  const char* error() const override { return err_.c_str(); }
  // the run's device state record (clock, counters, status), one copy
  int run_state(RunState* h) {
    SFLOW_CU(cudaMemcpyAsync(h, st_, sizeof(RunState), cudaMemcpyDeviceToHost, stream_));
    SFLOW_CU(cudaStreamSynchronize(stream_));
    return SFLOW_OK;
  }
  int64_t cells_total() override {
    RunState h;
    if (cudaMemcpy(&h, st_, sizeof(RunState), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return h.cells_total;
  }
  int64_t border_total() override {
    RunState h;
    if (cudaMemcpy(&h, st_, sizeof(RunState), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return h.border_total;
  }

 private:
  static constexpr int kChunk = 16;   // steps per captured graph
  HostSetup hs_;
  int pitch_ = 0;
  int64_t plane_ = 0;
  int tile_h_ = kTileHDefault;   // cells per tile column (TileShape)
  int tiles_x_ = 0, tiles_y_ = 0;
  cudaStream_t stream_ = nullptr;
  R *q_ = nullptr, *rd_ = nullptr, *rn_ = nullptr, *qs_ = nullptr, *arc_ = nullptr, *hmax_ = nullptr, *pdynmax_ = nullptr, *mvmax_ = nullptr;
  double* deposit_ = nullptr;
  double *erosion_ = nullptr, *erodible_ = nullptr, *Bc_ = nullptr, *bsrc_tab_ = nullptr;
  R* bfrac_ = nullptr;
  uint32_t* vuln_ = nullptr;
  int vuln_words_ = 0;
  std::vector<double> erodible_user_;   // thickness set by set_erodible (else uniform)
  R* geo_[8];
  uint8_t *cflags_ = nullptr, *mask_ = nullptr, *tile_active_ = nullptr, *tile_wet_ = nullptr,
          *tile_static_ = nullptr;
  uint16_t* tile_count_ = nullptr;
  RunState* st_ = nullptr;
  double *stage_aos_ = nullptr, *stat_part_ = nullptr, *stat_out_ = nullptr;
  int nstat_blocks_ = 0;
  std::vector<void*> allocs_;
  char* arena_ = nullptr;   // one allocation carved by alloc()
  size_t arena_cap_ = 0, arena_used_ = 0, extra_bytes_ = 0;
  int64_t bytes_ = 0, launches_ = 0;
  KArgs<R> ka_;
  size_t smem_flux_ = 0;
  RunState hst_;
  bool uploaded_ = false, flux_ready_ = false;
  // t_stop / step_limit last written to the device (whole-state writes
  // clear limits_known_)
  bool limits_known_ = false;
  double limits_t_stop_ = 0.0;
  long long limits_steps_ = 0;
  double pending_dt_ = -1.0;
  cudaGraph_t graph_ = nullptr;
  cudaGraphExec_t graph_exec_ = nullptr;
  cudaGraph_t graph1_ = nullptr;
  cudaGraphExec_t graph1_exec_ = nullptr;
  cudaEvent_t ev_[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  void* flush_buf_ = nullptr;
  size_t flush_bytes_ = 0;
  KernelTable<R> tab_;

  cudaError_t prepare_timing(int flush) {
    if (!ev_[0])
      for (int k = 0; k < 5; ++k) {
        cudaError_t e = cudaEventCreate(&ev_[k]);
        if (e != cudaSuccess) return e;
      }
    if (flush && !flush_buf_) {
      flush_bytes_ = (size_t)512 << 20;   // 4x the 126 MB L2
      cudaError_t e = cudaMalloc(&flush_buf_, flush_bytes_);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  }
  cudaError_t flush_l2() {
    static int salt = 0;
    return cudaMemsetAsync(flush_buf_, (++salt) & 0xff, flush_bytes_, stream_);
  }
  cudaError_t build_graph1() {
    cudaError_t e = cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    const int64_t l0 = launches_;
    e = launch_step();
    launches_ = l0;
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(stream_, &g);
    if (e != cudaSuccess) { if (g) cudaGraphDestroy(g); return e; }
    if (e2 != cudaSuccess) return e2;
    graph1_ = g;
    return cudaGraphInstantiate(&graph1_exec_, graph1_, 0);
  }

  int steps_launches() const {
    const int topo = Bc_ ? 1 : 0;
    if (hs_.nrk == 2) return 4 + topo;
    int n = 3 + hs_.nrk + 1 + topo;
    const bool fused0 = hs_.a_dirk[0] == 0.0 && hs_.omega_tilde[0] > 0.0;
    for (int i = 0; i < hs_.nrk; ++i)
      if (hs_.omega_tilde[i] > 0.0 && !(i == 0 && fused0)) ++n;
    return n;
  }

  static unsigned long long bits_of(double x) {
    unsigned long long b;
    std::memcpy(&b, &x, sizeof(b));
    return b;
  }

  static constexpr size_t kArenaAlign = 256;
  bool in_arena(const void* p) const {
    return arena_ && (const char*)p >= arena_ && (const char*)p < arena_ + arena_cap_;
  }
  cudaError_t alloc(void** p, size_t bytes) {
    const size_t a = (bytes + kArenaAlign - 1) / kArenaAlign * kArenaAlign;
    if (arena_ && arena_used_ + a <= arena_cap_) {
      *p = arena_ + arena_used_;
      arena_used_ += a;
      bytes_ += (int64_t)bytes;
      return cudaSuccess;
    }
    cudaError_t e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) {
      allocs_.push_back(*p);
      bytes_ += (int64_t)bytes;
    }
    return e;
  }

  // per-tile bytes for the current tile height: activity; wet flags (the
  // batch's, then the single run's two step-parity buffers: 3 x tiles, all
  // "unknown" = 1); static-seed flags (host computed)
  cudaError_t alloc_tiles() {
    const size_t n = (size_t)tiles_x_ * tiles_y_;
    cudaError_t e = alloc((void**)&tile_active_, n);
    if (e == cudaSuccess) e = alloc((void**)&tile_wet_, 3 * n);
    if (e == cudaSuccess) e = alloc((void**)&tile_static_, n);
    if (e == cudaSuccess) e = alloc((void**)&tile_count_, n * sizeof(uint16_t));
    if (e == cudaSuccess) e = cudaMemset(tile_count_, 0, n * sizeof(uint16_t));
    if (e == cudaSuccess) e = cudaMemset(tile_active_, 0, n);
    if (e == cudaSuccess) e = cudaMemset(tile_wet_, 0xff, 3 * n);   // unknown
    if (e == cudaSuccess) {
      const std::vector<uint8_t> ts = tile_static_host();
      e = cudaMemcpy(tile_static_, ts.data(), n, cudaMemcpyHostToDevice);
    }
    return e;
  }
  // tiles with a border cell, a ring-boundary cell or a bottom-source cell
  // (seeds of every check_solve) within n_RK cells
  std::vector<uint8_t> tile_static_host() const {
    const int nx = hs_.nx, ny = hs_.ny, r = hs_.nrk, th = tile_h_;
    std::vector<uint8_t> ts((size_t)tiles_x_ * tiles_y_, 0);
    for (int ty = 0; ty < tiles_y_; ++ty)
      for (int tx = 0; tx < tiles_x_; ++tx) {
        const int j0 = tx * TX - r, j1 = std::min(nx, (tx + 1) * TX) - 1 + r;
        const int k0 = ty * th - r, k1 = std::min(ny, (ty + 1) * th) - 1 + r;
        uint8_t v = (j0 <= 0 || j1 >= nx - 1 || k0 <= 0 || k1 >= ny - 1) ? 1 : 0;
        if (!v && (hs_.p.radial_source_flag || hs_.p.bottom_radial_source_flag))
          for (int k = std::max(k0, 0); k <= std::min(k1, ny - 1) && !v; ++k)
            for (int j = std::max(j0, 0); j <= std::min(j1, nx - 1); ++j) {
              const uint8_t f = hs_.cflags[(size_t)k * nx + j];
              if ((f & 3) == 2 || (f & kFlagBottom)) { v = 1; break; }
            }
        ts[(size_t)ty * tiles_x_ + tx] = v;
      }
    return ts;
  }
  // the single run's wet flags back to "unknown" (the state changed on the
  // host, or a per-call entry point ran kernels that do not keep them)
  cudaError_t reset_wet_flags() {
    const size_t n = (size_t)tiles_x_ * tiles_y_;
    return cudaMemsetAsync(tile_wet_ + n, 0xff, 2 * n, stream_);
  }
  void free_tracked(void* p, size_t bytes) {
    if (in_arena(p)) {   // arena space is not reused; freed with the arena
      bytes_ -= (int64_t)bytes;
      return;
    }
    for (auto it = allocs_.begin(); it != allocs_.end(); ++it)
      if (*it == p) {
        allocs_.erase(it);
        break;
      }
    cudaFree(p);
    bytes_ -= (int64_t)bytes;
  }
  void drop_graphs() {
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (graph_) cudaGraphDestroy(graph_);
    if (graph1_exec_) cudaGraphExecDestroy(graph1_exec_);
    if (graph1_) cudaGraphDestroy(graph1_);
    graph_exec_ = nullptr;
    graph_ = nullptr;
    graph1_exec_ = nullptr;
    graph1_ = nullptr;
  }

  void release() {
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (graph_) cudaGraphDestroy(graph_);
    if (graph1_exec_) cudaGraphExecDestroy(graph1_exec_);
    if (graph1_) cudaGraphDestroy(graph1_);
    for (int k = 0; k < 5; ++k)
      if (ev_[k]) cudaEventDestroy(ev_[k]);
    if (flush_buf_) cudaFree(flush_buf_);
    for (void* p : allocs_) cudaFree(p);
    allocs_.clear();
    if (arena_) cudaFree(arena_);
    arena_ = nullptr;
    if (stage_aos_) cudaFree(stage_aos_);
    stage_aos_ = nullptr;
    if (stream_) cudaStreamDestroy(stream_);
  }

  // host-layout staging buffer, allocated on first use
  cudaError_t ensure_stage() {
    if (stage_aos_) return cudaSuccess;
    const size_t bytes = sizeof(double) * (size_t)hs_.nx * hs_.ny * (hs_.nv + 3);
    cudaError_t e = cudaMalloc((void**)&stage_aos_, bytes);
    if (e == cudaSuccess) bytes_ += (int64_t)bytes;
    return e;
  }

  // a per-cell FP64 host plane into a pitched device plane of R: read and
  // converted by the device where it can read host memory (asynchronous on
  // the run's stream; `src` must stay unchanged until the stream is
  // synchronised), else converted here and copied
  cudaError_t put_plane(R* dst, const std::vector<double>& src) {
    if (pageable_access() && src.size() == (size_t)hs_.nx * hs_.ny) {
      k_plane_to_pitched<R><<<(unsigned)(((size_t)plane_ + 255) / 256), 256, 0, stream_>>>(
          src.data(), dst, hs_.nx, hs_.ny, pitch_);
      ++launches_;
      return cudaGetLastError();
    }
    std::vector<R> buf((size_t)plane_, R(0));
    for (int k = 0; k < hs_.ny; ++k)
      for (int j = 0; j < hs_.nx; ++j) buf[(size_t)k * pitch_ + j] = (R)src[(size_t)k * hs_.nx + j];
    return cudaMemcpy(dst, buf.data(), sizeof(R) * plane_, cudaMemcpyHostToDevice);
  }

  // the flag bytes into their pitched plane (pad columns zero), in order
  // with the run's stream and finished on return: read by the device from
  // the host array where it can, else laid out here and copied
  cudaError_t put_flags() {
    const int nx = hs_.nx, ny = hs_.ny;
    if (pageable_access()) {
      k_bytes_to_pitched<<<(unsigned)(((size_t)plane_ + 255) / 256), 256, 0, stream_>>>(hs_.cflags.data(), cflags_,
                                                                                      nx, ny, pitch_);
      ++launches_;
      cudaError_t e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
      return e;
    }
    std::vector<uint8_t> f((size_t)plane_, 0);
    for (int k = 0; k < ny; ++k)
      for (int j = 0; j < nx; ++j) f[(size_t)k * pitch_ + j] = hs_.cflags[(size_t)k * nx + j];
    cudaError_t e = cudaStreamSynchronize(stream_);
    if (e == cudaSuccess) e = cudaMemcpy(cflags_, f.data(), plane_, cudaMemcpyHostToDevice);
    return e;
  }
  cudaError_t put_plane_d(double* dst, const std::vector<double>& src) {
    std::vector<double> buf((size_t)plane_, 0.0);
    for (int k = 0; k < hs_.ny; ++k)
      for (int j = 0; j < hs_.nx; ++j) buf[(size_t)k * pitch_ + j] = src[(size_t)k * hs_.nx + j];
    return cudaMemcpy(dst, buf.data(), sizeof(double) * plane_, cudaMemcpyHostToDevice);
  }
  cudaError_t get_plane_d(double* out, const double* src) {
    std::vector<double> buf((size_t)plane_);
    cudaError_t e = cudaStreamSynchronize(stream_);
    if (e == cudaSuccess) e = cudaMemcpy(buf.data(), src, sizeof(double) * plane_, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return e;
    for (int k = 0; k < hs_.ny; ++k)
      for (int j = 0; j < hs_.nx; ++j) out[(size_t)k * hs_.nx + j] = buf[(size_t)k * pitch_ + j];
    return cudaSuccess;
  }
  // erosion 0; erodible layer = erodible_fract * (1 - porosity) * thickness
  // (inpout_2d.f90:1983-1986), the thickness uniform or set by set_erodible
  cudaError_t reset_erosion() {
    const size_t N = (size_t)hs_.nx * hs_.ny;
    cudaError_t e = cudaStreamSynchronize(stream_);
    if (e == cudaSuccess) e = cudaMemset(erosion_, 0, sizeof(double) * plane_ * hs_.ns);
    std::vector<double> pl(N);
    for (int i = 0; i < hs_.ns && e == cudaSuccess; ++i) {
      const double f = hs_.erodible_fract[i] * (1.0 - hs_.erodible_porosity);
      for (size_t c = 0; c < N; ++c) pl[c] = f * (erodible_user_.empty() ? hs_.erodible_init : erodible_user_[c]);
      e = put_plane_d(erodible_ + (size_t)i * plane_, pl);
    }
    return e;
  }
  // B_cent and its topography terms as set up
  cudaError_t reset_topography() {
    cudaError_t e = cudaStreamSynchronize(stream_);
    if (e == cudaSuccess) e = put_plane_d(Bc_, hs_.B);
    if (e == cudaSuccess && hs_.Bx.empty()) {
      // a set-up without host topography terms: derive them from Bc_
      TopoPlanes<R> tp;
      for (int i = 0; i < 8; ++i) tp.p[i] = geo_[i];
      const int64_t n = (int64_t)hs_.nx * hs_.ny;
      k_topography_setup<R><<<(unsigned)((n + 255) / 256), 256, 0, stream_>>>(
          Bc_, hs_.nx, hs_.ny, (int64_t)pitch_, hs_.dx, hs_.dy, hs_.p.slope_correction_flag ? 1 : 0, tp);
      ++launches_;
      return cudaGetLastError();
    }
    const std::vector<double>* gsrc[8] = {&hs_.Bx, &hs_.By, &hs_.Bxx, &hs_.Bxy, &hs_.Byy, &hs_.gc, &hs_.dgcx, &hs_.dgcy};
    for (int i = 0; i < 8 && e == cudaSuccess; ++i)
      if (geo_[i]) e = put_plane(geo_[i], *gsrc[i]);
    return e;
  }
  cudaError_t launch_topography() {
    ++launches_;
    const int64_t n = (int64_t)hs_.nx * hs_.ny;
    return launch_step_kernel(k_topography<R>, dim3((unsigned)((n + 255) / 256)), dim3(256), 0, stream_, ka_.g.pdl, ka_);
  }

  static R thr(double x) {
    if constexpr (sizeof(R) == 8) return x;
    else return float_below(x);
  }

  template <class T>
  void fill_phys(Phys<T>& P) {
    const SflowParams& p = hs_.p;
    std::memset(&P, 0, sizeof(P));
    P.nv = hs_.nv; P.ns = hs_.ns; P.nrk = hs_.nrk;
    P.gas = p.gas_flag; P.liquid = p.liquid_flag; P.energy = p.energy_flag; P.alpha = p.alpha_flag;
    P.rheo = p.rheology_flag; P.rheo_model = p.rheology_model; P.slope_corr = p.slope_correction_flag;
    P.curv = p.curvature_term_flag; P.settling = p.settling_flag; P.entrain = p.entrainment_flag;
    P.collective = p.collective_settling_flag; P.radial_source = p.radial_source_flag;
    P.scheme = p.solver_scheme;
    P.eps_sing_d = hs_.eps_sing;
    auto th = [&](double x) -> T {
      if constexpr (sizeof(T) == 8) return x;
      else return float_below(x);
    };
    P.thr_eps = th(DBL_EPSILON);
    P.thr_eps_sing = th(hs_.eps_sing);
    P.thr_neg1e7 = th(-1.0e-7);
    P.thr_neg1e10 = th(-1.0e-10);
    P.thr_1em10 = th(1.0e-10);
    P.thr_1em7 = th(1.0e-7);
    P.thr_1em3 = th(1.0e-3);
    P.thr_273 = (T)273.0;
    P.eps_sing4 = (T)hs_.eps_sing4;
    P.inv_eps_sing = (T)(1.0 / hs_.eps_sing);
    P.sqrt2 = (T)std::sqrt(2.0);
    P.grav = (T)p.grav; P.pres = (T)p.pres; P.inv_pres = (T)(1.0 / p.pres);
    P.sp_heat_a = (T)p.sp_heat_a; P.sp_gas_const_a = (T)p.sp_gas_const_a; P.T_ambient = (T)p.T_ambient;
    P.rho_a_amb = (T)hs_.rho_a_amb;
    P.rho_l = (T)p.rho_l; P.inv_rho_l = (T)(p.rho_l != 0.0 ? 1.0 / p.rho_l : 0.0); P.sp_heat_l = (T)p.sp_heat_l;
    for (int i = 0; i < kMaxSolid; ++i) {
      P.rho_s[i] = (T)p.rho_s[i];
      P.inv_rho_s[i] = (T)(p.rho_s[i] != 0.0 ? 1.0 / p.rho_s[i] : 0.0);
      P.sp_heat_s[i] = (T)p.sp_heat_s[i];
      P.alphas_source[i] = (T)p.alphas_source[i];
      P.diam_s[i] = (T)p.diam_s[i];
    }
    P.h_source = (T)hs_.h_source; P.vel_source = (T)p.vel_source; P.T_source = (T)p.T_source;
    P.cell_area = (T)(hs_.dx * hs_.dy);
    P.src_rho_m = (T)hs_.src_rho_m; P.src_cp_mix = (T)hs_.src_cp_mix;
    P.mu = (T)p.mu; P.xi = (T)p.xi; P.friction_factor = (T)p.friction_factor;
    P.mu_s = (T)p.mu_s; P.mu_2 = (T)p.mu_2; P.I_0 = (T)p.I_0; P.muI_inf = (T)p.muI_inf;
    P.kin_visc_c = (T)hs_.kin_visc_c; P.loss_rate = (T)p.loss_rate;
    P.alphastot_min = (T)p.alphastot_min; P.max_packing = (T)p.maximum_solid_packing;
    P.A_drag = (T)p.A_drag; P.B_drag = (T)p.B_drag;
    P.coeff_porosity = (T)hs_.coeff_porosity; P.rho_c_sub = (T)hs_.rho_c_sub; P.T_erodible = (T)hs_.T_erodible;
    P.erodible_porosity = (T)hs_.erodible_porosity;
    P.erosion_coeff = (T)p.erosion_coeff;
    for (int i = 0; i < kMaxSolid; ++i) P.erodible_fract[i] = (T)hs_.erodible_fract[i];
    P.erodible_deposit = p.erodible_deposit_flag ? 1 : 0;
    P.topo_change = p.topo_change_flag ? 1 : 0;
    P.bottom_source = p.bottom_radial_source_flag ? 1 : 0;
    P.exchange = hs_.exchange;
    P.newton64 = p.fp32_newton_fp64 ? 1 : 0;
    P.nodata = 0;
    for (size_t c = 0; c < hs_.cflags.size(); ++c)
      if (hs_.cflags[c] & kFlagNodata) { P.nodata = 1; break; }
    // levels: a float h satisfies h >= level exactly when (double)h does,
    // with level rounded up to the next float
    auto up = [&](double x) -> T {
      if constexpr (sizeof(T) == 8) return x;
      else {
        float f = (float)x;
        if ((double)f < x) f = std::nextafterf(f, INFINITY);
        return f;
      }
    };
    P.n_thk = hs_.n_thk;
    P.n_dyn = hs_.n_dyn;
    for (int i = 0; i < SFLOW_MAX_LEVELS; ++i) {
      P.thk_levels[i] = up(hs_.thk_levels[i]);
      P.dyn_levels[i] = up(hs_.dyn_levels[i]);
    }
  }

  void fill_args() {
    const SflowParams& p = hs_.p;
    std::memset(&ka_, 0, sizeof(ka_));
    Grid<R>& g = ka_.g;
    g.nx = hs_.nx; g.ny = hs_.ny; g.pitch = pitch_; g.plane = plane_;
    g.tiles_x = tiles_x_; g.tiles_y = tiles_y_;
    g.x0 = p.x0; g.y0 = p.y0; g.dx = hs_.dx; g.dy = hs_.dy;
    g.rdx = (R)hs_.dx; g.rdy = (R)hs_.dy;
    g.x0r = (R)p.x0; g.y0r = (R)p.y0;
    g.dx2 = (R)(hs_.dx / 2.0); g.dy2 = (R)(hs_.dy / 2.0);
    g.one_by_dx = (R)(1.0 / hs_.dx); g.one_by_dy = (R)(1.0 / hs_.dy);
    g.rc = (R)p.reconstr_coeff; g.theta = (R)p.theta;
    g.cfl_dx = (R)(p.cfl * hs_.dx); g.cfl_dy = (R)(p.cfl * hs_.dy);
    for (int i = 0; i < hs_.nv; ++i) g.limiter[i] = p.limiter[i];
    g.limiter[hs_.nv] = p.limiter[1];
    g.limiter[hs_.nv + 1] = p.limiter[2];
    g.lim_all = g.limiter[0];
    for (int i = 1; i < hs_.nv + 2; ++i)
      if (g.limiter[i] != g.lim_all) g.lim_all = -1;
    g.cfl = p.cfl; g.max_dt = p.max_dt;
    // programmatic dependent launch of the step kernels (SFLOW_PDL=0: off)
    const char* pdl_env = std::getenv("SFLOW_PDL");
    g.pdl = (pdl_env && pdl_env[0] == '0') ? 0 : 1;
    fill_phys(ka_.pr);
    fill_phys(ka_.pd);
    for (int sd = 0; sd < 4; ++sd)
      for (int i = 0; i < kMaxVars; ++i) {
        ka_.bc.flag[sd][i] = p.bc[sd][i].flag;
        ka_.bc.value[sd][i] = (R)p.bc[sd][i].value;
      }
    g.k_off = hs_.row0;
    g.own_lo = hs_.own_lo;
    g.own_hi = hs_.own_hi;
    g.whole = (hs_.own_lo == 0 && hs_.own_hi == hs_.ny) ? 1 : 0;
    g.dry_bc = 1;
    for (int sd = 0; sd < 4; ++sd) {
      if ((sd < 2 && hs_.nx < 2) || (sd >= 2 && hs_.ny < 2)) continue;
      for (int i = 0; i < hs_.nv; ++i)
        if (!(p.bc[sd][i].flag == 1 && p.bc[sd][i].value == 0.0)) g.dry_bc = 0;
    }
    ka_.q = q_; ka_.rd = rd_; ka_.rn = rn_; ka_.qs = qs_;
    for (int i = 0; i < 16; ++i) { ka_.tableau_at[i] = hs_.a_tilde[i]; ka_.tableau_ad[i] = hs_.a_dirk[i]; }
    for (int i = 0; i < 4; ++i) { ka_.omega_t[i] = hs_.omega_tilde[i]; ka_.omega[i] = hs_.omega[i]; }
    for (int i = 0; i < 8; ++i) ka_.geo[i] = geo_[i];
    ka_.cflags = cflags_; ka_.arc = arc_; ka_.mask = mask_; ka_.tile_active = tile_active_;
    ka_.tile_wet = tile_wet_;
    ka_.tile_wet_step = tile_wet_ + (size_t)tiles_x_ * tiles_y_;
    ka_.tile_static = tile_static_;
    ka_.tile_count = tile_count_;
    ka_.hmax = hmax_; ka_.pdynmax = pdynmax_; ka_.mvmax = mvmax_; ka_.st = st_;
    ka_.deposit = deposit_;
    ka_.erosion = erosion_;
    ka_.erodible = erodible_;
    ka_.Bc = Bc_;
    ka_.bfrac = bfrac_;
    ka_.bsrc_tab = bsrc_tab_;
    ka_.vuln = vuln_;
    ka_.vuln_words = vuln_words_;
    ka_.take_last = hs_.take_last;
  }

  void init_state_host() {
    const SflowParams& p = hs_.p;
    std::memset(&hst_, 0, sizeof(hst_));
    hst_.t = p.t_start;
    hst_.dt = hst_.dt_old = hst_.dt_old_old = p.dt0;
    hst_.t_output = p.t_start + p.dt_output;
    hst_.t_end = p.t_end;
    hst_.t_stop = p.t_end;
    hst_.t_prev = p.t_start;
    hst_.dtmin_bits = bits_of(1.0e300);
    hst_.step_limit = (long long)1 << 62;
    for (int i = 0; i < 4; ++i) hst_.tp[i] = hs_.time_param[i];
    hst_.pi_g = hs_.pi_g;
  }

  cudaError_t set_limits(double t_stop, int64_t step_limit) {
    // write t_stop and step_limit into the device state without touching
    // the rest (the device owns t, dt and the counters); skipped when the
    // device already holds these values (only the host writes them)
    long long lim = step_limit < 0 ? ((long long)1 << 62) : (long long)step_limit;
    if (limits_known_ && t_stop == limits_t_stop_ && lim == limits_steps_) return cudaSuccess;
    cudaError_t e = cudaMemcpyAsync(&st_->t_stop, &t_stop, sizeof(double), cudaMemcpyHostToDevice, stream_);
    if (e != cudaSuccess) return e;
    static_assert(sizeof(lim) == sizeof(st_->step_limit), "step_limit size");
    e = cudaMemcpyAsync(&st_->step_limit, &lim, sizeof(lim), cudaMemcpyHostToDevice, stream_);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(stream_);
    if (e != cudaSuccess) return e;
    limits_known_ = true;
    limits_t_stop_ = t_stop;
    limits_steps_ = lim;
    return cudaSuccess;
  }


  cudaError_t set_smem_attr() { return tab_.set_smem(smem_flux_); }

  cudaError_t launch_mask(int solve_all) {
    ++launches_;
    return tab_.mask(ka_, dim3(tiles_x_, tiles_y_), stream_, solve_all);
  }
  cudaError_t launch_flux(int want_dt) {
    ++launches_;
    return tab_.flux(ka_, dim3(tiles_x_, tiles_y_), smem_flux_, stream_, q_, rd_, want_dt);
  }
  // mode -1: full fused epilogue; 0: stage only; 1: erosion only; 2: maps only
  cudaError_t launch_stage2(int mode) {
    ++launches_;
    return tab_.stage2(ka_, dim3(tiles_x_, tiles_y_), stream_, mode);
  }

  // one step; with a changing topography its terms are recomputed after it
  cudaError_t launch_step() {
    cudaError_t e;
    if (hs_.nrk == 2) {
      e = launch_mask(2);
      if (e == cudaSuccess) e = launch_flux(1);
      if (e == cudaSuccess) {
        e = launch_step_kernel(k_dt, dim3(1), dim3(1), 0, stream_, ka_.g.pdl, st_, hs_.p.max_dt);
        ++launches_;
      }
      if (e == cudaSuccess) e = launch_stage2(-1);
    } else {
      e = launch_step_general();
    }
    if (e == cudaSuccess && Bc_) e = launch_topography();
    return e;
  }

  // N_RK = 1, 3, 4: the timestep pass at q0 (fused with the stage-1 flux
  // when stage 1 is explicit and has a flux), then per stage the pointwise
  // stage kernel and, when omega_tilde > 0, the flux at the stage state.
  cudaError_t launch_step_general() {
    const int nv = hs_.nv;
    const int64_t sv = (int64_t)nv * plane_;
    const dim3 grid(tiles_x_, tiles_y_);
    const bool fused0 = hs_.a_dirk[0] == 0.0 && hs_.omega_tilde[0] > 0.0;
    cudaError_t e = launch_mask(0);
    if (e != cudaSuccess) return e;
    ++launches_;
    e = tab_.flux(ka_, grid, smem_flux_, stream_, q_, fused0 ? rd_ : nullptr, 1);
    if (e != cudaSuccess) return e;
    e = launch_step_kernel(k_dt, dim3(1), dim3(1), 0, stream_, ka_.g.pdl, st_, hs_.p.max_dt);
    ++launches_;
    if (e != cudaSuccess) return e;
    for (int i = 0; i < hs_.nrk; ++i) {
      ++launches_;
      e = tab_.stage(ka_, grid, stream_, i);
      if (e != cudaSuccess) return e;
      if (hs_.omega_tilde[i] > 0.0 && !(i == 0 && fused0)) {
        ++launches_;
        e = tab_.flux(ka_, grid, smem_flux_, stream_, qs_, rd_ + i * sv, 0);
        if (e != cudaSuccess) return e;
      }
    }
    ++launches_;
    return tab_.assemble(ka_, grid, stream_);
  }

  cudaError_t build_graph() {
    cudaError_t e = cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    const int64_t l0 = launches_;
    for (int i = 0; i < kChunk; ++i) {
      e = launch_step();
      if (e != cudaSuccess) {
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(stream_, &g);
        if (g) cudaGraphDestroy(g);
        return e;
      }
    }
    launches_ = l0;   // captured launches are counted when replayed
    e = cudaStreamEndCapture(stream_, &graph_);
    if (e != cudaSuccess) return e;
    return cudaGraphInstantiate(&graph_exec_, graph_, 0);
  }

  cudaError_t dispatch_init_maps(unsigned blocks) {
    ++launches_;
    return tab_.init_maps(ka_, blocks, stream_);
  }
  cudaError_t dispatch_qp(unsigned blocks) {
    ++launches_;
    return tab_.qp(ka_, blocks, stream_, stage_aos_);
  }
  cudaError_t dispatch_stats() {
    cudaError_t e = tab_.stats(ka_, nstat_blocks_, stream_, stat_part_);
    if (e != cudaSuccess) return e;
    k_stats_final<<<4, 256, 0, stream_>>>(stat_part_, nstat_blocks_, stat_out_);
    launches_ += 2;
    return cudaGetLastError();
  }
};

template <class R>
SolverBase* make_solver_impl(const HostSetup& s, std::string& err) {
  Solver<R>* sv = new Solver<R>(s);
  int rc = sv->init();
  if (rc != SFLOW_OK) {
    err = sv->err_;
    delete sv;
    return nullptr;
  }
  return sv;
}

}  // namespace sflow

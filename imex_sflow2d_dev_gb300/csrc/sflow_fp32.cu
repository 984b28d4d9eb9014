// sflow_fp32.cu -- FP32 bulk form of the solver: FP32 state, reconstruction,
// fluxes and explicit terms; FP64 implicit friction solve; FP64-equivalent
// wet/dry threshold tests; FP64 log sums.
#include "sflow_batch.cuh"
#include "sflow_solver.cuh"

namespace sflow {
SolverBase* make_solver_fp32(const HostSetup& s, std::string& err) {
  return make_solver_impl<float>(s, err);
}
BatchBase* make_batch_fp32(int max_runs, int64_t max_tiles, std::string& err) {
  return make_batch_impl<float>(max_runs, max_tiles, err);
}

// Self-check of f2d_exact / d2f_rn against the hardware conversions of
// this unit (compiled like the FP32 form: flush-to-zero): n seeded float and
// double bit patterns -- every exponent, rounding ties, the float range
// edges -- converted both ways; NaNs compare equal whatever their payload.
__device__ __forceinline__ unsigned long long conv_hash(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__global__ void k_check_conversions(long long n, unsigned long long seed, unsigned long long* bad) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long h = conv_hash(seed + (unsigned long long)i);
    // float -> double: any bit pattern
    const float f = __uint_as_float((unsigned)h);
    const double a = (double)f, b = f2d_exact(f);
    // subnormal floats: the helper flushes them (as the FP32 form does); the
    // hardware conversion may keep them
    const bool sub = ((unsigned)h & 0x7f800000u) == 0u;
    const bool fsame = (a == b && signbit(a) == signbit(b)) || (isnan(a) && isnan(b)) ||
                       (sub && b == 0.0 && signbit(b) == signbit(a));
    const bool fbad = !fsame;
    // double -> float: exponents around the float range, ties on every
    // fourth value
    unsigned long long db = h;
    const unsigned long long kind = (h >> 60) & 3ull;
    unsigned long long ex = 896ull - 40ull + ((h >> 40) % 336ull);   // float range +- margins
    if (kind == 0ull) ex = (h >> 40) & 0x7ffull;                      // any exponent
    db = (db & 0x800fffffffffffffull) | (ex << 52);
    if (kind == 1ull) db = (db & ~0x1fffffffull) | 0x10000000ull;     // exact tie
    const double d = __longlong_as_double((long long)db);
    const float c = (float)d, e = d2f_rn(d);
    // results below the float normal range: flushed by the helper, by the
    // hardware conversion possibly not
    const bool tiny = fabs(d) < 1.1754943508222875e-38;
    const bool dsame = __float_as_uint(c) == __float_as_uint(e) || (isnan(c) && isnan(e)) ||
                       (tiny && e == 0.0f && signbit(e) == signbit(c));
    const bool dbad = !dsame;
    if (fbad || dbad) atomicAdd(bad, 1ull);
  }
}
int check_conversions(long long n, unsigned long long seed, long long* mismatches) {
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return SFLOW_ECUDA;
  cudaMemset(d, 0, sizeof(*d));
  k_check_conversions<<<1024, 256>>>(n, seed, d);
  unsigned long long h = 0;
  const cudaError_t e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return SFLOW_ECUDA;
  *mismatches = (long long)h;
  return SFLOW_OK;
}
}  // namespace sflow

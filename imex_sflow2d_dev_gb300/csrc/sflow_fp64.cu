// sflow_fp64.cu -- plain FP64 form of the solver (compiled with --fmad=false
// so that the arithmetic follows the reference operation order exactly).
#include "sflow_batch.cuh"
#include "sflow_solver.cuh"

namespace sflow {
SolverBase* make_solver_fp64(const HostSetup& s, std::string& err) {
  return make_solver_impl<double>(s, err);
}
BatchBase* make_batch_fp64(int max_runs, int64_t max_tiles, std::string& err) {
  return make_batch_impl<double>(max_runs, max_tiles, err);
}

// The library's FP64 pow / log / cos (sflow_math.h) evaluated on the device,
// and CUDA's own functions beside them, for the test that compares the
// device bits with the host bits of the same functions.
__global__ void k_eval_math(int which, long long n, const double* x, const double* y, double* out) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double r;
    switch (which) {
      case 0: r = sfm_pow(x[i], y[i]); break;
      case 1: r = sfm_log(x[i]); break;
      case 2: r = sfm_cos(x[i]); break;
      case 3: r = pow(x[i], y[i]); break;
      case 4: r = log(x[i]); break;
      default: r = cos(x[i]); break;
    }
    out[i] = r;
  }
}
int eval_math(int which, long long n, const double* x, const double* y, double* out) {
  double *dx = nullptr, *dy = nullptr, *dout = nullptr;
  const size_t bytes = (size_t)(n > 0 ? n : 1) * sizeof(double);
  int rc = SFLOW_OK;
  if (cudaMalloc(&dx, bytes) != cudaSuccess || cudaMalloc(&dy, bytes) != cudaSuccess ||
      cudaMalloc(&dout, bytes) != cudaSuccess) {
    rc = SFLOW_ENOMEM;
  } else if (n > 0) {
    cudaMemcpy(dx, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice);
    if (y) cudaMemcpy(dy, y, (size_t)n * sizeof(double), cudaMemcpyHostToDevice);
    else cudaMemset(dy, 0, (size_t)n * sizeof(double));
    k_eval_math<<<608, 256>>>(which, n, dx, dy, dout);
    if (cudaMemcpy(out, dout, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) rc = SFLOW_ECUDA;
  }
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(dout);
  return rc;
}
}  // namespace sflow

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
}  // namespace sflow

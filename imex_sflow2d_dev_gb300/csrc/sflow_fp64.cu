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
}  // namespace sflow

// sflow_fp64.cu -- plain FP64 form of the solver (compiled with --fmad=false
// so that the arithmetic follows the reference operation order exactly).
#include "sflow_solver.cuh"

namespace sflow {
SolverBase* make_solver_fp64(const HostSetup& s, std::string& err) {
  return make_solver_impl<double>(s, err);
}
}  // namespace sflow

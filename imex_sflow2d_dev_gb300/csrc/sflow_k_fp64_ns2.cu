// sflow_k_fp64_ns2.cu -- kernels of the FP64 form with 2 solid classes.
#include "sflow_table_impl.cuh"

namespace sflow {
template KernelTable<double> make_table<double, 2>();
}  // namespace sflow

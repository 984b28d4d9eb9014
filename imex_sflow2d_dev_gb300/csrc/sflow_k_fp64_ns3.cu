// sflow_k_fp64_ns3.cu -- kernels of the FP64 form with 3 solid classes.
#include "sflow_table_impl.cuh"

namespace sflow {
template KernelTable<double> make_table<double, 3>();
}  // namespace sflow

// sflow_k_fp64_ns1.cu -- kernels of the FP64 form with 1 solid class.
#include "sflow_table_impl.cuh"

namespace sflow {
template KernelTable<double> make_table<double, 1>();
}  // namespace sflow

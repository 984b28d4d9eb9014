// sflow_k_fp32_ns2.cu -- kernels of the FP32 form with 2 solid classes.
#include "sflow_table_impl.cuh"

namespace sflow {
template KernelTable<float> make_table<float, 2>();
}  // namespace sflow

// sflow_k_fp32_ns1.cu -- kernels of the FP32 form with 1 solid class.
#include "sflow_table_impl.cuh"

namespace sflow {
template KernelTable<float> make_table<float, 1>();
}  // namespace sflow

// sflow_k_fp32_ns3.cu -- kernels of the FP32 form with 3 solid classes.
#include "sflow_table_impl.cuh"

namespace sflow {
template KernelTable<float> make_table<float, 3>();
}  // namespace sflow

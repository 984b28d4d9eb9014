// sflow_k_fp32_ns3_t4.cu -- 32 x 4 tiled kernels of the FP32 form with
// 3 solid classes.
#include "sflow_table_impl.cuh"

namespace sflow {
template void fill_tile_entries<float, 3, 4>(KernelTable<float>&);
}  // namespace sflow

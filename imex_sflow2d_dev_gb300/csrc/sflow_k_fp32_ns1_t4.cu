// sflow_k_fp32_ns1_t4.cu -- 32 x 4 tiled kernels of the FP32 form with
// 1 solid class.
#include "sflow_table_impl.cuh"

namespace sflow {
template void fill_tile_entries<float, 1, 4>(KernelTable<float>&);
}  // namespace sflow

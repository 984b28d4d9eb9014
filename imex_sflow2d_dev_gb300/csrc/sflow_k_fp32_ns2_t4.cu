// sflow_k_fp32_ns2_t4.cu -- 32 x 4 tiled kernels of the FP32 form with
// 2 solid classes.
#include "sflow_table_impl.cuh"

namespace sflow {
template void fill_tile_entries<float, 2, 4>(KernelTable<float>&);
}  // namespace sflow

// sflow_k_fp32_ns3.cu -- kernels of the FP32 form with 3 solid classes:
// the entries independent of the tile height and the 32 x 8 tiled kernels.
#include "sflow_table_impl.cuh"

namespace sflow {
template KernelTable<float> make_table<float, 3>();
template void fill_tile_entries<float, 3, 8>(KernelTable<float>&);
}  // namespace sflow

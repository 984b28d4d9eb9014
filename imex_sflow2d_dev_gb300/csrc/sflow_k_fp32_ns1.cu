// sflow_k_fp32_ns1.cu -- kernels of the FP32 form with 1 solid class:
// the entries independent of the tile height and the 32 x 8 tiled kernels.
#include "sflow_table_impl.cuh"

namespace sflow {
template KernelTable<float> make_table<float, 1>();
template void fill_tile_entries<float, 1, 8>(KernelTable<float>&);
}  // namespace sflow

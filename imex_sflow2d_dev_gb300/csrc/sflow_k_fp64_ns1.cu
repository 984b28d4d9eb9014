// sflow_k_fp64_ns1.cu -- kernels of the FP64 form with 1 solid class:
// the entries independent of the tile height and the 32 x 8 tiled kernels.
#include "sflow_table_impl.cuh"

namespace sflow {
template KernelTable<double> make_table<double, 1>();
template void fill_tile_entries<double, 1, 8>(KernelTable<double>&);
}  // namespace sflow

// sflow_k_fp64_ns3.cu -- kernels of the FP64 form with 3 solid classes:
// the entries independent of the tile height and the 32 x 8 tiled kernels.
#include "sflow_table_impl.cuh"

namespace sflow {
template KernelTable<double> make_table<double, 3>();
template void fill_tile_entries<double, 3, 8>(KernelTable<double>&);
}  // namespace sflow

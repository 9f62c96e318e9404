// Plain-FP64 instantiations of the advance kernel (FP64 gating).
#include "kernels.cu"
namespace gbrkc {
template int launch_pool<double>(int, const PoolView<double> &, int, int, int, size_t, void *, double, int, int, int);
template int prepare_pool_kernel<double>(int, int, size_t);
template int cluster_capacity<double>(int, int, size_t);
template int grid_capacity<double>(int);
template int launch_mega<double>(const MegaView<double> &, int, size_t, void *, double, int, int, int);
template int prepare_mega_kernel<double>(size_t, int *);
}  // namespace gbrkc

// Mixed-precision instantiations of the advance kernel (FP32 gating, FP32
// channel currents and b accumulation; FP64 voltage, stages and controller).
#include "kernels.cu"
namespace gbrkc {
template int launch_pool<float>(int, const PoolView<float> &, int, int, int, size_t, void *, double, int, int, int);
template int prepare_pool_kernel<float>(int, int, size_t);
template int cluster_capacity<float>(int, int, size_t);
template int grid_capacity<float>(int);
template int launch_mega<float>(const MegaView<float> &, int, size_t, void *, double, int, int, int);
template int prepare_mega_kernel<float>(size_t, int *);
}  // namespace gbrkc

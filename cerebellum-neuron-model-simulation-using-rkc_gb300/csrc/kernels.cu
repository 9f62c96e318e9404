// The advance kernel: one launch advances every system of a pool by n_iv
// output intervals (or initialises them), entirely on the device.  Teams of
// 4 or 32 lanes take many small systems per block; a whole block takes one
// large system at a time and loops over its share of systems (persistent).
//
// Built with -fmad=false (see integrator.cuh).  R selects FP64 or FP32
// gating; the instantiations live in kernels_fp64.cu / kernels_fp32.cu.
#include <cuda_runtime.h>

#include "integrator.cuh"

namespace gbrkc {

template <int CT, typename R, int TS>
__global__ void __launch_bounds__(256, 1) k_advance(const __grid_constant__ PoolView<R> P, double t0, int n_iv,
                                                 int iv0, int init) {
  extern __shared__ __align__(16) double smem[];
  if (TS == TEAM_BLOCK) {
    BlockTeam tm;
    for (int s = blockIdx.x; s < P.nsys; s += gridDim.x) {
      run_system<CT, R, BlockTeam>(P, tm, s, smem, t0, n_iv, iv0, init != 0);
      __syncthreads();
    }
  } else {
    constexpr int T = TS > 0 ? TS : 1;
    const int tiles = blockDim.x / T, tile = threadIdx.x / T;
    TileTeam<TS> tm;
    tm.r = threadIdx.x % T;
    tm.mask = (T == 32) ? 0xffffffffu : (((1u << T) - 1u) << ((threadIdx.x & 31) / T * T));
    // thread teams need no warp-level synchronisation at all
    if (T == 1) tm.mask = 1u << (threadIdx.x & 31);
    double *my = smem + (long)tile * P.ws_tile_doubles;
    for (int s = blockIdx.x * tiles + tile; s < P.nsys; s += gridDim.x * tiles)
      run_system<CT, R, TileTeam<TS>>(P, tm, s, my, t0, n_iv, iv0, init != 0);
  }
}

template <int CT, typename R>
static const void *kernel_for(int team) {
  switch (team) {
    case TEAM_THREAD: return (const void *)k_advance<CT, R, TEAM_THREAD>;
    case TEAM_TILE4: return (const void *)k_advance<CT, R, TEAM_TILE4>;
    case TEAM_WARP: return (const void *)k_advance<CT, R, TEAM_WARP>;
    default: return (const void *)k_advance<CT, R, TEAM_BLOCK>;
  }
}

template <typename R>
static const void *kernel_ptr(int type, int team) {
  switch (type) {
    case GR: return kernel_for<GR, R>(team);
    case GO: return kernel_for<GO, R>(team);
    case PKJ: return kernel_for<PKJ, R>(team);
    default: return kernel_for<IO, R>(team);
  }
}

template <typename R>
int prepare_pool_kernel(int type, int team, size_t smem) {
  const void *k = kernel_ptr<R>(type, team);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
  }
  return 0;
}

template <typename R>
int launch_pool(int type, const PoolView<R> &P, int team, int grid, int block, size_t smem, void *stream,
                double t0, int n_iv, int iv0, int init) {
  const void *k = kernel_ptr<R>(type, team);
  PoolView<R> Pc = P;
  void *args[] = {(void *)&Pc, (void *)&t0, (void *)&n_iv, (void *)&iv0, (void *)&init};
  cudaError_t e = cudaLaunchKernel(k, dim3(grid), dim3(block), args, smem, (cudaStream_t)stream);
  return (int)e;
}

}  // namespace gbrkc

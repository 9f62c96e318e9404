#include <type_traits>
// The advance kernels.  k_advance: one launch advances every system of one
// pool by n_iv output intervals (or initialises them), entirely on the
// device.  Single lanes take the tiniest systems (one system per thread),
// teams of 4 or 32 lanes small ones; a whole block takes one large system at
// a time and loops over its share of systems.  k_mega: one persistent launch
// for all pools, every CTA a role pulling systems from its role's queue.
//
// Built with -fmad=false (see integrator.cuh).  R selects FP64 or FP32
// gating; the instantiations live in kernels_fp64.cu / kernels_fp32.cu.
#include <algorithm>
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "integrator.cuh"
#include "lane_sys.cuh"

namespace gbrkc {

template <int CT, typename R, int TS>
__global__ void __launch_bounds__(256, 1) k_advance(const __grid_constant__ PoolView<R> P, double t0, int n_iv,
                                                 int iv0, int init) {
  extern __shared__ __align__(16) double smem[];
  if (TS == TEAM_THREAD || TS == TEAM_LANE4) {
    // the first P.lanes lanes of warp w of block b start at system
    // P.lanes (w * grid + b) + lane: the first warps of every block are
    // filled before any block's later warps
    const int first = (((int)threadIdx.x >> 5) * (int)gridDim.x + (int)blockIdx.x) * P.lanes + ((int)threadIdx.x & 31);
    const int stride = (int)gridDim.x * (MEGA_BLOCK / 32) * P.lanes;
    if (TS == TEAM_LANE4)
      run_lanes_regs<CT, R, MEGA_BLOCK, 4>(P, nullptr, first, stride, smem, t0, n_iv, iv0, init != 0);
    else
      run_lanes<CT, R, MEGA_BLOCK>(P, nullptr, first, stride, smem, t0, n_iv, iv0, init != 0);
  } else if (TS == TEAM_BLOCK) {
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
    double *my = smem + (long)tile * P.ws_tile_doubles;
    for (int s = blockIdx.x * tiles + tile; s < P.nsys; s += gridDim.x * tiles)
      run_system<CT, R, TileTeam<TS>>(P, tm, s, my, t0, n_iv, iv0, init != 0);
  }
}

// One large system per thread-block cluster of C CTAs (ClusterTeam): the
// cluster takes systems cid, cid + nclusters, ...
template <int CT, typename R, int C>
__global__ void __launch_bounds__(CLUSTER_BLOCK, 1) k_advance_cluster(const __grid_constant__ PoolView<R> P, double t0,
                                                                       int n_iv, int iv0, int init) {
  namespace cg = cooperative_groups;
  extern __shared__ __align__(16) double smem[];
  __shared__ double *s_bases[C];
  cg::cluster_group cl = cg::this_cluster();
  if (threadIdx.x < C) s_bases[threadIdx.x] = cl.map_shared_rank(smem, (int)threadIdx.x);
  cl.sync();
  const ClusterTeam<C> tm{(int)cl.block_rank(), s_bases, P.ws_tile_doubles};
  const int ncl = gridDim.x / C, cid = blockIdx.x / C;
  for (int s = cid; s < P.nsys; s += ncl) run_system<CT, R, ClusterTeam<C>>(P, tm, s, smem, t0, n_iv, iv0, init != 0);
  // no CTA leaves while a peer may still reach its shared memory
  cl.sync();
}

// One large system over every CTA of a cooperative launch (GridTeam): all
// CTAs take the pool's systems one after another.
template <int CT, typename R>
__global__ void __launch_bounds__(GRID_BLOCK, 1) k_advance_grid(const __grid_constant__ PoolView<R> P, double t0,
                                                                 int n_iv, int iv0, int init) {
  extern __shared__ __align__(16) double grid_smem[];
  __shared__ double s_wp[GRID_MAX_ROWS * 8];
  __shared__ double s_res;
  __shared__ unsigned long long s_epoch, s_lepoch;
  if (threadIdx.x == 0) s_epoch = s_lepoch = 0;     // counter and flags are zeroed before every launch
  __syncthreads();
  // the operator rows' copy: [rl] 1/Cm, [rl * maxdeg] g, [rl] counts, [rl * maxdeg] columns
  const long rl = P.grid_rl, md = P.grid_maxdeg;
  double *linv = grid_smem, *lg = grid_smem + rl;
  int *lcnt = (int *)(lg + rl * md), *lcol = lcnt + rl;
  const GridTeam tm{(GridBarrier *)P.grid_bar, P.grid_red, s_wp, &s_res, &s_epoch, P.grid_bw, P.grid_light,
                    P.grid_maxdeg, linv, lg, lcnt, lcol, P.grid_nbr, P.grid_flags, &s_lepoch};
  for (int s = 0; s < P.nsys; s++) run_system<CT, R, GridTeam>(P, tm, s, nullptr, t0, n_iv, iv0, init != 0);
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// a role of tile teams: every tile repeatedly takes the next system
template <int CT, typename R, int TS>
__device__ __forceinline__ void role_tiles(const PoolView<R> &P, int *q, double *smem, double t0, int n_iv,
                                           int iv0, int init) {
  const int tile = threadIdx.x / TS;
  TileTeam<TS> tm;
  tm.r = threadIdx.x % TS;
  tm.mask = (TS == 32) ? 0xffffffffu : (((1u << TS) - 1u) << ((threadIdx.x & 31) / TS * TS));
  double *my = smem + (long)tile * P.ws_tile_doubles;
  for (;;) {
    int s = 0;
    if (tm.r == 0) s = atomicAdd(q, 1);
    s = __shfl_sync(tm.mask, s, 0, TS);
    if (s >= P.nsys) break;
    run_system<CT, R, TileTeam<TS>>(P, tm, s, my, t0, n_iv, iv0, init != 0);
  }
}

// a role of whole blocks: the block takes the next system
template <int CT, typename R>
__device__ __forceinline__ void role_block(const PoolView<R> &P, int *q, double *smem, double t0, int n_iv,
                                           int iv0, int init) {
  __shared__ int s_next;
  BlockTeam tm;
  for (;;) {
    if (threadIdx.x == 0) s_next = atomicAdd(q, 1);
    __syncthreads();
    const int s = s_next;
    __syncthreads();
    if (s >= P.nsys) break;
    run_system<CT, R, BlockTeam>(P, tm, s, smem, t0, n_iv, iv0, init != 0);
    __syncthreads();
  }
}

template <typename R>
__global__ void __launch_bounds__(MEGA_BLOCK, 1) k_mega(const __grid_constant__ MegaView<R> M, double t0,
                                                         int n_iv, int iv0, int init) {
  extern __shared__ __align__(16) double smem[];
  if (threadIdx.x == 0) M.t_start[blockIdx.x] = global_ns();
  int role = 0;
  while (role < NTYPES - 1 && (int)blockIdx.x >= M.role_end[role]) role++;
  switch (role) {
    case GR:
      // single-lane granule systems on the CTA's first warps
      if ((int)(threadIdx.x >> 5) < M.lane_warps + ((int)blockIdx.x < M.lane_extra ? 1 : 0)) {
        if (M.gr_nc4)
          run_lanes_regs<GR, R, MEGA_BLOCK, 4>(M.pool[GR], M.queue + GR, 0, 0, smem, t0, n_iv, iv0, init != 0);
        else
          run_lanes<GR, R, MEGA_BLOCK>(M.pool[GR], M.queue + GR, 0, 0, smem, t0, n_iv, iv0, init != 0);
      }
      break;
    case GO: role_tiles<GO, R, TEAM_WARP>(M.pool[GO], M.queue + GO, smem, t0, n_iv, iv0, init); break;
    case PKJ: role_block<PKJ, R>(M.pool[PKJ], M.queue + PKJ, smem, t0, n_iv, iv0, init); break;
    default: role_block<IO, R>(M.pool[IO], M.queue + IO, smem, t0, n_iv, iv0, init); break;
  }
  __syncthreads();
  if (threadIdx.x == 0) M.t_end[blockIdx.x] = global_ns();
}

// The dynamic shared-memory limit is a per-kernel attribute shared by every
// engine in the process: only ever raise it, so that a later engine with
// smaller needs cannot break an earlier one's launches.
static cudaError_t raise_smem_limit(const void *k, size_t smem) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, k);
  if (e != cudaSuccess) return e;
  if ((size_t)a.maxDynamicSharedSizeBytes >= smem) return cudaSuccess;
  return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

template <typename R>
int prepare_mega_kernel(size_t smem, int *blocks_per_sm) {
  const void *k = (const void *)k_mega<R>;
  cudaError_t e = raise_smem_limit(k, smem);
  if (e != cudaSuccess) return (int)e;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, MEGA_BLOCK, smem);
  return (int)e;
}

template <typename R>
int launch_mega(const MegaView<R> &M, int grid, size_t smem, void *stream, double t0, int n_iv, int iv0,
                int init) {
  MegaView<R> Mc = M;
  void *args[] = {(void *)&Mc, (void *)&t0, (void *)&n_iv, (void *)&iv0, (void *)&init};
  cudaError_t e = cudaLaunchKernel((const void *)k_mega<R>, dim3(grid), dim3(MEGA_BLOCK), args, smem,
                                   (cudaStream_t)stream);
  return (int)e;
}

template <int CT, typename R>
static const void *kernel_for(int team) {
  switch (team) {
    case TEAM_GRID: return (const void *)k_advance_grid<CT, R>;
    case TEAM_CLUSTER8: return (const void *)k_advance_cluster<CT, R, 8>;
    case TEAM_CLUSTER16: return (const void *)k_advance_cluster<CT, R, 16>;
    case TEAM_LANE4:
      // instantiated for granule pools only (the others never have it)
      if constexpr (CT == GR) return (const void *)k_advance<CT, R, TEAM_LANE4>;
      return (const void *)k_advance<CT, R, TEAM_THREAD>;
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
    cudaError_t e = raise_smem_limit(k, smem);
    if (e != cudaSuccess) return (int)e;
  }
  if (team_cluster_size(team) > 8) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return (int)e;
  }
  return 0;
}

static cudaLaunchConfig_t cluster_config(int team, int grid, size_t smem, cudaStream_t stream,
                                         cudaLaunchAttribute *attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(CLUSTER_BLOCK);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = stream;
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = team_cluster_size(team);
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

// CTAs of the grid team's kernel the device co-schedules (cooperative
// launch: every CTA resident at once), 0 when it cannot launch cooperatively.
template <typename R>
int grid_capacity(int type) {
  int dev = 0, coop = 0, sms = 0, bps = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (!coop) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel_ptr<R>(type, TEAM_GRID), GRID_BLOCK, 0) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return sms * std::min(bps, 1);
}

template <typename R>
int cluster_capacity(int type, int team, size_t smem) {
  if (prepare_pool_kernel<R>(type, team, smem) != 0) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchAttribute attr[1];
  const cudaLaunchConfig_t cfg = cluster_config(team, team_cluster_size(team), smem, 0, attr);
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, kernel_ptr<R>(type, team), &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

template <typename R>
int launch_pool(int type, const PoolView<R> &P, int team, int grid, int block, size_t smem, void *stream,
                double t0, int n_iv, int iv0, int init) {
  const void *k = kernel_ptr<R>(type, team);
  PoolView<R> Pc = P;
  void *args[] = {(void *)&Pc, (void *)&t0, (void *)&n_iv, (void *)&iv0, (void *)&init};
  if (team == TEAM_GRID) {
    if (block < 32 || block > GRID_BLOCK || (block & (block - 1)) != 0 || block != P.grid_bw)
      return (int)cudaErrorInvalidConfiguration;
    return (int)cudaLaunchCooperativeKernel(k, dim3(grid), dim3(block), args, smem, (cudaStream_t)stream);
  }
  if (team_cluster_size(team) > 0) {
    if (block != CLUSTER_BLOCK || grid % team_cluster_size(team) != 0) return (int)cudaErrorInvalidConfiguration;
    cudaLaunchAttribute attr[1];
    const cudaLaunchConfig_t cfg = cluster_config(team, grid, smem, (cudaStream_t)stream, attr);
    return (int)cudaLaunchKernelExC(&cfg, k, args);
  }
  cudaError_t e = cudaLaunchKernel(k, dim3(grid), dim3(block), args, smem, (cudaStream_t)stream);
  return (int)e;
}

}  // namespace gbrkc

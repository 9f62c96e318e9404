// Device-resident RKC integrator (Sommeijer, Shampine & Verwer 1998) as the
// reference drives it: initial vectors and step (RKC_vec_initialize,
// solve_rkc.cu:438-560,757-791), nonlinear power method for the spectral
// radius (rkcrho, 563-754), Chebyshev stages (step, 816-906), error norm and
// step control (rkclow, 909-1096), dense output (rkcint, 795-813) and the
// per-interval driver with its ion-update clock (*_solve_by_rkc, 1122-1362).
//
// One "team" of threads integrates one system; the same code runs with a
// tile of 4 or 32 lanes, a whole block (large cells / networks), or a single
// lane (tiny cells: every thread its own system, the warp advancing 32
// systems side by side).  Every scalar of the controller is computed
// redundantly and identically by all team members, so control flow stays
// uniform within a team and needs no broadcast.  Every sum is the pairwise
// tree over compartment indices, the FP64 vector updates use the same
// explicit fused multiply-adds as the oracle's canonical mode, and the
// translation unit is built with -fmad=false: the plain-FP64 path reproduces
// the oracle bit for bit.
//
// The driver is flat: one call of tick() is one step attempt (rkclow's loop
// body) plus the bookkeeping after an accepted step, so independent systems
// sharing a warp move through their own attempt sequences without waiting
// for each other to accept.  A due ion update is returned to the caller
// (TICK_ION) instead of being run inside tick(): single-lane systems park
// until most of the warp's lanes have one due and then run them in one pass.
// On GB300 an FP64 warp instruction costs the same whatever its active-lane
// count, and the ion update is by far the longest path, so running it for 4
// lanes at a time would cost nearly as much as for 32.
#pragma once
#include <type_traits>
#include "engine.h"
#include "physics.cuh"

namespace gbrkc {

// A workspace vector: element i at p[i * LS] (LS = 1, or the block width for
// single-lane teams, whose workspaces interleave element by element so that a
// warp's 32 systems hit 32 consecutive shared-memory words).
template <int LS>
struct WVec {
  double *p;
  __device__ __forceinline__ double &operator[](int i) const { return p[(long)i * LS]; }
};

// Every team provides its workspace-vector type (Vec), builds the vector at
// a slot offset (vec_at) and gives the slot length for ncp elements
// (vstride).  CLUSTER > 0 marks a team spread over a thread-block cluster.
struct BlockTeam {
  static constexpr int LS = 1, NCF = 0, CLUSTER = 0, GRID = 0;
  typedef WVec<1> Vec;
  __device__ __forceinline__ Vec vec_at(double *W, long off) const { return Vec{W + off}; }
  __device__ __forceinline__ static long vstride(int ncp) { return ncp; }
  __device__ __forceinline__ int rank() const { return threadIdx.x; }
  __device__ __forceinline__ int size() const { return blockDim.x; }
  __device__ __forceinline__ void sync() const { __syncthreads(); }
};

template <int T>
struct TileTeam {
  static constexpr int LS = 1, NCF = 0, CLUSTER = 0, GRID = 0;
  typedef WVec<1> Vec;
  __device__ __forceinline__ Vec vec_at(double *W, long off) const { return Vec{W + off}; }
  __device__ __forceinline__ static long vstride(int ncp) { return ncp; }
  unsigned mask;
  int r;
  __device__ __forceinline__ int rank() const { return r; }
  __device__ __forceinline__ int size() const { return T; }
  __device__ __forceinline__ void sync() const {
    if (T > 1) __syncwarp(mask);
  }
};

// One thread, one system; workspaces interleaved across the block.  With
// NCF > 0 every system of the pool has exactly NCF compartments: the
// compartment loops unroll, values are computed into registers before they
// are stored (the rotating buffers are not known to be distinct, so stores
// would otherwise serialise the loop) and the pairwise sums run in registers.
template <int BLOCK, int NCF_ = 0>
struct LaneTeam {
  static constexpr int LS = BLOCK, NCF = NCF_, CLUSTER = 0, GRID = 0;
  typedef WVec<BLOCK> Vec;
  __device__ __forceinline__ Vec vec_at(double *W, long off) const { return Vec{W + off * BLOCK}; }
  __device__ __forceinline__ static long vstride(int ncp) { return ncp; }
  __device__ __forceinline__ int rank() const { return 0; }
  __device__ __forceinline__ int size() const { return 1; }
  __device__ __forceinline__ void sync() const {}
};

// One system on a thread-block cluster of C CTAs of CLUSTER_BLOCK threads.
// The workspace is spread block-cyclically over the CTAs' shared memory:
// element i sits in CTA (i mod 256C) / 256 at slot (i / 256C) * 256 + i mod
// 256, so the elements a thread owns in the team loops (i = rank + k * size)
// are in its own CTA; others (a compartment's neighbours) are read and
// written through distributed shared memory.  The team barrier is the
// cluster barrier.

template <int C>
struct CVec {
  long off;                    // slot offset within every CTA's workspace
  double *const *bases;        // workspace base of each CTA of the cluster
  __device__ __forceinline__ double &operator[](int i) const {
    constexpr int SZ = C * CLUSTER_BLOCK;
    const int q = (i & (SZ - 1)) / CLUSTER_BLOCK;
    const long l = (long)(i / SZ) * CLUSTER_BLOCK + (i & (CLUSTER_BLOCK - 1));
    return bases[q][off + l];
  }
};

template <int C>
struct ClusterTeam {
  static_assert((C & (C - 1)) == 0 && C <= 16, "cluster size must be a power of two up to 16");
  static constexpr int LS = 1, NCF = 0, CLUSTER = C, GRID = 0;
  typedef CVec<C> Vec;
  int crank;                   // this CTA's rank in the cluster
  double *const *bases;        // [C] workspace bases (distributed shared memory)
  long red_off;                // reduction area, after the workspace (CLUSTER_RED_DOUBLES)
  __device__ __forceinline__ Vec vec_at(double *, long off) const { return Vec{off, bases}; }
  __device__ __forceinline__ static long vstride(int ncp) {
    constexpr int SZ = C * CLUSTER_BLOCK;
    return (long)((ncp + SZ - 1) / SZ) * CLUSTER_BLOCK;
  }
  __device__ __forceinline__ int rank() const { return crank * CLUSTER_BLOCK + (int)threadIdx.x; }
  __device__ __forceinline__ int size() const { return C * CLUSTER_BLOCK; }
  __device__ __forceinline__ void sync() const {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
  }
};

// One system over every CTA of a cooperative launch (GridTeam): the
// workspace stays in global memory (the L2 holds it), element i is owned by
// thread i mod (gridDim * grid_bw) among each CTA's first grid_bw threads,
// and the team barrier is a software grid barrier: every CTA adds one to a
// counter (a reduction, no reply awaited) and polls it with acquire loads
// until it reaches gridDim times the CTA's own barrier count.  The wait is
// bounded: a CTA that waits more than GRID_SPIN_LIMIT polls raises the abort
// flag, after which no barrier waits and every CTA leaves its system at the
// next tick (status ST_BARRIER); the host reads the flag after the launch.
// A cooperative launch makes every CTA co-resident, so the bound is a guard,
// not a schedule.
constexpr long GRID_SPIN_LIMIT = 1L << 22;

__device__ __forceinline__ unsigned long long ld_acquire_gpu(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// epoch: this CTA's barrier count (shared memory, only thread 0 uses it).
// light: order the arrival with fence.acq_rel.gpu and rely on the acquire
// polls (the CTA's barrier carries both to its other threads); else
// fence.sc.gpu (__threadfence) before the arrival and after the wait.
__device__ __forceinline__ void grid_barrier(GridBarrier *b, unsigned long long *epoch, int light) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile GridBarrier *vb = b;
    if (!vb->abort) {
      const unsigned long long target = (*epoch += 1) * gridDim.x;
      if (light)
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
      else
        __threadfence();
      asm volatile("red.relaxed.gpu.global.add.u64 [%0], 1;" ::"l"(&b->count) : "memory");
      long it = 0;
      while (ld_acquire_gpu(&b->count) < target) {
        if (++it > GRID_SPIN_LIMIT || vb->abort) {
          atomicExch(&b->abort, 1);
          break;
        }
        if (it > 64) __nanosleep(32);
      }
      if (!light) __threadfence();
    }
  }
  __syncthreads();
}

// The grid team's stage barrier (grid_local_barrier): between the stages of
// one step a CTA reads only the elements of the CTAs that own its rows'
// neighbours (the operator is symmetric, so those are also the CTAs that
// read its elements), so it waits for those alone.  Each CTA publishes its
// stage count in its own flag (a release store on a 128-byte line) and warp
// 0's lanes poll the neighbours' flags with acquire loads, one flag a lane.
// nbr[b * (GRID_MAX_NBR + 1)] is CTA b's neighbour count, followed by the
// neighbours.  The wait is bounded like grid_barrier's and raises the same
// abort flag.
__device__ __forceinline__ void grid_local_barrier(GridBarrier *b, unsigned long long *flags, const int *nbr,
                                                   unsigned long long *lepoch) {
  __syncthreads();
  if (threadIdx.x < 32) {
    volatile GridBarrier *vb = b;
    if (!vb->abort) {
      const int lane = threadIdx.x;
      unsigned long long k = 0;
      if (lane == 0) {
        k = (*lepoch += 1);
        asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(flags + (long)blockIdx.x * 16), "l"(k)
                     : "memory");
      }
      k = __shfl_sync(0xffffffffu, k, 0);
      const int *my = nbr + (long)blockIdx.x * (GRID_MAX_NBR + 1);
      if (lane < my[0]) {
        const unsigned long long *f = flags + (long)my[1 + lane] * 16;
        long it = 0;
        while (ld_acquire_gpu(f) < k) {
          if (++it > GRID_SPIN_LIMIT || vb->abort) {
            atomicExch(&b->abort, 1);
            break;
          }
          if (it > 64) __nanosleep(32);
        }
      }
      __syncwarp();
    }
  }
  __syncthreads();
}

struct GridTeam {
  static constexpr int LS = 1, NCF = 0, CLUSTER = 0, GRID = 1;
  typedef WVec<1> Vec;
  GridBarrier *bar;
  double *red;                 // [2][GRID_MAX_BLOCKS] chunk sums (global)
  double *wp;                  // [GRID_MAX_ROWS][8] warp partials (shared)
  double *res;                 // the reduction's result (shared)
  unsigned long long *epoch;   // this CTA's barrier count (shared)
  int bw;                      // threads of each CTA that own elements
  int light;                   // the barrier's fences (grid_barrier)
  // the CTA's operator rows in shared memory (maxdeg 0: none): row slot
  // k * bw + t holds thread t's k-th element's entries
  int maxdeg;
  double *linv, *lg;           // [rl] 1/Cm, [rl * maxdeg] conductances
  int *lcnt, *lcol;            // [rl] entry counts, [rl * maxdeg] columns (system-wide)
  // stage barriers with the neighbouring CTAs only (nbr null: the grid barrier)
  const int *nbr;
  unsigned long long *flags;   // [gridDim * 16] stage counts, one 128-byte line a CTA
  unsigned long long *lepoch;  // this CTA's stage-barrier count (shared)
  __device__ __forceinline__ Vec vec_at(double *W, long off) const { return Vec{W + off}; }
  __device__ __forceinline__ static long vstride(int ncp) { return ncp; }
  // (the CTA has bw threads; a thread past bw would own nothing: a rank no
  // loop over the elements reaches)
  __device__ __forceinline__ int rank() const {
    return (int)threadIdx.x < bw ? (int)blockIdx.x * bw + (int)threadIdx.x : 0x3fffffff;
  }
  __device__ __forceinline__ int size() const { return (int)gridDim.x * bw; }
  __device__ __forceinline__ void sync() const { grid_barrier(bar, epoch, light); }
  __device__ __forceinline__ void sync_stage() const {
    if (nbr)
      grid_local_barrier(bar, flags, nbr, lepoch);
    else
      grid_barrier(bar, epoch, light);
  }
  __device__ __forceinline__ bool aborted() const { return ((volatile GridBarrier *)bar)->abort != 0; }
};

// pairwise tree over a[0..N) in registers, the same order as Sys::tree_sum
template <int N>
__device__ __forceinline__ double tree_regs(double (&a)[N]) {
#pragma unroll
  for (int stride = 1; stride < N; stride *= 2)
#pragma unroll
    for (int i = 0; i + stride < N; i += 2 * stride) a[i] = a[i] + a[i + stride];
  return a[0];
}

// logical vectors of the reference (param.h:21)
enum { LY = 0, LYN = 1, LFN = 2, LV1 = 3, LV2 = 4 };

constexpr int RKCLOW_LOOP_CAP = 1000;        // solve_rkc.cu:939
constexpr long STEPS_PER_INTERVAL_CAP = 200000;   // step attempts per 0.125 ms interval
constexpr int RHO_ITMAX = 1000;              // solve_rkc.cu:572
enum Tick { TICK_DONE = 0, TICK_MORE = 1, TICK_ION = 2 };
constexpr int ION_WAIT_MAX = 12;             // warp iterations a due ion update may wait

// One compartment's ion update (when update_ion) and its channel current
// term b (*_update_ion* and *_update_matrix of the reference), at pool
// compartment gi with stage voltage vyi.
template <int CT, typename R>
__device__ __forceinline__ double comp_ion_b_cell(const PoolView<R> &P, long gi, double vyi, double sum_dt,
                                                 bool update_ion) {
  const Slots<R> sl{P.ion, P.cond, P.stride, gi};
  if (CT == PKJ) {
    if (update_ion) {
      double ve = P.v[gi], ca = P.ca[gi], rv = P.rev[gi];
      Pkj<R>::ion(sl, ve, ca, rv, P.shell[gi], (P.flags[gi] & 1) != 0, vyi, sum_dt);
      P.v[gi] = ve; P.ca[gi] = ca; P.rev[gi] = rv;
    }
    return (double)Pkj<R>::b(sl, vyi, P.iext[gi], P.rev[gi]);
  } else if (CT == IO) {
    if (update_ion) {
      double ve = P.v[gi], ca = P.ca[gi];
      Io<R>::ion(sl, ve, ca, P.ctype[gi], vyi, sum_dt);
      P.v[gi] = ve; P.ca[gi] = ca;
    }
    return (double)Io<R>::b(sl, vyi, P.iext[gi]);
  } else if (CT == GR) {
    if (update_ion) {
      const int t = P.ctype[gi];
      double ve = P.v[gi];
      if (t >= 5) gr_na<R>(sl, P.na[t], vyi, ve, sum_dt);
      Gr<R>::ion(sl, ve, P.ca[gi], vyi, sum_dt);
      P.v[gi] = ve;
    }
    return (double)Gr<R>::b(sl, vyi, P.iext[gi]);
  } else {  // GO
    if (update_ion) {
      double ve = P.v[gi], ca = P.ca[gi], ca2 = P.ca2[gi], rv = P.rev[gi], cao = P.ca_old[gi];
      Go<R>::ion(sl, ve, ca, ca2, rv, P.area[gi], vyi, sum_dt);
      Go<R>::kahp(sl, ca, cao, sum_dt);
      P.v[gi] = ve; P.ca[gi] = ca; P.ca2[gi] = ca2; P.rev[gi] = rv; P.ca_old[gi] = cao;
    }
    return (double)Go<R>::b(sl, vyi, P.iext[gi], P.rev[gi]);
  }
}

// The synaptic current of compartment gi added to its b at an ion update
// (network mode), in the reference's expressions: b += g (V_y - E) per
// synapse for granule cells, b += the interval-start sum for Golgi cells,
// b += that sum * exp(-sum_dt / 0.6) for Purkinje cells (solve_rkc.cu:
// 201-224, 259-282, 348-360).  Synapses are added one by one in (kind, id)
// order; the reference's atomics leave that order open.
template <typename R>
__device__ __forceinline__ double syn_add(const PoolView<R> &P, long gi, double vyi, double sum_dt, double bi) {
  if (P.syn_mode == SYN_AT_ION) {
    for (int k = P.syn_row[gi]; k < P.syn_row[gi + 1]; k++) {
      const int s = P.syn_idx[k];
      bi = bi + P.syn_val[s] * (vyi - P.syn_e[s]);
    }
  } else if (P.syn_mode == SYN_BUFFERED) {
    bi = bi + P.syn_buf[gi];
  } else if (P.syn_mode == SYN_BUFFERED_DECAY) {
    bi = bi + P.syn_buf[gi] * mexp(-sum_dt / 0.6);
  }
  return bi;
}

// comp_ion_b_cell plus, at an ion update, the synaptic current (the
// reference's *_update_ion_and_matrix); initialisation (update_ion false)
// takes the channel current alone, as RKC_vec_initialize does.
template <int CT, typename R>
__device__ __forceinline__ double comp_ion_b(const PoolView<R> &P, long gi, double vyi, double sum_dt,
                                            bool update_ion) {
  double bi = comp_ion_b_cell<CT, R>(P, gi, vyi, sum_dt, update_ion);
  if (update_ion && P.syn_mode != SYN_NONE) bi = syn_add(P, gi, vyi, sum_dt, bi);
  return bi;
}

// Whether a launch has work for a system: an init launch initialises the
// systems waiting for it (ST_INIT); an advance steps the healthy systems
// with intervals left in their budget.
__device__ __forceinline__ bool system_selected(const Ctl &c, bool init, int n_iv) {
  if (init) return (c.status & ST_INIT) != 0;
  return c.status == 0 && n_iv > 0 && c.iv_left != 0;
}

// Device raster (output_file's rule, as in gr.cu:257 / pkj.cu:371): the
// cell's spike compartment went above the threshold at the end of the
// interval that ends at t, having been at or below it at the end of the
// previous one (main.cu:215 passes the interval's end time).
// The previous values are kept up to date whether or not the log is on.
template <typename R>
__device__ __forceinline__ void log_spike(const PoolView<R> &P, int pc, double t) {
  const double x = P.vnew[P.cell_spk[pc]];
  if (P.spk_log && x > P.spk_th && P.spk_prev[pc] <= P.spk_th) {
    const int k = atomicAdd(P.spk_count, 1);
    if (k < P.spk_cap) {
      P.spk_log[k].t = t;
      P.spk_log[k].cell = pc;
    }
  }
  P.spk_prev[pc] = x;
}

template <int CT, typename R, class Team>
struct Sys {
  static constexpr int LS = Team::LS, NCF = Team::NCF;
  static constexpr int NR = NCF > 0 ? NCF : 1;   // register staging width
  typedef typename Team::Vec V;
  const PoolView<R> &P;
  const Team &tm;
  int s, nc, ncp, ncell, ncomp, off, cell0;
  bool csr;
  const int *row, *col;
  const double *g, *invcm;
  const double *gc, *Gc;       // mixed precision: g / Cm and its row sums
  double *W;
  Ctl c;
  // flat driver state
  double t0;
  int k_iv, n_iv, iv0, rej_run;
  long long attempts0;
  mutable int red_buf = 0;     // cluster reductions: block-sum buffer in use

  __device__ Sys(const PoolView<R> &P_, const Team &tm_) : P(P_), tm(tm_) {}
  __device__ Sys(const PoolView<R> &P_, const Team &tm_, int s_, double *W_) : P(P_), tm(tm_) { bind(s_, W_); }

  __device__ __forceinline__ void bind(int s_, double *W_) {
    s = s_;
    W = W_;
    nc = P.sys_nc[s];
    ncp = (nc + 1) & ~1;
    ncell = P.sys_ncell[s];
    ncomp = P.sys_ncomp[s];
    off = P.sys_off[s];
    cell0 = P.sys_cell0[s];
    const int k = P.sys_csr[s];
    csr = k >= 0;
    if (csr) {
      row = P.s_row + P.s_row0[k];
      col = P.s_col + P.s_nz0[k];
      g = P.s_g + P.s_nz0[k];
      invcm = P.s_invcm + P.s_cm0[k];
      gc = P.s_gc + P.s_nz0[k];
      Gc = P.s_Gc + P.s_cm0[k];
    } else {
      const int t = P.sys_tmpl[s];
      row = P.t_row + P.t_row0[t];
      col = P.t_col + P.t_nz0[t];
      g = P.t_g + P.t_nz0[t];
      invcm = P.t_invcm + P.t_cm0[t];
      gc = P.t_gc + P.t_nz0[t];
      Gc = P.t_Gc + P.t_cm0[t];
    }
  }

  __device__ __forceinline__ V vec(int logical) const { return tm.vec_at(W, (long)c.map[logical] * Team::vstride(ncp)); }
  __device__ __forceinline__ V bvec() const { return tm.vec_at(W, (long)WS_B * Team::vstride(ncp)); }
  __device__ __forceinline__ V scratch() const { return tm.vec_at(W, (long)WS_SCRATCH * Team::vstride(ncp)); }

  // Grid team: copy this CTA's rows of the operator (the rows of the
  // elements its threads own, each thread its own) into shared memory, so
  // that a stage's dydt reads only the neighbours' values from L2.
  __device__ __forceinline__ void grid_rows_in() const {
    if constexpr (Team::GRID > 0) {
      if (tm.maxdeg == 0) return;
      const int md = tm.maxdeg;
      for (int i = tm.rank(), k = 0; i < nc; i += tm.size(), k++) {
        int j = i, base = 0;
        if (!(csr || ncell == 1)) {
          const int cidx = i / ncomp;
          j = i - cidx * ncomp;
          base = cidx * ncomp;
        }
        const int lr = k * tm.bw + (int)threadIdx.x;
        const int r0 = __ldg(row + j), r1 = __ldg(row + j + 1);
        tm.lcnt[lr] = r1 - r0;
        tm.linv[lr] = __ldg(invcm + j);
        for (int q = 0; q < r1 - r0; q++) {
          tm.lcol[lr * md + q] = base + __ldg(col + r0 + q);
          tm.lg[lr * md + q] = __ldg(g + r0 + q);
        }
      }
    }
  }

  // dydt at compartment i (solve_rkc.cu:178-196): (-b + sum g (y_j - y_i)) / Cm
  __device__ __forceinline__ double rhs(const V y, int i) const {
    if constexpr (Team::GRID > 0) {
      if (tm.maxdeg > 0) {
        // i is the calling thread's element: i = k * size + blockIdx * bw + t
        const int size = tm.size(), k = i / size;
        const int lr = k * tm.bw + (i - k * size - (int)blockIdx.x * tm.bw);
        double d = -(bvec()[i]);
        const double yi = y[i];
        const int n = tm.lcnt[lr];
        const int *cc = tm.lcol + lr * tm.maxdeg;
        const double *gg = tm.lg + lr * tm.maxdeg;
        for (int q = 0; q < n; q++) d = fma(gg[q], y[cc[q]] - yi, d);
        return d * tm.linv[lr];
      }
    }
    if constexpr (!std::is_same<R, double>::value) {
      // mixed precision: -b / Cm + sum (g / Cm) y_j - (sum g / Cm) y_i, the
      // same operator with one FP64 operation fewer per entry (the rounding
      // differs from the FP64 path's in the last bits)
      int j = i, base = 0;
      if (!(csr || ncell == 1)) {
        const int cidx = i / ncomp;
        j = i - cidx * ncomp;
        base = cidx * ncomp;
      }
      const int r0 = __ldg(row + j), r1 = __ldg(row + j + 1);
      double d = -(bvec()[i]) * __ldg(invcm + j);
      for (int k = r0; k < r1; k++) d = fma(__ldg(gc + k), y[base + __ldg(col + k)], d);
      return fma(-__ldg(Gc + j), y[i], d);
    }
    double d = -(bvec()[i]);
    const double yi = y[i];
    int r0, r1, base, j;
    if (csr || ncell == 1) {
      j = i;
      base = 0;
    } else {
      const int cidx = i / ncomp;
      j = i - cidx * ncomp;
      base = cidx * ncomp;
    }
    r0 = __ldg(row + j);
    r1 = __ldg(row + j + 1);
    for (int k = r0; k < r1; k++) d = fma(__ldg(g + k), y[base + __ldg(col + k)] - yi, d);
    return d * __ldg(invcm + j);
  }

  // pairwise tree over a[0..n): stride doubling, identical to the oracle
  __device__ __forceinline__ double tree_sum(const V a, int n) const {
    if constexpr (Team::CLUSTER > 0) return cluster_tree_sum(a, n);
    if constexpr (Team::GRID > 0) return grid_tree_sum(a, n);
    tm.sync();
    for (int stride = 1; stride < n; stride *= 2) {
      const int step = 2 * stride;
      for (int i = tm.rank() * step; i + stride < n; i += tm.size() * step) a[i] = a[i] + a[i + stride];
      tm.sync();
    }
    const double r = a[0];
    tm.sync();
    return r;
  }

  // tree_sum on a cluster team, the same additions in the same order with
  // one cluster barrier instead of one per level.  Element i is owned by the
  // thread that writes it in the team loops (every caller fills a[] that
  // way), and aligned blocks of CLUSTER_BLOCK elements lie in one CTA, one
  // element per thread: levels 0-4 are warp shuffles, 5-7 combine the 8 warp
  // partials of a block, and levels 8 and up combine block sums -- read by
  // one warp of every CTA through distributed shared memory after the
  // barrier, every CTA computing the same value.  The block sums are double
  // buffered: the next reduction's writes come after the next barrier, which
  // no CTA passes before every CTA has read this one's.
  __device__ __forceinline__ double cluster_tree_sum(const V a, int n) const {
    constexpr int C = Team::CLUSTER, B = CLUSTER_BLOCK, RR = (CLUSTER_MAX_ROWS * C + 31) / 32;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5, q = tm.crank;
    const int rows = (int)(Team::vstride(ncp) / B);
    double *red = tm.bases[q] + tm.red_off;
    double *wp = red + 2 * CLUSTER_MAX_ROWS, *res = wp + 8 * CLUSTER_MAX_ROWS;
    const int buf = red_buf;
    red_buf ^= 1;
    for (int k = 0; k < rows; k++) {
      const int i0 = (k * C + q) * B;
      if (i0 >= n) break;
      const int i = i0 + t;
      double x = (i < n) ? a[i] : 0.0;
#pragma unroll
      for (int st = 1; st < 32; st *= 2) {
        const double y = __shfl_down_sync(0xffffffffu, x, st);
        if ((lane & (2 * st - 1)) == 0 && i + st < n) x = x + y;
      }
      if (lane == 0) wp[k * 8 + warp] = x;
    }
    __syncthreads();
    if (t < rows) {
      const int i0 = (t * C + q) * B;
      if (i0 < n) {
        double w[8];
#pragma unroll
        for (int j = 0; j < 8; j++) w[j] = wp[t * 8 + j];
#pragma unroll
        for (int st = 1; st < 8; st *= 2)
#pragma unroll
          for (int j = 0; j + st < 8; j += 2 * st)
            if (i0 + (j + st) * 32 < n) w[j] = w[j] + w[j + st];
        red[buf * CLUSTER_MAX_ROWS + t] = w[0];
      }
    }
    tm.sync();
    if (warp == 0) {
      const int nb = (n + B - 1) / B;
      double v[RR];
#pragma unroll
      for (int r = 0; r < RR; r++) {
        const int b = lane + 32 * r;
        v[r] = (b < nb) ? tm.bases[b % C][tm.red_off + buf * CLUSTER_MAX_ROWS + b / C] : 0.0;
      }
#pragma unroll
      for (int st = 1; st < 32; st *= 2)
#pragma unroll
        for (int r = 0; r < RR; r++) {
          if (32 * r >= nb) break;
          const double y = __shfl_down_sync(0xffffffffu, v[r], st);
          if ((lane & (2 * st - 1)) == 0 && lane + 32 * r + st < nb) v[r] = v[r] + y;
        }
#pragma unroll
      for (int st = 1; st < RR; st *= 2)
#pragma unroll
        for (int r = 0; r + st < RR; r += 2 * st)
          if (32 * (r + st) < nb) v[r] = v[r] + v[r + st];
      if (lane == 0) *res = v[0];
    }
    __syncthreads();
    return *res;
  }

  // tree_sum on a grid team: the pairwise tree's additions in the same order.
  // Element i is owned by the thread that writes it in the team loops, so the
  // aligned chunk of bw elements (a power of two) starting at row k, CTA b
  // (chunk index k * gridDim + b) lies in CTA b, one element per thread:
  // levels 0-4 are warp shuffles, the next combine the chunk's bw / 32 warp
  // partials, the chunk sum goes to global memory, and after one grid barrier
  // warp 0 of every CTA combines all chunk sums (the remaining levels), every
  // CTA computing the same value.  The chunk sums are double-buffered, as on
  // a cluster.
  __device__ __forceinline__ double grid_tree_sum(const V a, int n) const {
    if constexpr (Team::GRID > 0) {
      constexpr int RR = GRID_MAX_BLOCKS / 32;
      const int t = threadIdx.x, lane = t & 31, warp = t >> 5, b = blockIdx.x, G = gridDim.x;
      const int B = tm.bw, nw = B >> 5;
      const int size = G * B;
      const int rows = (n + size - 1) / size;
      double *red = tm.red, *wp = tm.wp;
      const int buf = red_buf;
      red_buf ^= 1;
      if (t < B) {
        for (int k = 0; k < rows; k++) {
          const int i0 = k * size + b * B;
          if (i0 >= n) break;
          const int i = i0 + t;
          double x = (i < n) ? a[i] : 0.0;
#pragma unroll
          for (int st = 1; st < 32; st *= 2) {
            const double y = __shfl_down_sync(0xffffffffu, x, st);
            if ((lane & (2 * st - 1)) == 0 && i + st < n) x = x + y;
          }
          if (lane == 0) wp[k * 8 + warp] = x;
        }
      }
      __syncthreads();
      if (t < rows) {
        const int i0 = t * size + b * B;
        if (i0 < n) {
          double w[8];
#pragma unroll
          for (int j = 0; j < 8; j++) w[j] = (j < nw) ? wp[t * 8 + j] : 0.0;
#pragma unroll
          for (int st = 1; st < 8; st *= 2)
#pragma unroll
            for (int j = 0; j + st < 8; j += 2 * st)
              if (j + st < nw && i0 + (j + st) * 32 < n) w[j] = w[j] + w[j + st];
          red[buf * GRID_MAX_BLOCKS + t * G + b] = w[0];
        }
      }
      tm.sync();
      if (warp == 0) {
        const int nb = (n + B - 1) / B;
        double v[RR];
#pragma unroll
        for (int r = 0; r < RR; r++) {
          const int j = lane + 32 * r;
          v[r] = (j < nb) ? __ldcg(red + buf * GRID_MAX_BLOCKS + j) : 0.0;
        }
#pragma unroll
        for (int st = 1; st < 32; st *= 2)
#pragma unroll
          for (int r = 0; r < RR; r++) {
            if (32 * r >= nb) break;
            const double y = __shfl_down_sync(0xffffffffu, v[r], st);
            if ((lane & (2 * st - 1)) == 0 && lane + 32 * r + st < nb) v[r] = v[r] + y;
          }
#pragma unroll
        for (int st = 1; st < RR; st *= 2)
#pragma unroll
          for (int r = 0; r + st < RR; r += 2 * st)
            if (32 * (r + st) < nb) v[r] = v[r] + v[r + st];
        if (lane == 0) *tm.res = v[0];
      }
      __syncthreads();
      return *tm.res;
    } else {
      return 0.0;
    }
  }

  template <class A>
  __device__ __forceinline__ double sumsq(const A a) const {
    if constexpr (NCF > 0) {
      double q[NR];
#pragma unroll
      for (int i = 0; i < NCF; i++) q[i] = a[i] * a[i];
      return tree_regs<NR>(q);
    }
    V sc = scratch();
    for (int i = tm.rank(); i < nc; i += tm.size()) sc[i] = a[i] * a[i];
    return tree_sum(sc, nc);
  }

  // ---------------------------------------------------------------- rkcrho
  __device__ __forceinline__ void rkcrho() {
    const double uround = UROUND, sqrtu = sqrt(UROUND), small = 1.0 / 0.125;
    V yn = vec(LYN), fn = vec(LFN), v1 = vec(LV1), v2 = vec(LV2), sc = scratch();
    double *ede = P.ede + off;
    double sprad_old[3] = {0.0, 0.0, 0.0};
    c.n_rho++;
    const double ynrm = sqrt(sumsq(yn));
    const double vnrm = sqrt(sumsq(ede));
    double dynrm;
    if (ynrm != 0.0 && vnrm != 0.0) {
      dynrm = ynrm * sqrtu;
      const double al = dynrm / vnrm;
      for (int i = tm.rank(); i < nc; i += tm.size()) v1[i] = fma(al, ede[i], yn[i]);
    } else if (ynrm != 0.0) {
      dynrm = ynrm * sqrtu;
      for (int i = tm.rank(); i < nc; i += tm.size()) v1[i] = fma(sqrtu, yn[i], yn[i]);
    } else if (vnrm != 0.0) {
      dynrm = uround;
      const double al = dynrm / vnrm;
      for (int i = tm.rank(); i < nc; i += tm.size()) v1[i] = al * ede[i];
    } else {
      dynrm = uround;
      for (int i = tm.rank(); i < nc; i += tm.size()) v1[i] = dynrm;
    }
    tm.sync();
    double sigma = 0.0, sigmal;
    for (int iter = 0; iter < RHO_ITMAX; iter++) {
      c.n_rho_iter++;
      // v2 = F(v1); dam = v2 - fn; squares into the scratch
      double dfsq;
      if constexpr (NCF > 0) {
        double f[NR], q[NR];
#pragma unroll
        for (int i = 0; i < NCF; i++) {
          f[i] = rhs(v1, i);
          const double dm = -1.0 * fn[i] + f[i];
          q[i] = dm * dm;
        }
#pragma unroll
        for (int i = 0; i < NCF; i++) v2[i] = f[i];
        dfsq = tree_regs<NR>(q);
      } else {
        for (int i = tm.rank(); i < nc; i += tm.size()) {
          const double f = rhs(v1, i);
          v2[i] = f;
          const double dm = -1.0 * fn[i] + f;
          sc[i] = dm * dm;
        }
        dfsq = tree_sum(sc, nc);
      }
      const double dfnrm = sqrt(dfsq);
      sigmal = sigma;
      sigma = dfnrm / dynrm;
      sprad_old[0] = sprad_old[1];
      sprad_old[1] = sprad_old[2];
      sprad_old[2] = c.sprad;
      c.sprad = 1.2 * sigma;
      if (iter >= 1 && fabs(sigma - sigmal) <= ((sigma > small) ? sigma : small) * 0.001) {
        for (int i = tm.rank(); i < nc; i += tm.size()) ede[i] = -1.0 * yn[i] + v1[i];
        tm.sync();
        return;
      }
      if (iter > RHO_ITMAX / 2) {
        if ((fabs(sprad_old[2] - sprad_old[0]) < 0.00001) && (fabs(sprad_old[1] - c.sprad) < 0.00001)) {
          c.sprad = (c.sprad + sprad_old[2]) / 2.0;
          for (int i = tm.rank(); i < nc; i += tm.size()) ede[i] = -1.0 * yn[i] + v1[i];
          tm.sync();
          return;
        }
      }
      if (dfnrm != 0.0) {
        const double al = dynrm / dfnrm;
        if constexpr (NCF > 0) {
          double w[NR];
#pragma unroll
          for (int i = 0; i < NCF; i++) w[i] = fma(al, fn[i] - v2[i], yn[i]);
#pragma unroll
          for (int i = 0; i < NCF; i++) v1[i] = w[i];
        } else {
          for (int i = tm.rank(); i < nc; i += tm.size()) v1[i] = fma(al, fn[i] - v2[i], yn[i]);
        }
      } else {
        const int idx = iter % nc;
        if (tm.rank() == 0) v1[idx] = 2.0 * yn[idx] - v1[idx];
      }
      tm.sync();
    }
    c.idid = 6;
  }

  // the barrier between a step's stages: a stage reads its rows'
  // neighbours only, so a grid team waits for the CTAs that own them
  __device__ __forceinline__ void stage_sync() const {
    if constexpr (Team::GRID > 0)
      tm.sync_stage();
    else
      tm.sync();
  }

  // ----------------------------------------------------------------- step
  __device__ __forceinline__ bool step(double h, int m) {
    if (m > P.coef_mmax) {
      c.status |= ST_COEF_TABLE;
      return false;
    }
    const double *T = P.coef + P.coef_off[m];
    {
      V yn = vec(LYN), fn = vec(LFN), v1 = vec(LV1), v2 = vec(LV2);
      const double hm = h * __ldg(T);
      if constexpr (NCF > 0) {
        double a[NR], b[NR];
#pragma unroll
        for (int i = 0; i < NCF; i++) {
          a[i] = yn[i];
          b[i] = fma(hm, fn[i], a[i]);
        }
#pragma unroll
        for (int i = 0; i < NCF; i++) {
          v2[i] = a[i];
          v1[i] = b[i];
        }
      } else {
        for (int i = tm.rank(); i < nc; i += tm.size()) {
          v2[i] = yn[i];
          v1[i] = fma(hm, fn[i], yn[i]);
        }
      }
    }
    stage_sync();
    for (int j = 1; j < m; j++) {
      const double *q = T + 1 + 5 * (j - 1);
      const double mu = __ldg(q), nu = __ldg(q + 1), omn = __ldg(q + 2), mus = __ldg(q + 3), ajm1 = __ldg(q + 4);
      const double hm = h * mus;
      V y = vec(LY), yn = vec(LYN), fn = vec(LFN), v1 = vec(LV1), v2 = vec(LV2);
      if constexpr (NCF > 0) {
        double out[NR];
#pragma unroll
        for (int i = 0; i < NCF; i++) {
          const double f = rhs(v1, i);
          double t = mu * v1[i];
          t = fma(nu, v2[i], t);
          t = fma(omn, yn[i], t);
          const double u = fma(-ajm1, fn[i], f);
          out[i] = fma(hm, u, t);
        }
#pragma unroll
        for (int i = 0; i < NCF; i++) y[i] = out[i];
      } else {
        for (int i = tm.rank(); i < nc; i += tm.size()) {
          const double f = rhs(v1, i);
          double t = mu * v1[i];
          t = fma(nu, v2[i], t);
          t = fma(omn, yn[i], t);
          const double u = fma(-ajm1, fn[i], f);
          y[i] = fma(hm, u, t);
        }
      }
      const int t2 = c.map[LV2];
      c.map[LV2] = c.map[LV1];
      c.map[LV1] = c.map[LY];
      c.map[LY] = t2;
      stage_sync();
    }
    const int t3 = c.map[LY];
    c.map[LY] = c.map[LV1];
    c.map[LV1] = c.map[LV2];
    c.map[LV2] = t3;
    c.n_stage += m;
    return true;
  }

  // ------------------------------------------------------ rkclow, flat
  // One pass of rkclow's loop body (solve_rkc.cu:939-1096): returns
  // ATT_ACCEPT (the step was taken, c.idid = 1 or 2), ATT_REJECT (absh was
  // reduced; call again) or ATT_FAIL (c.status set).  rej_run counts the
  // attempts of the current rkclow call, bounded like the reference's loop.
  enum { ATT_FAIL = -1, ATT_REJECT = 0, ATT_ACCEPT = 1 };

  __device__ __forceinline__ int attempt() {
    const double hmax = H_MAX, hmin = c.hmin;
    if (c.newspc) {
      rkcrho();
      c.jacatt = 1;
    }
    c.last = 0;
    if (1.1 * c.absh >= fabs(c.tend - c.lt)) {
      c.absh = fabs(c.tend - c.lt);
      c.last = 1;
    }
    const double marg = sqrt(1.54 * c.absh * c.sprad + 1.0);
    if (!(marg < 1.0e9)) {
      c.status |= ST_NAN;
      return ATT_FAIL;
    }
    int m = 1 + (int)(marg);
    if (m > c.mmax) {
      m = (int)c.mmax;
      c.absh = (m * m - 1) / (1.54 * c.sprad);
      c.last = 0;
    }
    double h = 1.0 * c.absh;
    if (h <= hmin) h = hmin;
    if (!step(h, m)) return ATT_FAIL;
    c.n_steps++;
    // F(y) into vtemp1 and the error terms, fused
    double err;
    {
      V y = vec(LY), yn = vec(LYN), fn = vec(LFN), v1 = vec(LV1), sc = scratch();
      const double h04 = 0.4 * h;
      if constexpr (NCF > 0) {
        double f[NR], q[NR];
#pragma unroll
        for (int i = 0; i < NCF; i++) {
          f[i] = rhs(y, i);
          const double ay = fabs(y[i]), ayn = fabs(yn[i]);
          const double wt = fma(c.tol, (ay > ayn) ? ay : ayn, c.tol);
          const double est = fma(h04, fn[i] + f[i], 0.8 * (yn[i] - y[i]));
          const double qv = est / wt;
          q[i] = qv * qv;
        }
#pragma unroll
        for (int i = 0; i < NCF; i++) v1[i] = f[i];
        err = tree_regs<NR>(q);
      } else {
        for (int i = tm.rank(); i < nc; i += tm.size()) {
          const double f = rhs(y, i);
          v1[i] = f;
          const double ay = fabs(y[i]), ayn = fabs(yn[i]);
          const double wt = fma(c.tol, (ay > ayn) ? ay : ayn, c.tol);
          const double est = fma(h04, fn[i] + f, 0.8 * (yn[i] - y[i]));
          const double qv = est / wt;
          sc[i] = qv * qv;
        }
        err = tree_sum(sc, nc);
      }
    }
    // division by a power of two is exact scaling: multiply instead (the
    // same correctly rounded value, without the long FP64 divide)
    if ((nc & (nc - 1)) == 0)
      err = sqrt(err * __longlong_as_double((long long)(1023 - (__ffs(nc) - 1)) << 52));  // 2^-log2(nc)
    else
      err = sqrt(err / (double)nc);
    if (!(err == err)) {
      c.status |= ST_NAN;
      return ATT_FAIL;
    }
    // err^(1/3), shared by the reject and accept paths (one evaluation per
    // attempt whichever way the lanes of a warp go)
    const double cr = cm_cbrt(err);
    if (err > 1.0) {
      c.absh = 0.8 * c.absh / cr;
      c.n_rej++;
      if (c.absh < hmin) {
        c.idid = 4;
      } else {
        c.newspc = !c.jacatt;
        if (++rej_run >= RKCLOW_LOOP_CAP) {
          c.status |= ST_LOOP_CAP;
          return ATT_FAIL;
        }
        return ATT_REJECT;
      }
    }
    rej_run = 0;
    c.naccpt += 1;
    c.lt += h;
    c.gt = c.lt;
    c.jacatt = 0;
    c.newspc = 0;  // nstsig never advances (solve_rkc.cu:1024-1026)
    c.hw0 = h;
    c.hw1 = c.lt;
    {
      const int tmp = c.map[LV2];
      c.map[LV2] = c.map[LFN];
      c.map[LFN] = c.map[LV1];
      c.map[LV1] = c.map[LYN];
      c.map[LYN] = c.map[LY];
      c.map[LY] = tmp;
    }
    // err^(2/3) as the square of err^(1/3); errold^(1/3) carried over
    double fac = 10.0, temp1, temp2;
    if (c.naccpt == 1) {
      temp2 = cr;
      if (0.8 < fac * temp2) fac = 0.8 / temp2;
    } else {
      temp1 = 0.8 * c.absh * c.cbrt_errold;
      temp2 = fabs(c.hold) * (cr * cr);
      if (temp1 < fac * temp2) fac = temp1 / temp2;
    }
    c.cbrt_errold = cr;
    c.absh = ((0.1 > fac) ? 0.1 : fac) * c.absh;
    {
      const double mn = fmin(hmax, c.absh);
      c.absh = (hmin > mn) ? hmin : mn;
    }
    c.errold = err;
    c.hold = h;
    c.idid = c.last ? 1 : 2;
    // A grid team skips this barrier: every thread reads and writes only its
    // own elements until the next step's first barrier, the error norm's
    // grid barrier has already ordered every neighbour read of this attempt,
    // and its chunk sums are double-buffered.
    if constexpr (Team::GRID == 0) tm.sync();
    return ATT_ACCEPT;
  }

  // ------------------------------------------ ion update + current vector b
  __device__ __forceinline__ void ion_and_b(double sum_dt, bool update_ion, bool with_gap = true) {
    const V vy = vec(LY);
    const V b = bvec();
    for (int i = tm.rank(); i < nc; i += tm.size()) b[i] = comp_ion_b<CT, R>(P, off + i, vy[i], sum_dt, update_ion);
    if (CT == IO && with_gap && P.sys_ngap[s] > 0) {
      // io_gap_update + add_io_gap_val: per receiving dendrite, its four
      // edges in order (the reference adds them with atomics)
      tm.sync();
      const int e0 = P.sys_gap0[s], ne = P.sys_ngap[s];
      for (int cell = tm.rank(); cell < ne / 4; cell += tm.size()) {
        const int post = P.gap_post[e0 + 4 * cell];
        double acc = b[post];
        for (int k = 0; k < 4; k++) {
          const int e = e0 + 4 * cell + k;
          const int pre = P.gap_pre[e];
          const double diff = (pre > -1) ? (P.v[off + post] - P.v[off + pre]) : 0.0;
          acc += io_gap_current(P.gap_g[e], diff);
        }
        b[post] = acc;
      }
    }
    if (update_ion) c.n_ion++;
    tm.sync();
  }

  // ----------------------------------------------------- initialisation
  // RKC_vec_initialize: b from the initial V, vectors, rho, first step
  __device__ __forceinline__ void initialize() {
    V y = vec(LY), yn = vec(LYN), fn = vec(LFN), v1 = vec(LV1), v2 = vec(LV2);
    double *ede = P.ede + off;
    for (int i = tm.rank(); i < nc; i += tm.size()) {
      const double v0 = P.v[off + i];
      P.vnew[off + i] = v0;
      y[i] = v0;
      yn[i] = v0;
      v1[i] = 0.0;
      v2[i] = 0.0;
    }
    tm.sync();
    // b from the initial voltage (update_matrix only, no gap currents):
    // the b pass reads vec(LY) = initial V
    ion_and_b(0.0, false, false);
    for (int i = tm.rank(); i < nc; i += tm.size()) {
      const double f = rhs(yn, i);
      fn[i] = f;
      ede[i] = f;
    }
    tm.sync();
    rkcrho();
    // set_initial_absh (solve_rkc.cu:493-560)
    double absh = H_MAX;
    if (c.sprad * absh > 1.0) absh = 1.0 / c.sprad;
    absh = (absh > c.hmin) ? absh : c.hmin;
    for (int i = tm.rank(); i < nc; i += tm.size()) v1[i] = fma(absh, fn[i], yn[i]);
    tm.sync();
    V sc = scratch();
    int bad = 0;
    for (int i = tm.rank(); i < nc; i += tm.size()) {
      const double f = rhs(v1, i);
      v2[i] = f;
      const double wt = fma(c.tol, fabs(yn[i]), c.tol);
      if (wt == 0.0) bad = 1;
      const double dm = (f - fn[i]) * (1.0 / wt);
      sc[i] = dm * dm;
    }
    double est = tree_sum(sc, nc);
    if (bad) c.idid = 3.0;
    est = absh * sqrt(est / nc);
    if (0.1 * absh < H_MAX * sqrt(est)) {
      const double a2 = 0.1 * absh / sqrt(est);
      absh = (a2 > c.hmin) ? a2 : c.hmin;
    } else {
      absh = H_MAX;
    }
    c.absh = absh;
    {
      const double x = sqrt(c.tol / (10.0 * UROUND));
      c.mmax = (x - (double)(int)x < 0.5) ? (double)(int)x : (double)(int)(x + 0.9);
    }
  }

  // ------------------------------------------------------- flat driver
  // *_set_current at t, then the start of *_solve_by_rkc
  // (solve_rkc.cu:1122-1150); TICK_ION if the ion update left pending by
  // the previous interval is due before the first attempt.
  __device__ __forceinline__ int begin_interval(double t) {
    if (P.stim_on) {
      for (int cc = tm.rank(); cc < ncell; cc += tm.size()) {
        const int pc = cell0 + cc;
        const int comp = P.stim_comp[pc];
        if (comp >= 0) {
          const long gi = off + (long)cc * ncomp + comp;
          P.iext[gi] = 0;
          if (P.stim_t0[pc] <= t && t < P.stim_t1[pc]) P.iext[gi] = P.stim_amp[pc];
        }
      }
      tm.sync();
    }
    // Golgi / Purkinje synaptic current taken at the interval's start, before
    // the pending ion update (go_solve_by_rkc 1199-1200, pkj_solve_by_rkc
    // 1266-1269): sum of g (V_y - E) from zero, synapse by synapse
    if (P.syn_mode == SYN_BUFFERED || P.syn_mode == SYN_BUFFERED_DECAY) {
      const V vy = vec(LY);
      for (int i = tm.rank(); i < nc; i += tm.size()) {
        const long gi = off + i;
        double acc = 0.0;
        for (int k = P.syn_row[gi]; k < P.syn_row[gi + 1]; k++) {
          const int sid = P.syn_idx[k];
          acc = acc + P.syn_val[sid] * (vy[i] - P.syn_e[sid]);
        }
        P.syn_buf[gi] = acc;
      }
      tm.sync();
    }
    attempts0 = c.n_steps;
    rej_run = 0;
    return (c.sum_dt != 0.0) ? TICK_ION : TICK_MORE;
  }

  // the ion update and new current vector a TICK_ION asked for
  __device__ __forceinline__ void ion_due() {
    ion_and_b(c.sum_dt, true);
    c.sum_dt = 0.0;
  }

  // rkcint at the interval's end (solve_rkc.cu:795-813) and the soma record
  __device__ __forceinline__ void end_interval() {
    const double hlast = c.hw0, tlast = c.hw1 - hlast;
    const double sv = (c.gt_old - tlast) / hlast;
    const double a1 = (1.0 + 2.0 * sv) * (sv - 1.0) * (sv - 1.0);
    const double a2 = (3.0 - 2.0 * sv) * sv * sv;
    const double b1 = hlast * sv * (sv - 1.0) * (sv - 1.0);
    const double b2 = hlast * (sv - 1.0) * sv * sv;
    const V v1 = vec(LV1), v2 = vec(LV2), yn = vec(LYN), fn = vec(LFN);
    for (int i = tm.rank(); i < nc; i += tm.size())
      P.vnew[off + i] = fma(b2, fn[i], fma(b1, v2[i], fma(a2, yn[i], a1 * v1[i])));
    c.tend += H_MAX;
    tm.sync();
    if (P.soma_out) {
      for (int cc = tm.rank(); cc < ncell; cc += tm.size()) {
        const int pc = cell0 + cc;
        for (int k = 0; k < P.rec_w; k++)
          P.soma_out[((long)(iv0 + k_iv) * P.ncell_pool + pc) * P.rec_w + k] = P.vnew[P.cell_soma[pc] + k];
      }
    }
    if (P.spk_prev) {
      const double t = t0 + (k_iv + 1) * H_MAX;
      for (int cc = tm.rank(); cc < ncell; cc += tm.size()) log_spike(P, cell0 + cc, t);
    }
    if (c.iv_left > 0) c.iv_left--;
  }

  // Start advancing by n intervals from t: TICK_DONE if there is nothing to
  // do, else what begin_interval returns.
  __device__ __forceinline__ int start(double t, int n, int iv0_global) {
    if (c.iv_left >= 0 && n > c.iv_left) n = c.iv_left;
    t0 = t;
    n_iv = n;
    iv0 = iv0_global;
    k_iv = 0;
    if (c.status != 0 || n <= 0) return TICK_DONE;
    return begin_interval(t0);
  }

  // One step attempt and what follows it (the loop of *_solve_by_rkc,
  // solve_rkc.cu:1150-1362): TICK_MORE (attempt again), TICK_ION (run
  // ion_due() first) or TICK_DONE (intervals finished, or c.status set).
  __device__ __forceinline__ int tick() {
    const int a = attempt();
    if (a == ATT_REJECT) return TICK_MORE;
    if (a == ATT_FAIL) return TICK_DONE;
    if (c.n_steps - attempts0 > STEPS_PER_INTERVAL_CAP) {
      c.status |= ST_LOOP_CAP;
      return TICK_DONE;
    }
    c.sum_dt += c.gt - c.gt_old;
    c.gt_old = c.gt;
    const bool ge = (CT == GO || CT == PKJ);
    const bool trig = ge ? (c.sum_dt >= c.integ) : (c.sum_dt > c.integ);
    if (c.idid == 2.0) return trig ? TICK_ION : TICK_MORE;
    if (c.idid != 1.0) {
      c.status |= ST_IDID;
      return TICK_DONE;
    }
    end_interval();
    if (++k_iv >= n_iv) return TICK_DONE;
    return begin_interval(t0 + k_iv * H_MAX);
  }
};

// Stage a system's workspace between HBM (contiguous) and shared memory
// (element stride LS).
template <class Team>
__device__ __forceinline__ void ws_in(const Team &tm, double *dst, const double *src, long n) {
  if constexpr (Team::CLUSTER > 0) {
    // n = WS_VECS slots of ncp elements; each thread copies the elements it owns
    const int ncp = (int)(n / WS_VECS);
    for (int k = 0; k < WS_VECS; k++) {
      const typename Team::Vec v = tm.vec_at(dst, (long)k * Team::vstride(ncp));
      for (int i = tm.rank(); i < ncp; i += tm.size()) v[i] = src[(long)k * ncp + i];
    }
  } else {
    for (long i = tm.rank(); i < n; i += tm.size()) dst[i * Team::LS] = src[i];
  }
  tm.sync();
}
template <class Team>
__device__ __forceinline__ void ws_out(const Team &tm, double *dst, const double *src, long n) {
  if constexpr (Team::CLUSTER > 0) {
    const int ncp = (int)(n / WS_VECS);
    for (int k = 0; k < WS_VECS; k++) {
      const typename Team::Vec v = tm.vec_at(const_cast<double *>(src), (long)k * Team::vstride(ncp));
      for (int i = tm.rank(); i < ncp; i += tm.size()) dst[(long)k * ncp + i] = v[i];
    }
  } else {
    for (long i = tm.rank(); i < n; i += tm.size()) dst[i] = src[i * Team::LS];
  }
  tm.sync();
}

// Advance one system by n_iv intervals starting at t0 (or initialise it).
template <int CT, typename R, class Team>
__device__ __forceinline__ void run_system(const PoolView<R> &P, const Team &tm, int s, double *smem_ws, double t0,
                                           int n_iv, int iv0_global, bool init) {
  if (!system_selected(P.ctl[s], init, n_iv)) return;
  const long wsn = (long)WS_VECS * (long)((P.sys_nc[s] + 1) & ~1);
  double *gws = P.ws + P.sys_ws[s];
  double *W = P.ws_in_smem ? smem_ws : gws;
  if (P.ws_in_smem) ws_in(tm, W, gws, wsn);
  Sys<CT, R, Team> S(P, tm, s, W);
  S.c = P.ctl[s];
  S.grid_rows_in();
  if (init) {
    S.initialize();
    S.c.status &= ~ST_INIT;
    if constexpr (Team::GRID > 0)
      if (tm.aborted()) S.c.status |= ST_BARRIER;
  } else {
    int r = S.start(t0, n_iv, iv0_global);
    while (r != TICK_DONE) {
      if constexpr (Team::GRID > 0) {
        if (tm.aborted()) {
          S.c.status |= ST_BARRIER;
          break;
        }
      }
      if (r == TICK_ION) {
        S.ion_due();
        r = TICK_MORE;
      } else {
        r = S.tick();
      }
    }
  }
  tm.sync();
  if (P.ws_in_smem) ws_out(tm, gws, W, wsn);
  if (tm.rank() == 0) P.ctl[s] = S.c;
}

// Single-lane systems: every thread of the first `lanes` threads of the block
// integrates its own systems, taken from *q (or, with q null, the static
// sequence first, first + stride, ...).  A lane whose system has finished
// writes it back and takes the next one at once, so the warp keeps 32
// systems in flight until the queue runs dry.  A lane whose ion update is due
// parks; the warp runs the parked lanes' updates together once every live
// lane is parked or the oldest has waited ION_WAIT_MAX iterations.  Parking
// only delays a system; its own sequence of operations is unchanged.
// Workspaces always sit in shared memory, interleaved (Team::LS = BLOCK).
template <int CT, typename R, int BLOCK, int NCF = 0>
__device__ __forceinline__ void run_lanes(const PoolView<R> &P, int *q, int first, int stride, double *smem,
                                          double t0, int n_iv, int iv0_global, bool init) {
  typedef LaneTeam<BLOCK, NCF> Team;
  Team tm;
  double *W = smem + threadIdx.x;
  Sys<CT, R, Team> S(P, tm);
  // only the warp's first P.lanes lanes take systems (fewer systems per warp
  // diverge less: a warp runs the union of its lanes' paths)
  int s = ((int)(threadIdx.x & 31) >= P.lanes) ? P.nsys : (q ? atomicAdd(q, 1) : first);
  int r = TICK_DONE;
  // take systems until one needs stepping (or the queue is empty)
  auto acquire = [&]() {
    while (s < P.nsys) {
      S.bind(s, W);
      S.c = P.ctl[s];
      if (!system_selected(S.c, init, n_iv)) {
      } else if (init) {
        ws_in(tm, W, P.ws + P.sys_ws[s], (long)WS_VECS * S.ncp);
        S.initialize();
        S.c.status &= ~ST_INIT;
        ws_out(tm, P.ws + P.sys_ws[s], W, (long)WS_VECS * S.ncp);
        P.ctl[s] = S.c;
      } else {
        ws_in(tm, W, P.ws + P.sys_ws[s], (long)WS_VECS * S.ncp);
        r = S.start(t0, n_iv, iv0_global);
        if (r != TICK_DONE) return;
        ws_out(tm, P.ws + P.sys_ws[s], W, (long)WS_VECS * S.ncp);
        P.ctl[s] = S.c;
      }
      s = q ? atomicAdd(q, 1) : s + stride;
    }
    r = TICK_DONE;
  };
  acquire();
  int wait = 0;
  for (;;) {
    __syncwarp();
    const unsigned live = __ballot_sync(0xffffffffu, r != TICK_DONE);
    if (!live) break;
    const unsigned parked = __ballot_sync(0xffffffffu, r == TICK_ION);
    if (parked && (parked == live || ++wait > ION_WAIT_MAX)) {
      wait = 0;
      if (r == TICK_ION) {
        S.ion_due();
        r = TICK_MORE;
      }
      __syncwarp();
    }
    if (r == TICK_MORE) {
      r = S.tick();
      if (r == TICK_DONE) {
        ws_out(tm, P.ws + P.sys_ws[s], W, (long)WS_VECS * S.ncp);
        P.ctl[s] = S.c;
        s = q ? atomicAdd(q, 1) : s + stride;
        acquire();
      }
    }
  }
}

}  // namespace gbrkc

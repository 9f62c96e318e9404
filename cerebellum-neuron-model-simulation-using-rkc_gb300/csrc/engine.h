// Device-side data layout of the RKC engine (shared by the host runtime and
// the kernels).  All cells of one type live in a "pool"; a pool holds many
// independent RKC systems (a system is what the reference integrates with one
// step size: all cells of a reference type block, or one cell, or one
// inferior-olive gap-junction network).
//
// Layout in HBM, per pool:
//   * per-system workspace, system-major: [PHYS0..PHYS4, B, SCRATCH] x nc
//     FP64 -- the five rotating RKC vectors (y, yn, fn, vtemp1, vtemp2 of
//     param.h:21, rotated by index like the reference's pointer swaps), the
//     frozen current b and a reduction scratch.  Staged into shared memory
//     for the whole launch when it fits.
//   * per-compartment SoA state: elem v, Ca, Ca2, rev_ca2, Ca_old, i_ext
//     (FP64), gating slots ion[k][i] and conductances cond[k][i] (R = FP64 or
//     FP32), the eigenvector estimate ede and the output v_new (FP64).
//   * per-template CSR of one cell's axial operator (diagonal dropped, rows
//     sorted by column, RKC sign), 1/Cm per template compartment; multi-cell
//     systems with linear gap junctions carry a system CSR instead.
#pragma once
#include <stdint.h>

#include "model.h"

namespace gbrkc {

enum { WS_PHYS = 5, WS_B = 5, WS_SCRATCH = 6, WS_VECS = 7 };

// status bits written by the kernel (never a trap)
enum Status : int {
  ST_OK = 0,
  ST_NAN = 1,          // non-finite error norm or step
  ST_LOOP_CAP = 2,     // step loop exceeded its iteration bound
  ST_COEF_TABLE = 4,   // stage count beyond the coefficient table
  ST_IDID = 8,         // rkclow returned an idid other than 1/2 (solve_rkc.cu:1155)
  ST_INIT = 16,        // waiting for initialisation (set by the host; cleared by the init launch)
  ST_BARRIER = 32,     // a grid-team barrier gave up waiting (bounded spin)
};

// One threshold crossing of a cell's spike compartment, logged on the device
// at the end of an interval: the interval's end time and the pool cell.
struct SpikeRec {
  double t;
  int cell;
  int pad;
};

// Controller state of one RKC system (h_others / h_work / h_bool of
// solve_rkc.cu, plus the driver's static sum_dt and counters).
struct Ctl {
  double absh, sprad, naccpt, errold, hold, lt, tend, gt, gt_old, idid, mmax, hw0, hw1;
  double sum_dt, integ, hmin, tol;
  double cbrt_errold;  // errold^(1/3), carried from the last accepted step
  int map[5];          // logical {y, yn, fn, vtemp1, vtemp2} -> physical buffer
  int newspc, jacatt, last, status;
  int iv_left;         // intervals this system may still advance (-1: no limit)
  long long n_steps, n_rej, n_stage, n_rho, n_rho_iter, n_ion;
};

// Everything a kernel needs for one pool (passed by value).
template <typename R>
struct PoolView {
  int type, nsys;
  long stride;                        // pool compartment count (SoA stride)
  // per system
  const int *sys_off, *sys_nc, *sys_ncell, *sys_ncomp, *sys_tmpl, *sys_csr, *sys_cell0;
  const int *sys_gap0, *sys_ngap;
  const long *sys_ws;                 // workspace offset (doubles)
  Ctl *ctl;
  double *ws;
  // per compartment
  double *ede, *vnew, *v, *ca, *ca2, *rev, *ca_old, *iext;
  const double *shell, *area;
  const uint8_t *ctype, *flags;       // compartment type; bit0 = PKJ fixed Nernst
  R *ion;
  const R *cond;
  // templates
  const int *t_row0, *t_nz0, *t_cm0;  // per template offsets
  const int *t_row, *t_col;
  const double *t_g, *t_invcm;
  const double *t_gc, *t_Gc;          // mixed precision: g / Cm per entry, their row sums (like t_invcm)
  // system CSRs (multi-cell systems with linear gap junctions)
  const int *s_row0, *s_nz0, *s_cm0;
  const int *s_row, *s_col;
  const double *s_g, *s_invcm;
  const double *s_gc, *s_Gc;
  // IO nonlinear gap junctions: per system edge list (post compartment, pre or -1)
  const int *gap_pre, *gap_post;
  const double *gap_g;
  // per cell (pool cell index)
  const int *stim_comp;
  const double *stim_amp, *stim_t0, *stim_t1;
  int stim_on;
  // stage coefficients, per m: [h*mus factor of stage 1, then (mu, nu, 1-mu-nu, mus, ajm1) per stage]
  const double *coef;
  const long *coef_off;
  int coef_mmax;
  NaPar na[9];
  // outputs
  double *soma_out;                   // [interval][pool cell][rec_w] or null
  const int *cell_soma;               // per pool cell: first recorded compartment (pool index)
  int rec_w;                          // compartments recorded per cell
  int ncell_pool;
  // device raster: per pool cell the spike compartment and its value at the
  // previous interval's end; an upward crossing of spk_th appends a SpikeRec
  // (entries past spk_cap are counted, not written)
  const int *cell_spk;
  double *spk_prev;
  SpikeRec *spk_log;
  int *spk_count;
  int spk_cap;
  double spk_th;
  int lanes;                          // single-lane pools: lanes of each warp that take systems
  int ws_in_smem;                     // stage the workspace in shared memory
  long ws_tile_doubles;               // shared-memory workspace per team
  // chemical synapses onto this pool (network mode; syn_mode 0 = none)
  int syn_mode;                       // SYN_AT_ION, SYN_BUFFERED or SYN_BUFFERED_DECAY
  const int *syn_row;                 // [stride + 1] CSR over post compartments
  const int *syn_idx;                 // synapse ids, per compartment in (kind, id) order
  const double *syn_val;              // per synapse: conductance value (engine-wide table)
  const double *syn_e;                // per synapse: reversal potential
  double *syn_buf;                    // [stride] synaptic current taken at interval start
  // grid team (one system over every CTA of a cooperative launch): block
  // sums of the reductions, double-buffered, and the grid barrier's words
  double *grid_red;                   // [2][GRID_MAX_BLOCKS]
  unsigned *grid_bar;                 // GridBarrier
  int grid_bw;                        // threads of each CTA that own elements (a power of two, 32..GRID_BLOCK)
  int grid_light;                     // grid barrier: acq_rel fence + acquire polls (1) or sc fences (0)
  // grid team: each CTA's rows of the operator in shared memory (grid_rl
  // row slots of grid_maxdeg entries each); grid_maxdeg 0 = read the rows
  // from global memory
  int grid_rl, grid_maxdeg;
  // grid team: per CTA its neighbour CTAs ([ctas][GRID_MAX_NBR + 1]: count,
  // then the list) and the stage-count flags ([ctas * 16]); grid_nbr null:
  // every stage barrier is the grid barrier
  const int *grid_nbr;
  unsigned long long *grid_flags;
};

// How a pool takes its synaptic current (solve_rkc.cu): granule cells add
// every synapse's g (V_y - E) to b at each ion update (add_mfgr_val,
// add_gogr_val, 1100-1120); Golgi cells take the sum at the start of the
// interval and add it at each ion update (add_grgo_val_new +
// go_update_matrix_new, 1199-1200, 1180); Purkinje cells likewise, scaled by
// exp(-sum_dt / 0.6) (add_grpkj_val_new + pkj_update_matrix_new, 1266-1269,
// 1247-1250).
enum SynMode { SYN_NONE = 0, SYN_AT_ION = 1, SYN_BUFFERED = 2, SYN_BUFFERED_DECAY = 3 };

// Synapse kinds of the reference's RKC network path (syn.cu) and their
// per-synapse state: MF->GrC (AMPA, NMDA), GrC->GoC (AMPA, NMDA1, NMDA2),
// GoC->GrC (GABA_A, GABA_B), GrC->PC (AMPA).
enum SynKind { SYN_MFGR = 0, SYN_GRGO = 1, SYN_GOGR = 2, SYN_GRPKJ = 3, SYN_KINDS = 4 };

// The engine-wide synapse table for the per-interval update kernel.
struct SynView {
  int n;
  const int *kind, *grp;
  const int *pre_type;                // pool of the presynaptic compartment (-1: Poisson input)
  const long *pre_gi;                 // presynaptic compartment, pool index
  const double *w;
  double *s0, *s1, *s2, *val, *old_v;
  const double *pre_v[NTYPES];        // elem v of every pool
  unsigned long long *ring;           // per synapse: the last 64 intervals' events, newest in bit 0 (or null)
  const unsigned char *delay;         // per synapse: intervals between an event and its effect
  const double *grp_rate;             // per group: base rate, stimulus rate [Hz], window t0, t1 [ms]
  const unsigned long long *grp_seed;
  double decay[8];                    // exp(-RKC_DT / tau) per state, in SynKind order
};

int launch_syn_update(const SynView &S, void *stream, double t, long long interval);

// Team shapes the kernels are instantiated for: one thread (tiny cells, 32
// systems per warp, blocks of MEGA_BLOCK threads with interleaved shared
// workspaces), 4 or 32 lanes per system, or a whole block per system.
// TEAM_LANE4: one thread per system for pools whose systems all have exactly
// 4 compartments (loops unrolled at compile time).
// TEAM_CLUSTER8 / TEAM_CLUSTER16: one system per cluster of 8 / 16 CTAs
// (very large systems; 16 is a non-portable cluster size, used where the
// device can co-schedule it).
// TEAM_GRID: one system over every CTA of a cooperative launch (a system
// that is alone in its engine and larger than a cluster holds efficiently).
enum TeamKind {
  TEAM_THREAD = 1, TEAM_LANE4 = 2, TEAM_TILE4 = 4, TEAM_WARP = 32, TEAM_BLOCK = 0,
  TEAM_CLUSTER8 = 108, TEAM_CLUSTER16 = 116, TEAM_GRID = 200
};
constexpr int team_cluster_size(int team) {
  return team == TEAM_CLUSTER8 ? 8 : team == TEAM_CLUSTER16 ? 16 : 0;
}

// All pools in one persistent launch: CTA b < role_end[0] integrates granule
// systems (one per lane, on the CTA's first warps), then Golgi
// (32-lane warps), Purkinje and olive (whole blocks).  Each role pulls
// systems from its own atomic queue.
template <typename R>
struct MegaView {
  PoolView<R> pool[NTYPES];
  int role_end[NTYPES];
  int lane_warps, lane_extra;  // granule CTA b runs lane_warps (+1 if b < lane_extra) warps
  int gr_nc4;                 // every granule system has 4 compartments
  int *queue;                 // [NTYPES] next-system counters, zeroed per launch
  unsigned long long *t_start; // [grid] globaltimer at each CTA's start
  unsigned long long *t_end;   // [grid] globaltimer at each CTA's finish
};

constexpr int MEGA_BLOCK = 256;
// Cluster teams: CTAs of CLUSTER_BLOCK threads; at most CLUSTER_MAX_ROWS rows
// of CLUSTER_BLOCK elements per CTA and vector (the workspace of WS_VECS
// vectors fits 200 KB of shared memory), followed by the reduction area:
// block sums (double-buffered), warp partials, result.
constexpr int CLUSTER_BLOCK = 256;
constexpr int CLUSTER_MAX_ROWS = 14;
constexpr int CLUSTER_RED_DOUBLES = 2 * CLUSTER_MAX_ROWS + 8 * CLUSTER_MAX_ROWS + 2;
constexpr int LANE_MAX_NC = 8;   // largest system integrated by a single lane
// Grid team: CTAs of GRID_BLOCK threads, of which the first grid_bw (a power
// of two) own elements: element i of a workspace vector is owned by thread
// (i mod gridDim * grid_bw) of that numbering; a reduction covers at most
// GRID_MAX_BLOCKS chunks of grid_bw elements and GRID_MAX_ROWS rows of
// gridDim * grid_bw elements.
constexpr int GRID_BLOCK = 256;
constexpr int GRID_MAX_BLOCKS = 256;
constexpr int GRID_MAX_ROWS = 8;
constexpr int GRID_MAX_NBR = 32;   // neighbour CTAs a CTA's stage barrier can wait for (one a lane)
constexpr size_t GRID_ROWS_SMEM_MAX = 160 * 1024;   // shared memory for a CTA's operator rows
// bytes of that copy: per row slot its entry count, 1/Cm, and maxdeg
// (column, conductance) pairs
constexpr size_t grid_rows_smem(long rl, long maxdeg) { return (size_t)rl * (12 + 12 * (size_t)maxdeg); }
// The grid barrier's words, each on its own 128-byte line: the count of
// arrivals since the launch began (a CTA's k-th barrier ends when it reaches
// k * gridDim) and the abort flag.
struct GridBarrier {
  unsigned long long count;
  unsigned long long pad0[15];
  int abort;
  int pad1[31];
};

template <typename R>
int launch_mega(const MegaView<R> &M, int grid, size_t smem, void *stream, double t0, int n_iv, int iv0,
                int init);
template <typename R>
int prepare_mega_kernel(size_t smem, int *blocks_per_sm);

// Launch the advance / initialise kernel of one pool (kernels.cu).
template <typename R>
int launch_pool(int type, const PoolView<R> &P, int team, int grid, int block, size_t smem,
                void *stream, double t0, int n_iv, int iv0, int init);
template <typename R>
int prepare_pool_kernel(int type, int team, size_t smem);
// How many clusters of a cluster team's kernel the device can run at once
// with this shared memory (0: the shape does not fit).
template <typename R>
int cluster_capacity(int type, int team, size_t smem);
// CTAs of the grid team's cooperative launch (0: the device cannot launch it).
template <typename R>
int grid_capacity(int type);

}  // namespace gbrkc

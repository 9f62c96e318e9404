/*
 * gbrkc_compat.h -- the reference simulator's per-type entry points
 * (TairaKobayashi/Cerebellum-neuron-model-simulation-using-RKC), served by
 * the gbrkc engine.  A caller written against the reference -- its main.cu --
 * drives GrC, GoC, PC and IO blocks through these exact names, argument
 * meanings and call order; only the RKC solver is provided (the BE / CN
 * solvers are the reference's comparators and are not part of this library).
 *
 * Everything is exported with C linkage.  The state structs keep the layout
 * of the reference's param.h:27-46 so that the fields its main.cu reads
 * (n, nx, ny, nc, n_solver, DT, elem[v], elem[i_ext], vec[v_new]) are where
 * it expects them; those pointers are device addresses, as in the reference.
 * Each type runs as one RKC system of nx*ny cells with its gap junctions,
 * in FP64, on its own engine, exactly as the reference integrates it.
 *
 * Model files are read from the working directory under the reference's
 * names (Gr.txt, Go_131.txt, Pkj.txt, Pkj_GJ.csv, IO.txt), or from the
 * directory named by the GBRKC_MODEL_DIR environment variable.
 *
 * Errors follow the reference: a message on stdout and exit(1) (an unknown
 * solver name, an unreadable model file, a failed device call).
 */
#ifndef GBRKC_COMPAT_H
#define GBRKC_COMPAT_H

#include <stdio.h>
#ifndef __cplusplus
#include <stdbool.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define RKC_DT (0.125) /* [ms] output interval (param.h:12) */
#ifndef H_MAX
#define H_MAX (RKC_DT) /* solve_rkc.cuh:23 */
#endif
#define GBRKC_MAX_BUF 1024

/* param.h:15-21 */
typedef enum { kBE, kCN, kRKC, kSolver_num } kSolver_type;
typedef enum { N_TYPE_GR, N_TYPE_GO, N_TYPE_PKJ, N_TYPE_IO, NEURON_TYPE } neuron_type_t;
typedef enum { v, Ca, Cm, area, connect, compart, i_ext, n_elem } elem_t;
typedef enum { y, yn_r, fn, vtemp1, vtemp2, ede, v_new, n_vec_RKC } vec_RKC_t;

/* param.h:27-34.  elem is a host table of n_elem device arrays (v, Ca and
 * i_ext are provided; the others are NULL); ion, cond, ca2, rev_ca2, ca_old
 * and shell are NULL (the state lives in the engine). */
typedef struct {
  int n_solver, neuron_type;
  int n, nx, ny, nc;
  double **elem, **ion, **cond;
  double *ca2, *rev_ca2, *ca_old;
  double *shell;
  double DT;
} neuron_t;

/* param.h:36-46.  vec is a host table of n_vec_RKC device arrays; only
 * vec[v_new] (voltage at the end of the last interval) is provided. */
typedef struct {
  int nnz;
  double *val, *val_ori, *b;
  int *col, *row, *dig;
  double **vec;
  double *h_work, *h_others;
  bool *h_bool;
  double *dammy;
  int numThreadsPerBlock, numBlocks;
  char type[GBRKC_MAX_BUF];
} neuron_solve_t;

typedef struct _synapse_t synapse_t;
typedef struct _gap_t gap_t;

/* Block set-up: X_initialize reads the model, draws the initial-voltage
 * jitter from the process's rand() stream (one draw per cell, in the
 * reference's formula and order: gr_ion.cu:642, go_ion.cu:598,
 * pkj_ion.cu:367, io_ion.cu:172; the caller seeds it, main.cu:38 with
 * srand(0)),
 * builds and initialises the system and fills the caller's host mirror p;
 * it returns the device-side neuron_t.  (gr.cu:152, go.cu:161, pkj.cu:241,
 * io.cu:163) */
neuron_t *gr_initialize(const int nx, const int ny, const char *type, neuron_t *p);
neuron_t *go_initialize(const int nx, const int ny, const char *type, neuron_t *p);
neuron_t *pkj_initialize(const int nx, const int ny, const char *type, neuron_t *p);
neuron_t *io_initialize(const int nx, const int ny, const char *type, neuron_t *p);

/* Fill the caller's host mirror p_solve (vec[v_new]); returns the device-side
 * neuron_solve_t.  (gr_solve.cu:171, go_solve.cu:248, pkj_solve.cu:286,
 * io_solve.cu:196) */
neuron_solve_t *gr_solve_initialize(neuron_solve_t *p_solve, const char *type, neuron_t *p, neuron_t *d);
neuron_solve_t *go_solve_initialize(neuron_solve_t *p_solve, const char *type, neuron_t *p, neuron_t *d);
neuron_solve_t *pkj_solve_initialize(neuron_solve_t *p_solve, const char *type, neuron_t *p, neuron_t *d);
neuron_solve_t *io_solve_initialize(neuron_solve_t *p_solve, const char *type, neuron_t *p, neuron_t *d);

/* Advance the block by one output interval (H_MAX = 0.125 ms) after any
 * stimulus kernel the caller launched on the default stream; on return
 * p_solve->vec[v_new] holds the new voltages.  The coupling objects are the
 * ones the constructors below return (or NULL); in network mode the first
 * call of an interval advances every block and the synapses together, and
 * the others of that interval return at once.  (gr_solve.cu:293,
 * go_solve.cu:362, pkj_solve.cu:395, io_solve.cu:300) */
void gr_solve_update_v(neuron_t *d, neuron_solve_t *d_solve, neuron_t *p, neuron_solve_t *p_solve, synapse_t *mfgr,
                       synapse_t *gogr);
void go_solve_update_v(neuron_t *d, neuron_solve_t *d_solve, neuron_t *p, neuron_solve_t *p_solve, synapse_t *grgo);
void pkj_solve_update_v(neuron_t *d, neuron_solve_t *d_solve, neuron_t *p, neuron_solve_t *p_solve,
                        synapse_t *grpkj, synapse_t *mlipkj);
void io_solve_update_v(neuron_t *d, neuron_solve_t *d_solve, neuron_t *p, neuron_solve_t *p_solve, gap_t *io_gap);

/* The RKC drivers X_solve_update_v runs for an RKC block (solve_rkc.cuh:23-26,
 * solve_rkc.cu:1122-1362): the same one-interval advance. */
void gr_solve_by_rkc(neuron_t *d, neuron_solve_t *d_solve, neuron_t *p, neuron_solve_t *p_solve, synapse_t *mfgr,
                     synapse_t *gogr);
void go_solve_by_rkc(neuron_t *d, neuron_solve_t *d_solve, neuron_t *p, neuron_solve_t *p_solve, synapse_t *grgo);
void pkj_solve_by_rkc(neuron_t *d, neuron_solve_t *d_solve, neuron_t *p, neuron_solve_t *p_solve, synapse_t *grpkj,
                      synapse_t *mlipkj);
void io_solve_by_rkc(neuron_t *d, neuron_solve_t *d_solve, neuron_t *p, neuron_solve_t *p_solve, gap_t *io_gap);

/* The reference's stimulus protocols, as kernels over the device neuron_t
 * (launch <<<n / 128 + 1, 128>>> on the default stream, as main.cu does) and
 * as host launchers for callers without a CUDA compiler.  GrC: 0.01 nA at the
 * soma for 50 <= t < 100 ms (gr.cu:244-253); GoC: 0.2 nA at compartment 30
 * for 800 <= t < 1100 (go.cu:257-267); PC: 0.1 nA at the soma for
 * 550 <= t < 1300 (pkj.cu:332-343); IO: 5.5 uA/cm^2 at the dendrite for
 * 800 <= t < 820 (io.cu:246-256).  Each is (t0, t1, amplitude). */
#define GBRKC_STIM_GR 50.0, 100.0, 0.01e-3
#define GBRKC_STIM_GO 800.0, 1100.0, 0.2e-3
#define GBRKC_STIM_PKJ 550.0, 1300.0, 0.1e-3
#define GBRKC_STIM_IO 800.0, 820.0, 5.5
#ifdef __CUDACC__
/* The kernels are defined here, not in the library: a caller's <<<>>>
 * launch then runs the caller's own copy through the caller's own CUDA
 * runtime, however each side links the runtime (a launch through another
 * module's kernel stub pairs the launch configuration across two runtimes
 * when they are linked statically). */
static __device__ __forceinline__ void gbrkc_set_current(neuron_t *d, int type, double t, double t0, double t1,
                                                         double amp) {
  const int id = threadIdx.x + blockIdx.x * blockDim.x;
  if (id < d->n) {
    const int ncomp = d->nc / d->n;
    /* GrC soma (16 in the reference's 578-compartment cell, else 1), GoC 30, PC soma (the last), IO 0 */
    const int comp = type == N_TYPE_IO ? 0 : type == N_TYPE_GO ? 30 : type == N_TYPE_PKJ ? ncomp - 1
                                                                                        : (ncomp == 578 ? 16 : 1);
    double *iv = &d->elem[i_ext][comp + id * ncomp];
    *iv = 0.0;
    if (t0 <= t && t < t1) *iv = amp;
  }
}
static __global__ void gr_set_current(neuron_t *d_gr, const double t) {
  gbrkc_set_current(d_gr, N_TYPE_GR, t, GBRKC_STIM_GR);
}
static __global__ void go_set_current(neuron_t *d_go, const double t) {
  gbrkc_set_current(d_go, N_TYPE_GO, t, GBRKC_STIM_GO);
}
static __global__ void pkj_set_current(neuron_t *d_pkj, const double t) {
  gbrkc_set_current(d_pkj, N_TYPE_PKJ, t, GBRKC_STIM_PKJ);
}
static __global__ void io_set_current(neuron_t *d_io, const double t) {
  gbrkc_set_current(d_io, N_TYPE_IO, t, GBRKC_STIM_IO);
}
#endif
void gr_set_current_launch(neuron_t *d_gr, const double t);
void go_set_current_launch(neuron_t *d_go, const double t);
void pkj_set_current_launch(neuron_t *d_pkj, const double t);
void io_set_current_launch(neuron_t *d_io, const double t);
/* The reference's alternative Purkinje stimulus (pkj.cu:346-368; its call
 * in main.cu, once per interval, is commented out): a 25 Hz Poisson train
 * for 350 <= t < 1000 ms, one rand() draw per call, filtered by
 * exp(-0.125 / 0.6 ms); every cell's soma gets 0.1 nA times the filtered
 * train.  The train's state is kept across calls, as the reference's. */
void pkj_set_current_Poisson(const int num, neuron_t *d_pkj, const double t);

/* One CSV row of soma voltages ("%lf," per value, t first; IO: its three
 * compartments per cell) and the raster lines "%lf,%d\n" of cells whose
 * spike compartment crossed the threshold since the previous call (GrC,
 * GoC, IO: 10 mV; PC: -10 mV).  v_host is the block's vec[v_new] copied to
 * the host; raster_prev holds one value per cell (the reference starts it at
 * 100).  (gr.cu:257, go.cu:271, pkj.cu:371, io.cu:260) */
void gr_output_file(neuron_t *p, double *v_host, double *raster_prev, const double t, FILE *f_v, FILE *f_raster);
void go_output_file(neuron_t *p, double *v_host, double *raster_prev, const double t, FILE *f_v, FILE *f_raster);
void pkj_output_file(neuron_t *p, double *v_host, double *raster_prev, const double t, FILE *f_v, FILE *f_raster);
void io_output_file(neuron_t *p, double *v_host, double *raster_prev, const double t, FILE *f_v, FILE *f_raster);

/* Release the block and close its files (gr.cu:221, go.cu:233, pkj.cu:309,
 * io.cu:225) and its solver mirror (gr_solve.cu:261, go_solve.cu:335,
 * pkj_solve.cu:368, io_solve.cu:272). */
void gr_finalize(neuron_t *p, neuron_t *d, FILE *f_v, FILE *f_raster);
void go_finalize(neuron_t *p, neuron_t *d, FILE *f_v, FILE *f_raster);
void pkj_finalize(neuron_t *p, neuron_t *d, FILE *f_v, FILE *f_raster);
void io_finalize(neuron_t *p, neuron_t *d, FILE *f_v, FILE *f_raster);
void gr_solve_finalize(const int n, neuron_solve_t *d_solve, neuron_solve_t *p_solve);
void go_solve_finalize(const int n, neuron_solve_t *d_solve, neuron_solve_t *p_solve);
void pkj_solve_finalize(const int n, neuron_solve_t *d_solve, neuron_solve_t *p_solve);
void io_solve_finalize(const int n, neuron_solve_t *d_solve, neuron_solve_t *p_solve);

/* Coupling objects (syn.cuh:84-104, gap.cuh:19-21).  The constructors record
 * the synapse families (mfgr_create and grpkj_create take a rand() seed, as
 * the reference does).  Network mode (main.cu's network_sim) starts with the
 * first X_synapse_update, after the first interval: the blocks then move into
 * one engine, wired by the reference's rules (syn.cu:43-84, 146-262, 295-410,
 * 455-619; GrC -> PC targets from Pkj_location_info.csv, drawn with a
 * SplitMix64 stream seeded by that rand() value instead of cuRAND).  That
 * engine replays the first interval, which is bit-identical because the
 * synapses are still 0 in it, and from then on advances all blocks and
 * updates the synapses in one call per interval.  The wiring needs the
 * reference's 578-compartment granule cell (its axon compartments).  In
 * network mode a stimulus kernel must come before the interval's first
 * update call.  mlipkj is never updated or applied on the reference's RKC
 * path and is accepted only.  The IO gap junctions are part of the IO system
 * itself (built at io_initialize with the reference's conductance);
 * io_gap_create returns a handle for the caller to pass back and free. */
synapse_t *mfgr_create(const int n);
synapse_t *gogr_create(const int go_x, const int go_y, const int gr_x, const int gr_y);
synapse_t *grgo_create(const int gr_x, const int gr_y, const int go_x, const int go_y);
synapse_t *grpkj_create(const int gr_x, const int gr_y, const int pkj_x, const int pkj_y);
synapse_t *mlipkj_create(const int n_pkj, const int n_gr);
void mfgr_finalize(synapse_t *s, const int n);
void gogr_finalize(synapse_t *s, const int n);
void grgo_finalize(synapse_t *s, const int n);
void grpkj_finalize(synapse_t *s, const int n);
void mlipkj_finalize(synapse_t *s, const int n);
/* mfgr_create (with granule cells) and mlipkj_create (with granule and
 * Purkinje cells) open MF_RASTER.csv and MLI_RASTER.csv, as syn.cu:76, 726
 * do.  These append one row to them: the time, then one "%lf," conductance
 * per synapse in the reference's order (syn.cu:114, 804; main.cu:215 has
 * the first call, commented out).  Mossy-fibre values are 0 until network
 * mode starts, then the states of the last synapse update before the
 * current interval.  MLI synapses are never updated on the RKC path, so
 * their values are 0. */
void mf_output_file(synapse_t *mfgr, const double t, neuron_t *p_gr);
void mli_output_file(synapse_t *mlipkj, const double t, neuron_t *p_pkj);
void gr_synapse_update(const double t, const double DT, synapse_t *mfgr, synapse_t *gogr, neuron_t *d_go,
                       neuron_solve_t *p_gr_solve);
void go_synapse_update(const double t, const double DT, synapse_t *grgo, neuron_t *d_gr, neuron_solve_t *p_go_solve);
void pkj_synapse_update(const double t, const double DT, synapse_t *grpkj, synapse_t *mlipkj, neuron_t *d_gr,
                        neuron_solve_t *p_pkj_solve);
gap_t *io_gap_create(const int nx, const int ny);
void io_gap_finalize(gap_t *g);

/* Batched output -- this library's addition, no counterpart in the
 * reference.  Advance the type's block by n intervals in one device launch:
 * its stimulus protocol (the X_set_current rule above) is applied on the
 * device at each interval start, the output_file columns (the soma; IO: its
 * three compartments per cell) are recorded on the device for every
 * interval into rows (n x cells x columns doubles, interval-major), and the
 * raster crossings are found on the device (output_file's rule) and written
 * as (interval end time, cell) pairs sorted by time then cell.  The values
 * are the ones the per-interval path gives, bit for bit.  Returns the number
 * of crossings (at most spk_cap), GBRKC_ESOLVER (-5) when the block stopped
 * (a non-finite voltage), GBRKC_EOVERFLOW (-6) when spk_cap was too small,
 * GBRKC_EINVAL (-1) on bad arguments. */
long gbrkc_compat_advance_batch(int type, int n, double *rows, long row_cap, double *spk_t, int *spk_cell,
                                long spk_cap);

/* comptime.csv row (output.cu:3-36). */
void output_time(const int n_gr, const char *type1, const int n_go, const char *type2, const int n_pkj,
                 const char *type3, const int n_io, const char *type4, const double comp_time, const int sim_time);
void output_time2(const int n_gr, const char *type1, const int n_go, const char *type2, const int n_pkj,
                  const char *type3, const int n_io, const char *type4, const double comp_time,
                  const double comp_time_half, const int sim_time);

/* Golgi raster from the voltage file after a run (output.cu:38-81; its call
 * in main.cu is commented out): reads go_v_by_<S>.csv and writes
 * go_raster_by_<S>.csv as one row per interval, "t," then for each cell
 * "i," where its voltage crossed 0 mV upward (from -70 mV before the first
 * row) and "," otherwise.  S is picked from type by the reference's names
 * (BACKWARD_EULER, CRANK_NICOLSON, FORWARD_EULER, RUNGE_KUTTA_4 or RKC);
 * another name stops with the reference's message.  The reference's read
 * loop ends every file with "raster_FILE_ERROR1" and exit(1); this one
 * returns at the end of the file. */
void raster_plot(const int n_go, const char *type);

#ifdef __cplusplus
}
#endif

#endif /* GBRKC_COMPAT_H */

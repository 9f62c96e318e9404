/*
 * CPU oracle for the explicit Runge-Kutta-Chebyshev (RKC) hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file and rkc_oracle.c are a plain-C, FP64
 * restatement of the reference simulator's RKC path (controller, stages,
 * power iteration, dense output, the four cell types' setup, gating, current
 * assembly and the inferior-olive gap junctions).  They exist to check the
 * CUDA product against; nothing in the product links, loads or calls them.
 *
 * Pinning: the gating/ion kernels and the per-compartment setup are compared
 * bit-for-bit against the reference's own sources compiled for the host
 * (oracle/ref_harness, outputs in oracle/_ref); the full controller path is
 * pinned end-to-end by the reference's only checked-in artefact
 * (io_raster_by_RKC.csv: 8x8 IO cells, one spike each, 807.625-808.125 ms).
 *
 * Build with -ffp-contract=off so x86 and aarch64 hosts give identical bits.
 */
#ifndef RKC_ORACLE_H
#define RKC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* cell types, numbered like the reference's neuron_type_t (param.h:17) */
enum { ORC_GR = 0, ORC_GO = 1, ORC_PKJ = 2, ORC_IO = 3 };

/* fields per morphology row, per type, in the reference file formats:
 *  GR  (Gr.txt, gr.cu:31-35):      i1 i2 d1 d2 d3 d4 i3 + 10 densities  = 17
 *  GO  (Go_131.txt, go.cu:33-38):  i1 i2 d1 d2 d3 d4 i3 + 13 densities  = 20
 *  PKJ (Pkj.txt, pkj.cu:35-40):    i1 i2 x y z d i3                     = 7
 *  IO  (IO.txt, io.cu:28-33):      i1 i2 d1 d2 d4 i3                    = 6 */
int orc_row_fields(int type);

typedef struct orc_sys orc_sys;

typedef struct {
  int type;            /* ORC_* */
  int nx, ny;          /* grid of cells forming ONE RKC system */
  int ncomp;           /* compartments per cell */
  const double *rows;  /* ncomp * orc_row_fields(type) */
  const int *gj_pairs; /* PKJ only: 2*n_gj_pairs (pre, post) per cell pair (Pkj_GJ.csv) */
  int n_gj_pairs;
  const double *jitter;/* n = nx*ny per-cell V0 jitter (init_v_rand of *_initialize_ion) */
  /* stimulus: per cell one step current (compartment, amplitude, [t_on, t_off)) */
  const int *stim_comp;   /* n entries, -1 = none */
  const double *stim_amp, *stim_t0, *stim_t1;
  const double *io_gap_g; /* IO only: 4*n edge conductances, NULL = reference G_C */
  double tol;          /* <= 0: reference per-type default */
  double hmin;         /* <= 0: reference per-type default */
  int io_gap;          /* IO: 1 = build the nonlinear gap network (reference: n > 1) */
  int go_gj, pkj_gj;   /* 1 = add the linear GJ entries to the CSR (reference: n > 1) */
  int canon;           /* 1 = canonical arithmetic (canon_math.h), bit-comparable with
                          the GPU plain-FP64 path; 0 = the reference's literal expressions */
  const double *cond_scale; /* n factors on every channel density of a cell, NULL = 1
                          (synthetic variation; the reference's densities are fixed) */
  const double *cond_scale_ch; /* n*ncond factors, one per channel density of each cell
                          (replaces cond_scale), or NULL */
} orc_desc;

orc_sys *orc_create(const orc_desc *d);
void orc_destroy(orc_sys *s);

/* RKC_vec_initialize (solve_rkc.cu:757-791); returns idid (3 = failure) */
int orc_init(orc_sys *s);

/* one reference outer interval: *_set_current(t) then *_solve_by_rkc
 * (solve_rkc.cu:1122-1362); returns 0 or an idid error code */
int orc_advance(orc_sys *s, double t);

int orc_nc(const orc_sys *s);
int orc_n(const orc_sys *s);
const double *orc_vnew(const orc_sys *s);   /* vec[v_new] after the interval */
const double *orc_elem_v(const orc_sys *s); /* elem[v] */
const double *orc_b(const orc_sys *s);
const double *orc_ion(const orc_sys *s, int k);
const double *orc_ca(const orc_sys *s);
/* controller scalars: absh sprad naccpt errold hold lt tend sum_dt */
void orc_ctl(const orc_sys *s, double *out8);
/* counters: steps, rejects, stage evals (sum of m), rho calls, ion updates,
 * power-iteration RHS evaluations */
void orc_stats(const orc_sys *s, long long *out6);
/* Network mode: systems advanced together with the reference's chemical
 * synapses (syn.cu).  Systems advance in the order added; kinds 0..3 are
 * MF->GrC, GrC->GoC, GoC->GrC, GrC->PC; rates all 0 = the reference's
 * 5 / 60 Hz over 900-1000 ms.  Fields of orc_net_syn: 0 val, 1..3 states,
 * 4 old_v.  The network does not own its systems. */
typedef struct orc_net orc_net;
orc_net *orc_net_create(void);
int orc_net_add_system(orc_net *n, orc_sys *s);
/* per-synapse transmission delays (0..63 intervals) of synapses first ..
 * first+count-1; 0 (the default) is the reference's rule */
int orc_net_set_delays(orc_net *n, int first, int count, const int *delay);
int orc_net_add_synapses(orc_net *n, int kind, int count, const int *pre_sys, const int *pre_comp,
                         const int *post_sys, const int *post_comp, const double *w, double rate_base,
                         double rate_stim, double t0, double t1, unsigned long long seed);
int orc_net_build(orc_net *n);
int orc_net_advance(orc_net *n, double t);
int orc_net_nsyn(const orc_net *n);
const double *orc_net_syn(const orc_net *n, int field);
void orc_net_destroy(orc_net *n);

/* Row swaps taken by the Na / KAHP Markov solvers so far (process-wide). */
long long orc_pivot_swaps(void);
/* The canonical exp / log / pow of canon_math.h. */
double orc_cm_exp(double x);
double orc_cm_log(double x);
double orc_cm_pow(double x, double y);
double orc_cm_cbrt(double x);

/* static setup, for the setup pins: Cm, area, cond k, shell, CSR */
const double *orc_cm(const orc_sys *s);
const double *orc_area(const orc_sys *s);
const double *orc_cond(const orc_sys *s, int k);
int orc_ncond(const orc_sys *s);
int orc_nion(const orc_sys *s);
const double *orc_shell(const orc_sys *s);
const double *orc_rev_ca2(const orc_sys *s);
int orc_nnz(const orc_sys *s);
const int *orc_row(const orc_sys *s);
const int *orc_col(const orc_sys *s);
const double *orc_val(const orc_sys *s);

/* Ion-kernel probe: run one RKC ion update (the *_update_ion_RKC family)
 * on the current state with an explicit vnew and DT, without b.  Used to
 * compare against the reference's ion kernels compiled for the host. */
void orc_ion_update(orc_sys *s, const double *vnew, double dt);
void orc_update_b(orc_sys *s, const double *vy);
/* set state arrays directly (probe setup) */
void orc_set_elem_v(orc_sys *s, const double *v);
void orc_set_ion(orc_sys *s, int k, const double *x);
void orc_set_ca(orc_sys *s, const double *x);

/* per-cell V0 jitter drawn from libc rand() with the type's formula
 * (gr_ion.cu:642, go_ion.cu:598, pkj_ion.cu:367, io_ion.cu:172) */
void orc_draw_jitter(int type, int n, double *out);

#ifdef __cplusplus
}
#endif
#endif

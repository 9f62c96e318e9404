/*
 * gbrkc: GB300-native explicit Runge-Kutta-Chebyshev (RKC) solver for the
 * reference's cerebellar multi-compartment cell models -- C ABI.
 *
 * An engine owns device memory for many RKC "systems".  A system is what the
 * reference integrates with one step size: the nx*ny cells of one type with
 * their gap junctions (the reference's per-type block, main.cu:105-134), or a
 * single cell, or one inferior-olive gap-junction network.  Every system
 * keeps its own step size, stage count, spectral radius and ion-update clock,
 * exactly as the reference's *_solve_by_rkc does for its one system per type
 * (solve_rkc.cu:1122-1362); batching only changes packing.
 *
 * All functions return 0 on success or a negative GBRKC_E* code; the message
 * is available from gbrkc_last_error().  Plain pointers and sizes only.
 */
#ifndef GBRKC_H
#define GBRKC_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbrkc_engine gbrkc_engine;

enum { GBRKC_GR = 0, GBRKC_GO = 1, GBRKC_PKJ = 2, GBRKC_IO = 3 };
enum { GBRKC_FP64 = 0, GBRKC_MIXED = 1 };
enum {
  GBRKC_OK = 0,
  GBRKC_EINVAL = -1,   /* bad argument */
  GBRKC_ECUDA = -2,    /* CUDA error (no device, launch failure, ...) */
  GBRKC_ESTATE = -3,   /* call out of order (e.g. add after build) */
  GBRKC_ENOMEM = -4,   /* device or host allocation failed */
  GBRKC_ESOLVER = -5,  /* a system stopped: see gbrkc_system_ctl status */
  GBRKC_EOVERFLOW = -6 /* a fixed-size log or queue was full: entries were lost */
};
/* fields readable with gbrkc_read */
enum {
  GBRKC_F_VNEW = 0,    /* vec[v_new]: voltage at the end of the last interval */
  GBRKC_F_V = 1,       /* elem[v]: voltage the gating last saw */
  GBRKC_F_CA = 2,      /* elem[Ca] */
  GBRKC_F_B = 3,       /* frozen current vector b */
  GBRKC_F_ION = 4,     /* gating slot k (as FP64) */
  GBRKC_F_REV = 5,     /* Ca reversal potential (GO, PKJ) */
  GBRKC_F_YN = 6,      /* RKC solution vector yn */
  GBRKC_F_IEXT = 7     /* elem[i_ext]: injected current (device pointer only) */
};

typedef struct gbrkc_system_desc {
  int cell_type;            /* GBRKC_GR .. GBRKC_IO */
  int nx, ny;               /* cells of the system, on an nx x ny grid */
  int ncomp;                /* compartments per cell */
  const double *rows;       /* ncomp rows in the reference's parameter-file layout
                               (Gr.txt 17, Go_131.txt 20, Pkj.txt 7, IO.txt 6 fields) */
  const int *gj_pairs;      /* PKJ: (pre, post) compartment pairs between x-neighbours */
  int n_gj_pairs;
  int gap_junctions;        /* 1: the reference's gap junctions for this type when
                               nx*ny > 1 (GO and PKJ linear in the operator, IO nonlinear) */
  const double *io_gap_g;   /* IO: 4*nx*ny edge conductances, or NULL for the reference's */
  const double *jitter;     /* nx*ny initial-voltage jitters (init_v_rand of *_initialize_ion) */
  const int *stim_comp;     /* nx*ny stimulated compartment per cell or -1; NULL: no stimulus */
  const double *stim_amp;   /* step current amplitude ... */
  const double *stim_t0;    /* ... switched on at t0 (ms) ... */
  const double *stim_t1;    /* ... and off at t1, evaluated at each interval start */
  double tol;               /* RKC rtol = atol; <= 0: reference per-type value */
  double hmin;              /* minimum step (ms); <= 0: reference per-type value */
  const double *cond_scale; /* nx*ny factors on every channel density of the cell, or NULL
                               (no counterpart in the reference: its densities are fixed) */
  int idle;                 /* nonzero: a free slot -- neither initialised nor advanced
                               until gbrkc_systems_reset fills it */
  const double *cond_scale_ch; /* nx*ny*NCOND factors, one per channel density of each
                               cell in the type's conductance order (GrC 10, GoC 13,
                               PC 11, IO 8), replacing cond_scale; or NULL (no
                               counterpart in the reference) */
} gbrkc_system_desc;

/* Create an engine on the current CUDA device.  precision: GBRKC_FP64 (plain
 * FP64 everywhere) or GBRKC_MIXED (FP32 gating, channel currents and b; FP64
 * voltage, stages, spectral radius and step control). */
int gbrkc_engine_create(int precision, gbrkc_engine **out);
void gbrkc_engine_destroy(gbrkc_engine *e);

/* Register a system (host copies are taken); returns its id. */
int gbrkc_add_system(gbrkc_engine *e, const gbrkc_system_desc *d, int *sys_id);

/* Allocate and upload everything, then initialise every system on the device
 * (RKC_vec_initialize, solve_rkc.cu:757-791). */
int gbrkc_build(gbrkc_engine *e);

/* Advance every system by n_intervals output intervals of 0.125 ms, the
 * first one starting at time t0 (ms), in one device-resident launch per cell
 * type.  Equivalent to the reference's main loop calling *_set_current and
 * *_solve_update_v once per interval (main.cu:182-311).  A system whose step
 * becomes non-finite stops (the reference exits, main.cu:202); here it is
 * retired -- kept readable, skipped afterwards -- and GBRKC_ESOLVER reports
 * the systems that stopped during this call while all others advanced. */
int gbrkc_advance(gbrkc_engine *e, double t0, int n_intervals);
/* Number of retired systems so far. */
int gbrkc_retired_systems(gbrkc_engine *e);

/* Measure and keep the best number of granule systems per warp (cells per
 * warp, hence per CTA, of the persistent launch): the launch that
 * gbrkc_advance(e, t0, n_intervals) would make runs once per candidate (32,
 * 16, 8 lanes; twice each, the shorter time counts) from a device snapshot
 * of the engine, and the fastest is kept for the following advances.  The
 * engine's state, its CTA split between cell types and its soma / spike
 * records are restored, so the simulation is where it was; results never
 * depend on the choice (scheduling only).  Allocates the snapshot (the
 * engine's device footprint) for the duration of the call.  Engines with
 * synapses are refused.  *lanes_out receives the kept count (unchanged
 * when the engine has no granule lanes).  No counterpart in the reference,
 * whose launch shape is fixed at 128 threads (gr_solve.cu:198-199). */
int gbrkc_autotune(gbrkc_engine *e, double t0, int n_intervals, int *lanes_out);

/* Copy n values of a per-compartment field of one system to host memory. */
int gbrkc_read(gbrkc_engine *e, int sys_id, int field, int k, double *host, long n);

/* Controller scalars (absh sprad naccpt errold hold lt tend sum_dt), counters
 * (steps rejects stages rho_calls ion_updates rho_iterations) and status. */
int gbrkc_system_ctl(gbrkc_engine *e, int sys_id, double *ctl8, long long *stats6, int *status);
int gbrkc_system_nc(gbrkc_engine *e, int sys_id);

/* Record the soma voltage of every cell at the end of each interval for the
 * next n_intervals_max intervals (0 disables); read them per system as
 * [interval][cell]. */
int gbrkc_record_soma(gbrkc_engine *e, int n_intervals_max);
int gbrkc_read_soma(gbrkc_engine *e, int sys_id, int n_intervals, double *host);

/* Replace the step-current table of one system (host buffers, nx*ny each);
 * takes effect from the next interval. */
int gbrkc_set_stim(gbrkc_engine *e, int sys_id, const int *comp, const double *amp,
                   const double *t0, const double *t1);

/* The same for every cell of one type at once: arrays of gbrkc_type_cells()
 * entries, cells in system order (bulk host-to-device copies). */
int gbrkc_type_cells(gbrkc_engine *e, int cell_type);
int gbrkc_set_stim_type(gbrkc_engine *e, int cell_type, const int *comp, const double *amp,
                        const double *t0, const double *t1);
/* Soma recording of every cell of one type, [interval][cell] (one copy), and
 * restart of the recording window without reallocating. */
int gbrkc_read_soma_type(gbrkc_engine *e, int cell_type, int n_intervals, double *host);
/* Record `width` compartments per cell of a type instead of the soma: the
 * cell's compartments 0 .. width-1 (the IO output_file writes all three).
 * Call before gbrkc_record_soma; the soma reads then return
 * [interval][cell][width]. */
int gbrkc_record_width(gbrkc_engine *e, int cell_type, int width);
int gbrkc_rewind_soma(gbrkc_engine *e);

/* Device time of the last gbrkc_advance (CUDA events on the launching
 * streams): whole advance, and the kernel of one cell type. */
float gbrkc_last_advance_ms(gbrkc_engine *e);
float gbrkc_last_kernel_ms(gbrkc_engine *e, int cell_type);

/* Launch layout: returns 1 when all cell types advance in one persistent
 * launch (CTAs per type written to ctas_per_type[4]), 0 when each type has
 * its own launch (entries: that launch's CTAs, 0 for an empty type),
 * negative on error. */
int gbrkc_launch_layout(gbrkc_engine *e, int *ctas_per_type);

/* How a cell type's systems are integrated, for reports: GBRKC_TEAM_MEGA (the
 * persistent mixed-role launch), GBRKC_TEAM_GRID (one system over the SMs of a
 * cooperative launch), GBRKC_TEAM_CLUSTER (one system per thread-block
 * cluster) or GBRKC_TEAM_POOL (the type's own launch: a lane, warp or CTA per
 * system); 0 for an empty type, negative on error. */
enum { GBRKC_TEAM_MEGA = 1, GBRKC_TEAM_GRID = 2, GBRKC_TEAM_CLUSTER = 3, GBRKC_TEAM_POOL = 4 };
int gbrkc_type_team(gbrkc_engine *e, int cell_type);

/* The grid team's launch shape for a lone system of nc compartments on at
 * most max_ctas co-resident CTAs (the engine uses the device's SM count):
 * CTAs of threads_per_cta threads (a power of two, 32..256), each thread
 * owning elements i with i mod (ctas * threads_per_cta) its index.  The rule
 * minimises the busiest CTA's elements, then the CTA count, within 256
 * chunks of threads_per_cta elements and 8 elements a thread.  Host only
 * (no device needed); GBRKC_EINVAL when no shape holds nc. */
int gbrkc_grid_shape(long long nc, int max_ctas, int *threads_per_cta, int *ctas);

/* ---- chemical synapses (network mode) ----------------------------------
 * The reference's RKC network path (syn.cu; main.cu:300-305 with
 * network_sim true): mossy fibre -> granule (Poisson input), granule ->
 * Golgi, Golgi -> granule and granule (parallel fibre) -> Purkinje.  Every
 * 0.125 ms interval, all systems advance, then each synapse decays its
 * states by exp(-0.125 / tau), steps them by one when its presynaptic
 * compartment's voltage crossed 0 mV upward (or its Poisson fibre fired) and
 * recomputes its conductance (syn.cu:86-111, 263-288, 412-437, 646-668).
 * Granule cells add g (V - E) of each synapse to b at every ion update;
 * Golgi and Purkinje cells take the synaptic current at the start of the
 * interval and add it at each ion update, Purkinje cells scaled by
 * exp(-sum_dt / 0.6) (solve_rkc.cu:198-360, 1100-1120, 1180-1270).
 * The micro-circuit's inhibition onto Purkinje cells is absent from the
 * reference's RKC path (never updated or applied) and is not provided.
 * Poisson draws use a counter-based generator (seed, synapse, interval)
 * instead of the reference's cuRAND streams.  Synapses make gbrkc_advance
 * run one launch per interval. */
enum { GBRKC_SYN_MFGR = 0, GBRKC_SYN_GRGO = 1, GBRKC_SYN_GOGR = 2, GBRKC_SYN_GRPKJ = 3 };
/* per-synapse state readable with gbrkc_read_synapses */
enum { GBRKC_SYNF_VAL = 0, GBRKC_SYNF_S0 = 1, GBRKC_SYNF_S1 = 2, GBRKC_SYNF_S2 = 3, GBRKC_SYNF_OLD_V = 4 };

typedef struct gbrkc_synapse_desc {
  int kind;                       /* GBRKC_SYN_* */
  int n;                          /* synapses in this group */
  const int *pre_system;          /* per synapse (unused for GBRKC_SYN_MFGR) */
  const int *pre_comp;            /* presynaptic compartment within its system */
  const int *post_system;         /* per synapse */
  const int *post_comp;           /* postsynaptic compartment within its system */
  const double *weight;           /* per synapse (the reference's W_* / count factors) */
  double rate_base, rate_stim;    /* GBRKC_SYN_MFGR firing rates [Hz]: rate_stim for */
  double stim_t0, stim_t1;        /*   stim_t0 <= t < stim_t1 [ms], else rate_base; all 0 = */
                                  /*   the reference's 5 / 60 Hz over 900-1000 ms */
  unsigned long long seed;        /* GBRKC_SYN_MFGR Poisson stream */
  const int *delay;               /* per synapse: transmission delay in 0.125 ms intervals,
                                     0..63, or NULL (0: the reference's same-interval rule).
                                     No counterpart in the reference (its synapses act in the
                                     interval of the presynaptic crossing or fibre draw) */
} gbrkc_synapse_desc;

/* Add a group of synapses between systems already added (before
 * gbrkc_build); *first_id receives the id of its first synapse (ids are
 * consecutive, in the engine-wide table).  Kinds fix the cell types:
 * MFGR onto granule cells, GRGO granule -> Golgi, GOGR Golgi -> granule,
 * GRPKJ granule -> Purkinje.  (mfgr_create, grgo_create, gogr_create,
 * grpkj_create: syn.cu:63, 183, 336, 520) */
int gbrkc_add_synapses(gbrkc_engine *e, const gbrkc_synapse_desc *d, int *first_id);

/* Copy one per-synapse field (GBRKC_SYNF_*) of the first n synapses. */
int gbrkc_read_synapses(gbrkc_engine *e, int field, double *host, long n);

/* gbrkc_advance for callers that must not trigger a device allocation
 * while they step: for example a host already running other GPU work under
 * its own memory allocator, whose budget or pool a library cudaMalloc would
 * break into, or a real-time stepping loop that cannot take the device-wide
 * synchronisation a cudaMalloc / cudaFree may impose.  This call makes no
 * device allocation of any kind, and on success no host allocation either
 * (only an error message is stored as a string).  The persistent launch's
 * scratch -- per-role work-queue counters and per-CTA timestamps -- comes
 * from one fixed array in the library's static device memory, sized for
 * launches of at most 1024 CTAs (16.6 KB, held on every GPU that loads the
 * library until the process exits); a larger launch is rejected with
 * GBRKC_EINVAL.  Engines advanced one pool per launch need no scratch and
 * take the same path as gbrkc_advance.
 *   - gbrkc_build looks the array's address up on the engine's device and
 *     keeps it in the engine; this call only reads it.  An engine built
 *     after a device reset gets the reloaded array's address.
 *   - The call waits for its launch to finish and reads the status words
 *     back (device synchronisation, no allocation).
 *   - Every call shares the one array: calls whose work overlaps on the GPU
 *     (e.g. two host threads advancing two engines at once) race on it and
 *     corrupt each other's scheduling.  Serialise them.
 *   - Results are the same as gbrkc_advance's, bit for bit.  Unlike it, this
 *     call does not update gbrkc_retired_systems; it returns GBRKC_ESOLVER
 *     whenever any system of the engine is stopped (the others advance).
 * Engines with synapses are refused (they step through gbrkc_advance).
 * The engine itself is still allocated by gbrkc_build.  No counterpart in
 * the reference (it allocates through cudaMalloc at initialisation only). */
int gbrkc_advance_noalloc(gbrkc_engine *e, double t0, int n_intervals);

/* Device address of one system's per-compartment array (GBRKC_F_VNEW, _V,
 * _CA, _REV or _IEXT; nc doubles, the system's compartments in order).  Valid
 * until the engine is destroyed; the array is written by gbrkc_advance and may
 * be read (or, for _IEXT, written) by the caller's own kernels between
 * advances.  Replaces the device pointers the reference exposes through
 * neuron_t::elem and neuron_solve_t::vec (param.h:27-46). */
int gbrkc_field_device_ptr(gbrkc_engine *e, int system_id, int field, double **device_ptr);

/* Compartment updates so far (sum over systems of (stage evaluations + step
 * attempts) x compartments; power iterations excluded), for one cell type
 * or, with cell_type = -1, all.  Negative on error. */
long long gbrkc_compartment_updates(gbrkc_engine *e, int cell_type);

/* Total compartments over all systems. */
long gbrkc_total_compartments(gbrkc_engine *e);
const char *gbrkc_last_error(void);

/* ---- slots: re-using built systems (the request server's arena) ----
 * A built system can be refilled in place with a new cell of the same shape
 * (same type, morphology, grid and tolerance): new initial-voltage jitters,
 * stimulus, conductance scales and, for IO networks, edge conductances.  It
 * is then initialised on the device at the start of the next advance (only
 * the reset systems are; RKC_vec_initialize, solve_rkc.cu:757-791) and
 * integrates exactly as a freshly built system would: its own clock starts
 * at 0, and only the stimulus windows use the advance's time.  An interval
 * budget stops a system after that many intervals (it stays readable);
 * a budget of 0 parks it. */
typedef struct gbrkc_reset_desc {
  const double *jitter;     /* one per cell of the systems, in order */
  const int *stim_comp;     /* per cell: stimulated compartment or -1; NULL: none */
  const double *stim_amp, *stim_t0, *stim_t1;  /* per cell (times as the advances pass them) */
  const double *cond_scale; /* per cell, or NULL (1) */
  const double *io_gap_g;   /* IO networks: 4 per cell, or NULL (keep) */
  int n_intervals;          /* budget from now on; -1: none */
  const double *cond_scale_ch; /* per cell and channel (as gbrkc_system_desc), or NULL */
} gbrkc_reset_desc;

/* Reset systems first_id .. first_id+n-1, which must be consecutive systems
 * of one cell type (one run of its pool).  Not for engines with synapses. */
int gbrkc_systems_reset(gbrkc_engine *e, int first_id, int n, const gbrkc_reset_desc *d);
/* A field (GBRKC_F_VNEW, _V, _CA or _REV) of systems first_id .. first_id+n-1
 * (one run) in one copy: their compartments in order; cap >= their count. */
int gbrkc_read_run(gbrkc_engine *e, int first_id, int n, int field, double *host, long cap);
/* Status words (0: healthy, else GBRKC solver stop bits) and interval budgets
 * left of one run of systems; either pointer may be NULL. */
int gbrkc_run_status(gbrkc_engine *e, int first_id, int n, int *status, int *iv_left);
/* Set the interval budget of systems first_id .. first_id+n-1 (one run). */
int gbrkc_set_budget(gbrkc_engine *e, int first_id, int n, int n_intervals);
/* Device bytes one system of this shape takes in an engine (an upper
 * estimate for admission control), or a negative error code. */
long long gbrkc_system_bytes(int precision, int cell_type, int ncomp, int ncell);
/* The RKC stage coefficients the kernels use for m stages (1 <= m <= 1024),
 * tabulated on the host by the recurrences of solve_rkc.cu:816-906: mu~_1,
 * then for each stage j = 2..m the five values mu_j, nu_j, 1 - mu_j - nu_j,
 * mu~_j and a_{j-1}.  Returns the count, 1 + 5 (m - 1), or a negative error
 * code.  Needs no device. */
long gbrkc_rkc_coefficients(int m, double *out, long cap);

/* ---- device raster ----
 * At the end of every interval each cell's spike compartment is compared
 * with the reference's output_file rule (value > threshold and the previous
 * interval's value <= threshold; GrC/GoC/IO 10 mV on compartments 77 / 30 /
 * 2 (GrC reduced cells: the last), PC -10 mV on the soma: gr.cu:257,
 * go.cu:271, pkj.cu:371, io.cu:260), on the device.  gbrkc_record_spikes
 * gives every cell type a log of `capacity` crossings (0 turns it off);
 * gbrkc_read_spikes drains one type's log, sorted by (time, cell), as
 * interval end times, engine system ids and cells within the system.
 * GBRKC_EOVERFLOW reports crossings lost to a full log or a short read. */
int gbrkc_record_spikes(gbrkc_engine *e, long capacity);
int gbrkc_read_spikes(gbrkc_engine *e, int cell_type, long cap, double *t, int *sys, int *cell, long *n);

/* ---- request server ----
 * Simulation jobs of uneven cell counts and durations, admitted into a
 * device-resident arena and advanced together (no counterpart in the
 * reference, which integrates one fixed block per type per process).
 *
 * A slot class is one system shape (a single cell, or an nx x ny network of
 * one type).  gbrkc_server_start sizes each class's arena -- explicit slot
 * counts first, then shares of the rest of the HBM budget (0: 80% of the
 * free device memory) -- and builds one engine holding every slot, idle.
 * A request names a class, a number of systems and a duration in 0.125 ms
 * intervals, with per-cell jitters, stimulus (times relative to the
 * request's start), conductance scales and IO edge conductances.  Each
 * gbrkc_request_advance is one serving round: admit the queued requests
 * whose systems fit the free slots (first come first served; a later
 * request that fits may overtake a head that does not, at most 8 times),
 * advance every resident request by the quantum in one persistent launch
 * (each stops at exactly its own interval count), route the device raster
 * to the requests, and complete the requests that are done.  A served
 * request's results are bit-identical to an engine of its own started at 0.
 * Latency is submission to completion, on the host's steady clock. */
typedef struct gbrkc_server gbrkc_server;
enum { GBRKC_REQ_QUEUED = 0, GBRKC_REQ_RESIDENT = 1, GBRKC_REQ_DONE = 2, GBRKC_REQ_FAILED = 3 };

typedef struct gbrkc_slot_class {
  gbrkc_system_desc shape;  /* type, grid, morphology, junctions, tol, hmin (per-cell inputs ignored) */
  long long slots;          /* systems to hold, or 0 ... */
  double share;             /* ... a fraction of the budget left after the explicit classes */
} gbrkc_slot_class;

typedef struct gbrkc_request_desc {
  int class_id;
  int n_systems;            /* systems of the class's shape */
  int n_intervals;          /* duration in 0.125 ms intervals */
  const double *jitter;     /* per cell (n_systems x cells per system) */
  const int *stim_comp;     /* per cell, or NULL */
  const double *stim_amp, *stim_t0, *stim_t1;  /* per cell; times from the request's start */
  const double *cond_scale; /* per cell, or NULL */
  const double *io_gap_g;   /* IO networks: 4 per cell, or NULL */
} gbrkc_request_desc;

typedef struct gbrkc_server_stats_t {
  long long submitted, admitted, completed, failed, cancelled, queued, resident, rounds;
  double p50_ms, p99_ms, mean_ms, max_ms;  /* latency of the completed requests */
  double busy_s;            /* host time inside gbrkc_request_advance */
  double advance_s;         /* of which inside the engine's advance */
  long long compartment_updates;
  long long hbm_reserved, hbm_in_use;      /* arena bytes: all slots, occupied slots */
  long long slots, free_slots;
  double sim_ms;            /* the server's clock */
  long long lost_spike_reads;
} gbrkc_server_stats_t;

int gbrkc_server_create(int precision, long long hbm_budget, int quantum_intervals, gbrkc_server **out);
int gbrkc_server_add_class(gbrkc_server *s, const gbrkc_slot_class *c, int *class_id);
int gbrkc_server_start(gbrkc_server *s);
int gbrkc_server_class_slots(gbrkc_server *s, int class_id, int *slots, int *first_system);
int gbrkc_request_create(gbrkc_server *s, const gbrkc_request_desc *d, int *req_id);
int gbrkc_request_advance(gbrkc_server *s, int *n_completed);
int gbrkc_request_state(gbrkc_server *s, int req_id, int *state, double *latency_ms, int *status);
/* final v_new of every compartment of the request, systems in order */
int gbrkc_request_read(gbrkc_server *s, int req_id, double *host, long cap);
/* threshold crossings: times from the request's start, cells in request order */
int gbrkc_request_spikes(gbrkc_server *s, int req_id, long cap, double *t, int *cell, long *n);
/* cancel a queued or resident request, or forget a finished one */
int gbrkc_request_destroy(gbrkc_server *s, int req_id);
int gbrkc_server_stats(gbrkc_server *s, gbrkc_server_stats_t *out);
gbrkc_engine *gbrkc_server_engine(gbrkc_server *s);
const char *gbrkc_server_last_error(void);
void gbrkc_server_destroy(gbrkc_server *s);

#ifdef __cplusplus
}
#endif
#endif

// The reference's per-type entry points (include/gbrkc_compat.h) over the
// gbrkc C ABI.  One engine and one FP64 system per cell type, as the
// reference integrates one block per type (main.cu:105-134); the host mirror
// structs hold device pointers into the engine's arrays, so a caller reads
// vec[v_new] with its own cudaMemcpy and writes elem[i_ext] with its own
// stimulus kernel, as it does with the reference.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/gbrkc.h"
#include "../../include/gbrkc_compat.h"

namespace {

constexpr int NTYPES = 4;
const char *TYPE_NAME[NTYPES] = {"gr", "go", "pkj", "io"};
// reference parameter files (gr.cuh, go.cuh:22, pkj.cuh, io.cuh)
const char *MODEL_FILE[NTYPES] = {"Gr.txt", "Go_131.txt", "Pkj.txt", "IO.txt"};
const int ROW_FIELDS[NTYPES] = {17, 20, 7, 6};
const int REF_NCOMP_GR = 578;

struct Block {
  gbrkc_engine *eng = nullptr;
  int sid = -1;
  int n = 0, ncomp = 0;
  int stim_comp = 0;              // compartment of every cell the protocol drives
  int batch_cap = 0;              // batched output: intervals the recorder holds
  double t = 0.0;                 // start of the next interval
  neuron_t *d_neuron = nullptr;   // device copy of the mirror (for stimulus kernels)
  double **d_elem = nullptr;      // device table behind d_neuron->elem
  double **h_elem = nullptr;      // host table behind p->elem
  double **h_vec = nullptr;       // host table behind p_solve->vec
  neuron_solve_t *d_solve = nullptr;
};
Block g_block[NTYPES];

[[noreturn]] void die(const char *what) {
  printf("%s\n", what);
  exit(1);
}

void check(int rc, const char *what) {
  if (rc != 0) {
    printf("%s: %s\n", what, gbrkc_last_error());
    exit(1);
  }
}

void cuda_check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) {
    printf("%s: %s\n", what, cudaGetErrorString(e));
    exit(1);
  }
}

std::string model_path(const char *name) {
  const char *dir = getenv("GBRKC_MODEL_DIR");
  std::string p = (dir && dir[0]) ? std::string(dir) + "/" : std::string("./");
  return p + name;
}

// whitespace-separated numbers of a reference parameter file
std::vector<double> read_numbers(const std::string &path, char sep_extra) {
  FILE *f = fopen(path.c_str(), "r");
  if (!f) {
    printf("cannot open %s\n", path.c_str());
    exit(1);
  }
  std::vector<double> out;
  std::string tok;
  int ch;
  while ((ch = fgetc(f)) != EOF) {
    if (ch == ' ' || ch == '\t' || ch == '\n' || ch == '\r' || ch == sep_extra) {
      if (!tok.empty()) out.push_back(strtod(tok.c_str(), nullptr));
      tok.clear();
    } else {
      tok.push_back((char)ch);
    }
  }
  if (!tok.empty()) out.push_back(strtod(tok.c_str(), nullptr));
  fclose(f);
  return out;
}

// compartment that is stimulated / written / tested for spikes, by the
// reference's rules (gr.cu:250,264,270; go.cu:263,280,286; pkj.cu:339,382,
// 404; io.cu:252,271-283); a granule cell of another size uses its second
// compartment as soma and its last as the spike site
int soma_comp(int type, int ncomp) {
  if (type == GBRKC_PKJ) return ncomp - 1;
  if (type == GBRKC_GO) return 30;
  if (type == GBRKC_GR) return ncomp == REF_NCOMP_GR ? 16 : 1;
  return 1;
}
int raster_comp(int type, int ncomp) {
  if (type == GBRKC_PKJ) return ncomp - 1;
  if (type == GBRKC_GO) return 30;
  if (type == GBRKC_GR) return ncomp == REF_NCOMP_GR ? 77 : ncomp - 1;
  return 2;
}
double raster_threshold(int type) { return type == GBRKC_PKJ ? -10.0 : 10.0; }

// initial-voltage jitter: one rand() per cell in the reference's formula
// (gr_ion.cu:642, pkj_ion.cu:367: (rand + 1) / (RAND_MAX + 2) - 0.5;
// go_ion.cu:598, io_ion.cu:172: rand / RAND_MAX - 0.5)
std::vector<double> draw_jitter(int type, int n) {
  std::vector<double> j(n);
  for (int c = 0; c < n; c++) {
    if (type == GBRKC_GR || type == GBRKC_PKJ)
      j[c] = (((double)rand() + 1.0) / ((double)RAND_MAX + 2.0)) - 0.5;
    else
      j[c] = ((double)rand() / RAND_MAX) - 0.5;
  }
  return j;
}

__device__ int d_stim_comp[NTYPES];

neuron_t *initialize(int type, int nx, int ny, const char *solver, neuron_t *p) {
  if (strncmp(solver, "RKC", 3) != 0) {
    printf("%s: solver %s is not provided (only RKC)\n", TYPE_NAME[type], solver);
    exit(1);
  }
  Block &B = g_block[type];
  if (B.eng) die("block initialised twice");
  const int n = nx * ny;
  memset(p, 0, sizeof *p);
  p->n_solver = kRKC;
  p->neuron_type = type;
  p->n = n;
  p->nx = nx;
  p->ny = ny;
  p->DT = RKC_DT;
  B.n = n;
  B.t = 0.0;
  B.h_elem = (double **)calloc(n_elem, sizeof(double *));
  p->elem = B.h_elem;
  if (n > 0) {
    const std::vector<double> rows = read_numbers(model_path(MODEL_FILE[type]), 0);
    if (rows.empty() || rows.size() % ROW_FIELDS[type]) die("model file has a partial row");
    B.ncomp = (int)(rows.size() / ROW_FIELDS[type]);
    std::vector<double> jitter = draw_jitter(type, n);
    std::vector<int> pairs;
    if (type == GBRKC_PKJ) {
      const std::vector<double> gj = read_numbers(model_path("Pkj_GJ.csv"), ',');
      if (gj.size() % 2) die("Pkj_GJ.csv has a partial pair");
      for (double x : gj) pairs.push_back((int)x);
    }
    check(gbrkc_engine_create(GBRKC_FP64, &B.eng), "engine");
    gbrkc_system_desc d;
    memset(&d, 0, sizeof d);
    d.cell_type = type;
    d.nx = nx;
    d.ny = ny;
    d.ncomp = B.ncomp;
    d.rows = rows.data();
    d.gj_pairs = pairs.empty() ? nullptr : pairs.data();
    d.n_gj_pairs = (int)pairs.size() / 2;
    d.gap_junctions = 1;
    d.jitter = jitter.data();
    check(gbrkc_add_system(B.eng, &d, &B.sid), "add system");
    check(gbrkc_build(B.eng), "build");
    p->nc = n * B.ncomp;
    check(gbrkc_field_device_ptr(B.eng, B.sid, GBRKC_F_V, &B.h_elem[v]), "elem[v]");
    check(gbrkc_field_device_ptr(B.eng, B.sid, GBRKC_F_CA, &B.h_elem[Ca]), "elem[Ca]");
    check(gbrkc_field_device_ptr(B.eng, B.sid, GBRKC_F_IEXT, &B.h_elem[i_ext]), "elem[i_ext]");
    const int sc = (type == GBRKC_IO) ? 0 : (type == GBRKC_GO) ? 30 : soma_comp(type, B.ncomp);
    cuda_check(cudaMemcpyToSymbol(d_stim_comp, &sc, sizeof(int), type * sizeof(int)), "stimulus site");
    B.stim_comp = sc;
  }
  // device mirror for the stimulus kernels
  cuda_check(cudaMalloc(&B.d_elem, n_elem * sizeof(double *)), "device table");
  cuda_check(cudaMemcpy(B.d_elem, B.h_elem, n_elem * sizeof(double *), cudaMemcpyHostToDevice), "device table");
  neuron_t h = *p;
  h.elem = B.d_elem;
  cuda_check(cudaMalloc(&B.d_neuron, sizeof(neuron_t)), "device mirror");
  cuda_check(cudaMemcpy(B.d_neuron, &h, sizeof h, cudaMemcpyHostToDevice), "device mirror");
  return B.d_neuron;
}

neuron_solve_t *solve_initialize(int type, neuron_solve_t *ps, const char *solver, neuron_t *p) {
  Block &B = g_block[type];
  if (strncmp(solver, "RKC", 3) != 0) {
    printf("%s: solver %s is not provided (only RKC)\n", TYPE_NAME[type], solver);
    exit(1);
  }
  memset(ps, 0, sizeof *ps);
  strncpy(ps->type, solver, GBRKC_MAX_BUF - 1);
  B.h_vec = (double **)calloc(n_vec_RKC, sizeof(double *));
  ps->vec = B.h_vec;
  if (p->n > 0) check(gbrkc_field_device_ptr(B.eng, B.sid, GBRKC_F_VNEW, &B.h_vec[v_new]), "vec[v_new]");
  cuda_check(cudaMalloc(&B.d_solve, sizeof(neuron_solve_t)), "device solver mirror");
  cuda_check(cudaMemcpy(B.d_solve, ps, sizeof *ps, cudaMemcpyHostToDevice), "device solver mirror");
  return B.d_solve;
}

void update_v(int type) {
  Block &B = g_block[type];
  if (B.n == 0) return;
  // the caller's stimulus kernel ran on the default stream
  cuda_check(cudaStreamSynchronize(0), "stimulus");
  const int rc = gbrkc_advance(B.eng, B.t, 1);
  if (rc != 0) {
    printf("%s: %s\n", TYPE_NAME[type], gbrkc_last_error());
    exit(1);
  }
  B.t += H_MAX;
}

// stimulus protocols of the reference's *_set_current kernels
struct Protocol {
  double t0, t1, amp;
};
__device__ __forceinline__ void set_current(neuron_t *d, int type, double t, Protocol pr) {
  const int id = threadIdx.x + blockIdx.x * blockDim.x;
  if (id < d->n) {
    const int ncomp = d->nc / d->n;
    double *iv = &d->elem[i_ext][d_stim_comp[type] + id * ncomp];
    *iv = 0.0;
    if (pr.t0 <= t && t < pr.t1) *iv = pr.amp;
  }
}

constexpr Protocol PR_GR{50.0, 100.0, 0.01e-3}, PR_GO{800.0, 1100.0, 0.2e-3}, PR_PKJ{550.0, 1300.0, 0.1e-3},
    PR_IO{800.0, 820.0, 5.5};

void output(int type, neuron_t *p, double *vh, double *rprev, double t, FILE *fv, FILE *fr) {
  const Block &B = g_block[type];
  const int nc = B.ncomp;
  fprintf(fv, "%lf,", t);
  for (int j = 0; j < p->n; j++) {
    if (type == GBRKC_IO) {
      for (int k = 0; k < 3; k++) fprintf(fv, "%lf,", vh[k + j * nc]);
    } else {
      fprintf(fv, "%lf,", vh[soma_comp(type, nc) + j * nc]);
    }
  }
  fprintf(fv, "\n");
  const double th = raster_threshold(type);
  const int rc = raster_comp(type, nc);
  for (int j = 0; j < p->n; j++) {
    const double x = vh[rc + j * nc];
    if (x > th && rprev[j] <= th) fprintf(fr, "%lf,%d\n", t, j);
    rprev[j] = x;
  }
}

void finalize(int type, neuron_t *p, FILE *fv, FILE *fr) {
  Block &B = g_block[type];
  if (B.eng) gbrkc_engine_destroy(B.eng);
  if (B.d_neuron) cudaFree(B.d_neuron);
  if (B.d_elem) cudaFree(B.d_elem);
  free(B.h_elem);
  if (p) free(p);
  if (fv) fclose(fv);
  if (fr) fclose(fr);
  B.eng = nullptr;
  B.d_neuron = nullptr;
  B.d_elem = nullptr;
  B.h_elem = nullptr;
}

void solve_finalize(int type, neuron_solve_t *ps) {
  Block &B = g_block[type];
  if (B.d_solve) cudaFree(B.d_solve);
  free(B.h_vec);
  if (ps) free(ps);
  B.d_solve = nullptr;
  B.h_vec = nullptr;
}

void launch_stim(int type, neuron_t *d, double t);

}  // namespace

struct _gap_t {
  int nx, ny;
};

extern "C" {

// exported (nvcc gives kernel stubs hidden visibility by default): a caller
// launches these with <<<>>> from its own translation unit, as main.cu does
#define GBRKC_EXPORT __attribute__((visibility("default")))
GBRKC_EXPORT __global__ void gr_set_current(neuron_t *d_gr, const double t) { set_current(d_gr, GBRKC_GR, t, PR_GR); }
GBRKC_EXPORT __global__ void go_set_current(neuron_t *d_go, const double t) { set_current(d_go, GBRKC_GO, t, PR_GO); }
GBRKC_EXPORT __global__ void pkj_set_current(neuron_t *d_pkj, const double t) {
  set_current(d_pkj, GBRKC_PKJ, t, PR_PKJ);
}
GBRKC_EXPORT __global__ void io_set_current(neuron_t *d_io, const double t) { set_current(d_io, GBRKC_IO, t, PR_IO); }

neuron_t *gr_initialize(const int nx, const int ny, const char *type, neuron_t *p) {
  return initialize(GBRKC_GR, nx, ny, type, p);
}
neuron_t *go_initialize(const int nx, const int ny, const char *type, neuron_t *p) {
  return initialize(GBRKC_GO, nx, ny, type, p);
}
neuron_t *pkj_initialize(const int nx, const int ny, const char *type, neuron_t *p) {
  return initialize(GBRKC_PKJ, nx, ny, type, p);
}
neuron_t *io_initialize(const int nx, const int ny, const char *type, neuron_t *p) {
  return initialize(GBRKC_IO, nx, ny, type, p);
}

neuron_solve_t *gr_solve_initialize(neuron_solve_t *ps, const char *type, neuron_t *p, neuron_t *) {
  return solve_initialize(GBRKC_GR, ps, type, p);
}
neuron_solve_t *go_solve_initialize(neuron_solve_t *ps, const char *type, neuron_t *p, neuron_t *) {
  return solve_initialize(GBRKC_GO, ps, type, p);
}
neuron_solve_t *pkj_solve_initialize(neuron_solve_t *ps, const char *type, neuron_t *p, neuron_t *) {
  return solve_initialize(GBRKC_PKJ, ps, type, p);
}
neuron_solve_t *io_solve_initialize(neuron_solve_t *ps, const char *type, neuron_t *p, neuron_t *) {
  return solve_initialize(GBRKC_IO, ps, type, p);
}

void gr_solve_update_v(neuron_t *, neuron_solve_t *, neuron_t *, neuron_solve_t *, synapse_t *mfgr, synapse_t *gogr) {
  if (mfgr || gogr) die("gr: network mode is not provided");
  update_v(GBRKC_GR);
}
void go_solve_update_v(neuron_t *, neuron_solve_t *, neuron_t *, neuron_solve_t *, synapse_t *grgo) {
  if (grgo) die("go: network mode is not provided");
  update_v(GBRKC_GO);
}
void pkj_solve_update_v(neuron_t *, neuron_solve_t *, neuron_t *, neuron_solve_t *, synapse_t *grpkj,
                        synapse_t *mlipkj) {
  if (grpkj || mlipkj) die("pkj: network mode is not provided");
  update_v(GBRKC_PKJ);
}
void io_solve_update_v(neuron_t *, neuron_solve_t *, neuron_t *, neuron_solve_t *, gap_t *) { update_v(GBRKC_IO); }

void gr_set_current_launch(neuron_t *d, const double t) { launch_stim(GBRKC_GR, d, t); }
void go_set_current_launch(neuron_t *d, const double t) { launch_stim(GBRKC_GO, d, t); }
void pkj_set_current_launch(neuron_t *d, const double t) { launch_stim(GBRKC_PKJ, d, t); }
void io_set_current_launch(neuron_t *d, const double t) { launch_stim(GBRKC_IO, d, t); }

void gr_output_file(neuron_t *p, double *vh, double *rp, const double t, FILE *fv, FILE *fr) {
  output(GBRKC_GR, p, vh, rp, t, fv, fr);
}
void go_output_file(neuron_t *p, double *vh, double *rp, const double t, FILE *fv, FILE *fr) {
  output(GBRKC_GO, p, vh, rp, t, fv, fr);
}
void pkj_output_file(neuron_t *p, double *vh, double *rp, const double t, FILE *fv, FILE *fr) {
  output(GBRKC_PKJ, p, vh, rp, t, fv, fr);
}
void io_output_file(neuron_t *p, double *vh, double *rp, const double t, FILE *fv, FILE *fr) {
  output(GBRKC_IO, p, vh, rp, t, fv, fr);
}

void gr_finalize(neuron_t *p, neuron_t *, FILE *fv, FILE *fr) { finalize(GBRKC_GR, p, fv, fr); }
void go_finalize(neuron_t *p, neuron_t *, FILE *fv, FILE *fr) { finalize(GBRKC_GO, p, fv, fr); }
void pkj_finalize(neuron_t *p, neuron_t *, FILE *fv, FILE *fr) { finalize(GBRKC_PKJ, p, fv, fr); }
void io_finalize(neuron_t *p, neuron_t *, FILE *fv, FILE *fr) { finalize(GBRKC_IO, p, fv, fr); }
void gr_solve_finalize(const int, neuron_solve_t *, neuron_solve_t *ps) { solve_finalize(GBRKC_GR, ps); }
void go_solve_finalize(const int, neuron_solve_t *, neuron_solve_t *ps) { solve_finalize(GBRKC_GO, ps); }
void pkj_solve_finalize(const int, neuron_solve_t *, neuron_solve_t *ps) { solve_finalize(GBRKC_PKJ, ps); }
void io_solve_finalize(const int, neuron_solve_t *, neuron_solve_t *ps) { solve_finalize(GBRKC_IO, ps); }

synapse_t *mfgr_create(const int) { return nullptr; }
synapse_t *gogr_create(const int, const int, const int, const int) { return nullptr; }
synapse_t *grgo_create(const int, const int, const int, const int) { return nullptr; }
synapse_t *grpkj_create(const int, const int, const int, const int) { return nullptr; }
synapse_t *mlipkj_create(const int, const int) { return nullptr; }
void mfgr_finalize(synapse_t *, const int) {}
void gogr_finalize(synapse_t *, const int) {}
void grgo_finalize(synapse_t *, const int) {}
void grpkj_finalize(synapse_t *, const int) {}
void mlipkj_finalize(synapse_t *, const int) {}
void gr_synapse_update(const double, const double, synapse_t *, synapse_t *, neuron_t *, neuron_solve_t *) {
  die("gr_synapse_update: network mode is not provided");
}
void go_synapse_update(const double, const double, synapse_t *, neuron_t *, neuron_solve_t *) {
  die("go_synapse_update: network mode is not provided");
}
void pkj_synapse_update(const double, const double, synapse_t *, synapse_t *, neuron_t *, neuron_solve_t *) {
  die("pkj_synapse_update: network mode is not provided");
}

gap_t *io_gap_create(const int nx, const int ny) {
  gap_t *g = (gap_t *)malloc(sizeof(gap_t));
  g->nx = nx;
  g->ny = ny;
  return g;
}
void io_gap_finalize(gap_t *g) { free(g); }

void output_time(const int n_gr, const char *type1, const int n_go, const char *type2, const int n_pkj,
                 const char *type3, const int n_io, const char *type4, const double comp_time, const int sim_time) {
  FILE *f = fopen("comptime.csv", "a");
  if (!f) {
    printf("go_time_file_open_error \n");
    return;
  }
  fprintf(f, "Gr,%d,%s,Go,%d,%s,Pkj,%d,%s,Io,%d,%s,CompTime,%lf,SimTime,%d\n", n_gr, type1, n_go, type2, n_pkj,
          type3, n_io, type4, comp_time, sim_time);
  fclose(f);
}

void output_time2(const int n_gr, const char *type1, const int n_go, const char *type2, const int n_pkj,
                  const char *type3, const int n_io, const char *type4, const double comp_time,
                  const double comp_time_half, const int sim_time) {
  FILE *f = fopen("comptime.csv", "a");
  if (!f) {
    printf("go_time_file_open_error \n");
    return;
  }
  fprintf(f, "Gr,%d,%s,Go,%d,%s,Pkj,%d,%s,Io,%d,%s,AllCompTime,%lf,0.5s-endCompTime,%lf,SimTime,%d\n", n_gr, type1,
          n_go, type2, n_pkj, type3, n_io, type4, comp_time, comp_time_half, sim_time);
  fclose(f);
}

}  // extern "C"

namespace {
void launch_stim(int type, neuron_t *d, double t) {
  const int n = g_block[type].n;
  if (n <= 0) return;
  const dim3 grid(n / 128 + 1), block(128);
  switch (type) {
    case GBRKC_GR: gr_set_current<<<grid, block>>>(d, t); break;
    case GBRKC_GO: go_set_current<<<grid, block>>>(d, t); break;
    case GBRKC_PKJ: pkj_set_current<<<grid, block>>>(d, t); break;
    default: io_set_current<<<grid, block>>>(d, t); break;
  }
  cuda_check(cudaGetLastError(), "stimulus launch");
}

constexpr Protocol protocol(int type) {
  return type == GBRKC_GR ? PR_GR : type == GBRKC_GO ? PR_GO : type == GBRKC_PKJ ? PR_PKJ : PR_IO;
}
}  // namespace

extern "C" long gbrkc_compat_advance_batch(int type, int n, double *rows, long row_cap, double *spk_t, int *spk_cell,
                                           long spk_cap) {
  if (type < 0 || type >= NTYPES || n <= 0 || !rows || spk_cap < 0) return GBRKC_EINVAL;
  Block &B = g_block[type];
  if (B.n == 0) return 0;
  const int cols = (type == GBRKC_IO) ? 3 : 1;
  if (row_cap < (long)n * B.n * cols) return GBRKC_EINVAL;
  if (n > B.batch_cap) {
    // the protocol as the engine's stimulus table, evaluated at every interval
    // start on the device exactly as X_set_current does before each advance
    const Protocol pr = protocol(type);
    std::vector<int> comp(B.n, B.stim_comp);
    std::vector<double> amp(B.n, pr.amp), t0(B.n, pr.t0), t1(B.n, pr.t1);
    check(gbrkc_set_stim(B.eng, B.sid, comp.data(), amp.data(), t0.data(), t1.data()), "stimulus table");
    if (cols > 1 && B.batch_cap == 0) check(gbrkc_record_width(B.eng, type, cols), "recorder");
    check(gbrkc_record_soma(B.eng, n), "recorder");
    check(gbrkc_record_spikes(B.eng, (long)B.n * (n / 2 + 1)), "raster");
    B.batch_cap = n;
  }
  check(gbrkc_rewind_soma(B.eng), "recorder");
  const int rc = gbrkc_advance(B.eng, B.t, n);
  if (rc == GBRKC_ESOLVER) return rc;
  check(rc, TYPE_NAME[type]);
  B.t += n * H_MAX;
  check(gbrkc_read_soma(B.eng, B.sid, n, rows), "recorder");
  std::vector<int> sys(spk_cap > 0 ? spk_cap : 1);
  long m = 0;
  const int src = gbrkc_read_spikes(B.eng, type, spk_cap, spk_t, sys.data(), spk_cell, &m);
  if (src == GBRKC_EOVERFLOW) return src;
  check(src, "raster");
  return m;
}

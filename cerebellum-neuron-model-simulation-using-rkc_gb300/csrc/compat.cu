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
#include "splitmix.h"

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
  int n = 0, ncomp = 0, nx = 0, ny = 0;
  int stim_comp = 0;              // compartment of every cell the protocol drives
  int batch_cap = 0;              // batched output: intervals the recorder holds
  std::vector<double> rows, jitter;  // the block's description, kept for network mode
  std::vector<int> pairs;
  bool shared = false;            // network mode: the block lives in the shared engine
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

// kBE, kCN or kRKC from a solver name, matched on its first letters as
// main.cu:60-102 does; -1 for anything else
int solver_kind(const char *solver) {
  if (!strncmp(solver, "BE", 2)) return kBE;
  if (!strncmp(solver, "CN", 2)) return kCN;
  if (!strncmp(solver, "RKC", 3)) return kRKC;
  return -1;
}

// Only RKC is provided.  A block without cells runs no solver, so BE and CN
// are accepted there (the reference's run scripts name them for the types
// they leave empty).
void check_solver(int type, const char *solver, int n) {
  const int kind = solver_kind(solver);
  if (kind == kRKC || (kind >= 0 && n <= 0)) return;
  printf("%s: solver %s is not provided (only RKC)\n", TYPE_NAME[type], solver);
  exit(1);
}

neuron_t *initialize(int type, int nx, int ny, const char *solver, neuron_t *p) {
  const int n = nx * ny;
  check_solver(type, solver, n);
  Block &B = g_block[type];
  if (B.eng) die("block initialised twice");
  memset(p, 0, sizeof *p);
  p->n_solver = solver_kind(solver);
  p->neuron_type = type;
  p->n = n;
  p->nx = nx;
  p->ny = ny;
  p->DT = RKC_DT;
  B.n = n;
  B.nx = nx;
  B.ny = ny;
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
    B.rows = rows;
    B.jitter = jitter;
    B.pairs = pairs;
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
    // the compartment the X_set_current kernels drive
    B.stim_comp = (type == GBRKC_IO) ? 0 : (type == GBRKC_GO) ? 30 : soma_comp(type, B.ncomp);
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
  check_solver(type, solver, p->n);
  memset(ps, 0, sizeof *ps);
  strncpy(ps->type, solver, GBRKC_MAX_BUF - 1);
  B.h_vec = (double **)calloc(n_vec_RKC, sizeof(double *));
  ps->vec = B.h_vec;
  if (p->n > 0) check(gbrkc_field_device_ptr(B.eng, B.sid, GBRKC_F_VNEW, &B.h_vec[v_new]), "vec[v_new]");
  cuda_check(cudaMalloc(&B.d_solve, sizeof(neuron_solve_t)), "device solver mirror");
  cuda_check(cudaMemcpy(B.d_solve, ps, sizeof *ps, cudaMemcpyHostToDevice), "device solver mirror");
  return B.d_solve;
}

void network_advance(Block &B);

void update_v(int type) {
  Block &B = g_block[type];
  if (B.n == 0) return;
  // the caller's stimulus kernel ran on the default stream
  cuda_check(cudaStreamSynchronize(0), "stimulus");
  if (B.shared) {
    network_advance(B);
    return;
  }
  const int rc = gbrkc_advance(B.eng, B.t, 1);
  if (rc != 0) {
    printf("%s: %s\n", TYPE_NAME[type], gbrkc_last_error());
    exit(1);
  }
  B.t += H_MAX;
}

// stimulus protocols of the reference's *_set_current kernels (the
// kernels themselves are defined in gbrkc_compat.h)
struct Protocol {
  double t0, t1, amp;
};
constexpr Protocol PR_GR{GBRKC_STIM_GR}, PR_GO{GBRKC_STIM_GO}, PR_PKJ{GBRKC_STIM_PKJ}, PR_IO{GBRKC_STIM_IO};

// pkj.cu:346-354: every Purkinje soma (the last compartment) gets 0.1 nA
// times the filtered Poisson train
__global__ void set_current_poisson(neuron_t *d_pkj, const double val_current) {
  const int id = threadIdx.x + blockIdx.x * blockDim.x;
  if (id < d_pkj->n) {
    const int ncomp = d_pkj->nc / d_pkj->n;
    d_pkj->elem[i_ext][ncomp - 1 + id * ncomp] = 0.1e-3 * val_current;
  }
}

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

void network_release();

void finalize(int type, neuron_t *p, FILE *fv, FILE *fr) {
  Block &B = g_block[type];
  if (B.eng) gbrkc_engine_destroy(B.eng);
  if (B.shared) network_release();
  B.shared = false;
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

struct _synapse_t {
  int kind;
  int n;        // synapses of the family where the constructor knows them (mfgr, mlipkj), else its pair count
  FILE *f_out;  // MF_RASTER.csv / MLI_RASTER.csv (syn.cu:76, 726), or NULL
};

namespace {

// ------------------------------------------------------------ network mode
// The reference's network path (main.cu with network_sim true): every
// interval each type advances, then gr/go/pkj_synapse_update refresh the
// synapses from the new voltages.  The blocks then have to share one engine
// (synapses join systems of different types), which the per-type
// initialisation could not know: on the first X_synapse_update the blocks
// move into one engine wired by the reference's rules (syn.cu's *_create),
// which replays the interval already run -- bit for bit the same, as every
// synaptic value is still 0 in it -- and from then on the first
// X_solve_update_v of an interval advances every block and the synapses
// together; the other calls of that interval have nothing left to do.
enum { SYN_K_MFGR = 0, SYN_K_GRGO = 1, SYN_K_GOGR = 2, SYN_K_GRPKJ = 3, SYN_K_MLIPKJ = 4 };

struct Net {
  bool on = false;
  bool made[5] = {};
  unsigned long long seed_mf = 0, seed_pk = 0;
  gbrkc_engine *eng = nullptr;
  int sid[NTYPES] = {-1, -1, -1, -1};
  double t = 0.0;  // start of the shared engine's next interval
  int refs = 0;
  // mossy-fibre states as of the last synapse update before the current
  // interval, for mf_output_file (the engine's own states are one update
  // ahead once the interval has run); kept while MF_RASTER.csv is open
  int mf_watch = 0;  // synapses of the open MF_RASTER.csv
  std::vector<double> mf_ampa, mf_nmda;
} g_net;

synapse_t *net_create(int kind, int n, const char *raster) {
  g_net.made[kind] = true;
  _synapse_t *s = new _synapse_t{kind, n, nullptr};
  if (n > 0 && raster) {
    s->f_out = fopen(raster, "w");
    if (!s->f_out) die("cannot open a synapse raster file");
    if (kind == SYN_K_MFGR) g_net.mf_watch = n;
  }
  // a non-empty random family seeds its cuRAND states with rand() here
  // (syn.cu:82, 623, 755)
  if (n > 0 && (kind == SYN_K_MFGR || kind == SYN_K_GRPKJ || kind == SYN_K_MLIPKJ)) {
    const unsigned long long r = (unsigned long long)rand();
    if (kind == SYN_K_MFGR) g_net.seed_mf = r;
    if (kind == SYN_K_GRPKJ) g_net.seed_pk = r;
  }
  return s;
}

void syn_free(synapse_t *s) {
  if (!s) return;
  if (s->f_out) fclose(s->f_out);
  if (s->kind == SYN_K_MFGR && s->f_out) g_net.mf_watch = 0;
  delete s;
}

// the mossy-fibre synapses are the shared engine's first (network_on adds
// them first): copy their states before the next update
void snapshot_mf() {
  const int n = g_net.mf_watch;
  if (n <= 0 || !g_net.made[SYN_K_MFGR] || g_block[GBRKC_GR].n * 4 != n) return;
  g_net.mf_ampa.resize(n);
  g_net.mf_nmda.resize(n);
  check(gbrkc_read_synapses(g_net.eng, GBRKC_SYNF_S0, g_net.mf_ampa.data(), n), "mossy-fibre states");
  check(gbrkc_read_synapses(g_net.eng, GBRKC_SYNF_S1, g_net.mf_nmda.data(), n), "mossy-fibre states");
}

// the reference's wiring (syn.cu:146-262, 295-410, 455-619) on the blocks'
// grids: granule cell i at 16 (i mod nx, i div nx) um, Golgi and Purkinje
// cells at 32 (i mod nx, i div nx) + 8 um
struct Wire {
  std::vector<int> pre_cell, pre_comp, post_cell, post_comp;
  std::vector<double> w;
};

void wire_grgo(int gx, int gy, int ox, int oy, Wire &W) {
  const int n_gr = gx * gy, n_go = ox * oy;
  std::vector<int> cnt(n_go, 0);
  for (int a = 0; a < n_gr; a++)
    for (int b = 0; b < n_go; b++) {
      const double xg = (a % gx) * 16.0, yg = (a / gx) * 16.0, xo = (b % ox) * 32.0 + 8.0, yo = (b / ox) * 32.0 + 8.0;
      if (fabs(xo - xg) < 16.0 && fabs(yo - yg) < 220.0) {
        const float diff = (float)(8.0 + (b / ox) * 32.0 - (a / gx) * 16.0);
        W.pre_cell.push_back(a);
        W.pre_comp.push_back(250 + 77 - (int)(diff / 10.0));
        W.post_cell.push_back(b);
        W.post_comp.push_back(0);
        cnt[b]++;
      }
    }
  for (int b : W.post_cell) W.w.push_back(64.0 / 4.0 / (cnt[b] * 1.0 / 4.0));  // W_GRGO / (n / 4)
}

void wire_gogr(int ox, int oy, int gx, int gy, Wire &W) {
  const int n_gr = gx * gy, n_go = ox * oy;
  std::vector<int> cnt(n_gr, 0);
  for (int b = 0; b < n_go; b++)
    for (int a = 0; a < n_gr; a++) {
      const double xg = (a % gx) * 16.0, yg = (a / gx) * 16.0, xo = (b % ox) * 32.0 + 8.0, yo = (b / ox) * 32.0 + 8.0;
      if (fabs(xo - xg) < 32.0 && fabs(yo - yg) < 32.0) {
        W.pre_cell.push_back(b);
        W.pre_comp.push_back(30);  // GO_COMP_DEND * 3
        W.post_cell.push_back(a);
        W.post_comp.push_back(16);
        cnt[a]++;
      }
    }
  for (int a : W.post_cell) W.w.push_back(160000.0 * 4.0 / (cnt[a] * 4.0));  // W_GOGR / (4 n)
}

void wire_grpkj(int gx, int gy, int px, int py, const std::vector<double> &x, unsigned long long seed, Wire &W) {
  const int n_gr = gx * gy, n_pkj = px * py;
  std::vector<std::pair<int, int>> pairs;
  std::vector<int> cnt(n_pkj, 0);
  for (int a = 0; a < n_gr; a++)
    for (int b = 0; b < n_pkj; b++) {
      const double xg = (a % gx) * 16.0, yg = (a / gx) * 16.0, xp = (b % px) * 32.0 + 8.0, yp = (b / px) * 32.0 + 8.0;
      if (fabs(xp - xg) < 120.0 && fabs(yp - yg) < 220.0) {
        pairs.push_back({a, b});
        cnt[b]++;
      }
    }
  long long k = 0;
  for (const auto &pr : pairs) {
    const int a = pr.first, b = pr.second;
    const double dx = (a % gx) * 16.0 - (8.0 + (b % px) * 32.0);
    const double dy = (a / gx) * 16.0 - (8.0 + (b / px) * 32.0);
    const int ax = 250 + 77 + (int)(dy / 10.0);
    int best = -1;
    double min_x = 1000000.0;
    for (int i = 0; i < 25; i++, k++) {  // N_Syn_Per_GRPKJ, the running minimum kept (syn.cu:489-499)
      const double f = gbrkc::splitmix_uniform(seed, k, 0) - 0.5;
      for (size_t c = 0; c < x.size(); c++) {
        const double d = fabs(x[c] - dx + 10.0 * f);
        if (d < min_x) {
          min_x = d;
          best = (int)c;
        }
      }
      W.pre_cell.push_back(a);
      W.pre_comp.push_back(ax);
      W.post_cell.push_back(b);
      W.post_comp.push_back(best);
      W.w.push_back(1000000.0 * 0.3 / (512.0 * cnt[b] * 1.0 * 1 / 10.0));  // W_GRPKJ / (512 n / 10)
    }
  }
}

void add_wire(gbrkc_engine *E, int kind, int pre_type, int post_type, const Wire &W, unsigned long long seed) {
  if (W.post_cell.empty()) return;
  const Block &Pre = g_block[pre_type < 0 ? GBRKC_GR : pre_type], &Post = g_block[post_type];
  const size_t n = W.post_cell.size();
  std::vector<int> ps(n), pc(n), qs(n, g_net.sid[post_type]), qc(n);
  for (size_t i = 0; i < n; i++) {
    qc[i] = W.post_cell[i] * Post.ncomp + W.post_comp[i];
    if (pre_type >= 0) {
      ps[i] = g_net.sid[pre_type];
      pc[i] = W.pre_cell[i] * Pre.ncomp + W.pre_comp[i];
    }
  }
  gbrkc_synapse_desc d;
  memset(&d, 0, sizeof d);
  d.kind = kind;
  d.n = (int)n;
  d.pre_system = pre_type >= 0 ? ps.data() : nullptr;
  d.pre_comp = pre_type >= 0 ? pc.data() : nullptr;
  d.post_system = qs.data();
  d.post_comp = qc.data();
  d.weight = W.w.data();
  d.seed = seed;
  check(gbrkc_add_synapses(E, &d, nullptr), "synapses");
}

void network_on() {
  if (g_net.on) return;
  // the blocks have run 0 or 1 intervals, all the same
  double t_done = -1.0;
  for (int k = 0; k < NTYPES; k++) {
    const Block &B = g_block[k];
    if (B.n == 0) continue;
    if (t_done < 0.0) t_done = B.t;
    if (B.t != t_done) die("network mode: the blocks have advanced unequally");
  }
  if (t_done < 0.0) return;
  if (t_done > H_MAX) die("network mode: synapse updates must start after the first interval");
  gbrkc_engine *E = nullptr;
  check(gbrkc_engine_create(GBRKC_FP64, &E), "engine");
  for (int k = 0; k < NTYPES; k++) {
    Block &B = g_block[k];
    if (B.n == 0) continue;
    gbrkc_system_desc d;
    memset(&d, 0, sizeof d);
    d.cell_type = k;
    d.nx = B.nx;
    d.ny = B.ny;
    d.ncomp = B.ncomp;
    d.rows = B.rows.data();
    d.gj_pairs = B.pairs.empty() ? nullptr : B.pairs.data();
    d.n_gj_pairs = (int)B.pairs.size() / 2;
    d.gap_junctions = 1;
    d.jitter = B.jitter.data();
    check(gbrkc_add_system(E, &d, &g_net.sid[k]), "add system");
  }
  const Block &GR = g_block[GBRKC_GR], &GO = g_block[GBRKC_GO], &PK = g_block[GBRKC_PKJ];
  const bool full_gr = GR.n == 0 || GR.ncomp >= 578;
  if (GR.n > 0 && g_net.made[SYN_K_MFGR]) {
    Wire W;
    for (int a = 0; a < GR.n; a++)
      for (int j = 0; j < 4; j++) {  // four fibres onto compartments 0-3, W_MFGR / 4 (syn.cu:43-62)
        W.post_cell.push_back(a);
        W.post_comp.push_back(j);
        W.w.push_back(40000.0 / 4.0);
      }
    add_wire(E, GBRKC_SYN_MFGR, -1, GBRKC_GR, W, g_net.seed_mf);
  }
  if (GR.n > 0 && GO.n > 0 && (g_net.made[SYN_K_GRGO] || g_net.made[SYN_K_GOGR])) {
    if (!full_gr) die("network mode: the granule -> Golgi wiring needs the 578-compartment granule cell");
    Wire A, B;
    if (g_net.made[SYN_K_GRGO]) wire_grgo(GR.nx, GR.ny, GO.nx, GO.ny, A);
    if (g_net.made[SYN_K_GOGR]) wire_gogr(GO.nx, GO.ny, GR.nx, GR.ny, B);
    add_wire(E, GBRKC_SYN_GRGO, GBRKC_GR, GBRKC_GO, A, 0);
    add_wire(E, GBRKC_SYN_GOGR, GBRKC_GO, GBRKC_GR, B, 0);
  }
  if (GR.n > 0 && PK.n > 0 && g_net.made[SYN_K_GRPKJ]) {
    if (!full_gr) die("network mode: the granule -> Purkinje wiring needs the 578-compartment granule cell");
    // Pkj_location_info.csv: index, x, y, z, type per Purkinje compartment (syn.cu:536-553)
    const std::vector<double> loc = read_numbers(model_path("Pkj_location_info.csv"), ',');
    if (loc.size() < (size_t)PK.ncomp * 5) die("Pkj_location_info.csv holds fewer rows than Pkj.txt");
    std::vector<double> x(PK.ncomp);
    for (int c = 0; c < PK.ncomp; c++) x[c] = loc[(size_t)c * 5 + 1];
    Wire W;
    wire_grpkj(GR.nx, GR.ny, PK.nx, PK.ny, x, g_net.seed_pk, W);
    add_wire(E, GBRKC_SYN_GRPKJ, GBRKC_GR, GBRKC_PKJ, W, 0);
  }
  check(gbrkc_build(E), "build");
  // replay the interval the blocks ran alone (no synaptic input yet), with
  // the synapse update that ends it
  if (t_done > 0.0) check(gbrkc_advance(E, 0.0, 1), "network advance");
  for (int k = 0; k < NTYPES; k++) {
    Block &B = g_block[k];
    if (B.n == 0) continue;
    check(gbrkc_field_device_ptr(E, g_net.sid[k], GBRKC_F_V, &B.h_elem[v]), "elem[v]");
    check(gbrkc_field_device_ptr(E, g_net.sid[k], GBRKC_F_CA, &B.h_elem[Ca]), "elem[Ca]");
    check(gbrkc_field_device_ptr(E, g_net.sid[k], GBRKC_F_IEXT, &B.h_elem[i_ext]), "elem[i_ext]");
    cuda_check(cudaMemcpy(B.d_elem, B.h_elem, n_elem * sizeof(double *), cudaMemcpyHostToDevice), "device table");
    if (B.h_vec) check(gbrkc_field_device_ptr(E, g_net.sid[k], GBRKC_F_VNEW, &B.h_vec[v_new]), "vec[v_new]");
    gbrkc_engine_destroy(B.eng);
    B.eng = nullptr;
    B.shared = true;
    g_net.refs++;
  }
  g_net.eng = E;
  g_net.t = t_done;
  g_net.on = true;
}

void network_advance(Block &B) {
  if (B.t >= g_net.t) {
    snapshot_mf();
    const int rc = gbrkc_advance(g_net.eng, g_net.t, 1);
    if (rc != 0) {
      printf("network: %s\n", gbrkc_last_error());
      exit(1);
    }
    g_net.t += H_MAX;
  }
  B.t += H_MAX;
}

void network_release() {
  if (--g_net.refs > 0) return;
  if (g_net.eng) gbrkc_engine_destroy(g_net.eng);
  g_net = Net();
}

}  // namespace

extern "C" {


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

// main.cu passes its coupling objects on every call, network_sim or not
// (main.cu:201, 227, 259, 285).  Their synaptic values stay 0 -- and the
// blocks independent -- until the first X_synapse_update starts network mode.
void gr_solve_update_v(neuron_t *, neuron_solve_t *, neuron_t *, neuron_solve_t *, synapse_t *, synapse_t *) {
  update_v(GBRKC_GR);
}
void go_solve_update_v(neuron_t *, neuron_solve_t *, neuron_t *, neuron_solve_t *, synapse_t *) { update_v(GBRKC_GO); }
void pkj_solve_update_v(neuron_t *, neuron_solve_t *, neuron_t *, neuron_solve_t *, synapse_t *, synapse_t *) {
  update_v(GBRKC_PKJ);
}
void io_solve_update_v(neuron_t *, neuron_solve_t *, neuron_t *, neuron_solve_t *, gap_t *) { update_v(GBRKC_IO); }
void gr_solve_by_rkc(neuron_t *, neuron_solve_t *, neuron_t *, neuron_solve_t *, synapse_t *, synapse_t *) {
  update_v(GBRKC_GR);
}
void go_solve_by_rkc(neuron_t *, neuron_solve_t *, neuron_t *, neuron_solve_t *, synapse_t *) { update_v(GBRKC_GO); }
void pkj_solve_by_rkc(neuron_t *, neuron_solve_t *, neuron_t *, neuron_solve_t *, synapse_t *, synapse_t *) {
  update_v(GBRKC_PKJ);
}
void io_solve_by_rkc(neuron_t *, neuron_solve_t *, neuron_t *, neuron_solve_t *, gap_t *) { update_v(GBRKC_IO); }

void gr_set_current_launch(neuron_t *d, const double t) { launch_stim(GBRKC_GR, d, t); }
void go_set_current_launch(neuron_t *d, const double t) { launch_stim(GBRKC_GO, d, t); }
void pkj_set_current_launch(neuron_t *d, const double t) { launch_stim(GBRKC_PKJ, d, t); }
void io_set_current_launch(neuron_t *d, const double t) { launch_stim(GBRKC_IO, d, t); }
void pkj_set_current_Poisson(const int num, neuron_t *d_pkj, const double t) {
  static double val_current = 0.0;
  const double fr = (350 <= t && t < 1000) ? 25.0 : 0.0;
  const double f = ((double)rand() + 1.0) / ((double)RAND_MAX + 2.0);
  const int firing_flag = (fr * 0.125 * 0.001 > f) ? 1 : 0;
  val_current = val_current * 0.81193634615 + firing_flag;  // exp(-0.125 / 0.6)
  if (num <= 0) return;
  set_current_poisson<<<(num + 127) / 128, 128>>>(d_pkj, val_current);
  cuda_check(cudaGetLastError(), "Poisson stimulus launch");
}

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

// The coupling objects only record which synapse families the caller asked
// for (and, like the reference, take a rand() seed for the random ones); the
// network is wired and built on the first X_synapse_update call.
// Four mossy fibres per granule cell and N_Syn_Per_MLIPKJ = 1 MLI synapse
// per Purkinje cell (syn.cu:66, 709; syn.cuh:52); those two families open
// their raster files when they have synapses (syn.cu:76, 726).
synapse_t *mfgr_create(const int n) { return net_create(SYN_K_MFGR, 4 * n, "MF_RASTER.csv"); }
synapse_t *gogr_create(const int go_x, const int go_y, const int gr_x, const int gr_y) {
  return net_create(SYN_K_GOGR, go_x * go_y * gr_x * gr_y, nullptr);
}
synapse_t *grgo_create(const int gr_x, const int gr_y, const int go_x, const int go_y) {
  return net_create(SYN_K_GRGO, go_x * go_y * gr_x * gr_y, nullptr);
}
synapse_t *grpkj_create(const int gr_x, const int gr_y, const int pkj_x, const int pkj_y) {
  return net_create(SYN_K_GRPKJ, gr_x * gr_y * pkj_x * pkj_y, nullptr);
}
synapse_t *mlipkj_create(const int n_pkj, const int n_gr) {
  return net_create(SYN_K_MLIPKJ, (n_pkj == 0 || n_gr == 0) ? 0 : n_pkj, "MLI_RASTER.csv");
}
void mfgr_finalize(synapse_t *s, const int) { syn_free(s); }
void gogr_finalize(synapse_t *s, const int) { syn_free(s); }
void grgo_finalize(synapse_t *s, const int) { syn_free(s); }
void grpkj_finalize(synapse_t *s, const int) { syn_free(s); }
void mlipkj_finalize(synapse_t *s, const int) { syn_free(s); }

// syn.cu:114-127: the time, then each mossy fibre's conductance
// (G_MFGR_AMPA 0.88 ampa + G_MFGR_NMDA 0.12 nmda) x weight x 1e6, in the
// reference's synapse order (granule cell i, fibre j at 4 i + j).  Before
// network mode the states are 0, as the reference's are without updates.
void mf_output_file(synapse_t *s, const double t, neuron_t *) {
  if (!s || !s->f_out) return;
  constexpr double G_MFGR_AMPA = 0.18e-9, G_MFGR_NMDA = 0.025e-9, W_MFGR = 40000.0;  // syn.cuh:13-14, 54
  const bool live = g_net.on && (int)g_net.mf_ampa.size() == s->n;
  fprintf(s->f_out, "%lf,", t);
  for (int j = 0; j < s->n; j++) {
    const double ampa = live ? g_net.mf_ampa[j] : 0.0, nmda = live ? g_net.mf_nmda[j] : 0.0;
    double val = G_MFGR_AMPA * 0.88 * ampa + G_MFGR_NMDA * 0.12 * nmda;
    val *= W_MFGR / 4.0 * 1000000;
    fprintf(s->f_out, "%lf,", val);
  }
  fprintf(s->f_out, "\n");
}

// syn.cu:804-817: the time, then each MLI synapse's G_MLIPKJ_GABA x gaba x
// weight x 1e6.  On the RKC path these synapses are never updated
// (syn.cu:912-916) and W_MLIPKJ is 0 (syn.cuh:59): every value is 0.
void mli_output_file(synapse_t *s, const double t, neuron_t *) {
  if (!s || !s->f_out) return;
  fprintf(s->f_out, "%lf,", t);
  for (int j = 0; j < s->n; j++) fprintf(s->f_out, "%lf,", 0.0);
  fprintf(s->f_out, "\n");
}
void gr_synapse_update(const double, const double, synapse_t *, synapse_t *, neuron_t *, neuron_solve_t *) {
  network_on();
}
void go_synapse_update(const double, const double, synapse_t *, neuron_t *, neuron_solve_t *) { network_on(); }
void pkj_synapse_update(const double, const double, synapse_t *, synapse_t *, neuron_t *, neuron_solve_t *) {
  network_on();
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

void raster_plot(const int n_go, const char *type) {
  if (n_go <= 0) return;
  // the reference's solver names and file names (output.cu:40-45)
  static const struct {
    const char *name;
    size_t len;
    const char *in, *out;
  } kFiles[] = {{"BACKWARD_EULER", 14, "go_v_by_BEm.csv", "go_raster_by_BEm.csv"},
                {"CRANK_NICOLSON", 14, "go_v_by_CNm.csv", "go_raster_by_CNm.csv"},
                {"FORWARD_EULER", 13, "go_v_by_FEm.csv", "go_raster_by_FEm.csv"},
                {"RUNGE_KUTTA_4", 13, "go_v_by_RK4m.csv", "go_raster_by_RK4.csv"},
                {"RKC", 3, "go_v_by_RKC.csv", "go_raster_by_RKC.csv"}};
  const char *in = nullptr, *out = nullptr;
  for (const auto &f : kFiles)
    if (!strncmp(type, f.name, f.len)) {
      in = f.in;
      out = f.out;
      break;
    }
  if (!in) {
    printf("go_initialization_error \n");
    exit(1);
  }
  FILE *fp = fopen(in, "r");
  FILE *fw = fopen(out, "w");
  if (!fp || !fw) die("raster_plot: cannot open the Golgi voltage or raster file");
  std::vector<double> v(n_go, -70.0), old_v(n_go, -70.0);
  printf("Debug for output \n");
  double t;
  while (fscanf(fp, "%lf,", &t) == 1) {
    fprintf(fw, "%lf,", t);
    for (int i = 0; i < n_go; i++) {
      if (fscanf(fp, "%lf,", &v[i]) != 1) {
        printf("raster_FILE_ERROR2\n");
        exit(1);
      }
      if (v[i] > 0.0 && old_v[i] < 0.0) {
        fprintf(fw, "%d,", i);
        printf("%d,", i);
      } else {
        fprintf(fw, ",");
      }
      old_v[i] = v[i];
    }
    fprintf(fw, "\n");
  }
  fclose(fp);
  fclose(fw);
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
  if (B.shared) return GBRKC_EINVAL;  // network mode advances all types together
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

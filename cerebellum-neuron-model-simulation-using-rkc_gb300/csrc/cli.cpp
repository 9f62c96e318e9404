// gbrkc_main: the reference's command line over gbrkc_compat.h.
//
//   gbrkc_main S_gr gx gy S_go ox oy S_pkj px py S_io ix iy [TS_ms [batch [network]]]
//
// S is the solver name per type, matched on its first letters as the
// reference does (main.cu:60-102); only RKC is provided, and BE or CN is
// accepted for a type with nx * ny == 0, which is skipped.  Each 0.125 ms interval: the type's stimulus
// protocol, one advance, the voltages copied back, one CSV row written; the
// files are the reference's: <type>_v_by_RKC.csv, <type>_raster_by_RKC.csv,
// comptime.csv (appended) and an empty debug_file.csv.  The jitter stream is
// seeded with srand(0) first, as main.cu:38 does.  TS_ms (default 1500, the
// reference's TS) is this tool's addition, and so is batch: with batch > 1
// each type advances `batch` intervals per device launch with its protocol,
// voltage record and raster evaluated on the device
// (gbrkc_compat_advance_batch), and a writer thread formats the same CSV
// rows from the recorded columns while the GPU runs the next batch.  The
// files are byte-identical to the per-interval path's.  network = 1 runs
// main.cu's network_sim branch: no stimulus kernels, and the synapse updates
// after every interval (batch must then be 1).  The coupling objects are
// created in either case, as main.cu:137-145 does.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/gbrkc_compat.h"

namespace {

struct TypeRun {
  const char *name;
  neuron_t *(*init)(int, int, const char *, neuron_t *);
  neuron_solve_t *(*solve_init)(neuron_solve_t *, const char *, neuron_t *, neuron_t *);
  void (*stim)(neuron_t *, double);
  void (*out)(neuron_t *, double *, double *, double, FILE *, FILE *);
  void (*fin)(neuron_t *, neuron_t *, FILE *, FILE *);
  void (*solve_fin)(int, neuron_solve_t *, neuron_solve_t *);
  char solver[GBRKC_MAX_BUF] = {};
  neuron_t *p = nullptr, *d = nullptr;
  neuron_solve_t *ps = nullptr, *ds = nullptr;
  FILE *fv = nullptr, *fr = nullptr;
  double *vh = nullptr, *raster = nullptr;
};

// the coupling objects, passed to every update call as main.cu:201-285 does
struct Coupling {
  synapse_t *mfgr = nullptr, *gogr = nullptr, *grgo = nullptr, *grpkj = nullptr, *mlipkj = nullptr;
  gap_t *io_gap = nullptr;
} g_cpl;

void gr_update(TypeRun &r) { gr_solve_update_v(r.d, r.ds, r.p, r.ps, g_cpl.mfgr, g_cpl.gogr); }
void go_update(TypeRun &r) { go_solve_update_v(r.d, r.ds, r.p, r.ps, g_cpl.grgo); }
void pkj_update(TypeRun &r) { pkj_solve_update_v(r.d, r.ds, r.p, r.ps, g_cpl.grpkj, g_cpl.mlipkj); }
void io_update(TypeRun &r) { io_solve_update_v(r.d, r.ds, r.p, r.ps, g_cpl.io_gap); }

// One batch of recorded output of one type, written by the writer thread in
// the order the batches were queued.
struct Batch {
  FILE *fv, *fr;
  int type, n, cells, cols;
  double t0;  // start of the batch's first interval
  std::vector<double> rows;
  std::vector<double> spk_t;
  std::vector<int> spk_cell;
};

class Writer {
 public:
  Writer() : th_([this] { run(); }) {}
  ~Writer() { finish(); }
  void push(Batch &&b) {
    std::lock_guard<std::mutex> g(m_);
    q_.push_back(std::move(b));
    cv_.notify_one();
  }
  void finish() {
    {
      std::lock_guard<std::mutex> g(m_);
      done_ = true;
      cv_.notify_one();
    }
    if (th_.joinable()) th_.join();
  }

 private:
  void run() {
    for (;;) {
      Batch b;
      {
        std::unique_lock<std::mutex> l(m_);
        cv_.wait(l, [this] { return done_ || !q_.empty(); });
        if (q_.empty()) return;
        b = std::move(q_.front());
        q_.pop_front();
      }
      write(b);
    }
  }
  // output_file's rows: "%lf," time then the columns; raster "%lf,%d\n"
  static void write(const Batch &b) {
    size_t s = 0;
    for (int i = 0; i < b.n; i++) {
      const double t = b.t0 + (i + 1) * H_MAX;
      fprintf(b.fv, "%lf,", t);
      const double *r = b.rows.data() + (size_t)i * b.cells * b.cols;
      for (int j = 0; j < b.cells * b.cols; j++) fprintf(b.fv, "%lf,", r[j]);
      fprintf(b.fv, "\n");
      while (s < b.spk_t.size() && b.spk_t[s] == t) fprintf(b.fr, "%lf,%d\n", t, b.spk_cell[s++]);
    }
  }
  std::mutex m_;
  std::condition_variable cv_;
  std::deque<Batch> q_;
  bool done_ = false;
  std::thread th_;
};

}  // namespace

int main(int argc, char **argv) {
  if (argc < 13) {
    printf("usage: %s S_gr gx gy S_go ox oy S_pkj px py S_io ix iy [TS_ms]\n", argv[0]);
    return 1;
  }
  const double ts = (argc > 13) ? atof(argv[13]) : 1500.0;
  const int batch = (argc > 14) ? atoi(argv[14]) : 1;
  const bool network = (argc > 15) && atoi(argv[15]) != 0;
  if (batch < 1 || (network && batch != 1)) {
    printf("batch must be >= 1 (and 1 in network mode)\n");
    return 1;
  }
  srand(0);  // the initial-voltage jitter stream, seeded as main.cu:38 does
  // the reference's console echo (main.cu:40-55)
  printf("argc = %d\n", argc);
  for (int i = 0; i < argc; i++) printf("argv[%d] = %s\n", i, argv[i]);
  static const char *const kEcho[4] = {"GR  solver -> ", "GO  solver -> ", "PKJ solver -> ", "IO  solver -> "};
  for (int k = 0; k < 4; k++) printf("%s%s\n", kEcho[k], argv[1 + 3 * k]);
  printf("\n");
  TypeRun runs[4] = {
      {"gr", gr_initialize, gr_solve_initialize, gr_set_current_launch, gr_output_file, gr_finalize, gr_solve_finalize},
      {"go", go_initialize, go_solve_initialize, go_set_current_launch, go_output_file, go_finalize, go_solve_finalize},
      {"pkj", pkj_initialize, pkj_solve_initialize, pkj_set_current_launch, pkj_output_file, pkj_finalize,
       pkj_solve_finalize},
      {"io", io_initialize, io_solve_initialize, io_set_current_launch, io_output_file, io_finalize, io_solve_finalize}};
  void (*update[4])(TypeRun &) = {gr_update, go_update, pkj_update, io_update};
  int nx[4], ny[4];
  for (int k = 0; k < 4; k++) {
    strncpy(runs[k].solver, argv[1 + 3 * k], GBRKC_MAX_BUF - 1);
    runs[k].solver[GBRKC_MAX_BUF - 1] = 0;
    nx[k] = atoi(argv[2 + 3 * k]);
    ny[k] = atoi(argv[3 + 3 * k]);
    // BE, CN or RKC, matched on the first letters (main.cu:60-102); the
    // reference's scripts name BE or CN for the types they leave empty
    const char *tag = !strncmp(runs[k].solver, "BE", 2)    ? "BE"
                      : !strncmp(runs[k].solver, "CN", 2)  ? "CN"
                      : !strncmp(runs[k].solver, "RKC", 3) ? "RKC"
                                                           : nullptr;
    if (!tag) {
      printf("Error!! -> set solver name in argv [ %d ]\n", 1 + 3 * k);
      return 0;
    }
    if (strcmp(tag, "RKC") != 0 && nx[k] * ny[k] > 0) {
      printf("%s: solver %s is not provided (only RKC)\n", runs[k].name, runs[k].solver);
      return 1;
    }
    char name[64];
    snprintf(name, sizeof name, "%s_v_by_%s.csv", runs[k].name, tag);
    runs[k].fv = fopen(name, "w");
    snprintf(name, sizeof name, "%s_raster_by_%s.csv", runs[k].name, tag);
    runs[k].fr = fopen(name, "w");
    if (!runs[k].fv || !runs[k].fr) {
      printf("cannot open the output files of %s\n", runs[k].name);
      return 1;
    }
  }
  for (int k = 0; k < 4; k++) {
    TypeRun &r = runs[k];
    r.p = (neuron_t *)malloc(sizeof(neuron_t));
    r.ps = (neuron_solve_t *)malloc(sizeof(neuron_solve_t));
    r.d = r.init(nx[k], ny[k], r.solver, r.p);
    r.ds = r.solve_init(r.ps, r.solver, r.p, r.d);
    r.vh = (double *)malloc((r.p->nc > 0 ? r.p->nc : 1) * sizeof(double));
    r.raster = (double *)malloc((r.p->n > 0 ? r.p->n : 1) * sizeof(double));
    for (int j = 0; j < r.p->n; j++) r.raster[j] = 100.0;
  }
  // the coupling objects (main.cu:137-145)
  synapse_t *mfgr = mfgr_create(runs[0].p->n);
  synapse_t *gogr = gogr_create(runs[1].p->nx, runs[1].p->ny, runs[0].p->nx, runs[0].p->ny);
  synapse_t *grgo = grgo_create(runs[0].p->nx, runs[0].p->ny, runs[1].p->nx, runs[1].p->ny);
  synapse_t *grpkj = grpkj_create(runs[0].p->nx, runs[0].p->ny, runs[2].p->nx, runs[2].p->ny);
  synapse_t *mlipkj = mlipkj_create(runs[2].p->n, runs[0].p->n);
  gap_t *io_gap = io_gap_create(nx[3], ny[3]);
  g_cpl = Coupling{mfgr, gogr, grgo, grpkj, mlipkj, io_gap};
  FILE *dbg = fopen("debug_file.csv", "w");
  if (dbg) fclose(dbg);

  double t = 0.0;
  const clock_t start = clock();
  clock_t half = start;
  if (batch > 1) {
    // intervals the per-interval loop below would run
    long total = 0;
    for (double tt = 0.0; tt < ts - 0.0001; tt += H_MAX) total++;
    Writer w;
    for (long done = 0; done < total;) {
      const int n = (int)std::min<long>(batch, total - done);
      for (int k = 0; k < 4; k++) {
        TypeRun &r = runs[k];
        if (r.p->n <= 0) continue;
        Batch b;
        b.fv = r.fv;
        b.fr = r.fr;
        b.type = k;
        b.n = n;
        b.cells = r.p->n;
        b.cols = (k == 3) ? 3 : 1;
        b.t0 = t;
        b.rows.resize((size_t)n * b.cells * b.cols);
        const long cap = (long)b.cells * (n / 2 + 1);
        b.spk_t.resize(cap);
        b.spk_cell.resize(cap);
        const long m = gbrkc_compat_advance_batch(k, n, b.rows.data(), (long)b.rows.size(), b.spk_t.data(),
                                                  b.spk_cell.data(), cap);
        if (m == -5) {
          w.finish();
          printf("isnan in %s, time=%f\n", r.name, t);
          return 1;
        }
        if (m < 0) {
          printf("batched advance of %s failed (%ld)\n", r.name, m);
          return 1;
        }
        b.spk_t.resize(m);
        b.spk_cell.resize(m);
        w.push(std::move(b));
      }
      const double t_prev = t;
      for (int i = 0; i < n; i++) t += H_MAX;
      if (t_prev < 500.0 && t >= 500.0) half = clock();
      done += n;
    }
    w.finish();
  }
  long t_count = 0;
  while (t < ts - 0.0001) {
    if (t_count++ % 400 == 0) {  // progress every 50 ms (main.cu:185-190)
      printf("time:%f\n", t);
      printf("Now compute time = %.2f \n", (double)(clock() - start) / CLOCKS_PER_SEC);
    }
    for (int k = 0; k < 4; k++) {
      TypeRun &r = runs[k];
      if (r.p->n <= 0) continue;
      if (!network) r.stim(r.d, t);
      update[k](r);
      if (cudaMemcpy(r.vh, r.ps->vec[v_new], r.p->nc * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) {
        printf("copy of %s voltages failed\n", r.name);
        return 1;
      }
      if (isnan(r.vh[1])) {
        printf("isnan in %s, time=%f\n", r.name, t);
        return 1;
      }
      r.out(r.p, r.vh, r.raster, t + H_MAX, r.fv, r.fr);
    }
    if (network) {  // main.cu:300-305
      gr_synapse_update(t, H_MAX, mfgr, gogr, runs[1].d, runs[0].ps);
      go_synapse_update(t, H_MAX, grgo, runs[0].d, runs[1].ps);
      pkj_synapse_update(t, H_MAX, grpkj, mlipkj, runs[0].d, runs[2].ps);
    }
    t += H_MAX;
    if (t >= 500.0 && 500.0 + H_MAX > t) half = clock();
  }
  const clock_t end = clock();
  const double comp = (double)(end - start) / CLOCKS_PER_SEC;
  printf("time:%f \ncomputational time = %.2f \n", t, comp);
  const int n[4] = {runs[0].p->n, runs[1].p->n, runs[2].p->n, runs[3].p->n};
  if (ts <= 500.0)
    output_time(n[0], runs[0].solver, n[1], runs[1].solver, n[2], runs[2].solver, n[3], runs[3].solver, comp, (int)ts);
  else
    output_time2(n[0], runs[0].solver, n[1], runs[1].solver, n[2], runs[2].solver, n[3], runs[3].solver, comp,
                 (double)(end - half) / CLOCKS_PER_SEC, (int)ts);
  mfgr_finalize(mfgr, n[0]);
  gogr_finalize(gogr, n[1] * n[0]);
  grgo_finalize(grgo, n[1] * n[0]);
  grpkj_finalize(grpkj, n[0] * n[2]);
  mlipkj_finalize(mlipkj, n[0] * n[2]);
  io_gap_finalize(io_gap);
  for (int k = 0; k < 4; k++) {
    TypeRun &r = runs[k];
    free(r.vh);
    free(r.raster);
    r.fin(r.p, r.d, r.fv, r.fr);
    r.solve_fin(n[k], r.ds, r.ps);
  }
  return 0;
}

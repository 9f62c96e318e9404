// Runs the reference simulator's own RKC path on the GPU -- its X_initialize
// / X_solve_initialize / X_set_current / X_solve_update_v / X_output_file
// entry points, compiled from its sources by this directory's Makefile --
// in the per-interval loop of its main.cu:182-311,
// with the simulated time, the stimulus and extra outputs chosen on the
// command line.  Test infrastructure and the reference baseline; not part of
// the product.
//
//   ref_rkc_run GRX GRY GOX GOY PKJX PKJY IOX IOY TS_MS STIM OUTDIR DUMP_IV
//               [SOLVERS [NETWORK]]
//
//   STIM    "ref": the reference's X_set_current protocols, as main.cu runs
//           them; "const:gr=A,go=A,pkj=A,io=A" (any subset): a current A
//           at the compartment each type's X_set_current stimulates (GrC 16,
//           GoC 30, PC 1599, IO 0; gr.cu:245, go.cu:258, pkj.cu:333,
//           io.cu:247), in the units of that type, for all t -- or from t0 on
//           with "A@t0"; none for the types not named.
//   OUTDIR  receives the reference's CSVs ({gr,go,pkj,io}_{v,raster}_by_RKC
//           .csv, written by its own X_output_file) and, for the first
//           DUMP_IV intervals, every compartment's v_new of every type as
//           raw float64 (<type>_vnew.bin, interval-major), and the initial
//           elem[v] (<type>_v0.bin).
//   SOLVERS "RKC" (default) or four comma-separated solver names for GrC,
//           GoC, PC and IO (RKC, CN or BE, as main.cu's arguments), e.g.
//           "CN,RKC,RKC,CN" as the reference's network1.sh runs them; a
//           BE / CN type takes DT = 0.025 ms sub-steps within each interval
//           (main.cu:193-200) and its voltage is read from elem[v].  The
//           CSV names carry each type's solver name, as main.cu's do.
//   NETWORK 1: main.cu's network branch -- no X_set_current, and after
//           every interval the three synapse updates of main.cu:302-306 --
//           which main.cu itself leaves off (network_sim = false, main.cu:39).
// Model files are read by the reference's loaders from the working
// directory.  srand(0) as main.cu:38, so the initial jitter follows its
// rand() order (GrC, GoC, PC, IO).  Prints one JSON line: the loop's wall
// time (device synchronised at both ends; the reference's D2H copy and CSV
// output of every interval included, as in main.cu) and the sizes.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "param.h"
#include "go.cuh"
#include "go_solve.cuh"
#include "go_ion.cuh"
#include "gr.cuh"
#include "gr_solve.cuh"
#include "gr_ion.cuh"
#include "pkj.cuh"
#include "pkj_solve.cuh"
#include "pkj_ion.cuh"
#include "io.cuh"
#include "io_solve.cuh"
#include "io_ion.cuh"
#include "solve_bem.cuh"
#include "solve_rkc.cuh"
#include "syn.cuh"
#include "gap.cuh"
#include "output.cuh"

__global__ void const_current(neuron_t *d, const int comp, const int ncomp, const double amp) {
  const int id = threadIdx.x + blockIdx.x * blockDim.x;
  if (id < d->n) d->elem[i_ext][comp + id * ncomp] = amp;
}

// the compartment and compartment count of each type's X_set_current
static const int STIM_COMP[4] = {16, GO_COMP_DEND * 3, 1599, 0};
static const int NCOMP[4] = {GR_COMP, GO_COMP, PKJ_COMP, IO_COMP};

static double now_s() {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static FILE *open_out(const char *dir, const char *name, const char *mode) {
  char path[2048];
  snprintf(path, sizeof path, "%s/%s", dir, name);
  FILE *f = fopen(path, mode);
  if (!f) {
    perror(path);
    exit(2);
  }
  return f;
}

struct TypeRun {
  const char *name;
  int n = 0, nc = 0;
  neuron_t *p = nullptr, *d = nullptr;
  neuron_solve_t *ps = nullptr, *ds = nullptr;
  double *host = nullptr, *raster = nullptr;
  FILE *fv = nullptr, *fr = nullptr, *fdump = nullptr;
};

int main(int argc, char **argv) {
  if (argc < 13) {
    fprintf(stderr, "usage: ref_rkc_run GRX GRY GOX GOY PKJX PKJY IOX IOY TS_MS STIM OUTDIR DUMP_IV\n");
    return 1;
  }
  int dims[8];
  for (int k = 0; k < 8; k++) dims[k] = atoi(argv[1 + k]);
  const double ts_ms = atof(argv[9]);
  const char *stim = argv[10];
  const char *dir = argv[11];
  const int dump_iv = atoi(argv[12]);
  double amp[4] = {0.0, 0.0, 0.0, 0.0}, t_on[4] = {0.0, 0.0, 0.0, 0.0};
  bool on[4] = {false, false, false, false};
  const bool ref_stim = strcmp(stim, "ref") == 0;
  if (!ref_stim) {
    if (strncmp(stim, "const:", 6) != 0) {
      fprintf(stderr, "STIM must be ref or const:TYPE=A,...\n");
      return 1;
    }
    char buf[512];
    snprintf(buf, sizeof buf, "%s", stim + 6);
    for (char *tok = strtok(buf, ","); tok; tok = strtok(nullptr, ",")) {
      char *eq = strchr(tok, '=');
      if (!eq) return 1;
      *eq = 0;
      int k = !strcmp(tok, "gr") ? 0 : !strcmp(tok, "go") ? 1 : !strcmp(tok, "pkj") ? 2 : !strcmp(tok, "io") ? 3 : -1;
      if (k < 0) {
        fprintf(stderr, "unknown type %s\n", tok);
        return 1;
      }
      on[k] = true;
      amp[k] = atof(eq + 1);
      if (const char *at = strchr(eq + 1, '@')) t_on[k] = atof(at + 1);
    }
  }
  char solvers[4][8] = {"RKC", "RKC", "RKC", "RKC"};
  if (argc > 13 && strcmp(argv[13], "RKC") != 0) {
    char buf[64];
    snprintf(buf, sizeof buf, "%s", argv[13]);
    int k = 0;
    for (char *tok = strtok(buf, ","); tok && k < 4; tok = strtok(nullptr, ","), k++) snprintf(solvers[k], 8, "%s", tok);
    if (k != 4) {
      fprintf(stderr, "SOLVERS: four names or RKC\n");
      return 1;
    }
  }
  const bool network = argc > 14 && atoi(argv[14]) != 0;
  srand(0);
  TypeRun T[4];
  const char *names[4] = {"gr", "go", "pkj", "io"};
  for (int k = 0; k < 4; k++) {
    T[k].name = names[k];
    T[k].p = (neuron_t *)malloc(sizeof(neuron_t));
    T[k].ps = (neuron_solve_t *)malloc(sizeof(neuron_solve_t));
  }
  // main.cu:105-134: each type initialised in this order (rand() order)
  T[0].d = gr_initialize(dims[0], dims[1], solvers[0], T[0].p);
  T[0].ds = gr_solve_initialize(T[0].ps, solvers[0], T[0].p, T[0].d);
  T[1].d = go_initialize(dims[2], dims[3], solvers[1], T[1].p);
  T[1].ds = go_solve_initialize(T[1].ps, solvers[1], T[1].p, T[1].d);
  T[2].d = pkj_initialize(dims[4], dims[5], solvers[2], T[2].p);
  T[2].ds = pkj_solve_initialize(T[2].ps, solvers[2], T[2].p, T[2].d);
  T[3].d = io_initialize(dims[6], dims[7], solvers[3], T[3].p);
  T[3].ds = io_solve_initialize(T[3].ps, solvers[3], T[3].p, T[3].d);
  // main.cu:137-145
  synapse_t *mfgr = mfgr_create(T[0].p->n);
  synapse_t *gogr = gogr_create(T[1].p->nx, T[1].p->ny, T[0].p->nx, T[0].p->ny);
  synapse_t *grgo = grgo_create(T[0].p->nx, T[0].p->ny, T[1].p->nx, T[1].p->ny);
  synapse_t *grpkj = grpkj_create(T[0].p->nx, T[0].p->ny, T[2].p->nx, T[2].p->ny);
  synapse_t *mlipkj = mlipkj_create(T[2].p->n, T[0].p->n);
  gap_t *io_gap = io_gap_create(dims[6], dims[7]);
  for (int k = 0; k < 4; k++) {
    TypeRun &R = T[k];
    R.n = R.p->n;
    R.nc = R.p->nc;
    char nm[64];
    snprintf(nm, sizeof nm, "%s_v_by_%s.csv", R.name, solvers[k]);
    R.fv = open_out(dir, nm, "w");
    snprintf(nm, sizeof nm, "%s_raster_by_%s.csv", R.name, solvers[k]);
    R.fr = open_out(dir, nm, "w");
    if (R.nc == 0) continue;
    R.host = (double *)malloc(sizeof(double) * R.nc);
    R.raster = (double *)malloc(sizeof(double) * R.n);
    for (int i = 0; i < R.n; i++) R.raster[i] = 100;
    cudaMemcpy(R.host, R.p->elem[v], sizeof(double) * R.nc, cudaMemcpyDeviceToHost);
    snprintf(nm, sizeof nm, "%s_v0.bin", R.name);
    FILE *f0 = open_out(dir, nm, "wb");
    fwrite(R.host, sizeof(double), R.nc, f0);
    fclose(f0);
    if (dump_iv > 0) {
      snprintf(nm, sizeof nm, "%s_vnew.bin", R.name);
      R.fdump = open_out(dir, nm, "wb");
    }
  }
  cudaDeviceSynchronize();
  const double w0 = now_s();
  double t = 0.0;
  int iv = 0, bad = -1;
  while (t < ts_ms - 0.0001 && bad < 0) {
    for (int k = 0; k < 4 && bad < 0; k++) {
      TypeRun &R = T[k];
      if (R.n == 0) continue;
      const int blocks = R.n / 128 + 1;
      // main.cu:193-200: sub-steps of the type's DT within the interval
      for (double l_dt = 0.0; l_dt < H_MAX; l_dt += R.p->DT) {
        if (network) {
        } else if (ref_stim) {
          switch (k) {
            case 0: gr_set_current<<<blocks, 128>>>(R.d, t + l_dt); break;
            case 1: go_set_current<<<blocks, 128>>>(R.d, t + l_dt); break;
            case 2: pkj_set_current<<<blocks, 128>>>(R.d, t + l_dt); break;
            default: io_set_current<<<blocks, 128>>>(R.d, t + l_dt); break;
          }
        } else if (on[k]) {
          const_current<<<blocks, 128>>>(R.d, STIM_COMP[k], NCOMP[k], (t + l_dt >= t_on[k]) ? amp[k] : 0.0);
        }
        switch (k) {
          case 0: gr_solve_update_v(R.d, R.ds, R.p, R.ps, mfgr, gogr); break;
          case 1: go_solve_update_v(R.d, R.ds, R.p, R.ps, grgo); break;
          case 2: pkj_solve_update_v(R.d, R.ds, R.p, R.ps, grpkj, mlipkj); break;
          default: io_solve_update_v(R.d, R.ds, R.p, R.ps, io_gap); break;
        }
      }
      if (R.p->n_solver == kRKC)
        cudaMemcpy(R.host, R.ps->vec[v_new], sizeof(double) * R.nc, cudaMemcpyDeviceToHost);
      else
        cudaMemcpy(R.host, R.p->elem[v], sizeof(double) * R.nc, cudaMemcpyDeviceToHost);
      if (isnan(R.host[1])) bad = k;
      switch (k) {
        case 0: gr_output_file(R.p, R.host, R.raster, t + H_MAX, R.fv, R.fr); break;
        case 1: go_output_file(R.p, R.host, R.raster, t + H_MAX, R.fv, R.fr); break;
        case 2: pkj_output_file(R.p, R.host, R.raster, t + H_MAX, R.fv, R.fr); break;
        default: io_output_file(R.p, R.host, R.raster, t + H_MAX, R.fv, R.fr); break;
      }
      if (R.fdump && iv < dump_iv) fwrite(R.host, sizeof(double), R.nc, R.fdump);
    }
    if (network && bad < 0) {
      // main.cu:302-306
      gr_synapse_update(t, H_MAX, mfgr, gogr, T[1].d, T[0].ps);
      go_synapse_update(t, H_MAX, grgo, T[0].d, T[1].ps);
      pkj_synapse_update(t, H_MAX, grpkj, mlipkj, T[0].d, T[2].ps);
    }
    iv++;
    t += H_MAX;
  }
  cudaDeviceSynchronize();
  const double wall = now_s() - w0;
  const cudaError_t err = cudaGetLastError();
  for (int k = 0; k < 4; k++) {
    fclose(T[k].fv);
    fclose(T[k].fr);
    if (T[k].fdump) fclose(T[k].fdump);
  }
  printf("{\"wall_s\": %.6f, \"intervals\": %d, \"ts_ms\": %.6f, \"nan_type\": %d, \"cuda\": \"%s\", "
         "\"solvers\": \"%s,%s,%s,%s\", \"network\": %d, "
         "\"nc\": {\"gr\": %d, \"go\": %d, \"pkj\": %d, \"io\": %d}, "
         "\"cells\": {\"gr\": %d, \"go\": %d, \"pkj\": %d, \"io\": %d}, \"stim\": \"%s\"}\n",
         wall, iv, t, bad, cudaGetErrorString(err), solvers[0], solvers[1], solvers[2], solvers[3], (int)network,
         T[0].nc, T[1].nc, T[2].nc, T[3].nc, T[0].n, T[1].n, T[2].n,
         T[3].n, stim);
  return bad >= 0 ? 3 : 0;
}

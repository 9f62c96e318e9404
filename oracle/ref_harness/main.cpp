// Command-line front end of the reference harness (test infrastructure).
//   ref_harness setup TYPE NX NY OUTDIR
//   ref_harness ion   TYPE NX NY SEED NSTEPS DT OUTDIR
// TYPE: 0 GR, 1 GO, 2 PKJ, 3 IO.  Morphology files are read by the
// reference's own loaders from the current directory.  Outputs are raw
// little-endian float64 / int32 files in OUTDIR.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "harness.h"

extern "C" void ref_host_setup_gr(int, int, struct ref_state *);
extern "C" void ref_host_setup_go(int, int, struct ref_state *);
extern "C" void ref_host_setup_pkj(int, int, struct ref_state *);
extern "C" void ref_host_setup_io(int, int, struct ref_state *);
extern "C" int ref_csr_gr(int, int, int *, int *, double *, int);
extern "C" int ref_csr_go(int, int, int *, int *, double *, int);
extern "C" int ref_csr_pkj(int, int, int *, int *, double *, int);
extern "C" int ref_csr_io(int, int, int *, int *, double *, int);

static const int NCOND[4] = {10, 13, 11, 8};
static const int NION[4] = {20, 24, 18, 10};
static const int NCOMP[4] = {578, 131, 1600, 3};

static void dump(const char *dir, const char *name, const void *p, size_t bytes) {
  char path[1024];
  snprintf(path, sizeof path, "%s/%s.bin", dir, name);
  FILE *f = fopen(path, "wb");
  if (!f) { perror(path); exit(2); }
  fwrite(p, 1, bytes, f);
  fclose(f);
}

static void setup(int type, int nx, int ny, struct ref_state *s) {
  memset(s, 0, sizeof *s);
  s->type = type; s->ncond = NCOND[type]; s->nion = NION[type];
  switch (type) {
    case 0: ref_host_setup_gr(nx, ny, s); break;
    case 1: ref_host_setup_go(nx, ny, s); break;
    case 2: ref_host_setup_pkj(nx, ny, s); break;
    case 3: ref_host_setup_io(nx, ny, s); break;
  }
}

static void dump_state(const char *dir, const char *tag, struct ref_state *s) {
  char nm[64];
  size_t B = sizeof(double) * s->nc;
  snprintf(nm, sizeof nm, "%s_v", tag); dump(dir, nm, s->elem[0], B);
  snprintf(nm, sizeof nm, "%s_ca", tag); dump(dir, nm, s->elem[1], B);
  for (int k = 0; k < s->nion; k++) { snprintf(nm, sizeof nm, "%s_ion%d", tag, k); dump(dir, nm, s->ion[k], B); }
  if (s->type == 1 || s->type == 2) { snprintf(nm, sizeof nm, "%s_rev", tag); dump(dir, nm, s->rev_ca2, B); }
  if (s->type == 1) {
    snprintf(nm, sizeof nm, "%s_ca2", tag); dump(dir, nm, s->ca2, B);
    snprintf(nm, sizeof nm, "%s_caold", tag); dump(dir, nm, s->ca_old, B);
  }
}

int main(int argc, char **argv) {
  if (argc < 5) { fprintf(stderr, "usage: see source\n"); return 1; }
  int type = atoi(argv[2]), nx = atoi(argv[3]), ny = atoi(argv[4]);
  struct ref_state s;
  setup(type, nx, ny, &s);
  if (!strcmp(argv[1], "setup")) {
    const char *dir = argv[5];
    size_t B = sizeof(double) * s.nc;
    dump(dir, "cm", s.elem[2], B);
    dump(dir, "area", s.elem[3], B);
    dump(dir, "compart", s.elem[5], B);
    for (int k = 0; k < s.ncond; k++) { char nm[32]; snprintf(nm, sizeof nm, "cond%d", k); dump(dir, nm, s.cond[k], B); }
    if (type == 2) dump(dir, "shell", s.shell, B);
    int cap = 8 * s.nc + 4096;
    int *row = (int *)calloc(s.nc + 1, sizeof(int)), *col = (int *)calloc(cap, sizeof(int));
    double *val = (double *)calloc(cap, sizeof(double));
    int nnz = 0;
    switch (type) {
      case 0: nnz = ref_csr_gr(nx, ny, row, col, val, cap); break;
      case 1: nnz = ref_csr_go(nx, ny, row, col, val, cap); break;
      case 2: nnz = ref_csr_pkj(nx, ny, row, col, val, cap); break;
      case 3: nnz = ref_csr_io(nx, ny, row, col, val, cap); break;
    }
    if (nnz < 0) { fprintf(stderr, "csr capacity\n"); return 3; }
    dump(dir, "row", row, sizeof(int) * (s.nc + 1));
    dump(dir, "col", col, sizeof(int) * nnz);
    dump(dir, "val", val, sizeof(double) * nnz);
    return 0;
  }
  if (!strcmp(argv[1], "ion")) {
    int seed = atoi(argv[5]), nsteps = atoi(argv[6]);
    double DT = atof(argv[7]);
    const char *dir = argv[8];
    srand(seed);
    ref_init_ion(&s);
    dump_state(dir, "init", &s);
    double *vnew = (double *)calloc(s.nc, sizeof(double));
    for (int k = 0; k < nsteps; k++) {
      for (int i = 0; i < s.nc; i++) {
        double x = (double)i * 0.6180339887498949 + (double)k * 0.2718281828459045;
        vnew[i] = -90.0 + 130.0 * (x - floor(x));
      }
      ref_ion_update(&s, vnew, DT);
    }
    dump_state(dir, "final", &s);
    return 0;
  }
  return 1;
}

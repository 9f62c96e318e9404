// Reference CSR build for one cell type (set_host_pkj_solve), compiled from
// the reference source where it lies (test infrastructure).
#include "pkj_solve.cu"
#include "harness.h"
extern "C" int ref_csr_pkj(int nx, int ny, int *row, int *col, double *val, int cap) {
  neuron_t t;
  memset(&t, 0, sizeof t);
  t.nx = nx; t.ny = ny; t.n = nx * ny; t.nc = t.n * PKJ_COMP;
  neuron_solve_t *s = set_host_pkj_solve("RKC", &t);
  int nnz = s->row[t.nc];
  if (nnz > cap) return -nnz;
  for (int i = 0; i <= t.nc; i++) row[i] = s->row[i];
  for (int i = 0; i < nnz; i++) { col[i] = s->col[i]; val[i] = s->val[i]; }
  return nnz;
}

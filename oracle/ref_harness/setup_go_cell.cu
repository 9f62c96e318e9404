// Reference static setup for one cell type, compiled from the reference
// source where it lies (test infrastructure).  Exposes initialize_host_go.
#include "go.cu"
#include "harness.h"
extern "C" void ref_host_setup_go(int nx, int ny, struct ref_state *s) {
  neuron_t *h = (neuron_t *)calloc(1, sizeof(neuron_t));
  h->nx = nx; h->ny = ny; h->n = nx * ny; h->nc = h->n * GO_COMP;
  initialize_host_go(h);
  s->n = h->n; s->nc = h->nc;
  for (int k = 0; k < n_elem; k++) s->elem[k] = h->elem[k];
  for (int k = 0; k < s->ncond; k++) s->cond[k] = h->cond[k];
  for (int k = 0; k < s->nion; k++) s->ion[k] = h->ion[k];
  s->ca2 = h->ca2; s->rev_ca2 = h->rev_ca2; s->ca_old = h->ca_old; s->shell = h->shell;
}

// Host driver for the reference's RKC ion kernels -- test infrastructure.
//
// Compiled with g++ together with the reference's gr_ion.cu, go_ion.cu,
// pkj_ion.cu and io_ion.cu (built where they lie, with shim/cuda_runtime.h
// standing in for CUDA), so each __global__ kernel body runs on the host once
// per compartment index.  Its outputs pin the oracle's gating code.
#include "param.h"
#include "gr.cuh"
#include "go.cuh"
#include "pkj.cuh"
#include "io.cuh"
#include "harness.h"

ref_dim3 threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0}, blockDim = {1, 1, 1}, gridDim = {1, 1, 1};

extern "C" {

static void fill_neuron(neuron_t *nt, ref_state *s, double **elem, double **cond, double **ion) {
  for (int k = 0; k < n_elem; k++) elem[k] = s->elem[k];
  for (int k = 0; k < s->ncond; k++) cond[k] = s->cond[k];
  for (int k = 0; k < s->nion; k++) ion[k] = s->ion[k];
  nt->elem = elem; nt->cond = cond; nt->ion = ion;
  nt->ca2 = s->ca2; nt->rev_ca2 = s->rev_ca2; nt->ca_old = s->ca_old; nt->shell = s->shell;
  nt->n = s->n; nt->nc = s->nc; nt->nx = s->n; nt->ny = 1;
}

// *_initialize_ion (host functions of the reference)
void ref_init_ion(ref_state *s) {
  neuron_t nt; double *elem[n_elem], *cond[24], *ion[24];
  fill_neuron(&nt, s, elem, cond, ion);
  switch (s->type) {
    case N_TYPE_GR: gr_initialize_ion(&nt); break;
    case N_TYPE_GO: go_initialize_ion(&nt); break;
    case N_TYPE_PKJ: pkj_initialize_ion(&nt); break;
    case N_TYPE_IO: io_initialize_ion(&nt); break;
  }
}

// the RKC ion-update kernels, in the order *_update_ion_and_matrix launches them
void ref_ion_update(ref_state *s, double *vnew, double DT) {
  neuron_t nt; double *elem[n_elem], *cond[24], *ion[24];
  fill_neuron(&nt, s, elem, cond, ion);
  neuron_solve_t ns;
  memset(&ns, 0, sizeof ns);
  switch (s->type) {
    case N_TYPE_GR:
      for (int id = 0; id < s->nc; id++) {
        blockIdx.x = id;
        gr_Na_update_2order(s->nc, vnew, elem[v], DT, elem[compart], ion[o_Na], ion[c1_Na],
                            ion[c2_Na], ion[c3_Na], ion[c4_Na], ion[c5_Na], ion[i1_Na],
                            ion[i2_Na], ion[i3_Na], ion[i4_Na], ion[i5_Na], ion[i6_Na]);
      }
      for (int id = 0; id < s->nc; id++) { blockIdx.x = id; gr_update_ion_RKC_exp_imp(&nt, &ns, vnew, DT); }
      break;
    case N_TYPE_GO:
      for (int id = 0; id < s->nc; id++) { blockIdx.x = id; go_update_ion_RKC_exp_imp(&nt, &ns, vnew, DT); }
      for (int id = 0; id < s->nc; id++) {
        blockIdx.x = id;
        go_KAHP_update_2order(s->n, elem[Ca], s->ca_old, ion[o1_KAHP_go], ion[o2_KAHP_go],
                              ion[c1_KAHP_go], ion[c2_KAHP_go], ion[c3_KAHP_go], ion[c4_KAHP_go], DT);
      }
      break;
    case N_TYPE_PKJ:
      for (int id = 0; id < s->nc; id++) { blockIdx.x = id; pkj_update_ion_RKC(&nt, &ns, vnew, DT); }
      break;
    case N_TYPE_IO:
      for (int id = 0; id < s->nc; id++) { blockIdx.x = id; io_update_ion_RKC(&nt, &ns, vnew, DT); }
      break;
  }
  blockIdx.x = 0;
}

}  // extern "C"

// Never-called definitions for CN-solver kernels that the reference's
// *_solve.cu files reference but that live in solve_cnm.cu (not built here).
// Test infrastructure only.
#include "param.h"
__global__ void gr_cnm_vec_initialize(neuron_t *, neuron_solve_t *) {}
__global__ void go_cnm_vec_initialize(neuron_t *, neuron_solve_t *) {}
__global__ void pkj_cnm_vec_initialize(neuron_t *, neuron_solve_t *) {}
__global__ void io_cnm_vec_initialize(neuron_t *, neuron_solve_t *) {}

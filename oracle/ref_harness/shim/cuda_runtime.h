/* Host-only stand-in for <cuda_runtime.h>, used to compile the reference's
 * *_ion.cu files with g++ so that their __global__ kernel bodies run as
 * plain host functions (one call per thread index).  Test infrastructure. */
#pragma once
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
struct ref_dim3 { unsigned int x, y, z; };
extern ref_dim3 threadIdx, blockIdx, blockDim, gridDim;
typedef int cudaError_t;

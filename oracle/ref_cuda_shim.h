// Host execution of the reference's CUDA kernels (TEST INFRASTRUCTURE ONLY).
//
// The kernels of src/gromacs/zeta_fmm/kernel.cu launch one thread per block,
// except p2p (64 threads per block that share nothing and never synchronise)
// and merge_bodies (independent threads); their __shared__ arrays are scratch
// of the block's single thread.  A host loop over blocks and threads therefore
// runs them exactly as written.  Host compilers see __global__, __device__ and
// __shared__ as ignored attributes through cuda_runtime.h; this header supplies
// the built-in launch indices, which the driver sets before each call.
#pragma once
#include <cuda_runtime.h>

extern uint3 threadIdx, blockIdx;
extern dim3 blockDim, gridDim;

// the integer max/min that CUDA declares at global scope for device code
static inline int max(int a, int b) { return a > b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }

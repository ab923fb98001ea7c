// Host compilation of device code for the CPU tests: the CUDA qualifiers and the block
// barrier become no-ops, so a file of __device__ functions (csrc/ros3.cuh, the generated
// mechanism routines) compiles with g++ and runs one cell at a time on the host.  The
// barrier is needed only between lanes, and a host run has one lane per call.
#pragma once
#define __device__
#define __host__
#define __global__
#define __noinline__ __attribute__((noinline))
#define __forceinline__ inline __attribute__((always_inline))
#define __constant__
#define __syncthreads() ((void)0)
#include <math.h>

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
#define __syncwarp(...) ((void)0)
#include <math.h>
// one lane of one block: the cooperative (per-warp) code paths compile but are not run
struct CudaHostIndex3 {
    unsigned x, y, z;
};
static const CudaHostIndex3 threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0}, blockDim = {32, 1, 1}, gridDim = {1, 1, 1};
// the intrinsics the device code names, with their IEEE meaning for one lane (a host float
// or double operation rounds to nearest like the _rn forms; warp votes and shuffles of a
// single lane return its own value)
#include <string.h>
inline double __longlong_as_double(long long x)
{
    double d;
    memcpy(&d, &x, sizeof d);
    return d;
}
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fadd_rn(float a, float b) { return a + b; }
inline double __dmul_rn(double a, double b) { return a * b; }
inline double __dadd_rn(double a, double b) { return a + b; }
inline bool __any_sync(unsigned, bool p) { return p; }
inline bool __all_sync(unsigned, bool p) { return p; }
inline unsigned __ballot_sync(unsigned, bool p) { return p ? 1u : 0u; }
template <class T> inline T __shfl_sync(unsigned, T v, int, int = 32) { return v; }
template <class T> inline T __shfl_xor_sync(unsigned, T v, int, int = 32) { return v; }
template <class T> inline T __shfl_down_sync(unsigned, T v, unsigned, int = 32) { return v; }

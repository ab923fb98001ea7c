// Measurement helpers (include/cmaqchem_diag.h).
#include <cuda_runtime.h>

#include <string>

#include "../../include/cmaqchem_diag.h"

#ifdef CHEM_PHASE_TIMING
// clock cycles per phase of the lock-stepped ROS3 attempt (ros3.cuh: CHEM_PHASE_MARK)
__device__ unsigned long long g_chem_phase_cycles[8];
#endif

namespace {

constexpr int CHAINS = 8;

// Each thread runs CHAINS independent dependent-FMA chains; the result is stored only
// when it matches an impossible value, so the work cannot be removed.
__global__ void k_fp64_fma(int iters, double b, double c, double* sink)
{
    double a[CHAINS];
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) a[k] = (double)(threadIdx.x + k) * 1.0e-3;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < CHAINS; ++k) a[k] = fma(a[k], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s += a[k];
    if (s == -1.2345e300) sink[threadIdx.x] = s;
}

// One warp; lanes below `active` run one dependent FMA chain of `iters` links; lane 0
// reports the clock cycles the chain took.
__global__ void k_fp64_issue(int active, int iters, double b, double c, double* sink, long long* cycles)
{
    const int lane = threadIdx.x & 31;
    double a = (double)lane * 1.0e-3;
    const long long t0 = clock64();
    if (lane < active)
        for (int i = 0; i < iters; ++i) a = fma(a, b, c);
    __syncwarp();
    const long long t1 = clock64();
    if (a == -1.2345e300) sink[lane] = a;
    if (lane == 0) *cycles = t1 - t0;
}

}  // namespace

extern "C" int cmaqchem_diag_fp64_issue(int device, int active_lanes, double* cycles_per_instruction)
{
    if (active_lanes < 1 || active_lanes > 32 || !cycles_per_instruction) return -1;
    if (cudaSetDevice(device) != cudaSuccess) return -1;
    double* sink = nullptr;
    long long* cyc = nullptr;
    if (cudaMalloc(&sink, 32 * sizeof(double)) != cudaSuccess) return -1;
    if (cudaMalloc(&cyc, sizeof(long long)) != cudaSuccess) {
        cudaFree(sink);
        return -1;
    }
    const int iters = 20000;
    k_fp64_issue<<<1, 32>>>(active_lanes, 64, 0.999999, 1.0e-7, sink, cyc);   // warm-up
    k_fp64_issue<<<1, 32>>>(active_lanes, iters, 0.999999, 1.0e-7, sink, cyc);
    long long c = 0;
    cudaError_t err = cudaMemcpy(&c, cyc, sizeof(long long), cudaMemcpyDeviceToHost);
    cudaFree(sink);
    cudaFree(cyc);
    if (err != cudaSuccess) return -1;
    *cycles_per_instruction = (double)c / iters;
    return 0;
}

namespace {

int fp64_peak_iters(int device, int iters, double* tflops, double* ms)
{
    if (cudaSetDevice(device) != cudaSuccess) return -1;
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    double* sink = nullptr;
    if (cudaMalloc(&sink, 1024 * sizeof(double)) != cudaSuccess) return -1;
    const int threads = 256, blocks = nsm * 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fp64_fma<<<blocks, threads>>>(64, 0.999999, 1.0e-7, sink);   // warm-up
    cudaEventRecord(e0);
    k_fp64_fma<<<blocks, threads>>>(iters, 0.999999, 1.0e-7, sink);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (err != cudaSuccess) return -1;
    const double flops = 2.0 * CHAINS * (double)iters * threads * blocks;
    if (tflops) *tflops = flops / (t * 1.0e-3) / 1.0e12;
    if (ms) *ms = t;
    return 0;
}

}  // namespace

extern "C" int cmaqchem_diag_fp64_peak(int device, double* tflops, double* ms)
{
    return fp64_peak_iters(device, 4096, tflops, ms);
}

extern "C" int cmaqchem_diag_fp64_peak_long(int device, double target_ms, double* tflops, double* ms)
{
    if (!(target_ms > 0.0)) return -1;
    double t = 0.0;
    if (fp64_peak_iters(device, 4096, nullptr, &t) != 0 || !(t > 0.0)) return -1;   // rate at 4096 links
    double scale = (target_ms < 10.0 ? 10.0 : (target_ms > 5000.0 ? 5000.0 : target_ms)) / t;
    const double iters = 4096.0 * scale;
    return fp64_peak_iters(device, iters > 1.0e9 ? 1000000000 : (iters < 64.0 ? 64 : (int)iters), tflops, ms);
}

extern "C" int cmaqchem_diag_phase_cycles(int device, unsigned long long* out, int reset)
{
#ifdef CHEM_PHASE_TIMING
    if (cudaSetDevice(device) != cudaSuccess) return -1;
    if (out && cudaMemcpyFromSymbol(out, g_chem_phase_cycles, 8 * sizeof(unsigned long long)) != cudaSuccess)
        return -1;
    if (reset) {
        const unsigned long long z[8] = {};
        if (cudaMemcpyToSymbol(g_chem_phase_cycles, z, sizeof(z)) != cudaSuccess) return -1;
    }
    return 0;
#else
    (void)device;
    (void)out;
    (void)reset;
    return -1;
#endif
}

namespace {

// `chains` independent FP64 chains per thread of one kind: 0 a*b+c (DFMA), 1 a*b, 2 a+c.
template <int CH, int OP>
__global__ void k_fp64_kind(int iters, double b, double c, double* sink)
{
    double a[CH];
#pragma unroll
    for (int k = 0; k < CH; ++k) a[k] = (double)(threadIdx.x + k) * 1.0e-3;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < CH; ++k) {
            if (OP == 0) a[k] = fma(a[k], b, c);
            else if (OP == 1) a[k] = a[k] * b;
            else a[k] = a[k] + c;
        }
    }
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < CH; ++k) t += a[k];
    if (t == -1.2345e300) sink[threadIdx.x] = t;
}

template <int CH>
cudaError_t launch_kind(int op, int blocks, int threads, int iters, double* sink)
{
    if (op == 0) k_fp64_kind<CH, 0><<<blocks, threads>>>(iters, 0.999999, 1.0e-7, sink);
    else if (op == 1) k_fp64_kind<CH, 1><<<blocks, threads>>>(iters, 0.999999, 1.0e-7, sink);
    else k_fp64_kind<CH, 2><<<blocks, threads>>>(iters, 0.999999, 1.0e-7, sink);
    return cudaGetLastError();
}

cudaError_t launch_chains(int chains, int op, int blocks, int threads, int iters, double* sink)
{
    switch (chains) {
    case 1: return launch_kind<1>(op, blocks, threads, iters, sink);
    case 2: return launch_kind<2>(op, blocks, threads, iters, sink);
    case 4: return launch_kind<4>(op, blocks, threads, iters, sink);
    case 8: return launch_kind<8>(op, blocks, threads, iters, sink);
    default: return launch_kind<16>(op, blocks, threads, iters, sink);
    }
}

}  // namespace

extern "C" int cmaqchem_diag_fp64_rate(int device, int op, int chains, int threads, int blocks_per_sm,
                                       double* ops_per_clk_per_sm, double* ms)
{
    if (op < 0 || op > 2 || (chains != 1 && chains != 2 && chains != 4 && chains != 8 && chains != 16)) return -1;
    if (threads < 32 || threads > 1024 || threads % 32 != 0 || blocks_per_sm < 1 || blocks_per_sm > 32) return -1;
    if (!ops_per_clk_per_sm) return -1;
    if (cudaSetDevice(device) != cudaSuccess) return -1;
    int nsm = 0, khz = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, device);
    double* sink = nullptr;
    if (cudaMalloc(&sink, 1024 * sizeof(double)) != cudaSuccess) return -1;
    const int blocks = nsm * blocks_per_sm, iters = 32768 / chains;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaError_t err = launch_chains(chains, op, blocks, threads, 64, sink);   // warm-up
    cudaEventRecord(e0);
    if (err == cudaSuccess) err = launch_chains(chains, op, blocks, threads, iters, sink);
    cudaEventRecord(e1);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float t = 0.0f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (err != cudaSuccess || !(t > 0.0f)) return -1;
    // lane operations per second / SMs / the device's maximum SM clock
    const double ops = (double)chains * iters * threads * blocks;
    *ops_per_clk_per_sm = ops / (t * 1.0e-3) / nsm / (khz * 1.0e3);
    if (ms) *ms = t;
    return 0;
}

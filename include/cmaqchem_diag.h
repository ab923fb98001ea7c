/*
 * cmaqchem_diag.h -- measurement helpers of libcmaqchem.so.  Not part of the CHEM
 * replacement (cmaqchem.h); used by the benchmark to measure the roofline peak.
 */
#ifndef CMAQCHEM_DIAG_H
#define CMAQCHEM_DIAG_H

#ifdef __cplusplus
extern "C" {
#endif

/* FP64 fused-multiply-add throughput of `device`, measured with independent FMA chains
 * on every SM: TFLOP/s (an FMA counts 2) and the kernel time in ms. */
int cmaqchem_diag_fp64_peak(int device, double* tflops, double* ms);

/* The same measurement with a kernel of about target_ms milliseconds (clamped to
 * 10-5000 ms), long enough for a clock sampler to record the SM clock it ran at. */
int cmaqchem_diag_fp64_peak_long(int device, double target_ms, double* tflops, double* ms);

/* Phase-timing builds (CHEM_PHASE_TIMING): clock cycles thread 0 of each block of the
 * lock-stepped work-queue kernel spent in each phase of a ROS3 attempt, summed over blocks:
 * out[0] f(Y) and the partial-derivative products, [1] Jacobian and LU, [2] stage 1 solve,
 * [3] stage 2's f, [4] stage 2 solve, [5] stage 3 solve, [6] error estimate, step update and
 * the refill of finished lanes; out[7] the number of block-attempts.  reset != 0 zeroes the
 * counters after reading.  Returns -1 in other builds. */
int cmaqchem_diag_phase_cycles(int device, unsigned long long* out, int reset);

/* FP64 lane operations per clock per SM, at the device's maximum SM clock, of `chains`
 * (1, 2, 4, 8 or 16) independent chains per thread of one kind (op 0: a*b+c, 1: a*b,
 * 2: a+c), `threads` per block and `blocks_per_sm` blocks per SM; ms: the kernel time.
 * The saturated value over the launch shapes is the FP64 pipe's rate. */
int cmaqchem_diag_fp64_rate(int device, int op, int chains, int threads, int blocks_per_sm,
                            double* ops_per_clk_per_sm, double* ms);

/* Clock cycles per link of a dependent FP64 FMA chain run by one warp with active_lanes
 * (1-32) lanes active: the latency a cell's sequential FP64 work pays per operation. */
int cmaqchem_diag_fp64_issue(int device, int active_lanes, double* cycles_per_instruction);

/* Scheduling knobs of a handle, for the autotuner: "night_pattern" (1: warps whose cells are
 * all dark use the smaller night LU pattern; 0: the day pattern always, same numbers),
 * "lockstep" (work-queue kernel: 0 free-running warps, 1 (default) the block's warps run
 * each step attempt together with barriers between its phases, 2 also between the
 * generated chunks), "block_warps" (2, 4 or 8 warps per block; 8 by default; 0 lockstep
 * needs 8), "blocks_per_sm" (cap on resident blocks per SM of the work-queue kernel,
 * 0 (default): as many as fit) and "adjoint_tape_mb" (device memory for the adjoint's
 * step tape; a synchronisation step whose tape is larger is processed in batches of
 * consecutive cells; 0 (default): the largest step's tape, halved until it fits) and
 * "ros3_dtmin_exp" (ROS3's minimum step is 10^value minutes; default -8, the reference's
 * DTMIN; a lower value lets tight tolerances pass the initial radical transient) and
 * "rconst_pass" (1, default when its arrays fit at set-up: the work-queue ROS3 call
 * evaluates CALC_RCONST of every cell in a pass of whole warps before the solver kernel,
 * which gathers the rates; 0: the solver kernel evaluates them in the lanes it refills;
 * same results) and
 * "queue_history" (0: clear the step counts the work queue is ordered by, so that the next
 * call is queued as a fresh run's first call; synchronises the device before and after) and
 * "host_chunks" (1-16, default 4: cmaqchem_step moves the grid in that many chunks of
 * consecutive cells so that copies overlap the integration of the previous chunk) and
 * "ebi_warp" (EBI solver: 1 (default) one cell per warp with its state in shared memory,
 * 0 one cell per lane; same results), "ebi_defer" (EBI: n > 0 runs one cell per lane and
 * hands the cells still iterating after n Backward-Euler iterations to the one-cell-per-warp
 * kernel, which integrates them from their inputs; default 100; 0: ebi_warp alone decides;
 * same results) and
 * "gear_warp" (SMVGEAR: 1 (default) one cell per warp with its workspace in shared memory,
 * 0 one cell per lane; same results). */
struct cmaqchem_handle;
int cmaqchem_diag_set_tuning(struct cmaqchem_handle* h, const char* key, int value);

#ifdef __cplusplus
}
#endif
#endif

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

#ifdef __cplusplus
}
#endif
#endif

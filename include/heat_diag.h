/*
 * heat_diag.h -- diagnostics of the GB300 heat solver library.
 *
 * No counterpart in the reference: the reference measures machine rates with
 * separate microbenchmarks (Kernel-Test/, Bandwidth_Measurements/).  These
 * calls give the FP64 execution-pipe rate of the current device, the ceiling
 * the FP64 stencil forms are held against next to the HBM roofline.
 */
#ifndef HEAT_DIAG_H
#define HEAT_DIAG_H

#ifdef __cplusplus
extern "C" {
#endif

/* Measured FP64 fused-multiply-add rate of the current device in giga
 * operations per second (one FMA counted as one operation), from eight
 * independent dependency chains per thread over all SMs, timed with CUDA
 * events.  Takes a few milliseconds.  Returns HEAT_OK or a HEAT_E* code.   */
int heat_diag_fp64_rate(double *gops_out);

#ifdef __cplusplus
}
#endif

#endif /* HEAT_DIAG_H */

/*
 * heat_diag.h -- diagnostics of the GB300 heat solver library.
 *
 * No counterpart in the reference: the reference measures machine rates with
 * separate microbenchmarks (Kernel-Test/, Bandwidth_Measurements/).  These
 * calls give the FP64 execution-pipe rate of the current device, the ceiling
 * the FP64 stencil forms are held against next to the HBM roofline, and check
 * the bounded device-side wait behind HEAT_ETIMEOUT.
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

/* Difference of the current fields of two contexts of the same grid, on the
 * device: max |a - b| and ||a - b||_2 / ||b||_2 over all points (b is the
 * reference side, as compare.py:47-76 of the reference's verify pipeline
 * treats its first argument).  Works across precision forms (an FP32C field
 * is widened to FP64 first).  Synchronises both contexts' streams.         */
struct heat_ctx;
int heat_diag_field_diff(struct heat_ctx *a, struct heat_ctx *b, double *max_abs,
                         double *rel_l2);

/* Bounded-wait check.  One block waits, with the same bounded mbarrier wait
 * the TMA kernels use (each attempt a try_wait of up to ~2 us), capped at
 * `attempts` tries (1 .. 2^22, the kernels' own limit; HEAT_EINVAL otherwise),
 * on an mbarrier that nothing arrives at.  The wait must give
 * up: *timed_out = 1 and the call returns HEAT_ETIMEOUT, the status a TMA
 * kernel's context reports when one of its waits runs out, and the device
 * stays usable.  HEAT_OK with *timed_out = 0 would mean the wait completed. */
int heat_diag_wait_timeout(unsigned attempts, int *timed_out);

/* Failure path of the product kernel itself.  Queues, on the context's
 * stream, one launch of the FP32C two-step kernel (the kernel heat_step uses
 * for HEAT_FP32C contexts) with its wait limit set to 0 attempts: its first
 * mbarrier wait gives up at once, it sets the context's error flag, waits
 * (with the full bounded wait) for its own loads in flight and returns
 * without writing any point.  The context's fields and step count are
 * unchanged.  The next call that synchronises the context -- heat_sync,
 * heat_norm, heat_get_field, or heat_batch_run of a batch holding it --
 * returns HEAT_ETIMEOUT, once.  HEAT_ESTATE for a context that does not step
 * with the two-step kernel (HEAT_FP64, a source term, HEAT_NO_TEMPORAL).    */
int heat_diag_fp32c_timeout(struct heat_ctx *c);

/* The same for the default FP64 form's TMA-staged launch (the kernel
 * heat_step uses for HEAT_FP64 contexts, with or without a source term): one
 * launch with its wait limit at 0 attempts gives up at its first wait in both
 * warpgroups, flags the context and returns without writing a point; the next
 * synchronising call reports HEAT_ETIMEOUT once.  HEAT_ESTATE for a context
 * that does not step with that launch (HEAT_BITEXACT, HEAT_NAIVE,
 * HEAT_HWFP64, HEAT_FP32C).                                                  */
int heat_diag_fp64_timeout(struct heat_ctx *c);

#ifdef __cplusplus
}
#endif

#endif /* HEAT_DIAG_H */

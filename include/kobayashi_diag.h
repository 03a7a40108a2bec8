/*
 * kobayashi_diag.h -- diagnostic entry points of libkobayashi_gpu.so.
 *
 * Not part of the reference's surface (jklae/CrystalGrowth has no
 * counterpart): they let tests check the device build of kg_math.h against
 * the host build, and let the benchmark measure the FP64 pipe it is bound by.
 */
#ifndef KOBAYASHI_DIAG_H
#define KOBAYASHI_DIAG_H
#include "kobayashi_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define KG_FN_ATAN 0  /* y = kg_atan(x) */
#define KG_FN_SIN 1   /* y = sin part of kg_sincos(x) */
#define KG_FN_COS 2   /* y = cos part of kg_sincos(x) */
#define KG_FN_DIV 4   /* y = x / b, the GPU's own IEEE division */
#define KG_FN_IDIV 5  /* y = kg_idiv(x, b): x / b through the integer-pipe path */
#define KG_FN_TWICE_PLUS 10 /* y[i] = kg_twice_plus(x[i], x[n-1-i]): 2 x + y in one FMA */
#define KG_FN_MUL2_ADD 11   /* y[i] = 2 x[i] + x[n-1-i], two hardware roundings */
#define KG_FN_GDIV 13       /* y[i] = kg_gdiv(x[i], x[n-1-i]): integer-pipe division, any divisor */
#define KG_FN_DIV_PAIR 14   /* y[i] = x[i] / x[n-1-i], the GPU's own IEEE division */

/* Evaluates function `fn` on n host values on the current device (synchronous). */
KG_API int kg_diag_eval(int fn, const double* x, double* y, long long n, double b);

/* Runs the batched kernel's bounded grid barrier on `blocks` CTAs while it
 * waits for one CTA more: every wait must give up after max_polls polls.
 * *timed_out = 1 when the error flag was raised (the expected outcome). */
KG_API int kg_diag_barrier_timeout(int blocks, long long max_polls, int* timed_out);

/* Waits, with the strip kernel's bounded wait, on an mbarrier that no bulk
 * copy completes: the wait must give up (about half a second) and raise the
 * flag.  *timed_out = 1 is the expected outcome. */
KG_API int kg_diag_mbar_timeout(int* timed_out);

/* Host-side fault injection: raises the handle's device error flag exactly as
 * a step kernel whose bounded bulk-copy wait ran out does (nothing runs on the
 * GPU, nothing faults).  The next kg_sync / kg_get_fields reports
 * KG_ERR_TIMEOUT, and kg_step then refuses until the state is replaced. */
KG_API int kg_diag_inject_timeout(kg_sim* h);

/* The same for a batch: raises the grid barrier's error flag as a persistent CTA whose wait ran out
 * does, and reads it back as kg_batch_step does (returns KG_ERR_TIMEOUT).  kg_batch_step then refuses
 * until every instance's state has been replaced. */
struct kg_batch;
KG_API int kg_diag_batch_inject_timeout(struct kg_batch* b);

/* FP64 pipe probe on the current device: every thread runs `chains` (4, 8 or
 * 16) independent dependency chains of one FP64 operation -- op 0: FMA,
 * 1: add, 2: multiply, 3: two adds per multiply -- in ctas_per_sm CTAs of
 * `threads` threads (64..512) on every SM.  Returns lane-operations per
 * second (CUDA events) and, if lanes_per_sm_clock is not NULL, lane-operations
 * per SM per SM clock cycle (from clock64 stamps of every CTA, independent of
 * the clock frequency). */
KG_API int kg_diag_fp64_probe(int op, int chains, int ctas_per_sm, int threads, double* lanes_per_s,
                              double* lanes_per_sm_clock);

/* The highest FP64 lane-operation rate of kg_diag_fp64_probe over ops 0..3, 8 and 16 chains and 2, 4
 * and 8 CTAs of 256 threads per SM. */
KG_API int kg_diag_fp64_peak(double* ops_per_s);

/* Copies `bytes` (a multiple of 16; both pointers 16-byte aligned) from src to dst with a kernel's
 * loads and stores instead of a copy engine, enqueued on `stream` (a cudaStream_t).  Either end may
 * be device memory or page-locked host memory; anything else is refused with KG_ERR_INVALID.  Used to
 * compare the two ways of moving a field to the host. */
KG_API int kg_diag_copy(void* dst, const void* src, long long bytes, void* stream);

#ifdef __cplusplus
}
#endif
#endif

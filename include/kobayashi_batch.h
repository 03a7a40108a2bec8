/*
 * kobayashi_batch.h -- batched ensemble of independent Kobayashi grids.
 *
 * No counterpart in the reference (jklae/CrystalGrowth runs one grid per
 * process, src/main.cpp:18): hundreds of instances of uneven sizes, each with
 * its own kg_params, advance together in one launch per step (or one
 * persistent launch per chunk).  Every instance computes exactly what a
 * kg_sim of the same size and parameters computes.  Conventions as in
 * kobayashi_gpu.h (int status, kg_last_error, one stream per handle).
 */
#ifndef KOBAYASHI_BATCH_H
#define KOBAYASHI_BATCH_H
#include "kobayashi_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define KG_BATCH_LAUNCH 0      /* one kernel per step over all strips, CUDA-graph chunks */
#define KG_BATCH_MAX_STREAMS 16
#define KG_BATCH_PERSISTENT 1  /* one cooperative kernel per chunk, bounded grid barrier between steps */

typedef struct kg_batch_tuning {
    int nt;     /* threads per strip CTA: 32, 64, 128 or 256 (strip width nt - 2 columns) */
    int bh;     /* rows per strip */
    int mode;   /* KG_BATCH_LAUNCH or KG_BATCH_PERSISTENT */
    int chunk;  /* steps per graph (launch mode) or per persistent launch */
    int streams; /* launch mode: instances split into this many groups of about equal cells, each
                    group stepped on its own stream (1..KG_BATCH_MAX_STREAMS); 1 in persistent mode */
    int tblock; /* temporal blocking: time steps per pass over HBM, 1 or 2 (2 needs nt <= 128; the strip
                   is then nt - 6 columns wide and the halo 4 columns and 3 rows of phi per side) */
} kg_batch_tuning;

typedef struct kg_batch kg_batch;

/* n instances; instance k has size nx[k] x ny[k] and parameters params[k].
 * Every instance starts from the reference's 5-cell nucleus at its centre. */
KG_API int kg_batch_create(int n, const int* nx, const int* ny, const kg_params* params, kg_batch** out);
KG_API int kg_batch_destroy(kg_batch* b);
/* zero instance k's fields and seed disks (as kg_seed_disks) */
KG_API int kg_batch_seed_disks(kg_batch* b, int k, int n, const int* cx, const int* cy, const int* r);
/* advance every instance by nsteps */
KG_API int kg_batch_step(kg_batch* b, long long nsteps);
KG_API int kg_batch_sync(kg_batch* b);
KG_API int kg_batch_get_fields(kg_batch* b, int k, double* phi, double* T, double* theta);
KG_API int kg_batch_set_fields(kg_batch* b, int k, const double* phi, const double* T, const double* theta);
/* instance count, total cells, steps taken, strips in the work list */
KG_API int kg_batch_get_info(const kg_batch* b, int* n, long long* cells, long long* steps, int* nwork);
KG_API int kg_batch_set_tuning(kg_batch* b, const kg_batch_tuning* t);
KG_API int kg_batch_get_tuning(const kg_batch* b, kg_batch_tuning* t);
/* Times trial_steps steps of every (nt, bh, mode/streams, tblock) candidate
 * on this batch -- 150 candidates: nt 32/64/128, bh 4/8/16/32/64, launch mode on
 * 1/4/8/16 streams or persistent, 1 or 2 steps per pass -- installs the
 * fastest (keeping the current chunk) and restores the state it started from.
 * best / best_ms_per_step may be NULL. */
KG_API int kg_batch_autotune(kg_batch* b, int trial_steps, kg_batch_tuning* best, double* best_ms_per_step);
KG_API int kg_batch_get_stream(kg_batch* b, void** stream);

#ifdef __cplusplus
}
#endif
#endif

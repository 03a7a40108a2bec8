/*
 * kobayashi_gpu.h -- C ABI of the GB300 Kobayashi phase-field library
 * (libkobayashi_gpu.so).
 *
 * This is the drop-in boundary for the simulation core of jklae/CrystalGrowth.
 * The reference has no FFI: its boundary is the C++ class Kobayashi behind
 * DXViewer's ISimulation interface (src/Kobayashi.h:32-68).  Each entry point
 * below names the reference member it replaces.  include/kobayashi.hpp wraps
 * this ABI in a C++ class with the reference's method names.
 *
 * Conventions
 *   - Every function returns an int status: KG_OK (0) or a negative KG_ERR_*;
 *     nothing aborts or throws.  kg_last_error() returns a message for the
 *     calling thread's most recent failure.
 *   - Plain pointers and sizes only.  Host buffers belong to the caller; device
 *     memory belongs to the library.  Fields are row-major FP64, index
 *     i + nx*j (src/Kobayashi.h:91).
 *   - One handle = one CUDA stream on the current device; a handle is not
 *     thread-safe (the reference is single-threaded too).  kg_step and
 *     kg_update only enqueue work; calls that return host data synchronise.
 *   - Arithmetic is IEEE FP64 with the reference's operation order; atan, sin
 *     and cos are the library's own faithful implementations (kg_math.h), the
 *     same on the CPU oracle and the GPU.
 */
#ifndef KOBAYASHI_GPU_H
#define KOBAYASHI_GPU_H

#if defined(__GNUC__)
#define KG_API __attribute__((visibility("default")))
#else
#define KG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define KG_OK 0
#define KG_ERR_INVALID (-1)  /* bad argument (null pointer, size, parameter out of range) */
#define KG_ERR_CUDA (-2)     /* CUDA runtime error; see kg_last_error() */
#define KG_ERR_NOMEM (-3)    /* device or host allocation failed */
#define KG_ERR_TIMEOUT (-4)  /* a bounded device-side wait ran out (batched kernel) */

/* Model parameters.  Field meaning and defaults follow the reference's members
 * (src/Kobayashi.h:94-105, defaults src/Kobayashi.cpp:61-63,76-84).  theta0 (the
 * preferred growth angle) is an extension: eps = eps_bar (1 + delta cos(aniso
 * (theta - theta0))); theta0 = 0 reproduces the reference bit for bit. */
typedef struct kg_params {
    double dx, dy, dt;
    double tau, eps_bar, mu, K, delta, aniso, alpha, gamma, teq;
    double theta0;
} kg_params;

typedef struct kg_sim kg_sim;

/* Reference defaults: _parameterInit + the ctor's _dx/_dy/_dt
 * (src/Kobayashi.cpp:61-63,76-84); mu is kept although the step never reads it. */
KG_API int kg_params_default(kg_params* p, double dt);

/* Checks a parameter set: finite values, dx, dy, dt, tau > 0 (and within
 * [2^-100, 2^100]), eps_bar > 0, |theta0| <= 100, aniso an integer-valued
 * value in [1, 64]. */
KG_API int kg_params_validate(const kg_params* p);

/* The reference's parameter sliders (src/Kobayashi.cpp:12-59, 555-618): nine
 * integer positions in the order tau, eps_bar, mu, K, delta, aniso, alpha,
 * gamma, teq; value = (float)position * ratio as the slider's thumb-track
 * handler computes it (ratios 1e-4, 1e-3, 0.1, 0.1, 0.01, 1, 0.1, 1, 0.1).
 * kg_slider_range gives a slider's integer range and default position. */
#define KG_SLIDERS 9
KG_API int kg_slider_range(int which, int* lo, int* hi, int* def);
KG_API int kg_params_from_sliders(const int* pos, double dt, kg_params* p);

/* Kobayashi(int x, int y, float timeStep) + _vectorInit (src/Kobayashi.cpp:7-67,
 * 98-123): allocates the grid on the current device, zeroes phi, T and theta
 * and seeds the reference's 5-cell nucleus at (nx/2, ny/2).  nx, ny >= 1
 * (the nucleus wraps periodically; for nx, ny >= 3 it is the reference's). */
KG_API int kg_create(int nx, int ny, const kg_params* p, kg_sim** out);

/* ~Kobayashi (src/Kobayashi.cpp:69-71) */
KG_API int kg_destroy(kg_sim* h);

/* iResetSimulationState (src/Kobayashi.cpp:241-249) without the viewer calls:
 * _vectorInit again, step and frame counters back to 0; parameters persist. */
KG_API int kg_reset(kg_sim* h);

/* Generalised nucleus: zero all fields and set phi = 1 on n disks
 * {(i,j): di^2 + dj^2 <= r^2} around (cx[k], cy[k]), distances measured on the
 * periodic grid.  The reference's 5-cell nucleus (src/Kobayashi.cpp:116-123) is
 * the disk of radius 1.  Counters back to 0. */
KG_API int kg_seed_disks(kg_sim* h, int n, const int* cx, const int* cy, const int* r);

/* Parameter mutation (the reference mutates its float& slider targets,
 * src/Kobayashi.cpp:579-611). */
KG_API int kg_set_params(kg_sim* h, const kg_params* p);
KG_API int kg_get_params(const kg_sim* h, kg_params* p);

/* nsteps explicit Euler steps (_computeGradientLaplacian + _evolution,
 * src/Kobayashi.cpp:125-221), enqueued on the handle's stream, in CUDA-graph
 * chunks (kg_set_graph_chunk). */
KG_API int kg_step(kg_sim* h, long long nsteps);

/* iUpdate (src/Kobayashi.cpp:227-239): 10 steps and frame += 1. */
KG_API int kg_update(kg_sim* h);

/* Waits for the handle's stream; reports any asynchronous CUDA error. */
KG_API int kg_sync(kg_sim* h);

/* Host copies of the current state (synchronous); any pointer may be NULL. */
KG_API int kg_get_fields(kg_sim* h, double* phi, double* T, double* theta);
/* Overwrite the current state from host buffers (synchronous); NULL leaves a field as is. */
KG_API int kg_set_fields(kg_sim* h, const double* phi, const double* T, const double* theta);

/* iGetObjectCount (src/Kobayashi.cpp:363-366) */
KG_API int kg_get_size(const kg_sim* h, int* nx, int* ny);
/* steps taken since create/reset; frames = iUpdate calls (_simFrame, src/Kobayashi.h:81) */
KG_API int kg_get_counters(const kg_sim* h, long long* steps, long long* frames);

/* Device pointers of the current state (valid until the next step or reset)
 * and the handle's cudaStream_t, for consumers that stay on the GPU. */
KG_API int kg_device_fields(kg_sim* h, double** phi, double** T, double** theta);
KG_API int kg_get_stream(kg_sim* h, void** stream);

/* No counterpart in the reference.  For callers that cannot allocate device
 * memory when they step the model -- a viewer or game loop that owns the GPU
 * memory budget and allows no allocation inside a frame, a host recording its
 * work while a CUDA stream is being captured (cudaMalloc/cudaFree are illegal
 * then), a real-time loop that cannot afford cudaFree's device-wide
 * synchronisation: advances the caller's own device buffers phi, T, theta
 * (nx*ny FP64 each) in place by nsteps steps, enqueued on `stream`
 * (a cudaStream_t; NULL = the legacy default stream), and allocates nothing.
 * The second copy of the state lives in a fixed device array inside the
 * library (6 MiB per GPU that loads the library, held until exit), so grids
 * are limited to 262,144 cells (512 x 512); larger ones are refused with
 * KG_ERR_INVALID.  The first call on each device looks up that array's device
 * address and keeps it, and loads the step kernel: make that first call (any
 * nsteps, 0 included) before any stream capture.  The step uses per-lane row
 * loads only (no bulk copies, hence no bounded wait that could time out);
 * its results are those of kg_step, its speed may differ.  All
 * calls on a device share the array, so calls that overlap on the GPU (e.g. on
 * two streams at once) race and corrupt each other; nothing in the array needs
 * to start at zero, each call overwrites what it reads.  Returns once the work
 * is enqueued; synchronise the stream before reading the buffers. */
KG_API int kg_step_noalloc(int nx, int ny, const kg_params* p, double* phi, double* T, double* theta,
                           long long nsteps, void* stream);

/* Strip shape of the fused step: nt threads per CTA (32, 64, 128 or 256; the
 * strip is nt - 2 columns wide) and bh rows per strip.  kg_create picks 256 x 24,
 * 128 x 32 or 128 x 16 where that still gives at least 8,000 CTAs, else the
 * largest strips that give about 30,000.  Results do not depend on the shape;
 * two steps per pass (kg_set_tblock) use strips of at most 128 threads. */
KG_API int kg_set_tile(kg_sim* h, int nt, int bh);
KG_API int kg_get_tile(const kg_sim* h, int* nt, int* bh);

/* Temporal blocking factor k of kg_step: 1 (default) advances the grid one
 * step per pass over HBM; 2 advances it two steps per pass, holding the
 * intermediate step in shared memory (a halo of 4 columns and 3 rows of phi
 * each side, recomputed).  Results are identical for k = 1 and 2; k = 2 halves
 * the HBM traffic per step and costs extra FP64 work on the halo.  An odd
 * remainder of steps takes one k = 1 launch.  No counterpart in the reference
 * (it sweeps the whole grid twice per step, src/Kobayashi.cpp:227-239). */
KG_API int kg_set_tblock(kg_sim* h, int k);
KG_API int kg_get_tblock(const kg_sim* h, int* k);

/* Steps per captured CUDA graph used by kg_step (default 100; 0 = no graphs). */
KG_API int kg_set_graph_chunk(kg_sim* h, int chunk);

/* Snapshots (no counterpart in the reference, which keeps its state in memory
 * only): a 4096-byte JSON header (format, version, nx, ny, steps, frames,
 * params) followed by phi, T, theta as little-endian FP64 arrays.  kg_load
 * needs a handle of the same size and restores parameters and counters. */
KG_API int kg_save(kg_sim* h, const char* path);
KG_API int kg_load(kg_sim* h, const char* path);

/* Message of the calling thread's last failure ("" if none). */
KG_API const char* kg_last_error(void);

/* Build/version string of the library. */
KG_API const char* kg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* KOBAYASHI_GPU_H */

/*
 * kg_common.h -- host-side helpers shared by the library's translation units:
 * error reporting, parameter validation and the preparation of the
 * per-parameter-set constants (KgDev) that the kernels read.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include "kobayashi_gpu.h"
#include "kg_device.cuh"

/* records a message for kg_last_error() and returns `code` */
int kg_fail(int code, const char* fmt, ...);

/* maps a CUDA error to KG_ERR_CUDA with a message naming `what` */
int kg_cuda_fail(cudaError_t e, const char* what);

#define KG_CUDA(call)                                              \
    do {                                                           \
        cudaError_t kg_e_ = (call);                                \
        if (kg_e_ != cudaSuccess)                                  \
            return kg_cuda_fail(kg_e_, #call);                     \
    } while (0)

/* A host<->device copy of `bytes`, enqueued on stream s as consecutive cudaMemcpyAsync calls of at
 * most 64 MiB each.  Measured on GB300 (Grace host link, pinned buffers): 64 MiB pieces held 186-192
 * GB/s in every run, while single 512 MiB copies issued right after long compute phases fell to
 * 6-60 GB/s. */
cudaError_t kg_copy_pieces(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s);

/* A copy between the device and caller-owned host memory, enqueued on stream s.  Page-locked host
 * memory (16-byte aligned ends, a multiple of 16 bytes) is moved by a copy kernel whose loads and
 * stores cross the host link themselves; anything else by the copy engine, in kg_copy_pieces.
 * Measured on GB300 after a minute of sustained stepping: copy-engine downloads into page-locked
 * memory ran at 14-20 GB/s (and uploads at times at 4-55 GB/s), the copy kernel at 118-192 GB/s. */
cudaError_t kg_copy_host(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s);

/* fills the derived constants of one parameter set; returns KG_OK or KG_ERR_INVALID */
int kg_prepare(const kg_params* p, KgDev* d);

/* strip width (threads) and height for a single nx x ny grid on the current device */
void kg_pick_tile(int nx, int ny, int* nt, int* bh);

/* phi -> RGBA float32 for nx*ny cells in the given order (kg_color.cu) */
int kg_color_launch(const double* phi, float* rgba, int nx, int ny, int order, cudaStream_t s);

/* zero fields and seed disks on the device (kg_common.cu) */
int kg_seed_device(double* phi, double* t, double* theta, int nx, int ny, int n, const int* cx, const int* cy,
                   const int* r, cudaStream_t s);

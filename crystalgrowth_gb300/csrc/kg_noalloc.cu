/*
 * kg_noalloc.cu -- the fused step on caller-owned device buffers, with no
 * device allocation at all.
 *
 * Some callers cannot allocate device memory when they want to step the
 * simulation: a viewer or game loop that owns the GPU's memory budget and
 * forbids allocations inside a frame, a host that records its per-frame work
 * while a CUDA stream is being captured (cudaMalloc and cudaFree are not
 * allowed then), or a real-time loop that cannot afford the device-wide
 * synchronisation cudaFree implies.  kg_step_noalloc serves them: the caller
 * passes its own phi, T and theta device buffers and a stream, and the second
 * ping-pong copy of the state that the step needs lives in a fixed,
 * library-owned device array instead of in cudaMalloc'd memory.
 *
 * Limit: grids of at most KG_NOALLOC_MAX_CELLS cells (512 x 512).  The array
 * (3 fields x 2^18 cells x 8 bytes = 6 MiB) is part of the library's device
 * image, so every GPU that loads the library holds it until the process exits.
 *
 * The step is the same fused strip as kg_step's, with per-lane row loads only
 * (no bulk copies, so it has no bounded wait that could time out) and a fixed
 * strip shape: results are identical to kg_step's, speed may differ.
 */
#include <mutex>
#include "kg_common.h"

#define KG_NOALLOC_MAX_CELLS (1 << 18)

/* the scratch copy of (phi, T, theta): shared by every call on a device */
static __device__ __align__(256) double kg_noalloc_scratch[3 * KG_NOALLOC_MAX_CELLS];

template <int NT>
__global__ void __launch_bounds__(NT) kg_noalloc_step_kernel(const __grid_constant__ KgDev P, int nx, int ny, int bh,
                                                             const double* __restrict__ phi_in,
                                                             const double* __restrict__ t_in,
                                                             const double* __restrict__ th_in,
                                                             double* __restrict__ phi_out, double* __restrict__ t_out,
                                                             double* __restrict__ th_out)
{
    __shared__ KgSmem<NT> sm;
    kg_strip<NT>(P, nx, ny, phi_in, t_in, th_in, phi_out, t_out, th_out, blockIdx.x * (NT - 2), blockIdx.y * bh, bh,
                 sm);
}

/* Device address of the scratch array on the current device.  Host code
 * cannot use kg_noalloc_scratch directly: on the host that name only stands
 * for the symbol.  The address is looked up once per device, with that device
 * current, and kept; the same first call also makes the runtime load the step
 * kernel (with lazy module loading it would otherwise load at its first
 * launch), so a first call with nsteps = 0 prepares the device completely. */
static int noalloc_scratch(double** out)
{
    static std::mutex mu;
    static double* addr[128] = {};
    int dev = 0;
    KG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128)
        return kg_fail(KG_ERR_INVALID, "kg_step_noalloc: device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, kg_noalloc_scratch);
        if (e != cudaSuccess)
            return kg_cuda_fail(e, "kg_step_noalloc: cudaGetSymbolAddress of the scratch array");
        cudaFuncAttributes fa;
        e = cudaFuncGetAttributes(&fa, kg_noalloc_step_kernel<128>);
        if (e != cudaSuccess)
            return kg_cuda_fail(e, "kg_step_noalloc: loading the step kernel");
        addr[dev] = (double*)p;
    }
    *out = addr[dev];
    return KG_OK;
}

extern "C" int kg_step_noalloc(int nx, int ny, const kg_params* p, double* phi, double* T, double* theta,
                               long long nsteps, void* stream)
{
    if (!phi || !T || !theta)
        return kg_fail(KG_ERR_INVALID, "kg_step_noalloc: phi, T and theta must be device pointers");
    if (nx < 1 || ny < 1 || nsteps < 0)
        return kg_fail(KG_ERR_INVALID, "kg_step_noalloc: bad grid size or step count");
    if ((long long)nx * ny > KG_NOALLOC_MAX_CELLS)
        return kg_fail(KG_ERR_INVALID,
                       "kg_step_noalloc: a %d x %d grid (%lld cells) exceeds the no-allocation limit of %d cells "
                       "(512 x 512); use kg_create/kg_step for larger grids",
                       nx, ny, (long long)nx * ny, KG_NOALLOC_MAX_CELLS);
    KgDev dev;
    int rc = kg_prepare(p, &dev);
    if (rc)
        return rc;
    double* s = nullptr;
    rc = noalloc_scratch(&s);
    if (rc)
        return rc;
    if (nsteps == 0)
        return KG_OK;
    const size_t N = (size_t)nx * ny;
    cudaStream_t st = (cudaStream_t)stream;
    double* A[3] = {phi, T, theta};
    double* B[3] = {s, s + N, s + 2 * N};
    const int NT = 128;
    const int bh = ny < 64 ? ny : 64;
    dim3 grid((nx + NT - 3) / (NT - 2), (ny + bh - 1) / bh);
    for (long long k = 0; k < nsteps; k++) {
        double* const* from = (k & 1) ? B : A;
        double* const* to = (k & 1) ? A : B;
        kg_noalloc_step_kernel<NT><<<grid, NT, 0, st>>>(dev, nx, ny, bh, from[0], from[1], from[2], to[0], to[1],
                                                        to[2]);
    }
    KG_CUDA(cudaGetLastError());
    if (nsteps & 1)
        for (int f = 0; f < 3; f++)
            KG_CUDA(cudaMemcpyAsync(A[f], B[f], N * sizeof(double), cudaMemcpyDeviceToDevice, st));
    return KG_OK;
}

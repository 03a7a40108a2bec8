/*
 * kg_diag.cu -- diagnostic kernels: device evaluation of kg_math.h for the
 * host-vs-device tests, and an FP64 FMA throughput probe.
 */
#include "kg_common.h"
#include <stdlib.h>
#include <string.h>
#include "kobayashi_diag.h"

__global__ void kg_diag_eval_kernel(int fn, const double* __restrict__ x, double* __restrict__ y, long long n, double b,
                                    kg_idivc ic)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double v = x[i], r = 0.0;
        if (fn == KG_FN_ATAN) {
            r = kg_atan(v);
        } else if (fn == KG_FN_SIN || fn == KG_FN_COS) {
            double s, c;
            kg_sincos(v, &s, &c);
            r = fn == KG_FN_SIN ? s : c;
        } else if (fn == KG_FN_IDIV) {
            r = kg_idiv(v, &ic);
        } else if (fn == KG_FN_DIV) {
            r = v / b;
        } else if (fn == KG_FN_TWICE_PLUS) {
            r = kg_twice_plus(v, x[n - 1 - i]);
        } else if (fn == KG_FN_MUL2_ADD) {
            r = __dadd_rn(__dmul_rn(2.0, v), x[n - 1 - i]);
        } else if (fn == KG_FN_GDIV) {
            r = kg_gdiv(v, x[n - 1 - i]);
        } else if (fn == KG_FN_DIV_PAIR) {
            r = v / x[n - 1 - i];
        }
        y[i] = r;
    }
}

extern "C" int kg_diag_eval(int fn, const double* x, double* y, long long n, double b)
{
    const bool known = fn == KG_FN_ATAN || fn == KG_FN_SIN || fn == KG_FN_COS || fn == KG_FN_DIV ||
                       fn == KG_FN_IDIV || fn == KG_FN_TWICE_PLUS || fn == KG_FN_MUL2_ADD || fn == KG_FN_GDIV ||
                       fn == KG_FN_DIV_PAIR;
    if (!known || n < 0 || (n > 0 && (!x || !y)))
        return kg_fail(KG_ERR_INVALID, "kg_diag_eval: bad arguments");
    kg_idivc ic;
    memset(&ic, 0, sizeof ic);
    if ((fn == KG_FN_DIV || fn == KG_FN_IDIV) && kg_idiv_prepare(b, &ic))
        return kg_fail(KG_ERR_INVALID, "kg_diag_eval: divisor outside [2^-100, 2^100]");
    if (n == 0)
        return KG_OK;
    double* d = nullptr;
    KG_CUDA(cudaMalloc(&d, sizeof(double) * 2 * (size_t)n));
    cudaError_t e = cudaMemcpy(d, x, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        int blocks = (int)((n + 255) / 256 < 152 * 8 ? (n + 255) / 256 : 152 * 8);
        kg_diag_eval_kernel<<<blocks, 256>>>(fn, d, d + n, n, b, ic);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpy(y, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess)
        return kg_cuda_fail(e, "kg_diag_eval");
    return KG_OK;
}

/*
 * FP64 pipe probe.  Every thread runs CHAINS independent dependency chains of
 * one FP64 operation (OP 0: FMA, 1: add, 2: multiply, 3: two adds and one
 * multiply, the step's own mix), KG_PEAK_ITERS times.  Thread 0 of each CTA
 * records its SM and the SM clock at its start and end, so the rate per SM
 * clock comes out without knowing the clock frequency.
 */
#define KG_PEAK_ITERS 4096

template <int OP, int CHAINS>
__global__ void kg_diag_fp64_kernel(double* out, double s, long long* stamps)
{
    long long t0 = clock64();
    double v[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; c++)
        v[c] = 1.0 + 1e-3 * (threadIdx.x + c);
    for (int i = 0; i < KG_PEAK_ITERS; i++) {
#pragma unroll
        for (int c = 0; c < CHAINS; c++) {
            if constexpr (OP == 0)
                v[c] = __fma_rn(v[c], s, 0.5);
            else if constexpr (OP == 1)
                v[c] = __dadd_rn(v[c], s);
            else if constexpr (OP == 2)
                v[c] = __dmul_rn(v[c], s);
            else
                v[c] = (c % 3 == 2) ? __dmul_rn(v[c], s) : __dadd_rn(v[c], s);
        }
    }
    double acc = 0;
#pragma unroll
    for (int c = 0; c < CHAINS; c++)
        acc += v[c];
    if (acc == 12345.678)
        out[0] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned smid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        stamps[3 * blockIdx.x] = smid;
        stamps[3 * blockIdx.x + 1] = t0;
        stamps[3 * blockIdx.x + 2] = clock64();
    }
}

typedef void (*kg_fp64_kernel_t)(double*, double, long long*);

static kg_fp64_kernel_t fp64_kernel(int op, int chains)
{
#define KG_K(o)                                                                       \
    (chains == 4 ? kg_diag_fp64_kernel<o, 4> : chains == 8 ? kg_diag_fp64_kernel<o, 8> \
                                                            : kg_diag_fp64_kernel<o, 16>)
    switch (op) {
    case 0: return KG_K(0);
    case 1: return KG_K(1);
    case 2: return KG_K(2);
    default: return KG_K(3);
    }
#undef KG_K
}

extern "C" int kg_diag_fp64_probe(int op, int chains, int ctas_per_sm, int threads, double* lanes_per_s,
                                  double* lanes_per_sm_clock)
{
    if (op < 0 || op > 3 || (chains != 4 && chains != 8 && chains != 16) || ctas_per_sm < 1 || ctas_per_sm > 16 ||
        (threads != 64 && threads != 128 && threads != 256 && threads != 512) || !lanes_per_s)
        return kg_fail(KG_ERR_INVALID, "kg_diag_fp64_probe: bad arguments");
    int dev = 0, sms = 0;
    KG_CUDA(cudaGetDevice(&dev));
    KG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * ctas_per_sm;
    kg_fp64_kernel_t k = fp64_kernel(op, chains);
    int fit = 0;
    KG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, k, threads, 0));
    if (fit < ctas_per_sm)
        return kg_fail(KG_ERR_INVALID, "kg_diag_fp64_probe: only %d CTAs of %d threads fit on an SM", fit, threads);
    double* out = nullptr;
    long long* stamps = nullptr;
    KG_CUDA(cudaMalloc(&out, sizeof(double)));
    cudaError_t e = cudaMalloc(&stamps, sizeof(long long) * 3 * blocks);
    cudaEvent_t a = nullptr, b = nullptr;
    if (e == cudaSuccess)
        e = cudaEventCreate(&a);
    if (e == cudaSuccess)
        e = cudaEventCreate(&b);
    float best = 1e30f;
    double best_clk = 0;
    long long* h = (long long*)malloc(sizeof(long long) * 3 * blocks);
    double* sm_lo = (double*)malloc(sizeof(double) * 3 * sms); /* per SM: first start, last end, CTAs */
    if (!h || !sm_lo)
        e = cudaErrorMemoryAllocation;
    for (int r = 0; r < 4 && e == cudaSuccess; r++) {
        cudaEventRecord(a);
        k<<<blocks, threads>>>(out, 0.999, stamps);
        cudaEventRecord(b);
        e = cudaEventSynchronize(b);
        if (e == cudaSuccess)
            e = cudaGetLastError();
        if (e != cudaSuccess || r == 0)
            continue; /* the first launch warms up */
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        e = cudaMemcpy(h, stamps, sizeof(long long) * 3 * blocks, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess)
            break;
        /* per SM: the lanes its CTAs ran between the first start and the last end (clock64 counts that
         * SM's own clock) */
        for (int i = 0; i < sms; i++) {
            sm_lo[3 * i] = 1e300;
            sm_lo[3 * i + 1] = -1e300;
            sm_lo[3 * i + 2] = 0;
        }
        for (int i = 0; i < blocks; i++) {
            int id = (int)h[3 * i];
            if (id < 0 || id >= sms)
                continue;
            if ((double)h[3 * i + 1] < sm_lo[3 * id])
                sm_lo[3 * id] = (double)h[3 * i + 1];
            if ((double)h[3 * i + 2] > sm_lo[3 * id + 1])
                sm_lo[3 * id + 1] = (double)h[3 * i + 2];
            sm_lo[3 * id + 2] += 1;
        }
        double rate = 0;
        int used = 0;
        const double lanes_per_cta = (double)threads * KG_PEAK_ITERS * chains;
        for (int i = 0; i < sms; i++)
            if (sm_lo[3 * i + 1] > sm_lo[3 * i]) {
                used++;
                rate += sm_lo[3 * i + 2] * lanes_per_cta / (sm_lo[3 * i + 1] - sm_lo[3 * i]);
            }
        if (ms < best) {
            best = ms;
            best_clk = used ? rate / used : 0;
        }
    }
    free(h);
    free(sm_lo);
    if (a)
        cudaEventDestroy(a);
    if (b)
        cudaEventDestroy(b);
    cudaFree(out);
    cudaFree(stamps);
    if (e != cudaSuccess)
        return kg_cuda_fail(e, "kg_diag_fp64_probe");
    *lanes_per_s = (double)blocks * threads * KG_PEAK_ITERS * chains / (best * 1e-3);
    if (lanes_per_sm_clock)
        *lanes_per_sm_clock = best_clk;
    return KG_OK;
}

/* the best FP64 lane rate over a sweep of operations, chain counts and CTAs per SM */
extern "C" int kg_diag_fp64_peak(double* ops_per_s)
{
    if (!ops_per_s)
        return kg_fail(KG_ERR_INVALID, "kg_diag_fp64_peak: null pointer");
    double best = 0;
    const int ctas[3] = {2, 4, 8};
    for (int op = 0; op < 4; op++)
        for (int chains : {8, 16})
            for (int c : ctas) {
                double v = 0;
                int rc = kg_diag_fp64_probe(op, chains, c, 256, &v, nullptr);
                if (rc == KG_ERR_INVALID)
                    continue; /* that many CTAs do not fit */
                if (rc)
                    return rc;
                if (v > best)
                    best = v;
            }
    *ops_per_s = best;
    return KG_OK;
}

/* An mbarrier that no copy ever completes: the strip kernel's bounded wait
 * must give up, raise the flag and return. */
__global__ void kg_diag_mbar_kernel(unsigned* err)
{
    __shared__ unsigned long long mbar;
    if (threadIdx.x == 0) {
        kg_mbar_init(&mbar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    kg_mbar_wait(&mbar, 0, err);
}

extern "C" int kg_diag_mbar_timeout(int* timed_out)
{
    if (!timed_out)
        return kg_fail(KG_ERR_INVALID, "kg_diag_mbar_timeout: null pointer");
    unsigned* d = nullptr;
    KG_CUDA(cudaMalloc(&d, sizeof(unsigned)));
    cudaError_t e = cudaMemset(d, 0, sizeof(unsigned));
    if (e == cudaSuccess) {
        kg_diag_mbar_kernel<<<1, 32>>>(d);
        e = cudaGetLastError();
    }
    unsigned h = 0;
    if (e == cudaSuccess)
        e = cudaMemcpy(&h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess)
        return kg_cuda_fail(e, "kg_diag_mbar_timeout");
    *timed_out = h != 0;
    return KG_OK;
}

/* Copies `bytes` (a multiple of 16, both ends 16-byte aligned) with SM loads and stores instead of a
 * copy engine: the GPU writes the destination directly (for page-locked host memory, over the host
 * link). */
__global__ void kg_diag_copy_kernel(uint4* __restrict__ dst, const uint4* __restrict__ src, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

extern "C" int kg_diag_copy(void* dst, const void* src, long long bytes, void* stream)
{
    if (!dst || !src || bytes < 0 || (bytes & 15) || ((uintptr_t)dst & 15) || ((uintptr_t)src & 15))
        return kg_fail(KG_ERR_INVALID, "kg_diag_copy: pointers must be 16-byte aligned and bytes a multiple of 16");
    /* both ends must be addresses the device can use: device memory, or page-locked host memory (whose
     * device address is looked up, not assumed) */
    void* ends[2] = {dst, (void*)src};
    for (int k = 0; k < 2; k++) {
        cudaPointerAttributes a;
        KG_CUDA(cudaPointerGetAttributes(&a, ends[k]));
        if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeHost && a.type != cudaMemoryTypeManaged)
            return kg_fail(KG_ERR_INVALID, "kg_diag_copy: %s is not device or page-locked host memory",
                           k ? "src" : "dst");
        if (!a.devicePointer)
            return kg_fail(KG_ERR_INVALID, "kg_diag_copy: %s has no device address", k ? "src" : "dst");
        ends[k] = a.devicePointer;
    }
    if (bytes == 0)
        return KG_OK;
    kg_diag_copy_kernel<<<152 * 8, 256, 0, (cudaStream_t)stream>>>((uint4*)ends[0], (const uint4*)ends[1], bytes / 16);
    KG_CUDA(cudaGetLastError());
    return KG_OK;
}

/*
 * kg_diag.cu -- diagnostic kernels: device evaluation of kg_math.h for the
 * host-vs-device tests, and an FP64 FMA throughput probe.
 */
#include "kg_common.h"
#include <string.h>
#include "kobayashi_diag.h"

__global__ void kg_diag_eval_kernel(int fn, const double* __restrict__ x, double* __restrict__ y, long long n, double b,
                                    double yh, double yl, kg_idivc ic)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double v = x[i], r = 0.0;
        if (fn == KG_FN_ATAN) {
            r = kg_atan(v);
        } else if (fn == KG_FN_SIN || fn == KG_FN_COS) {
            double s, c;
            kg_sincos(v, &s, &c);
            r = fn == KG_FN_SIN ? s : c;
        } else if (fn == KG_FN_CDIV) {
            r = kg_cdiv(v, b, yh, yl);
        } else if (fn == KG_FN_IDIV) {
            r = kg_idiv(v, &ic);
        } else if (fn == KG_FN_IADD) {
            r = kg_iadd(v, x[n - 1 - i]);
        } else if (fn == KG_FN_ADD) {
            r = __dadd_rn(v, x[n - 1 - i]);
        } else if (fn == KG_FN_IMUL2) {
            r = kg_imul2(v);
        } else if (fn == KG_FN_MUL2) {
            r = __dmul_rn(2.0, v);
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
    if (fn < KG_FN_ATAN || fn > KG_FN_DIV_PAIR || fn == 12 || n < 0 || (n > 0 && (!x || !y)))
        return kg_fail(KG_ERR_INVALID, "kg_diag_eval: bad arguments");
    double yh = 0, yl = 0;
    kg_idivc ic;
    memset(&ic, 0, sizeof ic);
    if ((fn == KG_FN_CDIV || fn == KG_FN_DIV || fn == KG_FN_IDIV) &&
        (kg_cdiv_prepare(b, &yh, &yl) || kg_idiv_prepare(b, &ic)))
        return kg_fail(KG_ERR_INVALID, "kg_diag_eval: divisor outside [2^-100, 2^100]");
    if (n == 0)
        return KG_OK;
    double* d = nullptr;
    KG_CUDA(cudaMalloc(&d, sizeof(double) * 2 * (size_t)n));
    cudaError_t e = cudaMemcpy(d, x, sizeof(double) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        int blocks = (int)((n + 255) / 256 < 152 * 8 ? (n + 255) / 256 : 152 * 8);
        kg_diag_eval_kernel<<<blocks, 256>>>(fn, d, d + n, n, b, yh, yl, ic);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpy(y, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess)
        return kg_cuda_fail(e, "kg_diag_eval");
    return KG_OK;
}

#define KG_PEAK_CHAINS 8
#define KG_PEAK_ITERS 4096

__global__ void kg_diag_fma_kernel(double* out, double s)
{
    double v[KG_PEAK_CHAINS];
    for (int c = 0; c < KG_PEAK_CHAINS; c++)
        v[c] = 1.0 + 1e-3 * (threadIdx.x + c);
    for (int i = 0; i < KG_PEAK_ITERS; i++) {
#pragma unroll
        for (int c = 0; c < KG_PEAK_CHAINS; c++)
            v[c] = __fma_rn(v[c], s, 0.5);
    }
    double acc = 0;
    for (int c = 0; c < KG_PEAK_CHAINS; c++)
        acc += v[c];
    if (acc == 12345.678)
        out[0] = acc;
}

extern "C" int kg_diag_fp64_peak(double* ops_per_s)
{
    if (!ops_per_s)
        return kg_fail(KG_ERR_INVALID, "kg_diag_fp64_peak: null pointer");
    int dev = 0, sms = 0;
    KG_CUDA(cudaGetDevice(&dev));
    KG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* out = nullptr;
    KG_CUDA(cudaMalloc(&out, sizeof(double)));
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const int blocks = sms * 4, threads = 256;
    kg_diag_fma_kernel<<<blocks, threads>>>(out, 0.999);
    float best = 1e30f;
    for (int r = 0; r < 3; r++) {
        cudaEventRecord(a);
        kg_diag_fma_kernel<<<blocks, threads>>>(out, 0.999);
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        if (ms < best)
            best = ms;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(out);
    if (e != cudaSuccess)
        return kg_cuda_fail(e, "kg_diag_fp64_peak");
    *ops_per_s = (double)blocks * threads * KG_PEAK_ITERS * KG_PEAK_CHAINS / (best * 1e-3);
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

/*
 * kg_color.cu -- the reference's phi -> colour ramp as a headless device
 * buffer.
 *
 * The reference colours every cell on the CPU before each Direct3D draw
 * (Kobayashi::iUpdateConstantBuffer, src/Kobayashi.cpp:309-345): three linear
 * segments of the colour ramp with breaks at 0.9, 0.99 and 1.0 (float
 * literals), alpha = 1.  Here one kernel writes all cells' RGBA (float32) at
 * once, into device memory (for a renderer that stays on the GPU) or, through
 * the host entry point, into a host buffer.  The arithmetic follows the
 * reference's FP64 build (the float literals promoted to double, the ramp in
 * double, rounded to float at the end), so the output equals the reference's
 * colours for the same phi bit for bit.
 *
 * Two cell orders:
 *   KG_COLOR_GRID    rgba[4 (i + nx j) + c] is the colour of cell (i, j);
 *   KG_COLOR_VIEWER  the order of the viewer's constant buffers, including the
 *                    reference's transposition j = i / s, k = i % s with
 *                    s = sqrt(nx ny) (src/Kobayashi.cpp:311-315): square grids only.
 */
#include <math.h>
#include "kg_common.h"
#include "kobayashi_color.h"

/* the ramp's float literals (src/Kobayashi.cpp:318-325), as the FP64 build sees them */
__device__ __forceinline__ void kg_ramp(double phi, double* r, double* g, double* b)
{
    const double c1x = (double)0.2505490f, c1y = (double)0.5f, c1z = (double)0.9882353f;
    const double c2x = (double)0.3607843f, c2y = (double)1.0f, c2z = (double)0.9882353f;
    const double c3x = (double)0.9005490f, c3y = (double)1.0f, c3z = (double)0.9882353f;
    const double b1 = (double)0.9f, b2 = (double)0.99f, b3 = (double)1.0f;
    double ratio;
    if (phi <= b1) {
        ratio = phi * (1.0 / b1);
        /* c0 * (1 - ratio) + c1 * ratio with c0 = 0 */
        *r = 0.0 * (1.0 - ratio) + c1x * ratio;
        *g = 0.0 * (1.0 - ratio) + c1y * ratio;
        *b = 0.0 * (1.0 - ratio) + c1z * ratio;
    } else if (phi > b1 && phi <= b2) {
        ratio = (phi - b1) * (1.0 / (b2 - b1));
        *r = c1x * (1.0 - ratio) + c2x * ratio;
        *g = c1y * (1.0 - ratio) + c2y * ratio;
        *b = c1z * (1.0 - ratio) + c2z * ratio;
    } else {
        ratio = (phi - b2) * (1.0 / (b3 - b2));
        *r = c2x * (1.0 - ratio) + c3x * ratio;
        *g = c2y * (1.0 - ratio) + c3y * ratio;
        *b = c2z * (1.0 - ratio) + c3z * ratio;
    }
}

__global__ void kg_color_kernel(const double* __restrict__ phi, float4* __restrict__ out, int nx, int ny, int order,
                                int side)
{
    long long N = (long long)nx * ny;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
        long long src = i;
        if (order == KG_COLOR_VIEWER) {
            long long j = i / side, k = i % side;
            src = j + (long long)nx * k;
        }
        double r, g, b;
        kg_ramp(phi[src], &r, &g, &b);
        out[i] = make_float4((float)r, (float)g, (float)b, 1.0f);
    }
}

int kg_color_launch(const double* phi, float* rgba, int nx, int ny, int order, cudaStream_t s)
{
    if (order != KG_COLOR_GRID && order != KG_COLOR_VIEWER)
        return kg_fail(KG_ERR_INVALID, "colormap: unknown cell order %d", order);
    int side = 0;
    if (order == KG_COLOR_VIEWER) {
        side = (int)sqrt((double)nx * ny);
        if (nx != ny || (long long)side * side != (long long)nx * ny)
            return kg_fail(KG_ERR_INVALID, "colormap: the viewer order needs a square grid (got %d x %d)", nx, ny);
    }
    if (((uintptr_t)rgba & 15) != 0)
        return kg_fail(KG_ERR_INVALID, "colormap: the RGBA buffer must be 16-byte aligned");
    long long N = (long long)nx * ny;
    int blocks = (int)((N + 255) / 256 < 152 * 16 ? (N + 255) / 256 : 152 * 16);
    kg_color_kernel<<<blocks, 256, 0, s>>>(phi, (float4*)rgba, nx, ny, order, side);
    KG_CUDA(cudaGetLastError());
    return KG_OK;
}

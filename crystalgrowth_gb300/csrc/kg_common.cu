/*
 * kg_common.cu -- error reporting, parameter checks, derived constants and
 * the nucleus seeding kernel.
 */
#include <math.h>
#include <string.h>
#include "kg_common.h"

static thread_local char g_err[512];

int kg_fail(int code, const char* fmt, ...)
{
    /* formatted into a local buffer first: a caller may pass kg_last_error() itself as an argument */
    char buf[sizeof g_err];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    memcpy(g_err, buf, sizeof g_err);
    return code;
}

int kg_cuda_fail(cudaError_t e, const char* what)
{
    /* the error is handled here: clear it from the runtime's per-thread last error, or the next
     * launch check (cudaGetLastError) would report it again (a failed cudaMalloc leaves it there) */
    (void)cudaGetLastError();
    return kg_fail(e == cudaErrorMemoryAllocation ? KG_ERR_NOMEM : KG_ERR_CUDA, "%s: %s (%s)", what,
                   cudaGetErrorString(e), cudaGetErrorName(e));
}

extern "C" const char* kg_last_error(void) { return g_err; }

/* grid-stride copy of n 16-byte units */
__global__ void kg_copy_kernel(uint4* __restrict__ dst, const uint4* __restrict__ src, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

cudaError_t kg_copy_host(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s)
{
    if (bytes == 0)
        return cudaSuccess;
    const void* host = kind == cudaMemcpyDeviceToHost ? dst : src;
    cudaPointerAttributes a;
    if (((uintptr_t)dst & 15) == 0 && ((uintptr_t)src & 15) == 0 && (bytes & 15) == 0 &&
        cudaPointerGetAttributes(&a, host) == cudaSuccess && a.type == cudaMemoryTypeHost && a.devicePointer) {
        /* page-locked: the kernel uses the buffer's device address, looked up above, never the host one */
        uint4* d = (uint4*)(kind == cudaMemcpyDeviceToHost ? a.devicePointer : dst);
        const uint4* sp = (const uint4*)(kind == cudaMemcpyDeviceToHost ? src : a.devicePointer);
        kg_copy_kernel<<<152 * 8, 256, 0, s>>>(d, sp, (long long)(bytes / 16));
        return cudaGetLastError();
    }
    (void)cudaGetLastError(); /* a pointer query on ordinary host memory may leave an error behind */
    return kg_copy_pieces(dst, src, bytes, kind, s);
}

cudaError_t kg_copy_pieces(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s)
{
    const size_t piece = (size_t)64 << 20;
    for (size_t off = 0; off < bytes; off += piece) {
        const size_t n = bytes - off < piece ? bytes - off : piece;
        cudaError_t e = cudaMemcpyAsync((char*)dst + off, (const char*)src + off, n, kind, s);
        if (e != cudaSuccess)
            return e;
    }
    return cudaSuccess;
}

extern "C" const char* kg_version(void) { return "kobayashi-gb300 0.1 (sm_103a, FP64)"; }

/* _parameterInit and the ctor's grid spacing (src/Kobayashi.cpp:61-63,76-84) */
extern "C" int kg_params_default(kg_params* p, double dt)
{
    if (!p)
        return kg_fail(KG_ERR_INVALID, "kg_params_default: null pointer");
    p->dx = 0.03;
    p->dy = 0.03;
    p->dt = dt;
    p->tau = 0.0003;
    p->eps_bar = 0.010;
    p->mu = 1.0;
    p->K = 1.6;
    p->delta = 0.05;
    p->aniso = 6.0;
    p->alpha = 0.9;
    p->gamma = 10.0;
    p->teq = 1.0;
    p->theta0 = 0.0;
    return KG_OK;
}

/* The reference's slider model (src/Kobayashi.cpp:12-59): per parameter the
 * integer slider range, its default position (_parameterInit, :87-95) and the
 * ratio that turns a position into a value (value = (float)position * ratio,
 * the SB_THUMBTRACK branch of iWMHScroll, :587-591). */
static const struct {
    int lo, hi, def;
    float ratio;
} kg_sliders[KG_SLIDERS] = {
    {1, 9, 3, 0.0001f},  /* tau */
    {6, 15, 10, 0.001f}, /* eps_bar */
    {5, 14, 10, 0.1f},   /* mu */
    {10, 19, 16, 0.1f},  /* K */
    {1, 9, 5, 0.01f},    /* delta */
    {2, 8, 6, 1.0f},     /* aniso */
    {7, 12, 9, 0.1f},    /* alpha */
    {10, 20, 10, 1.0f},  /* gamma */
    {5, 15, 10, 0.1f},   /* teq */
};

extern "C" int kg_slider_range(int which, int* lo, int* hi, int* def)
{
    if (which < 0 || which >= KG_SLIDERS)
        return kg_fail(KG_ERR_INVALID, "kg_slider_range: slider %d out of range [0, %d)", which, KG_SLIDERS);
    if (lo)
        *lo = kg_sliders[which].lo;
    if (hi)
        *hi = kg_sliders[which].hi;
    if (def)
        *def = kg_sliders[which].def;
    return KG_OK;
}

extern "C" int kg_params_from_sliders(const int* pos, double dt, kg_params* p)
{
    if (!pos || !p)
        return kg_fail(KG_ERR_INVALID, "kg_params_from_sliders: null pointer");
    float v[KG_SLIDERS];
    for (int k = 0; k < KG_SLIDERS; k++) {
        if (pos[k] < kg_sliders[k].lo || pos[k] > kg_sliders[k].hi)
            return kg_fail(KG_ERR_INVALID, "kg_params_from_sliders: slider %d at %d outside [%d, %d]", k, pos[k],
                           kg_sliders[k].lo, kg_sliders[k].hi);
        v[k] = (float)pos[k] * kg_sliders[k].ratio;
    }
    int rc = kg_params_default(p, dt);
    if (rc)
        return rc;
    p->tau = v[0];
    p->eps_bar = v[1];
    p->mu = v[2];
    p->K = v[3];
    p->delta = v[4];
    p->aniso = v[5];
    p->alpha = v[6];
    p->gamma = v[7];
    p->teq = v[8];
    return kg_params_validate(p);
}

static bool finite_all(const kg_params* p)
{
    const double v[] = {p->dx, p->dy, p->dt, p->tau, p->eps_bar, p->mu, p->K, p->delta, p->aniso, p->alpha,
                        p->gamma, p->teq, p->theta0};
    static_assert(sizeof v == sizeof(kg_params), "every kg_params member is checked");
    for (double x : v)
        if (!isfinite(x))
            return false;
    return true;
}

extern "C" int kg_params_validate(const kg_params* p)
{
    if (!p)
        return kg_fail(KG_ERR_INVALID, "params: null pointer");
    if (!finite_all(p))
        return kg_fail(KG_ERR_INVALID, "params: every field must be finite");
    const double lo = 1e-12, hi = 1e12;
    if (!(p->dx >= lo && p->dx <= hi && p->dy >= lo && p->dy <= hi))
        return kg_fail(KG_ERR_INVALID, "params: dx, dy must lie in [1e-12, 1e12]");
    if (!(p->dt > 0 && p->dt <= hi))
        return kg_fail(KG_ERR_INVALID, "params: dt must be > 0");
    if (!(p->tau >= lo && p->tau <= hi))
        return kg_fail(KG_ERR_INVALID, "params: tau must lie in [1e-12, 1e12]");
    if (!(p->eps_bar > 0))
        return kg_fail(KG_ERR_INVALID, "params: eps_bar must be > 0");
    if (!(p->aniso >= 1 && p->aniso <= 64 && p->aniso == floor(p->aniso)))
        return kg_fail(KG_ERR_INVALID, "params: aniso (mode number j) must be an integer in [1, 64]");
    if (!(fabs(p->theta0) <= 100.0))
        return kg_fail(KG_ERR_INVALID, "params: |theta0| must be <= 100");
    return KG_OK;
}

int kg_prepare(const kg_params* p, KgDev* d)
{
    int rc = kg_params_validate(p);
    if (rc)
        return rc;
    memset(d, 0, sizeof *d);
    d->dx = p->dx;
    d->dy = p->dy;
    d->dt = p->dt;
    d->tau = p->tau;
    d->eps_bar = p->eps_bar;
    d->K = p->K;
    d->delta = p->delta;
    d->aniso = p->aniso;
    d->alpha = p->alpha;
    d->gamma = p->gamma;
    d->teq = p->teq;
    d->theta0 = p->theta0;
    d->lap_den = 3.0 * p->dx * p->dx;
    if (kg_idiv_prepare(p->dx, &d->idx) || kg_idiv_prepare(p->dy, &d->idy) || kg_idiv_prepare(d->lap_den, &d->ilap) ||
        kg_idiv_prepare(p->tau, &d->itau))
        return kg_fail(KG_ERR_INVALID, "params: dx, dy, 3 dx^2 and tau must lie in [2^-100, 2^100]");
    d->c_epsd = -p->eps_bar * p->aniso * p->delta;
    d->a_pi = p->alpha / KG_PI;
    /* memo for theta == 0: the same operations the kernel would do */
    d->arg0 = p->aniso * (0.0 - p->theta0);
    double s, c;
    kg_sincos(d->arg0, &s, &c);
    d->s0 = s;
    d->c0 = c;
    d->eps0 = p->eps_bar * (1.0 + p->delta * c);
    d->epsd0 = d->c_epsd * s;
    d->e2_0 = d->eps0 * d->eps0;
    d->ee0 = d->eps0 * d->epsd0;
    /* memo for T == 0 */
    d->u0 = p->gamma * (p->teq - 0.0);
    d->m0 = d->a_pi * kg_atan(d->u0);
    d->t_small = kg_absorb_bound(p->teq);
    d->zk = kg_bits(p->K * 0.0);
    d->ebk = (int)((kg_bits(p->K) >> 52) & 0x7ff);
    /* 1 - phi == 1 needs |phi| <= bound(1) = 2^-55, phi - 0.5 == -0.5 needs bound(0.5) = 2^-56 */
    d->phi_small = kg_absorb_bound(0.5);
    d->r0 = -0.5 + d->m0;
    return KG_OK;
}

/* Strip shape for one grid.  The first of 256 x 24, 128 x 32 and 128 x 16 that still gives at least
 * 8,000 CTAs (256 x 24 for 8192^2 and up, 128 x 16 for 4096^2).  Measured on GB300 at 8192^2
 * (cell-updates/s over steps 0-1000 / 4000-5000 / 8000-9000): 256 x 24 2.497e10 / 1.175e10 / 9.875e9,
 * 128 x 32 2.497e10 / 1.137e10 / 9.517e9, 128 x 16 2.485e10 / - / 9.279e9: wider and taller strips
 * recompute fewer halo columns and rows, and half as many CTAs start.  At 4096^2 late in the
 * trajectory 128 x 16 beat 128 x 32 (1.01e10 against 9.7e9).  Smaller grids: the largest strips that
 * still give about 30,000 CTAs (below that, strips covering the growing crystals finish last and the
 * SMs idle; above it, the repeated halo rows of short strips cost more than they save), down to
 * one-warp strips of 4 rows. */
void kg_pick_tile(int nx, int ny, int* nt, int* bh)
{
    const int big[3][2] = {{256, 24}, {128, 32}, {128, 16}};
    for (int k = 0; k < 3; k++) {
        const int t = big[k][0], h = big[k][1];
        if ((long long)((nx + t - 3) / (t - 2)) * ((ny + h - 1) / h) >= 8000) {
            *nt = t;
            *bh = h < ny ? h : ny;
            return;
        }
    }
    const long long want = 30000;
    const int shapes[8][2] = {{128, 64}, {128, 32}, {128, 16}, {64, 16}, {64, 8}, {32, 8}, {32, 4}};
    for (int k = 0; k < 7; k++) {
        int t = shapes[k][0], h = shapes[k][1];
        long long ctas = (long long)((nx + t - 3) / (t - 2)) * ((ny + h - 1) / h);
        if (ctas >= want || k == 6) {
            *nt = t;
            *bh = h < ny ? h : ny;
            return;
        }
    }
}

__global__ void kg_seed_kernel(double* phi, double* t, double* theta, int nx, int ny, int n, const int* cx,
                               const int* cy, const int* r)
{
    long long N = (long long)nx * ny;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        int i = (int)(c % nx), j = (int)(c / nx);
        double v = 0.0;
        for (int k = 0; k < n; k++) {
            int di = (i - cx[k]) % nx;
            if (di < 0)
                di += nx;
            if (di > nx / 2)
                di -= nx;
            int dj = (j - cy[k]) % ny;
            if (dj < 0)
                dj += ny;
            if (dj > ny / 2)
                dj -= ny;
            if ((long long)di * di + (long long)dj * dj <= (long long)r[k] * r[k]) {
                v = 1.0;
                break;
            }
        }
        phi[c] = v;
        t[c] = 0.0;
        theta[c] = 0.0;
    }
}

int kg_seed_device(double* phi, double* t, double* theta, int nx, int ny, int n, const int* cx, const int* cy,
                   const int* r, cudaStream_t s)
{
    if (n < 0 || (n > 0 && (!cx || !cy || !r)))
        return kg_fail(KG_ERR_INVALID, "seed: bad disk list");
    for (int k = 0; k < n; k++)
        if (r[k] < 0)
            return kg_fail(KG_ERR_INVALID, "seed: negative radius");
    int* d = nullptr;
    if (n > 0) {
        KG_CUDA(cudaMalloc(&d, sizeof(int) * 3 * (size_t)n));
        cudaError_t e = cudaMemcpyAsync(d, cx, sizeof(int) * n, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d + n, cy, sizeof(int) * n, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d + 2 * n, r, sizeof(int) * n, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) {
            cudaFree(d);
            return kg_cuda_fail(e, "seed: copy disks");
        }
    }
    long long N = (long long)nx * ny;
    int blocks = (int)((N + 255) / 256 < 152 * 16 ? (N + 255) / 256 : 152 * 16);
    kg_seed_kernel<<<blocks, 256, 0, s>>>(phi, t, theta, nx, ny, n, d, d ? d + n : nullptr, d ? d + 2 * n : nullptr);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (d)
        cudaFree(d);
    if (e != cudaSuccess)
        return kg_cuda_fail(e, "seed kernel");
    return KG_OK;
}

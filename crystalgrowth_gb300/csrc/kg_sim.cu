/*
 * kg_sim.cu -- the single-grid simulation handle (kg_sim) and its step kernel.
 *
 * State lives in HBM as two ping-pong copies of (phi, T, theta), nx*ny FP64
 * each, row-major like the reference's std::vector fields
 * (src/Kobayashi.h:107-115).  kg_step launches one fused kernel per time step
 * (kg_device.cuh) and replays them as CUDA graphs of `chunk` steps.
 */
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <new>
#include "kg_common.h"
#include "kobayashi_color.h"
#include "kobayashi_diag.h"


#define KG_STEP_BOUNDS(NT) __launch_bounds__(NT)

/* rows of phi and T reach shared memory by bulk (TMA) copies where the strip allows it (1), or by
 * per-lane loads everywhere (0) */
#ifndef KG_TMA
#define KG_TMA 1
#endif

template <int NT>
__global__ void KG_STEP_BOUNDS(NT) kg_step_kernel(const __grid_constant__ KgDev P, int nx, int ny, int bh,
                                                     const double* __restrict__ phi_in, const double* __restrict__ t_in,
                                                     const double* __restrict__ th_in, double* __restrict__ phi_out,
                                                     double* __restrict__ t_out, double* __restrict__ th_out,
                                                     unsigned* err)
{
    __shared__ KgSmem<NT> sm;
    const int i0 = blockIdx.x * (NT - 2);
    /* bulk copies need 16-byte aligned rows (nx even) and a strip that does not wrap left/right */
    const bool tma = KG_TMA && (nx % 2 == 0) && i0 >= 2 && i0 + NT <= nx;
    kg_strip<NT>(P, nx, ny, phi_in, t_in, th_in, phi_out, t_out, th_out, i0, blockIdx.y * bh, bh, sm, nullptr, tma,
                 err);
}

/* two steps per launch (temporal blocking, k = 2); per-lane loads only */
template <int NT>
__global__ void KG_STEP_BOUNDS(NT) kg_step2_kernel(const __grid_constant__ KgDev P, int nx, int ny, int bh,
                                                      const double* __restrict__ phi_in, const double* __restrict__ t_in,
                                                      const double* __restrict__ th_in, double* __restrict__ phi_out,
                                                      double* __restrict__ t_out, double* __restrict__ th_out)
{
    __shared__ KgSmem2<NT> sm;
    kg_strip2<NT>(P, nx, ny, phi_in, t_in, th_in, phi_out, t_out, th_out, blockIdx.x * (NT - 6), blockIdx.y * bh, bh,
                  sm);
}

struct kg_sim {
    int nx = 0, ny = 0;
    kg_params p{};
    KgDev dev{};
    double* buf[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
    int cur = 0;
    cudaStream_t stream = nullptr;
    long long steps = 0, frames = 0;
    int chunk = 100;
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    int nt = 128; /* threads per strip CTA (strip width nt - 2 columns) */
    int bh = 64;  /* rows per strip */
    int tblock = 1; /* time steps per launch: 1, or 2 (temporal blocking) */
    float* color = nullptr; /* RGBA staging buffer for kg_colormap, allocated on first use */
    unsigned* err = nullptr; /* raised by a kernel whose bounded wait ran out */
    /* set once a bounded wait ran out: the state is unreliable, and kg_step refuses until the state
     * is replaced (kg_reset, kg_seed_disks, kg_set_fields with all three fields, kg_load) */
    bool failed = false;
};

/* Destroys the instantiated graphs.  A graph launched earlier may still be running on the
 * handle's stream, so the stream is drained first. */
static void drop_graphs(kg_sim* h)
{
    if (!h->graph[0] && !h->graph[1])
        return;
    if (h->stream)
        cudaStreamSynchronize(h->stream);
    for (int k = 0; k < 2; k++)
        if (h->graph[k]) {
            cudaGraphExecDestroy(h->graph[k]);
            h->graph[k] = nullptr;
        }
}

/* one launch advancing `k` (1 or 2) steps from ping-pong copy `from` into copy from ^ 1 */
static int launch_step(kg_sim* h, int from, int k = 1)
{
    double* const* a = h->buf[from];
    double* const* b = h->buf[from ^ 1];
    if (k == 2) {
        /* the two-step pass holds two pipelines' rings: strips of at most 128 threads */
        const int nt2 = h->nt > 128 ? 128 : h->nt;
        dim3 grid((h->nx + nt2 - 7) / (nt2 - 6), (h->ny + h->bh - 1) / h->bh);
        if (nt2 == 32)
            kg_step2_kernel<32><<<grid, 32, 0, h->stream>>>(h->dev, h->nx, h->ny, h->bh, a[0], a[1], a[2], b[0], b[1],
                                                             b[2]);
        else if (nt2 == 64)
            kg_step2_kernel<64><<<grid, 64, 0, h->stream>>>(h->dev, h->nx, h->ny, h->bh, a[0], a[1], a[2], b[0], b[1],
                                                             b[2]);
        else
            kg_step2_kernel<128><<<grid, 128, 0, h->stream>>>(h->dev, h->nx, h->ny, h->bh, a[0], a[1], a[2], b[0],
                                                               b[1], b[2]);
    } else {
        dim3 grid((h->nx + h->nt - 3) / (h->nt - 2), (h->ny + h->bh - 1) / h->bh);
        if (h->nt == 32)
            kg_step_kernel<32><<<grid, 32, 0, h->stream>>>(h->dev, h->nx, h->ny, h->bh, a[0], a[1], a[2], b[0], b[1],
                                                            b[2], h->err);
        else if (h->nt == 64)
            kg_step_kernel<64><<<grid, 64, 0, h->stream>>>(h->dev, h->nx, h->ny, h->bh, a[0], a[1], a[2], b[0], b[1],
                                                            b[2], h->err);
        else if (h->nt == 256)
            kg_step_kernel<256><<<grid, 256, 0, h->stream>>>(h->dev, h->nx, h->ny, h->bh, a[0], a[1], a[2], b[0],
                                                              b[1], b[2], h->err);
        else
            kg_step_kernel<128><<<grid, 128, 0, h->stream>>>(h->dev, h->nx, h->ny, h->bh, a[0], a[1], a[2], b[0],
                                                              b[1], b[2], h->err);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return kg_cuda_fail(e, k == 2 ? "kg_step2_kernel launch" : "kg_step_kernel launch");
    return KG_OK;
}

/* launches that advance n steps with the handle's temporal blocking factor */
static long long launches_for(const kg_sim* h, long long n) { return h->tblock == 2 ? n / 2 + (n & 1) : n; }

/* enqueues n steps from copy `from`; the result lies in copy from ^ (launches_for(n) & 1) */
static int enqueue_steps(kg_sim* h, int from, long long n)
{
    int c = from;
    for (long long s = 0; s < n;) {
        const int k = (h->tblock == 2 && n - s >= 2) ? 2 : 1;
        int rc = launch_step(h, c, k);
        if (rc)
            return rc;
        c ^= 1;
        s += k;
    }
    return KG_OK;
}

/* a graph of h->chunk consecutive steps starting from ping-pong copy `from` */
static int build_graph(kg_sim* h, int from)
{
    cudaGraph_t g = nullptr;
    KG_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_steps(h, from, h->chunk);
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (rc != KG_OK) {
        if (g)
            cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess)
        return kg_cuda_fail(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&h->graph[from], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        h->graph[from] = nullptr;
        return kg_cuda_fail(e, "cudaGraphInstantiate");
    }
    return KG_OK;
}

static int check(const kg_sim* h)
{
    if (!h)
        return kg_fail(KG_ERR_INVALID, "null kg_sim handle");
    return KG_OK;
}

extern "C" int kg_destroy(kg_sim* h)
{
    if (!h)
        return KG_OK;
    if (h->stream)
        cudaStreamSynchronize(h->stream);
    drop_graphs(h);
    for (int k = 0; k < 2; k++)
        for (int f = 0; f < 3; f++)
            if (h->buf[k][f])
                cudaFree(h->buf[k][f]);
    if (h->color)
        cudaFree(h->color);
    if (h->err)
        cudaFree(h->err);
    if (h->stream)
        cudaStreamDestroy(h->stream);
    delete h;
    return KG_OK;
}

extern "C" int kg_seed_disks(kg_sim* h, int n, const int* cx, const int* cy, const int* r)
{
    int rc = check(h);
    if (rc)
        return rc;
    double* const* a = h->buf[h->cur];
    rc = kg_seed_device(a[0], a[1], a[2], h->nx, h->ny, n, cx, cy, r, h->stream);
    if (rc)
        return rc;
    h->failed = false;
    h->steps = 0;
    h->frames = 0;
    return KG_OK;
}

extern "C" int kg_reset(kg_sim* h)
{
    int rc = check(h);
    if (rc)
        return rc;
    /* _createNucleus(nx/2, ny/2): the centre and its four neighbours (src/Kobayashi.cpp:113-123) */
    int cx = h->nx / 2, cy = h->ny / 2, r = 1;
    return kg_seed_disks(h, 1, &cx, &cy, &r);
}

extern "C" int kg_create(int nx, int ny, const kg_params* p, kg_sim** out)
{
    if (!out)
        return kg_fail(KG_ERR_INVALID, "kg_create: null output pointer");
    *out = nullptr;
    if (nx < 1 || ny < 1 || (long long)nx * ny > (1ll << 34))
        return kg_fail(KG_ERR_INVALID, "kg_create: grid %d x %d out of range", nx, ny);
    KgDev dev;
    int rc = kg_prepare(p, &dev);
    if (rc)
        return rc;
    kg_sim* h = new (std::nothrow) kg_sim();
    if (!h)
        return kg_fail(KG_ERR_NOMEM, "kg_create: host allocation");
    h->nx = nx;
    h->ny = ny;
    h->p = *p;
    h->dev = dev;
    kg_pick_tile(nx, ny, &h->nt, &h->bh);
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    size_t bytes = sizeof(double) * (size_t)nx * ny;
    for (int k = 0; k < 2 && e == cudaSuccess; k++)
        for (int f = 0; f < 3 && e == cudaSuccess; f++)
            e = cudaMalloc(&h->buf[k][f], bytes);
    if (e == cudaSuccess)
        e = cudaMalloc(&h->err, sizeof(unsigned));
    if (e == cudaSuccess)
        e = cudaMemset(h->err, 0, sizeof(unsigned));
    if (e != cudaSuccess) {
        rc = kg_cuda_fail(e, "kg_create: device allocation");
        kg_destroy(h);
        return rc;
    }
    rc = kg_reset(h);
    if (rc) {
        kg_destroy(h);
        return rc;
    }
    *out = h;
    return KG_OK;
}

extern "C" int kg_set_params(kg_sim* h, const kg_params* p)
{
    int rc = check(h);
    if (rc)
        return rc;
    KgDev dev;
    rc = kg_prepare(p, &dev);
    if (rc)
        return rc;
    h->p = *p;
    h->dev = dev;
    drop_graphs(h);
    return KG_OK;
}

extern "C" int kg_get_params(const kg_sim* h, kg_params* p)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (!p)
        return kg_fail(KG_ERR_INVALID, "kg_get_params: null pointer");
    *p = h->p;
    return KG_OK;
}

extern "C" int kg_set_graph_chunk(kg_sim* h, int chunk)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (chunk < 0 || chunk > 100000)
        return kg_fail(KG_ERR_INVALID, "kg_set_graph_chunk: chunk %d out of range", chunk);
    h->chunk = chunk;
    drop_graphs(h);
    return KG_OK;
}

extern "C" int kg_set_tile(kg_sim* h, int nt, int bh)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (nt != 32 && nt != 64 && nt != 128 && nt != 256)
        return kg_fail(KG_ERR_INVALID, "kg_set_tile: nt must be 32, 64, 128 or 256");
    if (bh < 1 || bh > 65536)
        return kg_fail(KG_ERR_INVALID, "kg_set_tile: bh must lie in [1, 65536]");
    KG_CUDA(cudaStreamSynchronize(h->stream));
    h->nt = nt;
    h->bh = bh < h->ny ? bh : h->ny;
    drop_graphs(h);
    return KG_OK;
}

extern "C" int kg_set_tblock(kg_sim* h, int k)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (k != 1 && k != 2)
        return kg_fail(KG_ERR_INVALID, "kg_set_tblock: the temporal blocking factor must be 1 or 2");
    h->tblock = k;
    drop_graphs(h);
    return KG_OK;
}

extern "C" int kg_get_tblock(const kg_sim* h, int* k)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (!k)
        return kg_fail(KG_ERR_INVALID, "kg_get_tblock: null pointer");
    *k = h->tblock;
    return KG_OK;
}

extern "C" int kg_get_tile(const kg_sim* h, int* nt, int* bh)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (nt)
        *nt = h->nt;
    if (bh)
        *bh = h->bh;
    return KG_OK;
}

extern "C" int kg_step(kg_sim* h, long long nsteps)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (nsteps < 0)
        return kg_fail(KG_ERR_INVALID, "kg_step: negative step count");
    if (h->failed)
        return kg_fail(KG_ERR_TIMEOUT, "kg_step: an earlier step's bounded wait ran out and the state is "
                                       "unreliable; replace it first (kg_reset, kg_seed_disks, kg_set_fields, kg_load)");
    while (h->chunk > 0 && nsteps >= h->chunk) {
        if (!h->graph[h->cur]) {
            rc = build_graph(h, h->cur);
            if (rc)
                return rc;
        }
        cudaError_t e = cudaGraphLaunch(h->graph[h->cur], h->stream);
        if (e != cudaSuccess)
            return kg_cuda_fail(e, "cudaGraphLaunch");
        h->cur ^= (int)(launches_for(h, h->chunk) & 1);
        h->steps += h->chunk;
        nsteps -= h->chunk;
    }
    if (nsteps > 0) {
        rc = enqueue_steps(h, h->cur, nsteps);
        if (rc)
            return rc;
        h->cur ^= (int)(launches_for(h, nsteps) & 1);
        h->steps += nsteps;
    }
    return KG_OK;
}

extern "C" int kg_update(kg_sim* h)
{
    int rc = kg_step(h, 10);
    if (rc)
        return rc;
    h->frames++;
    return KG_OK;
}

/* waits for the stream and reports (then clears) a bounded wait that ran out */
static int sync_and_check(kg_sim* h)
{
    unsigned flag = 0;
    KG_CUDA(cudaMemcpyAsync(&flag, h->err, sizeof flag, cudaMemcpyDeviceToHost, h->stream));
    KG_CUDA(cudaStreamSynchronize(h->stream));
    if (flag) {
        cudaMemsetAsync(h->err, 0, sizeof(unsigned), h->stream);
        cudaStreamSynchronize(h->stream);
        h->failed = true;
        return kg_fail(KG_ERR_TIMEOUT, "kg_step: a bulk-copy wait in the step kernel ran out; the state is unreliable");
    }
    if (h->failed)
        return kg_fail(KG_ERR_TIMEOUT, "the state is unreliable after a bounded wait ran out; replace it first "
                                       "(kg_reset, kg_seed_disks, kg_set_fields, kg_load)");
    return KG_OK;
}

/* Host-side fault injection for tests: raises the handle's device error flag as a kernel whose bounded
 * wait ran out would (no kernel runs, nothing faults). */
extern "C" int kg_diag_inject_timeout(kg_sim* h)
{
    int rc = check(h);
    if (rc)
        return rc;
    const unsigned one = 1;
    KG_CUDA(cudaMemcpyAsync(h->err, &one, sizeof one, cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(cudaStreamSynchronize(h->stream));
    return KG_OK;
}

extern "C" int kg_sync(kg_sim* h)
{
    int rc = check(h);
    if (rc)
        return rc;
    return sync_and_check(h);
}

extern "C" int kg_get_fields(kg_sim* h, double* phi, double* T, double* theta)
{
    int rc = check(h);
    if (rc)
        return rc;
    size_t bytes = sizeof(double) * (size_t)h->nx * h->ny;
    double* dst[3] = {phi, T, theta};
    for (int f = 0; f < 3; f++)
        if (dst[f])
            KG_CUDA(kg_copy_host(dst[f], h->buf[h->cur][f], bytes, cudaMemcpyDeviceToHost, h->stream));
    return sync_and_check(h);
}

extern "C" int kg_set_fields(kg_sim* h, const double* phi, const double* T, const double* theta)
{
    int rc = check(h);
    if (rc)
        return rc;
    size_t bytes = sizeof(double) * (size_t)h->nx * h->ny;
    const double* src[3] = {phi, T, theta};
    for (int f = 0; f < 3; f++)
        if (src[f])
            KG_CUDA(kg_copy_host(h->buf[h->cur][f], src[f], bytes, cudaMemcpyHostToDevice, h->stream));
    KG_CUDA(cudaStreamSynchronize(h->stream));
    if (phi && T && theta)
        h->failed = false; /* the whole state was replaced */
    return KG_OK;
}

extern "C" int kg_get_size(const kg_sim* h, int* nx, int* ny)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (nx)
        *nx = h->nx;
    if (ny)
        *ny = h->ny;
    return KG_OK;
}

extern "C" int kg_get_counters(const kg_sim* h, long long* steps, long long* frames)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (steps)
        *steps = h->steps;
    if (frames)
        *frames = h->frames;
    return KG_OK;
}

extern "C" int kg_device_fields(kg_sim* h, double** phi, double** T, double** theta)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (phi)
        *phi = h->buf[h->cur][0];
    if (T)
        *T = h->buf[h->cur][1];
    if (theta)
        *theta = h->buf[h->cur][2];
    return KG_OK;
}

extern "C" int kg_get_stream(kg_sim* h, void** stream)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (!stream)
        return kg_fail(KG_ERR_INVALID, "kg_get_stream: null pointer");
    *stream = (void*)h->stream;
    return KG_OK;
}

extern "C" int kg_colormap_device(kg_sim* h, int order, float* rgba_device)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (!rgba_device)
        return kg_fail(KG_ERR_INVALID, "kg_colormap_device: null buffer");
    return kg_color_launch(h->buf[h->cur][0], rgba_device, h->nx, h->ny, order, h->stream);
}

extern "C" int kg_colormap(kg_sim* h, int order, float* rgba)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (!rgba)
        return kg_fail(KG_ERR_INVALID, "kg_colormap: null buffer");
    size_t bytes = sizeof(float) * 4 * (size_t)h->nx * h->ny;
    if (!h->color)
        KG_CUDA(cudaMalloc(&h->color, bytes));
    rc = kg_color_launch(h->buf[h->cur][0], h->color, h->nx, h->ny, order, h->stream);
    if (rc)
        return rc;
    KG_CUDA(kg_copy_host(rgba, h->color, bytes, cudaMemcpyDeviceToHost, h->stream));
    KG_CUDA(cudaStreamSynchronize(h->stream));
    return KG_OK;
}

/* ---- snapshots: a 4096-byte JSON header, then phi, T, theta as little-endian FP64 ---- */

#define KG_SNAP_HEADER 4096

/* the snapshot header's parameter keys and the kg_params member each one stores */
static const struct {
    const char* name;
    size_t off;
} kg_param_fields[] = {
    {"dx", offsetof(kg_params, dx)},         {"dy", offsetof(kg_params, dy)},
    {"dt", offsetof(kg_params, dt)},         {"tau", offsetof(kg_params, tau)},
    {"eps_bar", offsetof(kg_params, eps_bar)}, {"mu", offsetof(kg_params, mu)},
    {"K", offsetof(kg_params, K)},           {"delta", offsetof(kg_params, delta)},
    {"aniso", offsetof(kg_params, aniso)},   {"alpha", offsetof(kg_params, alpha)},
    {"gamma", offsetof(kg_params, gamma)},   {"teq", offsetof(kg_params, teq)},
    {"theta0", offsetof(kg_params, theta0)},
};
static const int kg_nparams = (int)(sizeof kg_param_fields / sizeof kg_param_fields[0]);
static_assert(sizeof(kg_params) == sizeof kg_param_fields / sizeof kg_param_fields[0] * sizeof(double),
              "every kg_params member must have a snapshot key");

static double* param_at(kg_params* p, int k) { return (double*)((char*)p + kg_param_fields[k].off); }

extern "C" int kg_save(kg_sim* h, const char* path)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (!path)
        return kg_fail(KG_ERR_INVALID, "kg_save: null path");
    char hdr[KG_SNAP_HEADER];
    memset(hdr, ' ', sizeof hdr);
    int n = snprintf(hdr, sizeof hdr,
                     "{\"format\": \"kobayashi-gb300-snapshot\", \"version\": 1, \"nx\": %d, \"ny\": %d, "
                     "\"steps\": %lld, \"frames\": %lld, \"dtype\": \"float64\", \"byteorder\": \"little\", "
                     "\"fields\": [\"phi\", \"T\", \"theta\"], \"header_bytes\": %d, \"params\": {",
                     h->nx, h->ny, h->steps, h->frames, KG_SNAP_HEADER);
    kg_params pc = h->p;
    for (int k = 0; k < kg_nparams; k++)
        n += snprintf(hdr + n, sizeof hdr - n, "%s\"%s\": %.17g", k ? ", " : "", kg_param_fields[k].name,
                      *param_at(&pc, k));
    n += snprintf(hdr + n, sizeof hdr - n, "}}");
    if (n >= KG_SNAP_HEADER - 1)
        return kg_fail(KG_ERR_INVALID, "kg_save: header overflow");
    hdr[n] = ' ';
    hdr[KG_SNAP_HEADER - 1] = '\n';
    FILE* f = fopen(path, "wb");
    if (!f)
        return kg_fail(KG_ERR_INVALID, "kg_save: cannot open %s for writing", path);
    size_t cells = (size_t)h->nx * h->ny;
    double* buf = (double*)malloc(cells * sizeof(double));
    rc = KG_OK;
    if (!buf)
        rc = kg_fail(KG_ERR_NOMEM, "kg_save: host buffer");
    if (rc == KG_OK && fwrite(hdr, 1, sizeof hdr, f) != sizeof hdr)
        rc = kg_fail(KG_ERR_INVALID, "kg_save: write failed");
    for (int fld = 0; fld < 3 && rc == KG_OK; fld++) {
        cudaError_t e = kg_copy_pieces(buf, h->buf[h->cur][fld], cells * sizeof(double), cudaMemcpyDeviceToHost,
                                       h->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess)
            rc = kg_cuda_fail(e, "kg_save: device copy");
        else if (fwrite(buf, sizeof(double), cells, f) != cells)
            rc = kg_fail(KG_ERR_INVALID, "kg_save: write failed");
    }
    free(buf);
    if (fclose(f) != 0 && rc == KG_OK)
        rc = kg_fail(KG_ERR_INVALID, "kg_save: close failed");
    return rc;
}

static int snap_int(const char* hdr, const char* key, long long* v)
{
    char pat[64];
    snprintf(pat, sizeof pat, "\"%s\": ", key);
    const char* p = strstr(hdr, pat);
    if (!p)
        return -1;
    return sscanf(p + strlen(pat), "%lld", v) == 1 ? 0 : -1;
}

static int snap_double(const char* hdr, const char* key, double* v)
{
    char pat[64];
    snprintf(pat, sizeof pat, "\"%s\": ", key);
    const char* p = strstr(hdr, pat);
    if (!p)
        return -1;
    return sscanf(p + strlen(pat), "%lf", v) == 1 ? 0 : -1;
}

extern "C" int kg_load(kg_sim* h, const char* path)
{
    int rc = check(h);
    if (rc)
        return rc;
    if (!path)
        return kg_fail(KG_ERR_INVALID, "kg_load: null path");
    FILE* f = fopen(path, "rb");
    if (!f)
        return kg_fail(KG_ERR_INVALID, "kg_load: cannot open %s", path);
    char hdr[KG_SNAP_HEADER + 1];
    size_t got = fread(hdr, 1, KG_SNAP_HEADER, f);
    hdr[got] = 0;
    long long nx = 0, ny = 0, steps = 0, frames = 0, version = 0;
    if (got != KG_SNAP_HEADER || !strstr(hdr, "\"format\": \"kobayashi-gb300-snapshot\"") ||
        snap_int(hdr, "version", &version) || version != 1 || snap_int(hdr, "nx", &nx) || snap_int(hdr, "ny", &ny) ||
        snap_int(hdr, "steps", &steps) || snap_int(hdr, "frames", &frames)) {
        fclose(f);
        return kg_fail(KG_ERR_INVALID, "kg_load: %s is not a kobayashi-gb300 snapshot", path);
    }
    if (nx != h->nx || ny != h->ny) {
        fclose(f);
        return kg_fail(KG_ERR_INVALID, "kg_load: snapshot is %lld x %lld, the handle is %d x %d", nx, ny, h->nx, h->ny);
    }
    kg_params p;
    memset(&p, 0, sizeof p);
    for (int k = 0; k < kg_nparams; k++)
        if (snap_double(hdr, kg_param_fields[k].name, param_at(&p, k))) {
            fclose(f);
            return kg_fail(KG_ERR_INVALID, "kg_load: parameter %s missing", kg_param_fields[k].name);
        }
    KgDev dev;
    rc = kg_prepare(&p, &dev);
    if (rc) {
        fclose(f);
        return rc;
    }
    size_t cells = (size_t)nx * ny;
    /* the whole payload must be present before anything reaches the device: a short file leaves the
     * handle as it was */
    if (fseek(f, 0, SEEK_END) != 0 || ftell(f) != (long)(KG_SNAP_HEADER + 3 * cells * sizeof(double)) ||
        fseek(f, KG_SNAP_HEADER, SEEK_SET) != 0) {
        fclose(f);
        return kg_fail(KG_ERR_INVALID, "kg_load: %s is truncated or too long for %lld x %lld", path, nx, ny);
    }
    double* buf = (double*)malloc(cells * sizeof(double));
    if (!buf) {
        fclose(f);
        return kg_fail(KG_ERR_NOMEM, "kg_load: host buffer");
    }
    for (int fld = 0; fld < 3 && rc == KG_OK; fld++) {
        if (fread(buf, sizeof(double), cells, f) != cells) {
            rc = kg_fail(KG_ERR_INVALID, "kg_load: %s is truncated", path);
            break;
        }
        cudaError_t e = kg_copy_pieces(h->buf[h->cur][fld], buf, cells * sizeof(double), cudaMemcpyHostToDevice,
                                       h->stream);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess)
            rc = kg_cuda_fail(e, "kg_load: device copy");
    }
    free(buf);
    fclose(f);
    if (rc)
        return rc;
    h->p = p;
    h->dev = dev;
    h->steps = steps;
    h->frames = frames;
    h->failed = false;
    drop_graphs(h);
    return KG_OK;
}

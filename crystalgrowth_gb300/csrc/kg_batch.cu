/*
 * kg_batch.cu -- many independent Kobayashi grids of uneven sizes, each with
 * its own parameters, advanced together.
 *
 * No counterpart in the reference, which simulates one grid per process; the
 * per-instance arithmetic is the same fused step (kg_device.cuh), so every
 * instance is bit-identical to a kg_sim run of the same grid.
 *
 * Layout: one device arena holds every instance's two ping-pong copies of
 * (phi, T, theta).  A work list enumerates strips (instance, first column,
 * first row), largest instances first so the longest strips start early.
 * Two execution modes, picked by kg_batch_autotune together with the strip
 * width NT and height BH:
 *   KG_BATCH_LAUNCH      one kernel per time step over the work list,
 *                        replayed as CUDA graphs of `chunk` steps;
 *   KG_BATCH_PERSISTENT  one cooperative launch per chunk: CTAs loop over
 *                        the work list, step after step, separated by a
 *                        grid-wide barrier whose waits are bounded (a CTA that
 *                        waits too long raises an error flag instead of
 *                        hanging; the host reports KG_ERR_TIMEOUT).
 */
#include <algorithm>
#include <new>
#include <type_traits>
#include <string.h>
#include <vector>
#include "kg_common.h"
#include "kobayashi_batch.h"
#include "kobayashi_diag.h"

struct KgInst {
    long long off;  /* offset of copy 0 in the arena (doubles); copy c at off + c*3*n, field f at + f*n */
    int nx, ny;
};

struct KgBarrier {
    unsigned count;
    unsigned gen;
    unsigned err;
    unsigned pad;
};

__device__ __forceinline__ void kg_inst_ptrs(const KgInst& in, double* arena, int from, const double** src, double** dst)
{
    long long n = (long long)in.nx * in.ny;
    double* a = arena + in.off + (long long)from * 3 * n;
    double* b = arena + in.off + (long long)(from ^ 1) * 3 * n;
    src[0] = a;
    src[1] = a + n;
    src[2] = a + 2 * n;
    dst[0] = b;
    dst[1] = b + n;
    dst[2] = b + 2 * n;
}

/* one strip of the work list.  COH: the persistent kernel, whose CTAs read in step s+1 what other CTAs
 * wrote in step s of the same launch, loads the fields through L2 only */
template <int NT, bool COH>
__device__ __forceinline__ void kg_batch_item(const int4 w, const KgDev* __restrict__ P, const KgInst* __restrict__ I,
                                              double* arena, int from, int bh, KgSmem<NT>& sm)
{
    const KgInst in = I[w.x];
    const double* s[3];
    double* d[3];
    kg_inst_ptrs(in, arena, from, s, d);
    kg_strip<NT, false, COH>(P[w.x], in.nx, in.ny, s[0], s[1], s[2], d[0], d[1], d[2], w.y, w.z, bh, sm);
}

/* the same with temporal blocking: two steps per pass (kg_strip2) */
template <int NT, bool COH>
__device__ __forceinline__ void kg_batch_item2(const int4 w, const KgDev* __restrict__ P, const KgInst* __restrict__ I,
                                               double* arena, int from, int bh, KgSmem2<NT>& sm)
{
    const KgInst in = I[w.x];
    const double* s[3];
    double* d[3];
    kg_inst_ptrs(in, arena, from, s, d);
    kg_strip2<NT, COH>(P[w.x], in.nx, in.ny, s[0], s[1], s[2], d[0], d[1], d[2], w.y, w.z, bh, sm);
}

/* one strip per CTA, one time step.  The bound of 1024 / NT resident CTAs per SM holds the kernel to
 * 64 registers: the parameters of each instance come from global memory rather than the constant bank,
 * and left to itself the compiler takes 70, which leaves 28 warps resident per SM instead of 32 (64
 * registers measured 0-1.6% faster on the 512-instance ensemble at 64- and 128-thread strips) */
template <int NT>
__global__ void __launch_bounds__(NT, 1024 / NT) kg_batch_step_kernel(const int4* __restrict__ work,
                                                                      const KgDev* __restrict__ P,
                                                                      const KgInst* __restrict__ I, double* arena,
                                                                      int from, int bh)
{
    __shared__ KgSmem<NT> sm;
    kg_batch_item<NT, false>(work[blockIdx.x], P, I, arena, from, bh, sm);
}

/* one strip per CTA, two time steps (temporal blocking) */
template <int NT>
__global__ void __launch_bounds__(NT) kg_batch_step2_kernel(const int4* __restrict__ work, const KgDev* __restrict__ P,
                                                            const KgInst* __restrict__ I, double* arena, int from,
                                                            int bh)
{
    __shared__ KgSmem2<NT> sm;
    kg_batch_item2<NT, false>(work[blockIdx.x], P, I, arena, from, bh, sm);
}

/* bounded grid barrier; returns false when the wait ran out (or another CTA's did) */
__device__ bool kg_grid_barrier(KgBarrier* bar, unsigned nblocks, long long max_polls)
{
    __shared__ unsigned ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* vgen = &bar->gen;
        volatile unsigned* verr = &bar->err;
        unsigned g = *vgen;
        __threadfence();
        unsigned arrived = atomicAdd(&bar->count, 1u);
        if (arrived == nblocks - 1) {
            atomicExch(&bar->count, 0u);
            __threadfence();
            atomicAdd(&bar->gen, 1u);
        } else {
            long long polls = 0;
            while (*vgen == g) {
                if (*verr || ++polls > max_polls) {
                    atomicExch(&bar->err, 1u);
                    break;
                }
                __nanosleep(256);
            }
        }
        __threadfence();
        ok = (*verr == 0);
    }
    __syncthreads();
    return ok != 0;
}

/* nlaunch passes of K (1 or 2) time steps each, separated by grid barriers */
template <int NT, int K>
__global__ void __launch_bounds__(NT) kg_batch_persistent_kernel(const int4* __restrict__ work, int nwork,
                                                                 const KgDev* __restrict__ P,
                                                                 const KgInst* __restrict__ I, double* arena, int from,
                                                                 int bh, int nlaunch, KgBarrier* bar,
                                                                 long long max_polls)
{
    __shared__ typename std::conditional<K == 2, KgSmem2<NT>, KgSmem<NT>>::type sm;
    for (int s = 0; s < nlaunch; s++) {
        for (int k = blockIdx.x; k < nwork; k += gridDim.x) {
            if constexpr (K == 2)
                kg_batch_item2<NT, true>(work[k], P, I, arena, from, bh, sm);
            else
                kg_batch_item<NT, true>(work[k], P, I, arena, from, bh, sm);
            __syncthreads();
        }
        from ^= 1;
        if (s + 1 < nlaunch && !kg_grid_barrier(bar, gridDim.x, max_polls))
            return;
    }
}

struct kg_batch {
    int n = 0;
    std::vector<KgInst> inst;
    std::vector<kg_params> params;
    long long arena_doubles = 0;
    double* arena = nullptr;
    KgDev* d_params = nullptr;
    KgInst* d_inst = nullptr;
    int4* d_work = nullptr;
    int nwork = 0;
    KgBarrier* d_bar = nullptr;
    cudaStream_t stream = nullptr;
    int cur = 0;
    long long steps = 0;
    kg_batch_tuning tune{128, 64, KG_BATCH_LAUNCH, 100, 1, 1};
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    long long cells = 0;
    /* launch mode with tune.streams > 1: the instances are split into groups of about equal cell
     * counts, each advanced on its own stream, so one group's next step overlaps another's tail */
    int ngroups = 1;
    int goff[KG_BATCH_MAX_STREAMS + 1] = {0};
    cudaStream_t gs[KG_BATCH_MAX_STREAMS] = {nullptr};
    cudaEvent_t fork_ev = nullptr;
    cudaEvent_t join_ev[KG_BATCH_MAX_STREAMS] = {nullptr};
    /* set when a grid-barrier wait ran out: kg_batch_step refuses until every instance's state has been
     * replaced since (kg_batch_seed_disks or kg_batch_set_fields with all three fields) */
    bool failed = false;
    std::vector<char> replaced;
};

/* Destroys the instantiated graphs after draining the handle's stream (a graph launched earlier may
 * still be running). */
static void batch_drop_graphs(kg_batch* b)
{
    if (!b->graph[0] && !b->graph[1])
        return;
    if (b->stream)
        cudaStreamSynchronize(b->stream);
    for (int k = 0; k < 2; k++)
        if (b->graph[k]) {
            cudaGraphExecDestroy(b->graph[k]);
            b->graph[k] = nullptr;
        }
}

static int batch_check(const kg_batch* b)
{
    if (!b)
        return kg_fail(KG_ERR_INVALID, "null kg_batch handle");
    return KG_OK;
}

static int valid_tuning(const kg_batch_tuning* t)
{
    if (!(t->nt == 32 || t->nt == 64 || t->nt == 128 || t->nt == 256))
        return kg_fail(KG_ERR_INVALID, "batch tuning: nt must be 32, 64, 128 or 256");
    if (t->bh < 4 || t->bh > 4096)
        return kg_fail(KG_ERR_INVALID, "batch tuning: bh must lie in [4, 4096]");
    if (t->mode != KG_BATCH_LAUNCH && t->mode != KG_BATCH_PERSISTENT)
        return kg_fail(KG_ERR_INVALID, "batch tuning: unknown mode");
    if (t->chunk < 1 || t->chunk > 100000)
        return kg_fail(KG_ERR_INVALID, "batch tuning: chunk must lie in [1, 100000]");
    if (t->streams < 1 || t->streams > KG_BATCH_MAX_STREAMS)
        return kg_fail(KG_ERR_INVALID, "batch tuning: streams must lie in [1, %d]", KG_BATCH_MAX_STREAMS);
    if (t->tblock != 1 && t->tblock != 2)
        return kg_fail(KG_ERR_INVALID, "batch tuning: tblock (steps per pass) must be 1 or 2");
    if (t->tblock == 2 && t->nt > 128)
        return kg_fail(KG_ERR_INVALID, "batch tuning: tblock 2 needs nt <= 128");
    return KG_OK;
}

/* strips of every instance for strip width nt-2 and height bh, largest instances first */
static int build_work(kg_batch* b)
{
    std::vector<int> order(b->n);
    for (int k = 0; k < b->n; k++)
        order[k] = k;
    auto cells = [&](int k) { return (long long)b->inst[k].nx * b->inst[k].ny; };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cells(x) > cells(y); });
    /* groups of about equal total cells (largest instance to the lightest group first) */
    int ng = b->tune.mode == KG_BATCH_LAUNCH ? b->tune.streams : 1;
    if (ng > b->n)
        ng = b->n;
    std::vector<std::vector<int>> groups(ng);
    std::vector<long long> load(ng, 0);
    for (int k : order) {
        int g = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        groups[g].push_back(k);
        load[g] += cells(k);
    }
    std::vector<int4> w;
    const int cw = b->tune.nt - 2 - 4 * (b->tune.tblock - 1); /* output columns per strip */
    for (int g = 0; g < ng; g++) {
        b->goff[g] = (int)w.size();
        for (int k : groups[g]) {
            const KgInst& in = b->inst[k];
            for (int j0 = 0; j0 < in.ny; j0 += b->tune.bh)
                for (int i0 = 0; i0 < in.nx; i0 += cw)
                    w.push_back(make_int4(k, i0, j0, 0));
        }
    }
    b->goff[ng] = (int)w.size();
    b->ngroups = ng;
    for (int g = 0; g < ng && ng > 1; g++) {
        if (!b->gs[g])
            KG_CUDA(cudaStreamCreateWithFlags(&b->gs[g], cudaStreamNonBlocking));
        if (!b->join_ev[g])
            KG_CUDA(cudaEventCreateWithFlags(&b->join_ev[g], cudaEventDisableTiming));
    }
    if (ng > 1 && !b->fork_ev)
        KG_CUDA(cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming));
    if (b->d_work)
        cudaFree(b->d_work);
    b->d_work = nullptr;
    b->nwork = (int)w.size();
    KG_CUDA(cudaMalloc(&b->d_work, sizeof(int4) * w.size()));
    KG_CUDA(cudaMemcpy(b->d_work, w.data(), sizeof(int4) * w.size(), cudaMemcpyHostToDevice));
    return KG_OK;
}

template <int NT, int K>
static cudaError_t launch_range(kg_batch* b, int first, int count, int from, cudaStream_t st)
{
    if constexpr (K == 2)
        kg_batch_step2_kernel<NT><<<count, NT, 0, st>>>(b->d_work + first, b->d_params, b->d_inst, b->arena, from,
                                                        b->tune.bh);
    else
        kg_batch_step_kernel<NT><<<count, NT, 0, st>>>(b->d_work + first, b->d_params, b->d_inst, b->arena, from,
                                                       b->tune.bh);
    return cudaGetLastError();
}

/* one launch of group g advancing k (1 or 2) steps from copy `from` */
static cudaError_t launch_group(kg_batch* b, int g, int from, int k, cudaStream_t st)
{
    int first = b->goff[g], count = b->goff[g + 1] - b->goff[g];
    if (count <= 0)
        return cudaSuccess;
    if (k == 2) {
        switch (b->tune.nt) {
        case 32: return launch_range<32, 2>(b, first, count, from, st);
        case 64: return launch_range<64, 2>(b, first, count, from, st);
        default: return launch_range<128, 2>(b, first, count, from, st);
        }
    }
    switch (b->tune.nt) {
    case 32: return launch_range<32, 1>(b, first, count, from, st);
    case 64: return launch_range<64, 1>(b, first, count, from, st);
    case 256: return launch_range<256, 1>(b, first, count, from, st);
    default: return launch_range<128, 1>(b, first, count, from, st);
    }
}

/* launches that advance n steps with the tuning's temporal blocking factor */
static long long batch_launches_for(const kg_batch* b, long long n)
{
    return b->tune.tblock == 2 ? n / 2 + (n & 1) : n;
}

/* n steps of group g from copy `from` on stream st: k = 2 launches, then a k = 1 launch for an odd rest */
static cudaError_t launch_group_steps(kg_batch* b, int g, int from, long long n, cudaStream_t st)
{
    cudaError_t e = cudaSuccess;
    int c = from;
    for (long long s = 0; s < n && e == cudaSuccess;) {
        const int k = (b->tune.tblock == 2 && n - s >= 2) ? 2 : 1;
        e = launch_group(b, g, c, k, st);
        c ^= 1;
        s += k;
    }
    return e;
}

/* nsteps consecutive steps from copy `from`: on the handle's stream, or forked
 * over the group streams and joined back onto it */
static int batch_launch_steps(kg_batch* b, int from, int nsteps)
{
    cudaError_t e = cudaSuccess;
    if (b->ngroups <= 1) {
        e = launch_group_steps(b, 0, from, nsteps, b->stream);
    } else {
        e = cudaEventRecord(b->fork_ev, b->stream);
        for (int g = 0; g < b->ngroups && e == cudaSuccess; g++) {
            e = cudaStreamWaitEvent(b->gs[g], b->fork_ev, 0);
            if (e == cudaSuccess)
                e = launch_group_steps(b, g, from, nsteps, b->gs[g]);
            if (e == cudaSuccess)
                e = cudaEventRecord(b->join_ev[g], b->gs[g]);
            if (e == cudaSuccess)
                e = cudaStreamWaitEvent(b->stream, b->join_ev[g], 0);
        }
    }
    if (e != cudaSuccess)
        return kg_cuda_fail(e, "kg_batch_step_kernel launch");
    return KG_OK;
}

template <int NT, int K>
static int persistent_run(kg_batch* b, int from, int nlaunch)
{
    int dev = 0, sms = 0, per_sm = 0, coop = 0;
    KG_CUDA(cudaGetDevice(&dev));
    KG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    KG_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop)
        return kg_fail(KG_ERR_CUDA, "persistent batch mode needs cooperative launch support");
    KG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kg_batch_persistent_kernel<NT, K>, NT, 0));
    int grid = std::min(b->nwork, std::max(1, per_sm) * sms);
    /* a wait longer than ~2 s means a CTA is missing: report instead of hanging */
    long long max_polls = 8ll << 20;
    KG_CUDA(cudaMemsetAsync(b->d_bar, 0, sizeof(KgBarrier), b->stream));
    void* args[] = {(void*)&b->d_work, (void*)&b->nwork, (void*)&b->d_params, (void*)&b->d_inst, (void*)&b->arena,
                    (void*)&from, (void*)&b->tune.bh, (void*)&nlaunch, (void*)&b->d_bar, (void*)&max_polls};
    KG_CUDA(cudaLaunchCooperativeKernel((const void*)kg_batch_persistent_kernel<NT, K>, dim3(grid), dim3(NT), args, 0,
                                        b->stream));
    return KG_OK;
}

/* one persistent launch of nlaunch passes of k steps each from copy `from` */
static int batch_persistent(kg_batch* b, int from, int nlaunch, int k)
{
    if (k == 2) {
        switch (b->tune.nt) {
        case 32: return persistent_run<32, 2>(b, from, nlaunch);
        case 64: return persistent_run<64, 2>(b, from, nlaunch);
        default: return persistent_run<128, 2>(b, from, nlaunch);
        }
    }
    switch (b->tune.nt) {
    case 32: return persistent_run<32, 1>(b, from, nlaunch);
    case 64: return persistent_run<64, 1>(b, from, nlaunch);
    case 256: return persistent_run<256, 1>(b, from, nlaunch);
    default: return persistent_run<128, 1>(b, from, nlaunch);
    }
}

static int batch_build_graph(kg_batch* b, int from)
{
    cudaGraph_t g = nullptr;
    KG_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    int rc = batch_launch_steps(b, from, b->tune.chunk);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc != KG_OK) {
        if (g)
            cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess)
        return kg_cuda_fail(e, "batch graph capture");
    e = cudaGraphInstantiate(&b->graph[from], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->graph[from] = nullptr;
        return kg_cuda_fail(e, "batch graph instantiate");
    }
    return KG_OK;
}

/* reads the barrier's error flag after a persistent chunk */
static int batch_check_barrier(kg_batch* b)
{
    KgBarrier h;
    KG_CUDA(cudaMemcpyAsync(&h, b->d_bar, sizeof h, cudaMemcpyDeviceToHost, b->stream));
    KG_CUDA(cudaStreamSynchronize(b->stream));
    if (h.err) {
        b->failed = true;
        std::fill(b->replaced.begin(), b->replaced.end(), 0);
        return kg_fail(KG_ERR_TIMEOUT, "batch: a grid-barrier wait ran out; the chunk did not complete");
    }
    return KG_OK;
}

/* Host-side fault injection for tests: raises the grid barrier's error flag as a CTA whose bounded wait
 * ran out would, and reads it back as kg_batch_step does after a persistent chunk (no kernel runs). */
extern "C" int kg_diag_batch_inject_timeout(kg_batch* b)
{
    if (!b)
        return kg_fail(KG_ERR_INVALID, "null kg_batch handle");
    KgBarrier h{0, 0, 1, 0};
    KG_CUDA(cudaMemcpyAsync(b->d_bar, &h, sizeof h, cudaMemcpyHostToDevice, b->stream));
    return batch_check_barrier(b);
}

/* instance k's state was replaced: the time-out latch clears once every instance's has been */
static void batch_replaced(kg_batch* b, int k)
{
    if (!b->failed)
        return;
    b->replaced[k] = 1;
    if (std::all_of(b->replaced.begin(), b->replaced.end(), [](char c) { return c != 0; }))
        b->failed = false;
}

extern "C" int kg_batch_step(kg_batch* b, long long nsteps)
{
    int rc = batch_check(b);
    if (rc)
        return rc;
    if (nsteps < 0)
        return kg_fail(KG_ERR_INVALID, "kg_batch_step: negative step count");
    if (b->failed)
        return kg_fail(KG_ERR_TIMEOUT, "kg_batch_step: an earlier grid-barrier wait ran out and the state is "
                                       "unreliable; replace it first (kg_batch_seed_disks / kg_batch_set_fields on "
                                       "every instance)");
    if (b->tune.mode == KG_BATCH_PERSISTENT) {
        while (nsteps > 0) {
            int s = (int)std::min<long long>(nsteps, b->tune.chunk);
            /* passes of tblock steps in one launch, then a one-step launch for an odd rest */
            const int k = b->tune.tblock;
            const int passes[2] = {s / k, s % k};
            for (int part = 0; part < 2; part++) {
                if (passes[part] == 0)
                    continue;
                rc = batch_persistent(b, b->cur, passes[part], part == 0 ? k : 1);
                if (rc)
                    return rc;
                rc = batch_check_barrier(b);
                if (rc)
                    return rc;
                b->cur ^= passes[part] & 1;
            }
            b->steps += s;
            nsteps -= s;
        }
        return KG_OK;
    }
    while (nsteps >= b->tune.chunk) {
        if (!b->graph[b->cur]) {
            rc = batch_build_graph(b, b->cur);
            if (rc)
                return rc;
        }
        KG_CUDA(cudaGraphLaunch(b->graph[b->cur], b->stream));
        b->cur ^= (int)(batch_launches_for(b, b->tune.chunk) & 1);
        b->steps += b->tune.chunk;
        nsteps -= b->tune.chunk;
    }
    if (nsteps > 0) {
        rc = batch_launch_steps(b, b->cur, (int)nsteps);
        if (rc)
            return rc;
        b->cur ^= (int)(batch_launches_for(b, nsteps) & 1);
        b->steps += nsteps;
    }
    return KG_OK;
}

extern "C" int kg_batch_destroy(kg_batch* b)
{
    if (!b)
        return KG_OK;
    if (b->stream)
        cudaStreamSynchronize(b->stream);
    batch_drop_graphs(b);
    cudaFree(b->arena);
    cudaFree(b->d_params);
    cudaFree(b->d_inst);
    cudaFree(b->d_work);
    cudaFree(b->d_bar);
    for (int g = 0; g < KG_BATCH_MAX_STREAMS; g++) {
        if (b->gs[g])
            cudaStreamDestroy(b->gs[g]);
        if (b->join_ev[g])
            cudaEventDestroy(b->join_ev[g]);
    }
    if (b->fork_ev)
        cudaEventDestroy(b->fork_ev);
    if (b->stream)
        cudaStreamDestroy(b->stream);
    delete b;
    return KG_OK;
}

extern "C" int kg_batch_create(int n, const int* nx, const int* ny, const kg_params* params, kg_batch** out)
{
    if (!out)
        return kg_fail(KG_ERR_INVALID, "kg_batch_create: null output pointer");
    *out = nullptr;
    if (n < 1 || !nx || !ny || !params)
        return kg_fail(KG_ERR_INVALID, "kg_batch_create: need n >= 1 instances with sizes and parameters");
    std::vector<KgDev> dev(n);
    kg_batch* b = new (std::nothrow) kg_batch();
    if (!b)
        return kg_fail(KG_ERR_NOMEM, "kg_batch_create: host allocation");
    b->n = n;
    b->inst.resize(n);
    b->replaced.assign(n, 0);
    b->params.assign(params, params + n);
    long long off = 0;
    for (int k = 0; k < n; k++) {
        if (nx[k] < 1 || ny[k] < 1 || (long long)nx[k] * ny[k] > (1ll << 32)) {
            delete b;
            return kg_fail(KG_ERR_INVALID, "kg_batch_create: instance %d has size %d x %d", k, nx[k], ny[k]);
        }
        int rc = kg_prepare(&params[k], &dev[k]);
        if (rc) {
            delete b;
            return kg_fail(rc, "kg_batch_create: instance %d: %s", k, kg_last_error());
        }
        b->inst[k].nx = nx[k];
        b->inst[k].ny = ny[k];
        b->inst[k].off = off;
        long long cells = (long long)nx[k] * ny[k];
        b->cells += cells;
        off += 6 * cells;
        off = (off + 31) & ~31ll; /* 256-byte aligned instances */
    }
    b->arena_doubles = off;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaMalloc(&b->arena, sizeof(double) * off);
    if (e == cudaSuccess)
        e = cudaMalloc(&b->d_params, sizeof(KgDev) * n);
    if (e == cudaSuccess)
        e = cudaMalloc(&b->d_inst, sizeof(KgInst) * n);
    if (e == cudaSuccess)
        e = cudaMalloc(&b->d_bar, sizeof(KgBarrier));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_params, dev.data(), sizeof(KgDev) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_inst, b->inst.data(), sizeof(KgInst) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemset(b->arena, 0, sizeof(double) * off);
    if (e == cudaSuccess)
        e = cudaMemset(b->d_bar, 0, sizeof(KgBarrier));
    if (e != cudaSuccess) {
        int rc = kg_cuda_fail(e, "kg_batch_create");
        kg_batch_destroy(b);
        return rc;
    }
    int rc = build_work(b);
    if (rc) {
        kg_batch_destroy(b);
        return rc;
    }
    /* every instance starts from the reference's nucleus */
    for (int k = 0; k < n && rc == KG_OK; k++) {
        int cx = nx[k] / 2, cy = ny[k] / 2, r = 1;
        rc = kg_batch_seed_disks(b, k, 1, &cx, &cy, &r);
    }
    if (rc) {
        kg_batch_destroy(b);
        return rc;
    }
    b->steps = 0;
    *out = b;
    return KG_OK;
}

static int inst_check(const kg_batch* b, int k)
{
    int rc = batch_check(b);
    if (rc)
        return rc;
    if (k < 0 || k >= b->n)
        return kg_fail(KG_ERR_INVALID, "batch: instance %d out of range [0, %d)", k, b->n);
    return KG_OK;
}

extern "C" int kg_batch_seed_disks(kg_batch* b, int k, int n, const int* cx, const int* cy, const int* r)
{
    int rc = inst_check(b, k);
    if (rc)
        return rc;
    const KgInst& in = b->inst[k];
    long long cells = (long long)in.nx * in.ny;
    double* a = b->arena + in.off + (long long)b->cur * 3 * cells;
    rc = kg_seed_device(a, a + cells, a + 2 * cells, in.nx, in.ny, n, cx, cy, r, b->stream);
    if (rc == KG_OK)
        batch_replaced(b, k);
    return rc;
}

extern "C" int kg_batch_get_fields(kg_batch* b, int k, double* phi, double* T, double* theta)
{
    int rc = inst_check(b, k);
    if (rc)
        return rc;
    const KgInst& in = b->inst[k];
    long long cells = (long long)in.nx * in.ny;
    double* a = b->arena + in.off + (long long)b->cur * 3 * cells;
    double* dst[3] = {phi, T, theta};
    for (int f = 0; f < 3; f++)
        if (dst[f])
            KG_CUDA(kg_copy_host(dst[f], a + f * cells, sizeof(double) * cells, cudaMemcpyDeviceToHost, b->stream));
    KG_CUDA(cudaStreamSynchronize(b->stream));
    return KG_OK;
}

extern "C" int kg_batch_set_fields(kg_batch* b, int k, const double* phi, const double* T, const double* theta)
{
    int rc = inst_check(b, k);
    if (rc)
        return rc;
    const KgInst& in = b->inst[k];
    long long cells = (long long)in.nx * in.ny;
    double* a = b->arena + in.off + (long long)b->cur * 3 * cells;
    const double* src[3] = {phi, T, theta};
    for (int f = 0; f < 3; f++)
        if (src[f])
            KG_CUDA(kg_copy_host(a + f * cells, src[f], sizeof(double) * cells, cudaMemcpyHostToDevice, b->stream));
    KG_CUDA(cudaStreamSynchronize(b->stream));
    if (phi && T && theta)
        batch_replaced(b, k);
    return KG_OK;
}

extern "C" int kg_batch_get_info(const kg_batch* b, int* n, long long* cells, long long* steps, int* nwork)
{
    int rc = batch_check(b);
    if (rc)
        return rc;
    if (n)
        *n = b->n;
    if (cells)
        *cells = b->cells;
    if (steps)
        *steps = b->steps;
    if (nwork)
        *nwork = b->nwork;
    return KG_OK;
}

extern "C" int kg_batch_set_tuning(kg_batch* b, const kg_batch_tuning* t)
{
    int rc = batch_check(b);
    if (rc)
        return rc;
    if (!t)
        return kg_fail(KG_ERR_INVALID, "kg_batch_set_tuning: null pointer");
    rc = valid_tuning(t);
    if (rc)
        return rc;
    KG_CUDA(cudaStreamSynchronize(b->stream));
    bool rework = t->nt != b->tune.nt || t->bh != b->tune.bh || t->streams != b->tune.streams ||
                  t->mode != b->tune.mode || t->tblock != b->tune.tblock;
    b->tune = *t;
    batch_drop_graphs(b);
    if (rework)
        return build_work(b);
    return KG_OK;
}

extern "C" int kg_batch_get_tuning(const kg_batch* b, kg_batch_tuning* t)
{
    int rc = batch_check(b);
    if (rc)
        return rc;
    if (!t)
        return kg_fail(KG_ERR_INVALID, "kg_batch_get_tuning: null pointer");
    *t = b->tune;
    return KG_OK;
}

extern "C" int kg_batch_sync(kg_batch* b)
{
    int rc = batch_check(b);
    if (rc)
        return rc;
    KG_CUDA(cudaStreamSynchronize(b->stream));
    return KG_OK;
}

extern "C" int kg_batch_get_stream(kg_batch* b, void** stream)
{
    int rc = batch_check(b);
    if (rc)
        return rc;
    if (!stream)
        return kg_fail(KG_ERR_INVALID, "kg_batch_get_stream: null pointer");
    *stream = (void*)b->stream;
    return KG_OK;
}

/*
 * The autotuner: times `trial_steps` steps of every candidate (strip width,
 * strip height, execution mode) on the batch itself, keeps the fastest, and
 * restores the state it started from, so tuning never changes results.
 */
extern "C" int kg_batch_autotune(kg_batch* b, int trial_steps, kg_batch_tuning* best_out, double* best_ms)
{
    int rc = batch_check(b);
    if (rc)
        return rc;
    if (trial_steps < 1 || trial_steps > 10000)
        return kg_fail(KG_ERR_INVALID, "kg_batch_autotune: trial_steps must lie in [1, 10000]");
    KG_CUDA(cudaStreamSynchronize(b->stream));
    double* saved = nullptr;
    size_t bytes = sizeof(double) * (size_t)b->arena_doubles;
    KG_CUDA(cudaMalloc(&saved, bytes));
    cudaError_t e = cudaMemcpyAsync(saved, b->arena, bytes, cudaMemcpyDeviceToDevice, b->stream);
    const int saved_cur = b->cur;
    const long long saved_steps = b->steps;
    const bool saved_failed = b->failed;
    const kg_batch_tuning orig = b->tune;
    kg_batch_tuning best = orig;
    float best_t = 1e30f;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    if (e == cudaSuccess)
        e = cudaEventCreate(&ev0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&ev1);
    if (e != cudaSuccess) {
        cudaFree(saved);
        return kg_cuda_fail(e, "kg_batch_autotune setup");
    }
    const int nts[3] = {32, 64, 128};
    const int bhs[5] = {4, 8, 16, 32, 64};
    /* (mode, streams): one launch per step; the same over 4, 8 or 16 group streams; persistent */
    const int modes[5][2] = {{KG_BATCH_LAUNCH, 1}, {KG_BATCH_LAUNCH, 4}, {KG_BATCH_LAUNCH, 8}, {KG_BATCH_LAUNCH, 16},
                             {KG_BATCH_PERSISTENT, 1}};
    /* the temporal blocking factor (steps per pass) sets the halo depth: 2 k rows/columns of phi, k of
     * T and theta per side */
    for (int kb = 1; kb <= 2 && rc == KG_OK; kb++)
    for (int mi = 0; mi < 5 && rc == KG_OK; mi++)
        for (int ni = 0; ni < 3 && rc == KG_OK; ni++)
            for (int hi = 0; hi < 5 && rc == KG_OK; hi++) {
                kg_batch_tuning t{nts[ni], bhs[hi], modes[mi][0], trial_steps, modes[mi][1], kb};
                rc = kg_batch_set_tuning(b, &t);
                if (rc)
                    break;
                /* warm-up run (builds the graph), then the timed run from the same state */
                for (int pass = 0; pass < 2 && rc == KG_OK; pass++) {
                    b->cur = saved_cur;
                    cudaMemcpyAsync(b->arena, saved, bytes, cudaMemcpyDeviceToDevice, b->stream);
                    if (pass == 0)
                        rc = kg_batch_step(b, trial_steps);
                }
                if (rc)
                    break;
                cudaEventRecord(ev0, b->stream);
                rc = kg_batch_step(b, trial_steps);
                cudaEventRecord(ev1, b->stream);
                if (rc)
                    break;
                e = cudaEventSynchronize(ev1);
                if (e != cudaSuccess) {
                    rc = kg_cuda_fail(e, "kg_batch_autotune trial");
                    break;
                }
                float ms = 0;
                cudaEventElapsedTime(&ms, ev0, ev1);
                if (ms < best_t) {
                    best_t = ms;
                    best = t;
                }
            }
    /* restore the state and install the winner with the caller's chunk length (a trial that timed out
     * only ran on a copy: the restored state is the caller's own) */
    b->cur = saved_cur;
    b->steps = saved_steps;
    b->failed = saved_failed;
    cudaMemcpyAsync(b->arena, saved, bytes, cudaMemcpyDeviceToDevice, b->stream);
    cudaStreamSynchronize(b->stream);
    cudaFree(saved);
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    if (rc)
        return rc;
    best.chunk = orig.chunk;
    rc = kg_batch_set_tuning(b, &best);
    if (rc)
        return rc;
    if (best_out)
        *best_out = best;
    if (best_ms)
        *best_ms = best_t / trial_steps;
    return KG_OK;
}

/* A grid barrier that can never complete (it expects one CTA more than the
 * grid has): every wait must run out after max_polls polls and raise the
 * error flag, and the kernel must end. */
__global__ void kg_diag_barrier_kernel(KgBarrier* bar, unsigned expect, long long max_polls)
{
    kg_grid_barrier(bar, expect, max_polls);
}

extern "C" int kg_diag_barrier_timeout(int blocks, long long max_polls, int* timed_out)
{
    if (blocks < 1 || blocks > 64 || max_polls < 1 || max_polls > (1ll << 26) || !timed_out)
        return kg_fail(KG_ERR_INVALID, "kg_diag_barrier_timeout: bad arguments");
    KgBarrier* bar = nullptr;
    KG_CUDA(cudaMalloc(&bar, sizeof(KgBarrier)));
    cudaError_t e = cudaMemset(bar, 0, sizeof(KgBarrier));
    if (e == cudaSuccess) {
        unsigned expect = (unsigned)blocks + 1;
        void* args[] = {(void*)&bar, (void*)&expect, (void*)&max_polls};
        e = cudaLaunchCooperativeKernel((const void*)kg_diag_barrier_kernel, dim3(blocks), dim3(32), args, 0, 0);
    }
    KgBarrier h{};
    if (e == cudaSuccess)
        e = cudaMemcpy(&h, bar, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(bar);
    if (e != cudaSuccess)
        return kg_cuda_fail(e, "kg_diag_barrier_timeout");
    *timed_out = h.err != 0;
    return KG_OK;
}

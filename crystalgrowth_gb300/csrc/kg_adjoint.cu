/*
 * kg_adjoint.cu -- hand-written reverse mode of the fused Kobayashi step.
 *
 * Forward step at a cell c (src/Kobayashi.cpp:139-215, theta0 extension):
 *   gx = (phi_E - phi_W)/dx, gy = (phi_N - phi_S)/dy, theta' = branch(gx, gy, theta)
 *   psi = j (theta' - theta0), eps = eb (1 + delta cos psi), eps' = -eb j delta sin psi
 *   e2 = eps^2, a = eps eps' gx, b = eps eps' gy
 *   R = (a_N - a_S)/dy - (b_E - b_W)/dx + e2 lap(phi) + gEx gx + gEy gy + W
 *       gEx = (e2_E - e2_W)/dx, gEy = (e2_N - e2_S)/dy, W = phi (1-phi)(phi - 1/2 + m)
 *   m = (alpha/pi) atan(gamma (Teq - T))
 *   phi' = phi + R dt / tau,  T' = T + lap(T) dt + K (phi' - phi)
 *
 * Reverse of one step, given the adjoints (lphi', lT', ltheta') of the next
 * state, in gather passes over the tape of the step (A and B run as one
 * kernel, kg_adj_pass_ab, which recomputes the neighbours' lR):
 *   A (local):  lR = (lphi' + K lT') dt/tau, the Laplacian seeds lR e2 and lT' dt,
 *               the local parts of lphi and lT, and the K, tau, gamma gradients;
 *   B (radius 1): the adjoints of e2, a, b gathered from the neighbours' lR,
 *               then eps, eps', psi, theta' and gx, gy; the delta and theta0
 *               gradients; ltheta (the dead zone passes ltheta' through);
 *   C (radius 1): lphi and lT gathered from the neighbours' gx/gy adjoints and
 *               Laplacian seeds.
 * The adjoint is checked against central finite differences and a separate
 * CPU tangent-linear model; it does not need to match anything bit for bit,
 * so its divisions by constants are multiplications by reciprocals.
 */
#include <math.h>
#include <new>
#include <string.h>
#include <vector>
#include "kg_common.h"
#include "kobayashi_adjoint.h"

#define KG_ADJ_BLOCKS 608
#define KG_ADJ_THREADS 256
#define KG_NPARAM 5 /* delta, K, theta0, tau, gamma */

struct KgAdj {
    double inv_dx, inv_dy, inv_lap, dt, dt_tau, tau, K, eb, delta, j, a_pi, gamma, teq, u0, inv0;
    /* products of parameters the reverse passes use per cell */
    double inv_tau, eb_delta, k_e, k_d, k_j, a_pi_gamma, a_pi_teq;
};

template <int NT>
__global__ void __launch_bounds__(NT) kg_tape_step_kernel(const __grid_constant__ KgDev P, int nx, int ny, int bh,
                                                          const double* __restrict__ phi_in,
                                                          const double* __restrict__ t_in,
                                                          const double* __restrict__ th_in, double* __restrict__ phi_out,
                                                          double* __restrict__ t_out, double* __restrict__ th_out,
                                                          const __grid_constant__ KgTape tape)
{
    __shared__ KgSmem<NT> sm;
    kg_strip<NT, true>(P, nx, ny, phi_in, t_in, th_in, phi_out, t_out, th_out, blockIdx.x * (NT - 2),
                       blockIdx.y * bh, bh, sm, &tape);
}

/* block sum of KG_NPARAM values into part[blockIdx.x * KG_NPARAM + k] (fixed order) */
__device__ void kg_block_accumulate(double v[KG_NPARAM], double* part)
{
    __shared__ double red[KG_ADJ_THREADS][KG_NPARAM];
    for (int k = 0; k < KG_NPARAM; k++)
        red[threadIdx.x][k] = v[k];
    __syncthreads();
    for (int s = KG_ADJ_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int k = 0; k < KG_NPARAM; k++)
                red[threadIdx.x][k] += red[threadIdx.x + s][k];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < KG_NPARAM; k++)
            part[blockIdx.x * KG_NPARAM + k] += red[0][k];
}

struct KgAdjWork {
    double *lLphi, *lLT, *lphi_loc, *lT_loc, *lgx, *lgy;
};

__device__ __forceinline__ long long kg_nb(int i, int j, int nx) { return (long long)j * nx + i; }

/* Passes A and B in one sweep: the neighbours' lR = (lphi' + K lT') dt/tau is
 * recomputed from the next step's adjoints instead of being read back. */
__global__ void __launch_bounds__(KG_ADJ_THREADS) kg_adj_pass_ab(const __grid_constant__ KgAdj A, int nx, int ny,
                                                                 const __grid_constant__ KgTape tp,
                                                                 const double* __restrict__ phi_next,
                                                                 const double* __restrict__ lphi1,
                                                                 const double* __restrict__ lt1,
                                                                 const double* __restrict__ lth1,
                                                                 double* __restrict__ lth0,
                                                                 const __grid_constant__ KgAdjWork w, double* part)
{
    const long long N = (long long)nx * ny;
    double g[KG_NPARAM] = {0, 0, 0, 0, 0};
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        int i = (int)(c % nx), j = (int)(c / nx);
        int ip = i + 1 == nx ? 0 : i + 1, im = i == 0 ? nx - 1 : i - 1;
        int jp = j + 1 == ny ? 0 : j + 1, jm = j == 0 ? ny - 1 : j - 1;
        long long cE = kg_nb(ip, j, nx), cW = kg_nb(im, j, nx), cN = kg_nb(i, jp, nx), cS = kg_nb(i, jm, nx);
        /* pass A at c (explicit FMAs: the adjoint is checked to a tolerance, not bit for bit) */
        double phi = tp.f[KG_TAPE_PHI][c], t = tp.f[KG_TAPE_T][c];
        double lap = tp.f[KG_TAPE_LAP][c], R = tp.f[KG_TAPE_RHS][c], m = tp.f[KG_TAPE_M][c];
        double s = tp.f[KG_TAPE_SIN][c], co = tp.f[KG_TAPE_COS][c];
        double eps = kg_fma(A.eb_delta, co, A.eb);
        double lp = lphi1[c], lt = lt1[c];
        double lRc = kg_fma(A.K, lt, lp) * A.dt_tau;
        double q = (phi - 0.5) + m;
        double pp = kg_fma(-phi, phi, phi);                  /* phi (1 - phi) */
        double dw = kg_fma(kg_fma(-2.0, phi, 1.0), q, pp);   /* (1 - 2 phi) q + phi (1 - phi) */
        double lm = lRc * pp;
        double u = A.gamma * (A.teq - t);
        double inv = (u == A.u0) ? A.inv0 : kg_gdiv(1.0, kg_fma(u, u, 1.0));
        double lmi = lm * inv;
        w.lLphi[c] = lRc * (eps * eps);
        w.lLT[c] = lt * A.dt;
        w.lphi_loc[c] = kg_fma(lRc, dw, lp);
        w.lT_loc[c] = kg_fma(-lmi, A.a_pi_gamma, lt);
        g[1] = kg_fma(lt, phi_next[c] - phi, g[1]);
        g[3] = kg_fma(-lRc, R * A.inv_tau, g[3]);
        g[4] = kg_fma(lmi, kg_fma(-A.a_pi, t, A.a_pi_teq), g[4]);
        /* pass B at c, with the neighbours' lR recomputed */
        double lRE = kg_fma(A.K, lt1[cE], lphi1[cE]) * A.dt_tau, lRW = kg_fma(A.K, lt1[cW], lphi1[cW]) * A.dt_tau;
        double lRN = kg_fma(A.K, lt1[cN], lphi1[cN]) * A.dt_tau, lRS = kg_fma(A.K, lt1[cS], lphi1[cS]) * A.dt_tau;
        const double* GX = tp.f[KG_TAPE_GX];
        const double* GY = tp.f[KG_TAPE_GY];
        double gx = GX[c], gy = GY[c];
        double dxx = kg_fma(lRW, GX[cW], -(lRE * GX[cE]));
        double dyy = kg_fma(lRS, GY[cS], -(lRN * GY[cN]));
        double le2 = kg_fma(dxx, A.inv_dx, kg_fma(dyy, A.inv_dy, lRc * lap));
        double la = (lRS - lRN) * A.inv_dy;
        double lb = (lRE - lRW) * A.inv_dx;
        double epsd = A.k_d * s;
        double ee = eps * epsd;
        double lq = kg_fma(la, gx, lb * gy);
        double leps = kg_fma(eps + eps, le2, epsd * lq);
        double lepsd = eps * lq;
        double lgx = kg_fma(lRc, tp.f[KG_TAPE_GEX][c], la * ee);
        double lgy = kg_fma(lRc, tp.f[KG_TAPE_GEY][c], lb * ee);
        double lpsi = kg_fma(leps, A.k_e * s, lepsd * (A.k_d * co));
        g[0] = kg_fma(leps, A.eb * co, kg_fma(lepsd, A.k_j * s, g[0]));
        g[2] = kg_fma(-A.j, lpsi, g[2]);
        double lthp = kg_fma(A.j, lpsi, lth1[c]);
        uint64_t bx = kg_bits(gx), by = kg_bits(gy);
        bool gx_small = kg_small(bx), gx_pos = kg_pos_big(bx), gx_neg = kg_neg_big(bx);
        bool gy_big = kg_pos_big(by) || kg_neg_big(by);
        double lth = 0.0;
        if (gx_neg || (gx_pos && gy_big)) {
            /* d atan(gy/gx) = (gx dgy - gy dgx) / (gx^2 + gy^2) */
            double tr = lthp * kg_gdiv(1.0, kg_fma(gx, gx, gy * gy));
            lgx = kg_fma(-gy, tr, lgx);
            lgy = kg_fma(gx, tr, lgy);
        } else if (!(gx_small && gy_big)) {
            lth = lthp;
        }
        w.lgx[c] = lgx;
        w.lgy[c] = lgy;
        lth0[c] = lth;
    }
    kg_block_accumulate(g, part);
}

__global__ void __launch_bounds__(KG_ADJ_THREADS) kg_adj_pass_c(const __grid_constant__ KgAdj A, int nx, int ny,
                                                                const __grid_constant__ KgAdjWork w,
                                                                double* __restrict__ lphi0, double* __restrict__ lt0)
{
    const long long N = (long long)nx * ny;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        int i = (int)(c % nx), j = (int)(c / nx);
        int ip = i + 1 == nx ? 0 : i + 1, im = i == 0 ? nx - 1 : i - 1;
        int jp = j + 1 == ny ? 0 : j + 1, jm = j == 0 ? ny - 1 : j - 1;
        long long cE = kg_nb(ip, j, nx), cW = kg_nb(im, j, nx), cN = kg_nb(i, jp, nx), cS = kg_nb(i, jm, nx);
        long long cNE = kg_nb(ip, jp, nx), cNW = kg_nb(im, jp, nx), cSE = kg_nb(ip, jm, nx), cSW = kg_nb(im, jm, nx);
        /* the transposed 9-point Laplacians (the stencil is symmetric), with explicit FMAs */
        double sp = kg_fma(2.0, (w.lLphi[cE] + w.lLphi[cW]) + (w.lLphi[cN] + w.lLphi[cS]),
                           (w.lLphi[cNE] + w.lLphi[cNW]) + (w.lLphi[cSE] + w.lLphi[cSW]));
        sp = kg_fma(-12.0, w.lLphi[c], sp);
        double st = kg_fma(2.0, (w.lLT[cE] + w.lLT[cW]) + (w.lLT[cN] + w.lLT[cS]),
                           (w.lLT[cNE] + w.lLT[cNW]) + (w.lLT[cSE] + w.lLT[cSW]));
        st = kg_fma(-12.0, w.lLT[c], st);
        double v = kg_fma(w.lgx[cW] - w.lgx[cE], A.inv_dx, w.lphi_loc[c]);
        v = kg_fma(w.lgy[cS] - w.lgy[cN], A.inv_dy, v);
        lphi0[c] = kg_fma(sp, A.inv_lap, v);
        lt0[c] = kg_fma(st, A.inv_lap, w.lT_loc[c]);
    }
}

/* lambda_phi = phi_N - target, lambda_T = lambda_theta = 0; block partial sums of 0.5 (phi_N - target)^2 */
__global__ void __launch_bounds__(KG_ADJ_THREADS) kg_adj_seed(long long N, const double* __restrict__ phi,
                                                              const double* __restrict__ target, double* lphi,
                                                              double* lt, double* lth, double* part)
{
    __shared__ double red[KG_ADJ_THREADS];
    double acc = 0.0;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < N; c += (long long)gridDim.x * blockDim.x) {
        double d = phi[c] - target[c];
        acc += 0.5 * d * d;
        if (lphi) {
            lphi[c] = d;
            lt[c] = 0.0;
            lth[c] = 0.0;
        }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = KG_ADJ_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        part[blockIdx.x] = red[0];
}

struct kg_adjoint {
    int nx = 0, ny = 0;
    long long N = 0, nsteps = 0;
    int k = 64, ncp = 0, nt = 128, bh = 64;
    kg_params p{};
    KgDev dev{};
    KgAdj adj{};
    cudaStream_t stream = nullptr;
    double* init = nullptr;   /* 3N */
    double* target = nullptr; /* N */
    double* cps = nullptr;    /* ncp * 3N */
    double* st = nullptr;     /* 2 * 3N */
    double* tape = nullptr;   /* k * KG_TAPE_FIELDS * N */
    double* lam = nullptr;    /* 2 * 3N */
    double* work = nullptr;   /* 6N */
    double* part = nullptr;   /* KG_ADJ_BLOCKS * KG_NPARAM + KG_ADJ_BLOCKS */
};

static int adj_prepare(kg_adjoint* a, const kg_params* p)
{
    KgDev dev;
    int rc = kg_prepare(p, &dev);
    if (rc)
        return rc;
    a->p = *p;
    a->dev = dev;
    KgAdj& A = a->adj;
    A.inv_dx = 1.0 / p->dx;
    A.inv_dy = 1.0 / p->dy;
    A.inv_lap = 1.0 / (3.0 * p->dx * p->dx);
    A.dt = p->dt;
    A.dt_tau = p->dt / p->tau;
    A.tau = p->tau;
    A.K = p->K;
    A.eb = p->eps_bar;
    A.delta = p->delta;
    A.j = p->aniso;
    A.a_pi = p->alpha / KG_PI;
    A.gamma = p->gamma;
    A.teq = p->teq;
    A.u0 = p->gamma * (p->teq - 0.0);
    A.inv0 = 1.0 / (1.0 + A.u0 * A.u0);
    A.inv_tau = 1.0 / p->tau;
    A.eb_delta = p->eps_bar * p->delta;            /* eps = eb + eb delta cos(psi) */
    A.k_e = -p->eps_bar * p->delta;                /* d eps / d psi = k_e sin(psi) */
    A.k_d = -p->eps_bar * p->aniso * p->delta;     /* eps' = k_d sin(psi); d eps'/d psi = k_d cos(psi) */
    A.k_j = -p->eps_bar * p->aniso;                /* d eps' / d delta = k_j sin(psi) */
    A.a_pi_gamma = A.a_pi * p->gamma;
    A.a_pi_teq = A.a_pi * p->teq;
    return KG_OK;
}

extern "C" int kg_adjoint_destroy(kg_adjoint* a)
{
    if (!a)
        return KG_OK;
    if (a->stream)
        cudaStreamSynchronize(a->stream);
    double* bufs[] = {a->init, a->target, a->cps, a->st, a->tape, a->lam, a->work, a->part};
    for (double* b : bufs)
        if (b)
            cudaFree(b);
    if (a->stream)
        cudaStreamDestroy(a->stream);
    delete a;
    return KG_OK;
}

extern "C" int kg_adjoint_create(int nx, int ny, const kg_params* p, long long nsteps, int checkpoint_every,
                                 kg_adjoint** out)
{
    if (!out)
        return kg_fail(KG_ERR_INVALID, "kg_adjoint_create: null output pointer");
    *out = nullptr;
    if (nx < 1 || ny < 1 || (long long)nx * ny > (1ll << 30) || nsteps < 1 || checkpoint_every < 1)
        return kg_fail(KG_ERR_INVALID, "kg_adjoint_create: bad sizes");
    kg_adjoint* a = new (std::nothrow) kg_adjoint();
    if (!a)
        return kg_fail(KG_ERR_NOMEM, "kg_adjoint_create: host allocation");
    int rc = adj_prepare(a, p);
    if (rc) {
        delete a;
        return rc;
    }
    a->nx = nx;
    a->ny = ny;
    a->N = (long long)nx * ny;
    a->nsteps = nsteps;
    a->k = (int)(checkpoint_every < nsteps ? checkpoint_every : nsteps);
    a->ncp = (int)((nsteps + a->k - 1) / a->k);
    kg_pick_tile(nx, ny, &a->nt, &a->bh);
    const size_t N = (size_t)a->N, d = sizeof(double);
    cudaError_t e = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaMalloc(&a->init, 3 * N * d);
    if (e == cudaSuccess)
        e = cudaMalloc(&a->target, N * d);
    if (e == cudaSuccess)
        e = cudaMalloc(&a->cps, (size_t)a->ncp * 3 * N * d);
    if (e == cudaSuccess)
        e = cudaMalloc(&a->st, 6 * N * d);
    if (e == cudaSuccess)
        e = cudaMalloc(&a->tape, (size_t)a->k * KG_TAPE_FIELDS * N * d);
    if (e == cudaSuccess)
        e = cudaMalloc(&a->lam, 6 * N * d);
    if (e == cudaSuccess)
        e = cudaMalloc(&a->work, 6 * N * d);
    if (e == cudaSuccess)
        e = cudaMalloc(&a->part, (KG_ADJ_BLOCKS * KG_NPARAM + KG_ADJ_BLOCKS) * d);
    if (e == cudaSuccess)
        e = cudaMemset(a->init, 0, 3 * N * d);
    if (e == cudaSuccess)
        e = cudaMemset(a->target, 0, N * d);
    if (e != cudaSuccess) {
        rc = kg_cuda_fail(e, "kg_adjoint_create");
        kg_adjoint_destroy(a);
        return rc;
    }
    *out = a;
    return KG_OK;
}

static int adj_check(const kg_adjoint* a)
{
    if (!a)
        return kg_fail(KG_ERR_INVALID, "null kg_adjoint handle");
    return KG_OK;
}

extern "C" int kg_adjoint_set_params(kg_adjoint* a, const kg_params* p)
{
    int rc = adj_check(a);
    return rc ? rc : adj_prepare(a, p);
}

extern "C" int kg_adjoint_set_initial(kg_adjoint* a, const double* phi0, const double* T0, const double* theta0)
{
    int rc = adj_check(a);
    if (rc)
        return rc;
    if (!phi0 || !T0)
        return kg_fail(KG_ERR_INVALID, "kg_adjoint_set_initial: phi0 and T0 are required");
    size_t bytes = sizeof(double) * (size_t)a->N;
    KG_CUDA(cudaMemcpyAsync(a->init, phi0, bytes, cudaMemcpyHostToDevice, a->stream));
    KG_CUDA(cudaMemcpyAsync(a->init + a->N, T0, bytes, cudaMemcpyHostToDevice, a->stream));
    if (theta0)
        KG_CUDA(cudaMemcpyAsync(a->init + 2 * a->N, theta0, bytes, cudaMemcpyHostToDevice, a->stream));
    else
        KG_CUDA(cudaMemsetAsync(a->init + 2 * a->N, 0, bytes, a->stream));
    KG_CUDA(cudaStreamSynchronize(a->stream));
    return KG_OK;
}

extern "C" int kg_adjoint_set_target(kg_adjoint* a, const double* phi_target)
{
    int rc = adj_check(a);
    if (rc)
        return rc;
    if (!phi_target)
        return kg_fail(KG_ERR_INVALID, "kg_adjoint_set_target: null pointer");
    KG_CUDA(cudaMemcpy(a->target, phi_target, sizeof(double) * (size_t)a->N, cudaMemcpyHostToDevice));
    return KG_OK;
}

extern "C" int kg_adjoint_get_stream(kg_adjoint* a, void** stream)
{
    int rc = adj_check(a);
    if (rc)
        return rc;
    if (!stream)
        return kg_fail(KG_ERR_INVALID, "kg_adjoint_get_stream: null pointer");
    *stream = (void*)a->stream;
    return KG_OK;
}

template <int NT>
__global__ void __launch_bounds__(NT) kg_adj_fwd_kernel(const __grid_constant__ KgDev P, int nx, int ny, int bh,
                                                        const double* __restrict__ phi_in,
                                                        const double* __restrict__ t_in,
                                                        const double* __restrict__ th_in, double* __restrict__ phi_out,
                                                        double* __restrict__ t_out, double* __restrict__ th_out)
{
    __shared__ KgSmem<NT> sm;
    kg_strip<NT>(P, nx, ny, phi_in, t_in, th_in, phi_out, t_out, th_out, blockIdx.x * (NT - 2), blockIdx.y * bh, bh,
                 sm);
}

static dim3 adj_grid(const kg_adjoint* a)
{
    return dim3((a->nx + a->nt - 3) / (a->nt - 2), (a->ny + a->bh - 1) / a->bh);
}

static double* st_ptr(kg_adjoint* a, int c) { return a->st + (size_t)c * 3 * a->N; }

/* forward rollout from the initial state with checkpoints; returns the index of the final state's copy */
static int adj_forward(kg_adjoint* a, int* cur_out)
{
    const size_t N = (size_t)a->N, bytes3 = 3 * N * sizeof(double);
    KG_CUDA(cudaMemcpyAsync(st_ptr(a, 0), a->init, bytes3, cudaMemcpyDeviceToDevice, a->stream));
    int cur = 0;
    for (long long n = 0; n < a->nsteps; n++) {
        if (n % a->k == 0)
            KG_CUDA(cudaMemcpyAsync(a->cps + (size_t)(n / a->k) * 3 * N, st_ptr(a, cur), bytes3,
                                    cudaMemcpyDeviceToDevice, a->stream));
        double* s = st_ptr(a, cur);
        double* d = st_ptr(a, cur ^ 1);
        if (a->nt == 32)
            kg_adj_fwd_kernel<32><<<adj_grid(a), 32, 0, a->stream>>>(a->dev, a->nx, a->ny, a->bh, s, s + N, s + 2 * N,
                                                                      d, d + N, d + 2 * N);
        else if (a->nt == 64)
            kg_adj_fwd_kernel<64><<<adj_grid(a), 64, 0, a->stream>>>(a->dev, a->nx, a->ny, a->bh, s, s + N, s + 2 * N,
                                                                      d, d + N, d + 2 * N);
        else
            kg_adj_fwd_kernel<128><<<adj_grid(a), 128, 0, a->stream>>>(a->dev, a->nx, a->ny, a->bh, s, s + N,
                                                                        s + 2 * N, d, d + N, d + 2 * N);
        cur ^= 1;
    }
    KG_CUDA(cudaGetLastError());
    *cur_out = cur;
    return KG_OK;
}

static int adj_loss(kg_adjoint* a, const double* phi, double* loss, bool seed)
{
    const size_t N = (size_t)a->N;
    kg_adj_seed<<<KG_ADJ_BLOCKS, KG_ADJ_THREADS, 0, a->stream>>>(a->N, phi, a->target, seed ? a->lam : nullptr,
                                                                 a->lam + N, a->lam + 2 * N,
                                                                 a->part + KG_ADJ_BLOCKS * KG_NPARAM);
    KG_CUDA(cudaGetLastError());
    std::vector<double> h(KG_ADJ_BLOCKS);
    KG_CUDA(cudaMemcpyAsync(h.data(), a->part + KG_ADJ_BLOCKS * KG_NPARAM, sizeof(double) * KG_ADJ_BLOCKS,
                            cudaMemcpyDeviceToHost, a->stream));
    KG_CUDA(cudaStreamSynchronize(a->stream));
    double s = 0.0;
    for (double v : h)
        s += v;
    *loss = s;
    return KG_OK;
}

extern "C" int kg_adjoint_forward(kg_adjoint* a, double* loss, double* phi_N, double* T_N, double* theta_N)
{
    int rc = adj_check(a);
    if (rc)
        return rc;
    int cur = 0;
    rc = adj_forward(a, &cur);
    if (rc)
        return rc;
    const size_t N = (size_t)a->N;
    double* s = st_ptr(a, cur);
    double l = 0.0;
    rc = adj_loss(a, s, &l, false);
    if (rc)
        return rc;
    if (loss)
        *loss = l;
    double* dst[3] = {phi_N, T_N, theta_N};
    for (int f = 0; f < 3; f++)
        if (dst[f])
            KG_CUDA(cudaMemcpyAsync(dst[f], s + f * N, N * sizeof(double), cudaMemcpyDeviceToHost, a->stream));
    KG_CUDA(cudaStreamSynchronize(a->stream));
    return KG_OK;
}

static KgTape tape_slot(kg_adjoint* a, int t)
{
    KgTape tp;
    for (int f = 0; f < KG_TAPE_FIELDS; f++)
        tp.f[f] = a->tape + ((size_t)t * KG_TAPE_FIELDS + f) * (size_t)a->N;
    return tp;
}

extern "C" int kg_adjoint_gradient(kg_adjoint* a, kg_grad_result* out, double* dL_dT0)
{
    int rc = adj_check(a);
    if (rc)
        return rc;
    if (!out)
        return kg_fail(KG_ERR_INVALID, "kg_adjoint_gradient: null result pointer");
    const size_t N = (size_t)a->N, bytes3 = 3 * N * sizeof(double);
    int cur = 0;
    rc = adj_forward(a, &cur);
    if (rc)
        return rc;
    double loss = 0.0;
    rc = adj_loss(a, st_ptr(a, cur), &loss, true);
    if (rc)
        return rc;
    KG_CUDA(cudaMemsetAsync(a->part, 0, sizeof(double) * KG_ADJ_BLOCKS * KG_NPARAM, a->stream));
    KgAdjWork w;
    w.lLphi = a->work;
    w.lLT = a->work + N;
    w.lphi_loc = a->work + 2 * N;
    w.lT_loc = a->work + 3 * N;
    w.lgx = a->work + 4 * N;
    w.lgy = a->work + 5 * N;
    int lc = 0; /* lam copy holding the adjoint of the state after the current step */
    for (int seg = a->ncp - 1; seg >= 0; seg--) {
        long long n0 = (long long)seg * a->k, n1 = n0 + a->k < a->nsteps ? n0 + a->k : a->nsteps;
        KG_CUDA(cudaMemcpyAsync(st_ptr(a, 0), a->cps + (size_t)seg * 3 * N, bytes3, cudaMemcpyDeviceToDevice,
                                a->stream));
        int c = 0;
        for (long long n = n0; n < n1; n++) {
            double* s = st_ptr(a, c);
            double* d = st_ptr(a, c ^ 1);
            if (a->nt == 32)
                kg_tape_step_kernel<32><<<adj_grid(a), 32, 0, a->stream>>>(a->dev, a->nx, a->ny, a->bh, s, s + N,
                                                                            s + 2 * N, d, d + N, d + 2 * N,
                                                                            tape_slot(a, (int)(n - n0)));
            else if (a->nt == 64)
                kg_tape_step_kernel<64><<<adj_grid(a), 64, 0, a->stream>>>(a->dev, a->nx, a->ny, a->bh, s, s + N,
                                                                            s + 2 * N, d, d + N, d + 2 * N,
                                                                            tape_slot(a, (int)(n - n0)));
            else
                kg_tape_step_kernel<128><<<adj_grid(a), 128, 0, a->stream>>>(a->dev, a->nx, a->ny, a->bh, s, s + N,
                                                                              s + 2 * N, d, d + N, d + 2 * N,
                                                                              tape_slot(a, (int)(n - n0)));
            c ^= 1;
        }
        KG_CUDA(cudaGetLastError());
        const double* phi_end = st_ptr(a, c); /* phi at step n1 */
        for (long long n = n1 - 1; n >= n0; n--) {
            KgTape tp = tape_slot(a, (int)(n - n0));
            const double* phi_next = (n + 1 == n1) ? phi_end : tape_slot(a, (int)(n + 1 - n0)).f[KG_TAPE_PHI];
            double* l1 = a->lam + (size_t)lc * 3 * N;
            double* l0 = a->lam + (size_t)(lc ^ 1) * 3 * N;
            kg_adj_pass_ab<<<KG_ADJ_BLOCKS, KG_ADJ_THREADS, 0, a->stream>>>(a->adj, a->nx, a->ny, tp, phi_next, l1,
                                                                            l1 + N, l1 + 2 * N, l0 + 2 * N, w, a->part);
            kg_adj_pass_c<<<KG_ADJ_BLOCKS, KG_ADJ_THREADS, 0, a->stream>>>(a->adj, a->nx, a->ny, w, l0, l0 + N);
            lc ^= 1;
        }
        KG_CUDA(cudaGetLastError());
    }
    std::vector<double> h(KG_ADJ_BLOCKS * KG_NPARAM);
    KG_CUDA(cudaMemcpyAsync(h.data(), a->part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, a->stream));
    if (dL_dT0)
        KG_CUDA(cudaMemcpyAsync(dL_dT0, a->lam + (size_t)lc * 3 * N + N, N * sizeof(double), cudaMemcpyDeviceToHost,
                                a->stream));
    KG_CUDA(cudaStreamSynchronize(a->stream));
    double g[KG_NPARAM] = {0, 0, 0, 0, 0};
    for (int b = 0; b < KG_ADJ_BLOCKS; b++)
        for (int k = 0; k < KG_NPARAM; k++)
            g[k] += h[b * KG_NPARAM + k];
    out->loss = loss;
    out->d_delta = g[0];
    out->d_K = g[1];
    out->d_theta0 = g[2];
    out->d_tau = g[3];
    out->d_gamma = g[4];
    return KG_OK;
}

/*
 * ko_oracle.c -- TEST INFRASTRUCTURE ONLY (the "O2" oracle).
 *
 * A plain-C, FP64 restatement of the reference's Kobayashi time step
 * (jklae/CrystalGrowth src/Kobayashi.cpp), used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 * It is never linked into the product library.
 *
 * It follows the reference loop by loop and operation by operation, so that,
 * with the C library's atan/sin/cos selected (libm = 1), it reproduces the
 * FP64 build of the reference's own code bit for bit:
 *   stage 1  _computeGradientLaplacian   src/Kobayashi.cpp:125-175
 *   stage 2  _evolution (in place)       src/Kobayashi.cpp:177-221
 * The only extension is theta0, the preferred growth angle: the anisotropy
 * argument is aniso*(theta - theta0), which is bit-identical to the
 * reference's aniso*theta when theta0 == 0.
 *
 * With libm = 0 the elementary functions come from kg_math.h, the definitions
 * the GPU kernels share; that is the configuration the GPU is compared with.
 * Build with -ffp-contract=off (no fused multiply-add contraction).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "../crystalgrowth_gb300/csrc/kg_math.h"

typedef struct ko_params {
    double dx, dy, dt;
    double tau, eps_bar, mu, K, delta, aniso, alpha, gamma, teq;
    double theta0;
} ko_params;

/* FLT_EPSILON (src/Kobayashi.cpp:154-167) as a double: 2^-23 */
#define KO_FLT_EPS 0x1p-23

static inline double ko_atan(double x, int libm) { return libm ? atan(x) : kg_atan(x); }

/* A one-entry memo of a pure function: the same argument bits give the same
 * result bits, so reusing the last result when the argument repeats changes
 * nothing.  It only saves time: most cells of a run share one sin/cos
 * argument (theta = 0) and one atan argument (T too small to change Teq - T). */
typedef struct ko_memo {
    uint64_t key;
    int valid;
    double a, b;
} ko_memo;

static inline uint64_t ko_bits(double x)
{
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
}

static inline void ko_sincos(double x, double* s, double* c, int libm)
{
    if (libm) {
        *s = sin(x);
        *c = cos(x);
    } else {
        kg_sincos(x, s, c);
    }
}

/* periodic neighbour indices, src/Kobayashi.cpp:133-136 */
#define KO_WRAP(i, n) (((i) % (n) + (n)) % (n))

static void ko_stage1(int nx, int ny, const ko_params* p, const double* phi, const double* t, double* angl,
                      double* gpx, double* gpy, double* lphi, double* lt, double* eps, double* epsd, int libm,
                      int nthreads)
{
    const double pi = KG_PI; /* PI_F: DXViewer's constant is not vendored; RN(pi) */
    (void)nthreads;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int j = 0; j < ny; j++) {
        ko_memo memo = {0, 0, 0.0, 0.0};
        for (int i = 0; i < nx; i++) {
            int ip = (i + 1) % nx;
            int im = ((i - 1) + nx) % nx;
            int jp = (j + 1) % ny;
            int jm = ((j - 1) + ny) % ny;
            size_t c = (size_t)i + (size_t)nx * j;
#define P(a, b) phi[(size_t)(a) + (size_t)nx * (b)]
#define TT(a, b) t[(size_t)(a) + (size_t)nx * (b)]
            gpx[c] = (P(ip, j) - P(im, j)) / p->dx;
            gpy[c] = (P(i, jp) - P(i, jm)) / p->dy;
            lphi[c] = (2.0 * (P(ip, j) + P(im, j) + P(i, jp) + P(i, jm)) + P(ip, jp) + P(im, jm) + P(im, jp) +
                       P(ip, jm) - 12.0 * P(i, j)) /
                      (3.0 * p->dx * p->dx);
            lt[c] = (2.0 * (TT(ip, j) + TT(im, j) + TT(i, jp) + TT(i, jm)) + TT(ip, jp) + TT(im, jm) + TT(im, jp) +
                     TT(ip, jm) - 12.0 * TT(i, j)) /
                    (3.0 * p->dx * p->dx);
#undef P
#undef TT
            double gx = gpx[c], gy = gpy[c];
            if (gx <= +KO_FLT_EPS && gx >= -KO_FLT_EPS) {
                if (gy < -KO_FLT_EPS)
                    angl[c] = -0.5 * pi;
                else if (gy > +KO_FLT_EPS)
                    angl[c] = 0.5 * pi;
            }
            if (gx > +KO_FLT_EPS) {
                if (gy < -KO_FLT_EPS)
                    angl[c] = 2.0 * pi + ko_atan(gy / gx, libm);
                else if (gy > +KO_FLT_EPS)
                    angl[c] = ko_atan(gy / gx, libm);
            }
            if (gx < -KO_FLT_EPS)
                angl[c] = pi + ko_atan(gy / gx, libm);

            double s, co;
            double arg = p->aniso * (angl[c] - p->theta0);
            if (memo.valid && memo.key == ko_bits(arg)) {
                s = memo.a;
                co = memo.b;
            } else {
                ko_sincos(arg, &s, &co, libm);
                memo.key = ko_bits(arg);
                memo.a = s;
                memo.b = co;
                memo.valid = 1;
            }
            eps[c] = p->eps_bar * (1.0 + p->delta * co);
            epsd[c] = -p->eps_bar * p->aniso * p->delta * s;
        }
    }
}

static void ko_stage2(int nx, int ny, const ko_params* p, double* phi, double* t, const double* gpx,
                      const double* gpy, const double* lphi, const double* lt, const double* eps,
                      const double* epsd, int libm, int nthreads)
{
    const double pi = KG_PI;
    (void)nthreads;
#pragma omp parallel for schedule(static) num_threads(nthreads)
    for (int j = 0; j < ny; j++) {
        ko_memo memo = {0, 0, 0.0, 0.0};
        for (int i = 0; i < nx; i++) {
            size_t ip = (size_t)((i + 1) % nx) + (size_t)nx * j;
            size_t im = (size_t)(((i - 1) + nx) % nx) + (size_t)nx * j;
            size_t jp = (size_t)i + (size_t)nx * ((j + 1) % ny);
            size_t jm = (size_t)i + (size_t)nx * (((j - 1) + ny) % ny);
            size_t c = (size_t)i + (size_t)nx * j;

            double gradEpsPowX = (eps[ip] * eps[ip] - eps[im] * eps[im]) / p->dx;
            double gradEpsPowY = (eps[jp] * eps[jp] - eps[jm] * eps[jm]) / p->dy;
            double term1 = (eps[jp] * epsd[jp] * gpx[jp] - eps[jm] * epsd[jm] * gpx[jm]) / p->dy;
            double term2 = -(eps[ip] * epsd[ip] * gpy[ip] - eps[im] * epsd[im] * gpy[im]) / p->dx;
            double term3 = gradEpsPowX * gpx[c] + gradEpsPowY * gpy[c];
            double u = p->gamma * (p->teq - t[c]);
            if (!(memo.valid && memo.key == ko_bits(u))) {
                memo.key = ko_bits(u);
                memo.a = ko_atan(u, libm);
                memo.valid = 1;
            }
            double m = p->alpha / pi * memo.a;
            double oldPhi = phi[c];
            double oldT = t[c];
            phi[c] = phi[c] + (term1 + term2 + eps[c] * eps[c] * lphi[c] + term3 +
                               oldPhi * (1.0 - oldPhi) * (oldPhi - 0.5 + m)) *
                                  p->dt / p->tau;
            t[c] = oldT + lt[c] * p->dt + p->K * (phi[c] - oldPhi);
        }
    }
}

/*
 * Advance (phi, T, theta) in place by nsteps explicit steps.
 * libm = 1: C library atan/sin/cos (the reference's own math);
 * libm = 0: kg_math.h (the GPU's math).  Returns 0, or -1 on bad input.
 */
int ko_run(int nx, int ny, const ko_params* p, double* phi, double* t, double* theta, long long nsteps, int libm,
           int nthreads)
{
    if (nx < 1 || ny < 1 || !p || !phi || !t || !theta || nsteps < 0)
        return -1;
    if (nthreads < 1)
        nthreads = 1;
    size_t n = (size_t)nx * (size_t)ny;
    double* w = (double*)malloc(6 * n * sizeof(double));
    if (!w)
        return -1;
    memset(w, 0, 6 * n * sizeof(double));
    double *gpx = w, *gpy = w + n, *lphi = w + 2 * n, *lt = w + 3 * n, *eps = w + 4 * n, *epsd = w + 5 * n;
    for (long long s = 0; s < nsteps; s++) {
        ko_stage1(nx, ny, p, phi, t, theta, gpx, gpy, lphi, lt, eps, epsd, libm, nthreads);
        ko_stage2(nx, ny, p, phi, t, gpx, gpy, lphi, lt, eps, epsd, libm, nthreads);
    }
    free(w);
    return 0;
}

/* kg_math.h entry points, for the elementary-function tests */
double ko_kg_atan(double x) { return kg_atan(x); }
void ko_kg_sincos(double x, double* s, double* c) { kg_sincos(x, s, c); }
/* host evaluation of kg_math.h over an array: fn 0 atan, 1 sin, 2 cos, 4 x / b, 5 kg_idiv(x, b),
 * 10 kg_twice_plus(x[i], x[n-1-i]), 11 2 x[i] + x[n-1-i] (two roundings), 12 kg_absorb_bound(x),
 * 13 kg_gdiv(x[i], x[n-1-i]), 14 x[i] / x[n-1-i] */
int ko_kg_eval(int fn, const double* x, double* y, long long n, double b)
{
    kg_idivc ic;
    if ((fn == 4 || fn == 5) && kg_idiv_prepare(b, &ic))
        return -1;
    for (long long i = 0; i < n; i++) {
        double s, c;
        switch (fn) {
        case 0: y[i] = kg_atan(x[i]); break;
        case 1: kg_sincos(x[i], &s, &c); y[i] = s; break;
        case 2: kg_sincos(x[i], &s, &c); y[i] = c; break;
        case 4: y[i] = x[i] / b; break;
        case 5: y[i] = kg_idiv(x[i], &ic); break;
        case 10: y[i] = kg_twice_plus(x[i], x[n - 1 - i]); break;
        case 11: y[i] = 2.0 * x[i] + x[n - 1 - i]; break;
        case 12: y[i] = kg_from_bits(kg_absorb_bound(x[i])); break;
        case 13: y[i] = kg_gdiv(x[i], x[n - 1 - i]); break;
        case 14: y[i] = x[i] / x[n - 1 - i]; break;
        default: return -1;
        }
    }
    return 0;
}

/*
 * Tangent-linear model of ko_run (kg_math functions): advances the state
 * (phi, T, theta) exactly as ko_run does, and alongside it the tangent
 * (dphi, dT, dtheta) -- the derivative of the state along a direction in
 * (initial state, delta, K, theta0, tau, gamma).  dparam = {d_delta, d_K,
 * d_theta0, d_tau, d_gamma}.  Written independently of the GPU adjoint: the
 * adjoint's <gradient, direction> must equal the final <phi_N - target, dphi_N>.
 * Branches of the angle are differentiated piecewise, as in the adjoint.
 */
int ko_tlm_run(int nx, int ny, const ko_params* p, const double* dparam, double* phi, double* t, double* theta,
               double* dphi, double* dt_, double* dtheta, long long nsteps, int nthreads)
{
    if (nx < 1 || ny < 1 || !p || !dparam || nsteps < 0)
        return -1;
    if (nthreads < 1)
        nthreads = 1;
    const double pi = KG_PI;
    const double d_delta = dparam[0], d_K = dparam[1], d_th0 = dparam[2], d_tau = dparam[3], d_gamma = dparam[4];
    size_t n = (size_t)nx * (size_t)ny;
    double* w = (double*)malloc(14 * n * sizeof(double));
    if (!w)
        return -1;
    double *gpx = w, *gpy = w + n, *lphi = w + 2 * n, *lt = w + 3 * n, *eps = w + 4 * n, *epsd = w + 5 * n;
    double *tgx = w + 6 * n, *tgy = w + 7 * n, *tlphi = w + 8 * n, *tlt = w + 9 * n, *teps = w + 10 * n,
           *tepsd = w + 11 * n;
    double *nphi = w + 12 * n, *ndphi = w + 13 * n;
    const double lap_den = 3.0 * p->dx * p->dx;
    for (long long step = 0; step < nsteps; step++) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (int j = 0; j < ny; j++) {
            for (int i = 0; i < nx; i++) {
                int ip = (i + 1) % nx, im = ((i - 1) + nx) % nx, jp = (j + 1) % ny, jm = ((j - 1) + ny) % ny;
                size_t c = (size_t)i + (size_t)nx * j;
#define A(arr, a, b) arr[(size_t)(a) + (size_t)nx * (b)]
                gpx[c] = (A(phi, ip, j) - A(phi, im, j)) / p->dx;
                gpy[c] = (A(phi, i, jp) - A(phi, i, jm)) / p->dy;
                tgx[c] = (A(dphi, ip, j) - A(dphi, im, j)) / p->dx;
                tgy[c] = (A(dphi, i, jp) - A(dphi, i, jm)) / p->dy;
                lphi[c] = (2.0 * (A(phi, ip, j) + A(phi, im, j) + A(phi, i, jp) + A(phi, i, jm)) + A(phi, ip, jp) +
                           A(phi, im, jm) + A(phi, im, jp) + A(phi, ip, jm) - 12.0 * A(phi, i, j)) / lap_den;
                lt[c] = (2.0 * (A(t, ip, j) + A(t, im, j) + A(t, i, jp) + A(t, i, jm)) + A(t, ip, jp) + A(t, im, jm) +
                         A(t, im, jp) + A(t, ip, jm) - 12.0 * A(t, i, j)) / lap_den;
                tlphi[c] = (2.0 * (A(dphi, ip, j) + A(dphi, im, j) + A(dphi, i, jp) + A(dphi, i, jm)) +
                            A(dphi, ip, jp) + A(dphi, im, jm) + A(dphi, im, jp) + A(dphi, ip, jm) -
                            12.0 * A(dphi, i, j)) / lap_den;
                tlt[c] = (2.0 * (A(dt_, ip, j) + A(dt_, im, j) + A(dt_, i, jp) + A(dt_, i, jm)) + A(dt_, ip, jp) +
                          A(dt_, im, jm) + A(dt_, im, jp) + A(dt_, ip, jm) - 12.0 * A(dt_, i, j)) / lap_den;
#undef A
                double gx = gpx[c], gy = gpy[c];
                int gx_small = gx <= KO_FLT_EPS && gx >= -KO_FLT_EPS;
                int gy_big = gy < -KO_FLT_EPS || gy > KO_FLT_EPS;
                if (gx_small) {
                    if (gy < -KO_FLT_EPS) {
                        theta[c] = -0.5 * pi;
                        dtheta[c] = 0.0;
                    } else if (gy > KO_FLT_EPS) {
                        theta[c] = 0.5 * pi;
                        dtheta[c] = 0.0;
                    }
                }
                if ((gx > KO_FLT_EPS && gy_big) || gx < -KO_FLT_EPS) {
                    double at = kg_atan(gy / gx);
                    if (gx < -KO_FLT_EPS)
                        theta[c] = pi + at;
                    else if (gy < -KO_FLT_EPS)
                        theta[c] = 2.0 * pi + at;
                    else
                        theta[c] = at;
                    dtheta[c] = (gx * tgy[c] - gy * tgx[c]) / (gx * gx + gy * gy);
                }
                double s, co;
                double psi = p->aniso * (theta[c] - p->theta0);
                double dpsi = p->aniso * (dtheta[c] - d_th0);
                kg_sincos(psi, &s, &co);
                eps[c] = p->eps_bar * (1.0 + p->delta * co);
                epsd[c] = -p->eps_bar * p->aniso * p->delta * s;
                teps[c] = p->eps_bar * (d_delta * co - p->delta * s * dpsi);
                tepsd[c] = -p->eps_bar * p->aniso * (d_delta * s + p->delta * co * dpsi);
            }
        }
#pragma omp parallel for schedule(static) num_threads(nthreads)
        for (int j = 0; j < ny; j++) {
            for (int i = 0; i < nx; i++) {
                size_t ip = (size_t)((i + 1) % nx) + (size_t)nx * j;
                size_t im = (size_t)(((i - 1) + nx) % nx) + (size_t)nx * j;
                size_t jp = (size_t)i + (size_t)nx * ((j + 1) % ny);
                size_t jm = (size_t)i + (size_t)nx * (((j - 1) + ny) % ny);
                size_t c = (size_t)i + (size_t)nx * j;
                double gEx = (eps[ip] * eps[ip] - eps[im] * eps[im]) / p->dx;
                double gEy = (eps[jp] * eps[jp] - eps[jm] * eps[jm]) / p->dy;
                double term1 = (eps[jp] * epsd[jp] * gpx[jp] - eps[jm] * epsd[jm] * gpx[jm]) / p->dy;
                double term2 = -(eps[ip] * epsd[ip] * gpy[ip] - eps[im] * epsd[im] * gpy[im]) / p->dx;
                double term3 = gEx * gpx[c] + gEy * gpy[c];
                double u = p->gamma * (p->teq - t[c]);
                double m = p->alpha / pi * kg_atan(u);
                double R = term1 + term2 + eps[c] * eps[c] * lphi[c] + term3 +
                           phi[c] * (1.0 - phi[c]) * (phi[c] - 0.5 + m);
                /* tangents */
#define DE2(x) (2.0 * eps[x] * teps[x])
#define DA(x) ((teps[x] * epsd[x] + eps[x] * tepsd[x]) * gpx[x] + eps[x] * epsd[x] * tgx[x])
#define DB(x) ((teps[x] * epsd[x] + eps[x] * tepsd[x]) * gpy[x] + eps[x] * epsd[x] * tgy[x])
                double dgEx = (DE2(ip) - DE2(im)) / p->dx;
                double dgEy = (DE2(jp) - DE2(jm)) / p->dy;
                double dt1 = (DA(jp) - DA(jm)) / p->dy;
                double dt2 = -(DB(ip) - DB(im)) / p->dx;
                double dt3 = dgEx * gpx[c] + gEx * tgx[c] + dgEy * gpy[c] + gEy * tgy[c];
                double du = d_gamma * (p->teq - t[c]) - p->gamma * dt_[c];
                double dm = p->alpha / pi * du / (1.0 + u * u);
                double ph = phi[c];
                double dW = ((1.0 - 2.0 * ph) * (ph - 0.5 + m) + ph * (1.0 - ph)) * dphi[c] + ph * (1.0 - ph) * dm;
                double dR = dt1 + dt2 + DE2(c) * lphi[c] + eps[c] * eps[c] * tlphi[c] + dt3 + dW;
#undef DE2
#undef DA
#undef DB
                double newphi = ph + R * p->dt / p->tau;
                double dnewphi = dphi[c] + dR * p->dt / p->tau - R * p->dt * d_tau / (p->tau * p->tau);
                double newt = t[c] + lt[c] * p->dt + p->K * (newphi - ph);
                double dnewt = dt_[c] + tlt[c] * p->dt + d_K * (newphi - ph) + p->K * (dnewphi - dphi[c]);
                nphi[c] = newphi;
                ndphi[c] = dnewphi;
                t[c] = newt;
                dt_[c] = dnewt;
            }
        }
        memcpy(phi, nphi, n * sizeof(double));
        memcpy(dphi, ndphi, n * sizeof(double));
    }
    free(w);
    return 0;
}

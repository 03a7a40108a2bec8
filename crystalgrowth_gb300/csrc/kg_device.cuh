/*
 * kg_device.cuh -- the fused Kobayashi step on sm_103a.
 *
 * One explicit step of the reference (src/Kobayashi.cpp:125-221) in one pass
 * over HBM: each CTA owns a strip of NT-2 columns and BH rows, and marches
 * down its rows.  At row r it computes the stage-1 quantities that neighbours
 * need (gradients, the persistent angle, eps, eps' and the products
 * eps^2, eps eps' phi_x, eps eps' phi_y) for its NT columns (one halo column
 * each side), keeps the vertical neighbours of those in registers and the
 * horizontal ones in shared memory, and finishes stage 2 (the Laplacians, the
 * divergence terms and the phi/T update) for row r-1.  Stage-1 work is
 * therefore done once per cell plus 2/BH rows and 2/(NT-2) columns of halo;
 * intermediate arrays never touch HBM (48 B/cell: phi, T, theta read and
 * written once).
 *
 * The arithmetic reproduces the reference operation for operation in IEEE
 * FP64 (this file is compiled with -fmad=false, so a*b+c is never fused
 * unless written as kg_fma), with these exact shortcuts:
 *   - divisions by dx, dy, 3 dx^2 and tau use kg_idiv: the IEEE quotient's
 *     bits from 64-bit integer arithmetic, off the FP64 pipe; the angle's
 *     gy/gx uses kg_gdiv, the same for a divisor that varies per cell;
 *   - eps, eps' for the angle value theta = 0 (every cell the front has not
 *     reached) come from a table computed once on the host with the same
 *     kg_sincos, keyed on the exact bits of the sine/cosine argument;
 *   - m = alpha/pi atan(gamma (Teq - T)) for the far-field argument
 *     gamma*Teq likewise; where |T| is small enough that Teq - T rounds to
 *     Teq (a bound from the host), the argument itself is not computed;
 *   - the Laplacians' 2 (E+W+N+S) + NE is one FMA: 2 x is exact, so the
 *     reference's two roundings are the FMA's one (kg_twice_plus);
 *   - where the E/W and N/S neighbours' eps^2 are equal (every cell whose
 *     neighbourhood the front has not reached), grad eps^2 is +0 and the term
 *     grad eps^2 . grad phi is a signed zero: its sign, and the sum it joins,
 *     are settled on bit patterns;
 *   - for |phi| <= 2^-56 the double well phi (1 - phi) (phi - 0.5 + m) is
 *     exactly phi (m - 0.5): the other factors round to 1 and -0.5;
 *   - quiet cells, whose 3x3 phi neighbourhood is all +0 (everywhere the
 *     front's far tail has not reached): every term of the phi update is a
 *     signed zero, so phi stays +0 and only T + lap_T dt is computed; with a
 *     +0 T neighbourhood as well, T stays +0 too.  Stage 1 of a cell whose
 *     four phi neighbours are +0 keeps theta and takes gx = gy = +0 without
 *     arithmetic;
 *   - the T update's latent-heat term K (phi' - phi) is not computed where
 *     a bound on the operands' exponents shows that adding it to
 *     T + lap_T dt cannot change the sum (kg_stage2).
 * Comparisons use the bit patterns (integer pipe), never the FP64 pipe: kg_bits
 * takes them through an inline-PTX move, so the optimiser cannot turn a bit
 * test back into an FP64 comparison.  atan, sin and cos (kg_math.h) run on
 * the integer pipes as well.
 */
#pragma once
#include <stdint.h>
#include "kg_math.h"

/* Everything the kernel needs about one parameter set, prepared on the host. */
struct KgDev {
    double dx, dy, dt, tau, eps_bar, K, delta, aniso, alpha, gamma, teq, theta0;
    kg_idivc idx, idy, ilap, itau; /* integer-pipe division by dx, dy, 3 dx^2, tau */
    double lap_den;   /* (3 dx) dx, src/Kobayashi.cpp:146 */
    double c_epsd;    /* ((-eps_bar) aniso) delta, src/Kobayashi.cpp:171 */
    double a_pi;      /* alpha / PI_F, src/Kobayashi.cpp:206 */
    double arg0;      /* aniso (0 - theta0): sin/cos argument of theta == 0 */
    double s0, c0;    /* sin(arg0), cos(arg0) */
    double eps0, epsd0, e2_0, ee0; /* eps, eps', eps^2, eps eps' at arg0 */
    double u0, m0;    /* gamma (Teq - 0) and (alpha/pi) atan(u0) */
    uint64_t zk;      /* bits of K * (+0): the T update's latent-heat term for a quiet cell */
    int ebk;          /* biased exponent field of K (0 for K = 0): bounds the latent-heat term */
    uint64_t t_small; /* |T| bit patterns up to this leave Teq - T == Teq, so u == u0 */
    uint64_t phi_small; /* |phi| bit patterns up to this leave 1 - phi == 1 and phi - 0.5 == -0.5 */
    double r0;          /* -0.5 + m0: the double-well factor (phi - 0.5 + m) of such a cell */
};

#define KG_ABS_MASK 0x7fffffffffffffffull
#define KG_EPS_BITS 0x3e80000000000000ull /* FLT_EPSILON = 2^-23 as a double */
#define KG_INF_BITS 0x7ff0000000000000ull

/* x <= +eps && x >= -eps */
__device__ __forceinline__ bool kg_small(uint64_t b) { return (b & KG_ABS_MASK) <= KG_EPS_BITS; }
/* x > +eps */
__device__ __forceinline__ bool kg_pos_big(uint64_t b) { return b > KG_EPS_BITS && b <= KG_INF_BITS; }
/* x < -eps */
__device__ __forceinline__ bool kg_neg_big(uint64_t b)
{
    return b > (0x8000000000000000ull | KG_EPS_BITS) && b <= 0xfff0000000000000ull;
}

/* The quiet-cell shortcut (exact; all-zero phi neighbourhoods): 0 off; 2 in the phi/T update only;
 * 3 as 2, and stage 1 of a cell with four +0 phi neighbours skips its two differences and the angle;
 * 1 as 3, and also settles that cell's eps eps' phi_x, eps eps' phi_y as signed zeros */
#ifndef KG_QUIET
#define KG_QUIET 3
#endif

/* 1: the latent-heat term K (phi' - phi) of the T update is skipped where a bound on exponents shows
 * that rounding absorbs it (exact); 0: always computed */
#ifndef KG_ABSORB
#define KG_ABSORB 1
#endif

/* 1: the angle's quotient gy/gx through kg_gdiv (the IEEE bits on the integer pipes); 0: the
 * hardware division */
#ifndef KG_GDIV
#define KG_GDIV 1
#endif

/* Stage-1 quantities of one cell that its neighbours read in stage 2. */
struct KgS1 {
    double gx, gy, e2, a, b; /* phi_x, phi_y, eps^2, eps eps' phi_x, eps eps' phi_y */
    double s, c;             /* sin, cos of aniso (theta - theta0) (kept for the adjoint's tape) */
};

/* Per-cell forward quantities the reverse (adjoint) step reads: one slot of
 * the tape, field f of cell i at f[k][i]. */
enum { KG_TAPE_PHI, KG_TAPE_T, KG_TAPE_GX, KG_TAPE_GY, KG_TAPE_SIN, KG_TAPE_COS, KG_TAPE_LAP, KG_TAPE_RHS,
       KG_TAPE_M, KG_TAPE_GEX, KG_TAPE_GEY, KG_TAPE_FIELDS };
struct KgTape {
    double* f[KG_TAPE_FIELDS];
};

/* stage-2 intermediates recorded on the tape */
struct KgS2Aux {
    double rhs, m, gex, gey;
};

/*
 * Stage 1 for one cell (src/Kobayashi.cpp:139-140,154-171): gradients, the
 * angle update (theta keeps its value in the FLT_EPSILON dead zone), eps, eps'.
 * theta is updated in place.
 */
__device__ __forceinline__ KgS1 kg_stage1(const KgDev& P, double pE, double pW, double pN, double pS, double& theta)
{
    KgS1 o;
    double gx, gy;
#if KG_QUIET == 1 || KG_QUIET == 3
    /* four +0 neighbours: both differences are +0 and the angle keeps its value (the dead zone) */
    const bool quiet = (kg_bits(pE) | kg_bits(pW) | kg_bits(pN) | kg_bits(pS)) == 0;
    if (quiet) {
        gx = 0.0;
        gy = 0.0;
    } else
#endif
    {
        gx = kg_idiv(pE - pW, &P.idx);
        gy = kg_idiv(pN - pS, &P.idy);
        uint64_t bx = kg_bits(gx), by = kg_bits(gy);
        /* the reference's three branches (src/Kobayashi.cpp:154-167) with one
         * shared atan call, so that lanes on different branches do not run it
         * one after the other; theta = off + atan(gy/gx), off in {0, pi, 2 pi}
         * (for off = 0 the atan value itself: adding +0 could turn -0 into +0) */
        bool gx_small = kg_small(bx), gx_pos = kg_pos_big(bx), gx_neg = kg_neg_big(bx);
        bool gy_pos = kg_pos_big(by), gy_neg = kg_neg_big(by);
        if (gx_small) {
            if (gy_neg)
                theta = -0.5 * KG_PI;
            else if (gy_pos)
                theta = 0.5 * KG_PI;
        }
        bool use_atan = gx_neg || (gx_pos && (gy_pos || gy_neg));
        if (use_atan) {
#if KG_GDIV
            double at = kg_atan(kg_gdiv(gy, gx));
#else
            double at = kg_atan(gy / gx);
#endif
            double s = (gx_neg ? KG_PI : 2.0 * KG_PI) + at;
            theta = (gx_neg || gy_neg) ? s : at;
        }
    }
    /* theta == +0 (every cell the front has not reached) gives arg0 exactly; skip the two FP64 ops */
    double arg = P.arg0;
    if (kg_bits(theta) != 0)
        arg = P.aniso * (theta - P.theta0);
    double e2, ee;
    if (kg_bits(arg) == kg_bits(P.arg0)) {
        e2 = P.e2_0;
        ee = P.ee0;
        o.s = P.s0;
        o.c = P.c0;
    } else {
        double s, c;
        kg_sincos(arg, &s, &c);
        double eps = P.eps_bar * (1.0 + P.delta * c);
        double epsd = P.c_epsd * s;
        e2 = eps * eps;
        ee = eps * epsd;
        o.s = s;
        o.c = c;
    }
    o.gx = gx;
    o.gy = gy;
    o.e2 = e2;
#if KG_QUIET == 1
    if (quiet && (kg_bits(ee) & KG_ABS_MASK) < KG_INF_BITS) {
        /* ee (+0) for a finite ee: a zero with ee's sign */
        o.a = kg_from_bits(kg_bits(ee) & ~KG_ABS_MASK);
        o.b = o.a;
    } else
#endif
    {
        o.a = ee * gx;
        o.b = ee * gy;
    }
    return o;
}

/* 1: kg_twice_plus in the Laplacians and the T bound for m (both exact); 0: the plain sequence */
#ifndef KG_FUSE
#define KG_FUSE 1
#endif
/* 1: the flat-eps^2 and small-phi shortcuts of stage 2 (both exact); 0: the plain sequence */
#ifndef KG_FAR
#define KG_FAR 1
#endif

/* 9-point Laplacian in the reference's summation order (src/Kobayashi.cpp:142-151). */
__device__ __forceinline__ double kg_lap(const KgDev& P, double c, double e, double w, double n, double s, double ne,
                                         double sw, double nw, double se)
{
    double v;
#if KG_FUSE
    v = kg_twice_plus(e + w + n + s, ne) + sw + nw + se - 12.0 * c;
#else
    v = 2.0 * (e + w + n + s) + ne + sw + nw + se - 12.0 * c;
#endif
    return kg_idiv(v, &P.ilap);
}

/*
 * Stage 2 for one cell (src/Kobayashi.cpp:190-215).  Neighbour stage-1 data:
 * e2 at E/W/N/S, a = eps eps' phi_x at N/S, b = eps eps' phi_y at E/W.
 */
__device__ __forceinline__ void kg_stage2(const KgDev& P, double e2c, double gx, double gy, double e2E, double e2W,
                                          double e2N, double e2S, double aN, double aS, double bE, double bW,
                                          double lap_phi, double lap_t, double& phi, double& t,
                                          KgS2Aux* aux = nullptr)
{
    double term1 = kg_idiv(aN - aS, &P.idy);
    double term2 = -kg_idiv(bE - bW, &P.idx);
    /* the reference's sum term1 + term2 + e2c lap + term3 + reaction, left to right */
    double acc = term1 + term2 + e2c * lap_phi;
    double gex, gey;
#if KG_FAR
    const uint64_t ue = kg_bits(e2E), un = kg_bits(e2N);
    if (ue == kg_bits(e2W) && un == kg_bits(e2S) && (ue & KG_ABS_MASK) < KG_INF_BITS &&
        (un & KG_ABS_MASK) < KG_INF_BITS && (kg_bits(gx) & KG_ABS_MASK) < KG_INF_BITS &&
        (kg_bits(gy) & KG_ABS_MASK) < KG_INF_BITS) {
        /* e2E - e2W = +0 and e2N - e2S = +0, so gex = gey = +0 and term3 = (+0 gx) + (+0 gy): a zero
         * that is -0 only when both products are, i.e. both gx and gy carry a sign bit.  Adding it
         * leaves a nonzero acc unchanged; for a zero acc the sum is -0 only if both are -0. */
        gex = 0.0;
        gey = 0.0;
        const uint64_t z3 = kg_bits(gx) & kg_bits(gy) & ~KG_ABS_MASK;
        const uint64_t ua = kg_bits(acc);
        if ((ua & KG_ABS_MASK) == 0)
            acc = kg_from_bits(ua & z3);
    } else
#endif
    {
        gex = kg_idiv(e2E - e2W, &P.idx);
        gey = kg_idiv(e2N - e2S, &P.idy);
        double term3 = gex * gx + gey * gy;
        acc = acc + term3;
    }
    double m = P.m0;
#if KG_FUSE
    if ((kg_bits(t) & KG_ABS_MASK) > P.t_small)
#endif
    {
        double u = P.gamma * (P.teq - t);
        if (kg_bits(u) != kg_bits(P.u0))
            m = P.a_pi * kg_atan(u);
    }
    double old_phi = phi;
    double old_t = t;
    double react;
#if KG_FAR
    if ((kg_bits(old_phi) & KG_ABS_MASK) <= P.phi_small)
        react = old_phi * (kg_bits(m) == kg_bits(P.m0) ? P.r0 : -0.5 + m);
    else
#endif
        react = old_phi * (1.0 - old_phi) * (old_phi - 0.5 + m);
    double rhs = acc + react;
    const double q = kg_idiv(rhs * P.dt, &P.itau);
    double new_phi = old_phi + q;
#if KG_ABSORB
    /* The reference's T' = (T + lap_T dt) + K (phi' - phi) = x + y.  With eb the biased exponent field
     * (|v| < 2^(eb - 1022) for every finite v): phi' - phi = q + e, |e| <= ulp(phi')/2 <=
     * 2^(max(eb_phi', 1) - 1076), so |d| = |RN(phi' - phi)| <= 2^(M + 1) with
     * M = max(eb_q - 1022, max(eb_phi', 1) - 1076), and |y| = |RN(K d)| <= 2^(eb_K - 1021 + M).  For a
     * normal x (2^(eb_x - 1023) <= |x|), eb_K + M + 56 < eb_x gives |y| < 2^(eb_x - 1077) = ulp(x)/4, so
     * RN(x + y) = x (a tie below a power of two rounds to x, whose significand is even).  Non-finite
     * q or phi' (eb = 2047) and zero, subnormal or non-finite x take the full expression. */
    const double x = old_t + lap_t * P.dt;
    const int ebx = (int)((kg_bits(x) >> 52) & 0x7ff);
    const int ebq = (int)((kg_bits(q) >> 52) & 0x7ff);
    const int ebn = max((int)((kg_bits(new_phi) >> 52) & 0x7ff), 1);
    const int M = max(ebq - 1022, ebn - 1076);
    if (ebx >= 1 && ebx <= 2046 && P.ebk + M + 56 < ebx)
        t = x;
    else
        t = x + P.K * (new_phi - old_phi);
#else
    t = old_t + lap_t * P.dt + P.K * (new_phi - old_phi);
#endif
    phi = new_phi;
    if (aux) {
        aux->rhs = rhs;
        aux->m = m;
        aux->gex = gex;
        aux->gey = gey;
    }
}

/*
 * The phi/T update of one cell from its 3x3 phi and T neighbourhoods (rows
 * below/at/above as pointers into shared memory, centre column k) and its
 * neighbours' stage-1 values, with the quiet-cell shortcut:
 *   all nine phi are +0, the neighbours' eps eps' phi_x (N, S) and
 *   eps eps' phi_y (E, W) are zeros, grad eps^2 is flat and finite, eps^2 is
 *   finite and T is not NaN.  Then term1, term2, eps^2 lap phi, term3 and the
 *   double well (+0 times a finite factor) are all zeros, so the phi update
 *   adds a zero to +0: phi stays +0.  T becomes (T + lap_T dt) + K (+0 - +0),
 *   whose last term is the zero P.zk; with nine +0 T values it is +0.
 * Everything else takes kg_stage2.
 */
__device__ __forceinline__ void kg_update_cell(const KgDev& P, const double* __restrict__ pS_, const double* __restrict__ p0,
                                               const double* __restrict__ pN_, const double* __restrict__ tS_,
                                               const double* __restrict__ t0, const double* __restrict__ tN_, int k,
                                               double e2c, double gx, double gy, double e2E, double e2W, double e2N,
                                               double e2S, double aN, double aS, double bE, double bW, double& phi,
                                               double& t)
{
#define KG_LAP9(r0, rN, rS) \
    kg_lap(P, r0[k], r0[k + 1], r0[k - 1], rN[k], rS[k], rN[k + 1], rS[k - 1], rN[k - 1], rS[k + 1])
#define KG_OR9(r0, rN, rS)                                                                                       \
    (kg_bits(r0[k]) | kg_bits(r0[k + 1]) | kg_bits(r0[k - 1]) | kg_bits(rN[k]) | kg_bits(rS[k]) |               \
     kg_bits(rN[k + 1]) | kg_bits(rS[k - 1]) | kg_bits(rN[k - 1]) | kg_bits(rS[k + 1]))
    phi = p0[k];
    t = t0[k];
#if KG_QUIET
    if (KG_OR9(p0, pN_, pS_) == 0) {
        const uint64_t ue = kg_bits(e2E), un = kg_bits(e2N);
        const bool quiet = ((kg_bits(aN) | kg_bits(aS) | kg_bits(bE) | kg_bits(bW)) & KG_ABS_MASK) == 0 &&
                           ue == kg_bits(e2W) && un == kg_bits(e2S) && (ue & KG_ABS_MASK) < KG_INF_BITS &&
                           (un & KG_ABS_MASK) < KG_INF_BITS && (kg_bits(e2c) & KG_ABS_MASK) < KG_INF_BITS &&
                           (kg_bits(t) & KG_ABS_MASK) <= KG_INF_BITS;
        if (quiet) {
            phi = 0.0;
            if (KG_OR9(t0, tN_, tS_) == 0) {
                t = 0.0;
            } else {
                const double x = t + KG_LAP9(t0, tN_, tS_) * P.dt;
                const uint64_t bx = kg_bits(x);
                if ((bx & KG_ABS_MASK) == 0)
                    t = kg_from_bits(bx & P.zk); /* a zero plus a zero: -0 only if both are */
                else if ((bx & KG_ABS_MASK) < KG_INF_BITS)
                    t = x;
                else
                    t = x + kg_from_bits(P.zk);
            }
            return;
        }
    }
#endif
    const double lap_phi = KG_LAP9(p0, pN_, pS_);
    const double lap_t = KG_LAP9(t0, tN_, tS_);
    kg_stage2(P, e2c, gx, gy, e2E, e2W, e2N, e2S, aN, aS, bE, bW, lap_phi, lap_t, phi, t);
#undef KG_LAP9
#undef KG_OR9
}

/* a global load: the plain (read-only cache) path, or with COH one that stays coherent with stores
 * other CTAs made earlier in the same kernel (L2 only) */
template <bool COH>
__device__ __forceinline__ double kg_ld(const double* p)
{
    if constexpr (COH)
        return __ldcg(p);
    else
        return *p;
}

__device__ __forceinline__ int kg_wrap(int i, int n)
{
    int r = i % n;
    return r < 0 ? r + n : r;
}

/*
 * The marching strip: one CTA of NT threads advances columns [i0, i0+NT-2)
 * (clipped to nx) and rows [j0, j0+bh) (clipped to ny) of one grid by one
 * step, reading (phi, T, theta) from `*_in` and writing `*_out`.
 * Shared memory: phi ring 8 x (NT+2), T ring 4 x NT, e2/b ring 2 x 2 x NT.
 */
template <int NT>
struct __align__(16) KgSmem {
    double phi[8][NT + 2]; /* column i0-2+k at [.][k]; rows by local index (row - (j0-2)) & 7 */
    double t[8][NT + 2];   /* same layout as phi */
    double e2[2][NT];
    double b[2][NT];
    unsigned long long mbar[16]; /* bulk-copy completion: [0..7] phi slots, [8..15] T slots */
};

/* ---- bulk (TMA) row copies into shared memory, completion tracked by mbarriers ---- */

__device__ __forceinline__ unsigned kg_smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void kg_mbar_init(unsigned long long* mbar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(kg_smem_addr(mbar)), "r"(count) : "memory");
}

/* one arrival that also announces `bytes` of transaction data */
__device__ __forceinline__ void kg_mbar_expect(unsigned long long* mbar, unsigned bytes)
{
    asm volatile("{\n\t.reg .b64 st;\n\t"
                 "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(kg_smem_addr(mbar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool kg_mbar_test(unsigned long long* mbar, unsigned parity)
{
    unsigned ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(kg_smem_addr(mbar)), "r"(parity)
                 : "memory");
    return ok != 0;
}

/* a bounded wait for phase `parity` of an mbarrier: about 0.7 s at most, then
 * the error flag is raised and false returned (nothing here waits forever) */
__device__ __forceinline__ bool kg_mbar_wait(unsigned long long* mbar, unsigned parity, unsigned* err)
{
    for (int i = 0; i < (1 << 24); i++) {
        if (kg_mbar_test(mbar, parity))
            return true;
        __nanosleep(32);
    }
    if (err)
        atomicExch(err, 1u);
    return false;
}

/* bytes (a multiple of 16) from 16-byte aligned global src to 16-byte aligned shared dst */
__device__ __forceinline__ void kg_bulk_copy(void* dst, const void* src, unsigned bytes, unsigned long long* mbar)
{
    unsigned long long gsrc;
    asm volatile("cvta.to.global.u64 %0, %1;" : "=l"(gsrc) : "l"(src));
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     kg_smem_addr(dst)),
                 "l"(gsrc), "r"(bytes), "r"(kg_smem_addr(mbar))
                 : "memory");
}

/*
 * The marching strip: one CTA of NT threads advances columns [i0, i0+NT-2)
 * (clipped to nx) and rows [j0, j0+bh) (clipped to ny) of one grid by one
 * step, reading (phi, T, theta) from `*_in` and writing `*_out`.
 *
 * Rows of phi and T reach shared memory in one of two ways.  With `tma`
 * (strips that do not wrap around the grid's left/right edge, nx even so
 * that every row starts 16-byte aligned) one thread issues a bulk copy of
 * each row segment, columns i0-2 .. i0+NT-1, one row ahead of use, and the
 * CTA waits on that row's mbarrier; otherwise every lane loads its own
 * column (wrapped).  Ring slots are indexed by the row's position in the
 * strip, (row - (j0-2)) & 7.  `err` (may be null) receives a time-out of a
 * bulk-copy wait.  With COH the per-lane loads bypass the SM's L1 and
 * read-only caches (a persistent kernel reads data other CTAs wrote earlier in
 * the same launch).
 */
template <int NT, bool TAPE = false, bool COH = false>
__device__ __forceinline__ void kg_strip(const KgDev& P, int nx, int ny, const double* __restrict__ phi_in,
                                         const double* __restrict__ t_in, const double* __restrict__ th_in,
                                         double* __restrict__ phi_out, double* __restrict__ t_out,
                                         double* __restrict__ th_out, int i0, int j0, int bh, KgSmem<NT>& sm,
                                         const KgTape* tape = nullptr, bool tma = false, unsigned* err = nullptr)
{
    const int L = threadIdx.x;
    const int jend = min(j0 + bh, ny);
    const int base = j0 - 2; /* row of ring slot index 0 */
    /* columns: smem index k <-> column i0-2+k; lane L <-> column i0-1+L <-> index L+1 */
    const int colA = kg_wrap(i0 - 2 + L, nx);
    const int colB = (L < 2) ? kg_wrap(i0 - 2 + NT + L, nx) : 0;
    const int col = kg_wrap(i0 - 1 + L, nx);
    const bool out_lane = (L >= 1) && (L <= NT - 2) && (i0 - 1 + L < nx);
    const unsigned row_bytes = (NT + 2) * sizeof(double);

    auto load_phi_row = [&](int q) {
        const double* row = phi_in + (size_t)kg_wrap(q, ny) * nx;
        sm.phi[(q - base) & 7][L] = kg_ld<COH>(row + colA);
        if (L < 2)
            sm.phi[(q - base) & 7][NT + L] = kg_ld<COH>(row + colB);
    };
    /* mbarriers count each ring's rows from the ring's first row (phi: j0-2, T: j0-1), so that the
     * k-th arrival at a barrier is its phase k: row q waits on phase (q - first) >> 3 */
    auto phi_bar = [&](int q) { return &sm.mbar[(q - base) & 7]; };
    auto phi_par = [&](int q) { return (unsigned)((q - base) >> 3) & 1u; };
    auto t_bar = [&](int q) { return &sm.mbar[8 + ((q - j0 + 1) & 7)]; };
    auto t_par = [&](int q) { return (unsigned)((q - j0 + 1) >> 3) & 1u; };
    auto issue_phi = [&](int q) {
        unsigned long long* mb = phi_bar(q);
        kg_mbar_expect(mb, row_bytes);
        kg_bulk_copy(sm.phi[(q - base) & 7], phi_in + (size_t)kg_wrap(q, ny) * nx + (i0 - 2), row_bytes, mb);
    };
    auto issue_t = [&](int q) {
        unsigned long long* mb = t_bar(q);
        kg_mbar_expect(mb, row_bytes);
        kg_bulk_copy(sm.t[(q - base) & 7], t_in + (size_t)kg_wrap(q, ny) * nx + (i0 - 2), row_bytes, mb);
    };
    bool ok = true;
    int r_fail = jend + 1;
    auto wait_phi = [&](int q) {
        if (!kg_mbar_wait(phi_bar(q), phi_par(q), err))
            ok = false;
    };
    auto wait_t = [&](int q) {
        if (!kg_mbar_wait(t_bar(q), t_par(q), err))
            ok = false;
    };

    if (tma) {
        if (L == 0) {
            for (int k = 0; k < 16; k++)
                kg_mbar_init(&sm.mbar[k], 1);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();
        if (L == 0) {
            issue_phi(j0 - 2);
            issue_phi(j0 - 1);
            issue_phi(j0);
            issue_t(j0 - 1);
        }
        /* the march waits for row r+1 at row r; the two rows above the strip are waited for here */
        wait_phi(j0 - 2);
        wait_phi(j0 - 1);
    } else {
        /* rows j0-2 and j0-1 of phi before the march */
        load_phi_row(j0 - 2);
        load_phi_row(j0 - 1);
    }

    /* registers: stage-1 results of this lane's column for rows r-2, r-1, r */
    double e2_m2 = 0, a_m2 = 0;
    double e2_m1 = 0, a_m1 = 0, gx_m1 = 0, gy_m1 = 0;
    for (int r = j0 - 1; r <= jend; r++) {
        const size_t roff = (size_t)kg_wrap(r, ny) * nx;
        if (tma) {
            /* prefetch phi row r+2 and T row r+1, then wait for phi row r+1 and T row r */
            if (L == 0) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                if (r + 2 <= jend + 1)
                    issue_phi(r + 2);
                if (r + 1 <= jend)
                    issue_t(r + 1);
            }
            wait_phi(r + 1);
            wait_t(r);
        } else {
            /* loads: phi row r+1, T row r */
            load_phi_row(r + 1);
            sm.t[(r - base) & 7][L + 1] = kg_ld<COH>(t_in + roff + col);
        }
        double theta = kg_ld<COH>(th_in + roff + col);
        /* the row barrier, which also makes a bulk-copy time-out a CTA-wide decision (a one-warp
         * strip, NT = 32, needs only a warp vote: warps never wait on each other) */
        bool fail;
        if constexpr (NT == 32) {
            __syncwarp();
            fail = __any_sync(0xffffffffu, !ok);
        } else
            fail = __syncthreads_or(!ok) != 0;
        if (fail) {
            r_fail = r;
            break;
        }

        const int rm = (r - 1 - base) & 7, r0 = (r - base) & 7, rp = (r + 1 - base) & 7;
        /* stage 1 at row r for all NT lanes */
        KgS1 s1 = kg_stage1(P, sm.phi[r0][L + 2], sm.phi[r0][L], sm.phi[rp][L + 1], sm.phi[rm][L + 1], theta);
        sm.e2[r & 1][L] = s1.e2;
        sm.b[r & 1][L] = s1.b;
        if (out_lane && r >= j0 && r < jend) {
            th_out[roff + col] = theta;
            if constexpr (TAPE) {
                tape->f[KG_TAPE_GX][roff + col] = s1.gx;
                tape->f[KG_TAPE_GY][roff + col] = s1.gy;
                tape->f[KG_TAPE_SIN][roff + col] = s1.s;
                tape->f[KG_TAPE_COS][roff + col] = s1.c;
            }
        }

        /* stage 2 at row s = r-1 for the output lanes */
        const int s = r - 1;
        if (out_lane && s >= j0) {
            const int sm1 = (s - 1 - base) & 7, s0 = (s - base) & 7, sp1 = (s + 1 - base) & 7;
            const int k = L + 1;
            const size_t soff = (size_t)kg_wrap(s, ny) * nx;
            double phi, t;
            if constexpr (TAPE) {
                double lap_phi = kg_lap(P, sm.phi[s0][k], sm.phi[s0][k + 1], sm.phi[s0][k - 1], sm.phi[sp1][k],
                                        sm.phi[sm1][k], sm.phi[sp1][k + 1], sm.phi[sm1][k - 1], sm.phi[sp1][k - 1],
                                        sm.phi[sm1][k + 1]);
                double lap_t = kg_lap(P, sm.t[s0][k], sm.t[s0][k + 1], sm.t[s0][k - 1], sm.t[sp1][k], sm.t[sm1][k],
                                      sm.t[sp1][k + 1], sm.t[sm1][k - 1], sm.t[sp1][k - 1], sm.t[sm1][k + 1]);
                phi = sm.phi[s0][k];
                t = sm.t[s0][k];
                KgS2Aux aux;
                tape->f[KG_TAPE_PHI][soff + col] = phi;
                tape->f[KG_TAPE_T][soff + col] = t;
                kg_stage2(P, e2_m1, gx_m1, gy_m1, sm.e2[s & 1][L + 1], sm.e2[s & 1][L - 1], s1.e2, e2_m2, s1.a, a_m2,
                          sm.b[s & 1][L + 1], sm.b[s & 1][L - 1], lap_phi, lap_t, phi, t, &aux);
                tape->f[KG_TAPE_LAP][soff + col] = lap_phi;
                tape->f[KG_TAPE_RHS][soff + col] = aux.rhs;
                tape->f[KG_TAPE_M][soff + col] = aux.m;
                tape->f[KG_TAPE_GEX][soff + col] = aux.gex;
                tape->f[KG_TAPE_GEY][soff + col] = aux.gey;
            } else {
                kg_update_cell(P, sm.phi[sm1], sm.phi[s0], sm.phi[sp1], sm.t[sm1], sm.t[s0], sm.t[sp1], k, e2_m1, gx_m1,
                               gy_m1, sm.e2[s & 1][L + 1], sm.e2[s & 1][L - 1], s1.e2, e2_m2, s1.a, a_m2,
                               sm.b[s & 1][L + 1], sm.b[s & 1][L - 1], phi, t);
            }
            phi_out[soff + col] = phi;
            t_out[soff + col] = t;
        }
        /* roll the vertical window */
        e2_m2 = e2_m1;
        a_m2 = a_m1;
        e2_m1 = s1.e2;
        a_m1 = s1.a;
        gx_m1 = s1.gx;
        gy_m1 = s1.gy;
    }
    if (tma && r_fail <= jend && L == 0) {
        /* a wait ran out: before the CTA leaves (its shared memory goes to the next CTA), give the
         * bulk copies still in flight -- at most the last 8 rows issued per ring -- a second bounded
         * wait */
        const int last_phi = min(r_fail + 2, jend + 1), last_t = min(r_fail + 1, jend);
        for (int q = max(j0 - 2, last_phi - 7); q <= last_phi; q++)
            kg_mbar_wait(phi_bar(q), phi_par(q), nullptr);
        for (int q = max(j0 - 1, last_t - 7); q <= last_t; q++)
            kg_mbar_wait(t_bar(q), t_par(q), nullptr);
    }
}

/*
 * Temporal blocking, k = 2: one CTA of NT threads advances columns
 * [i0, i0+NT-6) and rows [j0, j0+bh) (clipped to the grid) by TWO steps in one
 * pass over HBM.  Two marching pipelines share the row loop:
 *   pipeline 1 is the k = 1 strip on columns i0-3 .. i0+NT-4 (lane L <->
 *   column i0-3+L): at row r it runs stage 1 of step 1, and stage 2 of step 1
 *   for row r-1 on lanes 1..NT-2; the step-1 phi and T of that row go to
 *   shared-memory rings (phi1, t1) instead of HBM, and the step-1 theta of
 *   each lane's column waits two rows in registers;
 *   pipeline 2 runs stage 1 of step 2 for row r-2 (lanes 1..NT-2) from those
 *   rings, and stage 2 of step 2 for row r-3 on the output lanes 3..NT-4.
 * The halo is therefore 4 columns and 3 rows on each side for phi (2 per
 * step), and every cell of the intermediate step is computed with exactly the
 * operations of the k = 1 step, so results are bit-identical to two k = 1
 * steps.  One __syncthreads per row serves both pipelines: within a row's
 * compute no lane reads a ring slot or exchange slot another lane writes in
 * the same row, and the next row's loads only refill slots no longer read.
 * Shared memory: 41 KB at NT = 128.
 */
template <int NT>
struct __align__(16) KgSmem2 {
    double phi[8][NT + 2]; /* step-0 phi: column i0-4+k at [.][k]; row q at slot (q - (j0-4)) & 7 */
    double t[8][NT + 2];   /* step-0 T, same layout */
    double e2a[2][NT];     /* step-1 eps^2 and eps eps' phi_y of lane L at [row & 1][L] */
    double ba[2][NT];
    double phi1[8][NT];    /* step-1 phi of lane L's column at [slot][L] */
    double t1[8][NT];
    double e2b[2][NT];     /* step-2 exchange, as e2a/ba */
    double bb[2][NT];
};

template <int NT, bool COH = false>
__device__ __forceinline__ void kg_strip2(const KgDev& P, int nx, int ny, const double* __restrict__ phi_in,
                                          const double* __restrict__ t_in, const double* __restrict__ th_in,
                                          double* __restrict__ phi_out, double* __restrict__ t_out,
                                          double* __restrict__ th_out, int i0, int j0, int bh, KgSmem2<NT>& sm)
{
    static_assert(NT >= 8, "temporal blocking needs at least 8 lanes");
    const int L = threadIdx.x;
    const int jend = min(j0 + bh, ny);
    const int base = j0 - 4; /* row of ring slot 0 */
    const int colA = kg_wrap(i0 - 4 + L, nx);
    const int colB = (L < 2) ? kg_wrap(i0 - 4 + NT + L, nx) : 0;
    const int col = kg_wrap(i0 - 3 + L, nx);
    const bool lane1 = (L >= 1) && (L <= NT - 2);                                    /* step-1 stage 2, step-2 stage 1 */
    const bool out_lane = (L >= 3) && (L <= NT - 4) && (i0 - 3 + L < nx);           /* step-2 stage 2, outputs */
    auto load_phi_row = [&](int q) {
        const double* row = phi_in + (size_t)kg_wrap(q, ny) * nx;
        sm.phi[(q - base) & 7][L] = kg_ld<COH>(row + colA);
        if (L < 2)
            sm.phi[(q - base) & 7][NT + L] = kg_ld<COH>(row + colB);
    };
    load_phi_row(j0 - 4);
    load_phi_row(j0 - 3);

    /* pipeline 1 window (stage-1 results of rows r-2, r-1), pipeline 2 window, step-1 theta queue */
    double e2a_m2 = 0, aa_m2 = 0, e2a_m1 = 0, aa_m1 = 0, gxa_m1 = 0, gya_m1 = 0;
    double e2b_m2 = 0, ab_m2 = 0, e2b_m1 = 0, ab_m1 = 0, gxb_m1 = 0, gyb_m1 = 0;
    double th1_m1 = 0, th1_m2 = 0;
    for (int r = j0 - 3; r <= jend + 2; r++) {
        const size_t roff = (size_t)kg_wrap(r, ny) * nx;
        load_phi_row(r + 1);
        sm.t[(r - base) & 7][L + 1] = kg_ld<COH>(t_in + roff + col);
        double theta = kg_ld<COH>(th_in + roff + col);
        if constexpr (NT == 32)
            __syncwarp();
        else
            __syncthreads();

        /* ---- step 1: stage 1 at row r (all lanes) ---- */
        const int rm = (r - 1 - base) & 7, r0 = (r - base) & 7, rp = (r + 1 - base) & 7;
        KgS1 sa = kg_stage1(P, sm.phi[r0][L + 2], sm.phi[r0][L], sm.phi[rp][L + 1], sm.phi[rm][L + 1], theta);
        sm.e2a[r & 1][L] = sa.e2;
        sm.ba[r & 1][L] = sa.b;
        /* ---- step 1: stage 2 at row s = r-1 -> phi1, t1 ---- */
        const int s = r - 1;
        if (s >= j0 - 2) {
            const int ss = (s - base) & 7;
            double phi = 0.0, t = 0.0;
            if (lane1) {
                const int sm1 = (s - 1 - base) & 7, sp1 = (s + 1 - base) & 7;
                kg_update_cell(P, sm.phi[sm1], sm.phi[ss], sm.phi[sp1], sm.t[sm1], sm.t[ss], sm.t[sp1], L + 1, e2a_m1,
                               gxa_m1, gya_m1, sm.e2a[s & 1][L + 1], sm.e2a[s & 1][L - 1], sa.e2, e2a_m2, sa.a, aa_m2,
                               sm.ba[s & 1][L + 1], sm.ba[s & 1][L - 1], phi, t);
            }
            sm.phi1[ss][L] = phi;
            sm.t1[ss][L] = t;
        }
        e2a_m2 = e2a_m1;
        aa_m2 = aa_m1;
        e2a_m1 = sa.e2;
        aa_m1 = sa.a;
        gxa_m1 = sa.gx;
        gya_m1 = sa.gy;
        /* step-1 theta of row r-2 for this lane's column */
        double th1 = th1_m2;
        th1_m2 = th1_m1;
        th1_m1 = theta;

        /* ---- step 2: stage 1 at row q = r-2 from the step-1 rings ---- */
        const int q = r - 2;
        if (q >= j0 - 1) {
            const int qm = (q - 1 - base) & 7, q0 = (q - base) & 7, qp = (q + 1 - base) & 7;
            KgS1 sb{};
            if (lane1) {
                sb = kg_stage1(P, sm.phi1[q0][L + 1], sm.phi1[q0][L - 1], sm.phi1[qp][L], sm.phi1[qm][L], th1);
                sm.e2b[q & 1][L] = sb.e2;
                sm.bb[q & 1][L] = sb.b;
                if (out_lane && q >= j0 && q < jend)
                    th_out[(size_t)kg_wrap(q, ny) * nx + col] = th1;
            }
            /* ---- step 2: stage 2 at row u = r-3 -> outputs ---- */
            const int u = r - 3;
            if (out_lane && u >= j0 && u < jend) {
                const int um = (u - 1 - base) & 7, u0 = (u - base) & 7, up = (u + 1 - base) & 7;
                double phi, t;
                kg_update_cell(P, sm.phi1[um], sm.phi1[u0], sm.phi1[up], sm.t1[um], sm.t1[u0], sm.t1[up], L, e2b_m1,
                               gxb_m1, gyb_m1, sm.e2b[u & 1][L + 1], sm.e2b[u & 1][L - 1], sb.e2, e2b_m2, sb.a, ab_m2,
                               sm.bb[u & 1][L + 1], sm.bb[u & 1][L - 1], phi, t);
                const size_t uoff = (size_t)kg_wrap(u, ny) * nx;
                phi_out[uoff + col] = phi;
                t_out[uoff + col] = t;
            }
            e2b_m2 = e2b_m1;
            ab_m2 = ab_m1;
            e2b_m1 = sb.e2;
            ab_m1 = sb.a;
            gxb_m1 = sb.gx;
            gyb_m1 = sb.gy;
        }
    }
}

/*
 * kg_math.h -- the elementary functions of the Kobayashi step, written once
 * for host and device.
 *
 * The reference (src/Kobayashi.cpp:162,164,167,170,171,206) calls the C
 * library's atan, cos and sin.  The C library's double versions are not
 * correctly rounded and differ between libm builds (and between x86-64 and
 * aarch64), so a GPU kernel cannot reproduce them bit for bit.  This header
 * defines the functions instead: every result is a fixed sequence of 64-bit
 * integer operations or IEEE-754 double operations (add, mul, explicit fma,
 * one correctly rounded FP32 reciprocal as a seed), so the CUDA kernels and
 * the CPU oracle, which both include this file, compute identical bits on any
 * IEEE-754 machine as long as the compiler does not contract a*b+c (host:
 * -ffp-contract=off; device: -fmad=false).
 *
 * Methods (published; coefficients in kg_math_tables.h come from
 * gen_kg_math_tables.py, which evaluates the mathematics in 320-bit precision):
 *   kg_atan   table-driven Taylor expansion around c_k = k/128 (Gal's
 *             accurate-tables method), argument reduction atan(x) =
 *             pi/2 - atan(1/x) for |x| > 1, evaluated in 64-bit fixed point on
 *             the integer pipes (kg_atan_x).
 *   kg_sincos sin(nh + r) = S_n cos r + C_n sin r, h = pi/128, with tabulated
 *             S_n, C_n: kg_sincos_x reduces |x| < 64 exactly with a 192-bit
 *             product by 128/pi (Payne-Hanek style) and works in fixed point;
 *             64 <= |x| < 4096 takes kg_sincos_f64, a three-part Cody-Waite
 *             reduction in FP64.
 *   kg_idiv   the IEEE quotient a/b for a divisor fixed for a whole run, and
 *   kg_gdiv   for any divisor, both on the integer pipes.
 *
 * Accuracy: kg_atan_x < 0.55 ulp; kg_sincos_x absolute error < 2^-61 and
 * faithful where |value| >= 2^-9; kg_sincos_f64 about 1 ulp; kg_sincos
 * returns NaN for |x| >= 4096.
 *
 * This header is C99 and CUDA C++ at the same time (the oracle is plain C).
 */
#ifndef KG_MATH_H
#define KG_MATH_H

#include <math.h>
#include <stdint.h>
#include <string.h>
#include "kg_math_tables.h"

#if defined(__CUDACC__)
#define KG_HD static __host__ __device__ __forceinline__
#else
#define KG_HD static inline
#endif

#if defined(__CUDACC__)
__device__ static const double kg_atan_tab_dev[(KG_ATAN_N + 1) * KG_ATAN_STRIDE] = KG_ATAN_TAB_DATA;
__device__ static const double kg_sc_tab_dev[KG_SC_N * 4] = KG_SC_TAB_DATA;
#endif
static const double kg_atan_tab_host[(KG_ATAN_N + 1) * KG_ATAN_STRIDE] = KG_ATAN_TAB_DATA;
static const double kg_sc_tab_host[KG_SC_N * 4] = KG_SC_TAB_DATA;

KG_HD double kg_tab_atan(int i)
{
#if defined(__CUDA_ARCH__)
    return __ldg(&kg_atan_tab_dev[i]);
#else
    return kg_atan_tab_host[i];
#endif
}

KG_HD double kg_tab_sc(int i)
{
#if defined(__CUDA_ARCH__)
    return __ldg(&kg_sc_tab_dev[i]);
#else
    return kg_sc_tab_host[i];
#endif
}

#if defined(__CUDACC__)
__device__ static const uint64_t kg_atanx_tab_dev[(KG_ATAN_N + 1) * 8] = KG_ATANX_TAB_DATA;
__device__ static const uint64_t kg_scx_tab_dev[KG_SC_N * 2] = KG_SCX_TAB_DATA;
#endif
static const uint64_t kg_atanx_tab_host[(KG_ATAN_N + 1) * 8] = KG_ATANX_TAB_DATA;
static const uint64_t kg_scx_tab_host[KG_SC_N * 2] = KG_SCX_TAB_DATA;

KG_HD uint64_t kg_tab_atanx(int i)
{
#if defined(__CUDA_ARCH__)
    return __ldg(&kg_atanx_tab_dev[i]);
#else
    return kg_atanx_tab_host[i];
#endif
}

KG_HD int64_t kg_tab_scx(int i)
{
#if defined(__CUDA_ARCH__)
    return (int64_t)__ldg(&kg_scx_tab_dev[i]);
#else
    return (int64_t)kg_scx_tab_host[i];
#endif
}

/* 1: on the device the bit pattern comes through an inline-PTX move, which the optimiser cannot see
 * through; with a plain reinterpretation it may turn a test such as (bits & ~sign) == 0 or
 * (bits & ~sign) <= c back into a floating-point comparison, which on sm_103a runs on the narrow
 * FP64 pipe (measured: one FP64-pipe instruction per such test) */
#ifndef KG_BITS_ASM
#define KG_BITS_ASM 1
#endif

KG_HD uint64_t kg_bits(double x)
{
#if defined(__CUDA_ARCH__) && KG_BITS_ASM
    uint64_t u;
    asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
    return u;
#elif defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}

KG_HD double kg_from_bits(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double x;
    memcpy(&x, &u, sizeof x);
    return x;
#endif
}

/* fused multiply-add with a single rounding on both sides */
KG_HD double kg_fma(double a, double b, double c)
{
#if defined(__CUDA_ARCH__)
    return __fma_rn(a, b, c);
#else
    return fma(a, b, c);
#endif
}

KG_HD uint32_t kg_fbits(float x)
{
#if defined(__CUDA_ARCH__)
    return (uint32_t)__float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}

/*
 * The rare FP64 fallbacks of the integer-pipe routines (special operands,
 * overflow) call these.  On the device they are out-of-line functions, which
 * keeps the common path of every inlined call site short (measured: the
 * 4096^2 case at time steps 6000-7000 ran 3% faster than with the fallbacks
 * inlined).  Same IEEE operations either way.
 */
#ifndef KG_SLOW_NOINLINE
#define KG_SLOW_NOINLINE 1
#endif
#if defined(__CUDA_ARCH__) && KG_SLOW_NOINLINE
__device__ __noinline__ static double kg_div_slow_dev(double a, double b) { return a / b; }
__device__ __noinline__ static double kg_add_slow_dev(double a, double b) { return a + b; }
#endif

KG_HD double kg_div_slow(double a, double b)
{
#if defined(__CUDA_ARCH__) && KG_SLOW_NOINLINE
    return kg_div_slow_dev(a, b);
#else
    return a / b;
#endif
}

KG_HD double kg_add_slow(double a, double b)
{
#if defined(__CUDA_ARCH__) && KG_SLOW_NOINLINE
    return kg_add_slow_dev(a, b);
#else
    return a + b;
#endif
}

/* correctly rounded FP32 reciprocal (the same bits on host and device) */
KG_HD float kg_rcp_f(float x)
{
#if defined(__CUDA_ARCH__)
    return __frcp_rn(x);
#else
    return 1.0f / x;
#endif
}

/* round-to-nearest-even of an FP32 value to int (|v| < 2^23) */
KG_HD int kg_rint_f(float v)
{
#if defined(__CUDA_ARCH__)
    return __float2int_rn(v);
#else
    return (int)lrintf(v);
#endif
}

/*
 * sin(x) and cos(x) in FP64 arithmetic for |x| < 4096 (NaN outside).
 *   n = nearest integer to x*128/pi (picked in FP32; any nearby n is fine),
 *   r = x - n*H1 - n*H2 - n*H3 (three-part Cody-Waite; the first fma is exact), |r| <~ pi/256,
 *   sin x = S_n (1 - pc) + C_n (r + r*ps),  cos x = C_n (1 - pc) - S_n (r + r*ps)
 * with ps = sin(r)/r - 1 and pc = 1 - cos(r) as short Taylor polynomials in r^2.
 */
KG_HD void kg_sincos_f64(double x, double* s_out, double* c_out)
{
    if ((kg_bits(x) & 0x7fffffffffffffffull) >= 0x40b0000000000000ull) { /* |x| >= 4096, inf, NaN */
        double nan_ = kg_from_bits(0x7ff8000000000000ull);
        *s_out = nan_;
        *c_out = nan_;
        return;
    }
#if defined(__CUDA_ARCH__)
    int n = kg_rint_f(__fmul_rn(__double2float_rn(x), KG_SC_INV_H_F));
#else
    float xf = (float)x;
    float xn = xf * KG_SC_INV_H_F;
    int n = kg_rint_f(xn);
#endif
    double nd = (double)n;
    double r = kg_fma(-nd, KG_SC_H1, x);
    r = kg_fma(-nd, KG_SC_H2, r);
    r = kg_fma(-nd, KG_SC_H3, r);
    int b = (n & (KG_SC_N - 1)) * 4;
    double sh = kg_tab_sc(b + 0), sl = kg_tab_sc(b + 1);
    double ch = kg_tab_sc(b + 2), cl = kg_tab_sc(b + 3);
    double z = r * r;
    double ps = kg_fma(z, KG_S7, KG_S5);
    ps = kg_fma(z, ps, KG_S3);
    ps = z * ps;
    double pc = kg_fma(z, KG_C6, KG_C4);
    pc = kg_fma(z, pc, KG_C2);
    pc = z * pc;
    double rp = r * ps;
    double st = kg_fma(ch, rp, sl);
    st = kg_fma(-sh, pc, st);
    st = kg_fma(cl, r, st);
    st = kg_fma(ch, r, st);
    double ct = kg_fma(-sh, rp, cl);
    ct = kg_fma(-ch, pc, ct);
    ct = kg_fma(-sl, r, ct);
    ct = kg_fma(-sh, r, ct);
    *s_out = sh + st;
    *c_out = ch + ct;
}



/*
 * Integer-pipe division by a fixed divisor: the same bits as a / b (IEEE,
 * round to nearest even) computed with 64-bit integer arithmetic instead of
 * FP64 operations (on GB300 the FP64 pipe is the bottleneck and the integer
 * pipes are ~30x wider).
 *
 * With A, B the 53-bit significands of a and b (hidden bit included),
 * N = A' 2^52 where A' = 2A if A < B (so that N/B lies in [2^52, 2^53)), and
 * R = floor(2^116 / B), the estimate q = floor(A' R / 2^64) satisfies
 * floor(N/B) - 1 <= q <= floor(N/B) (the truncation of R costs less than
 * A'/2^64 < 2^-10).  One comparison of the exact remainder N - qB (computed
 * modulo 2^64: it lies in [0, 2B)) fixes q, and 2 rem > B decides the
 * rounding (an exact tie would need B = 2^52, i.e. b a power of two, which
 * is handled as an exact exponent shift).  Zero dividends return a;
 * subnormal, infinite and NaN dividends, and quotients that would be
 * subnormal or overflow, take the IEEE division.
 */
typedef struct kg_idivc {
    uint64_t B;  /* significand of b with the hidden bit */
    uint64_t R;  /* floor(2^116 / B); 0 for a power of two */
    double b;    /* the divisor itself, for the IEEE fallback */
    int eb;      /* biased exponent field of b */
    int pow2;    /* b is a power of two */
} kg_idivc;

KG_HD int kg_clz64(uint64_t x)
{
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

KG_HD uint64_t kg_umulhi64(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#elif defined(__SIZEOF_INT128__)
    return (uint64_t)(((unsigned __int128)a * b) >> 64);
#else
    uint64_t a0 = a & 0xffffffffull, a1 = a >> 32, b0 = b & 0xffffffffull, b1 = b >> 32;
    uint64_t p00 = a0 * b0, p01 = a0 * b1, p10 = a1 * b0, p11 = a1 * b1;
    uint64_t mid = (p00 >> 32) + (p01 & 0xffffffffull) + (p10 & 0xffffffffull);
    return p11 + (p01 >> 32) + (p10 >> 32) + (mid >> 32);
#endif
}

/* returns 0 for a positive normal b in [2^-100, 2^100], -1 otherwise */
KG_HD int kg_idiv_prepare(double b, kg_idivc* c)
{
    if (!(b >= 0x1p-100 && b <= 0x1p100))
        return -1;
    uint64_t ub = kg_bits(b);
    c->b = b;
    c->eb = (int)((ub >> 52) & 0x7ff);
    c->B = (ub & 0x000fffffffffffffull) | 0x0010000000000000ull;
    c->pow2 = (c->B == 0x0010000000000000ull);
    if (c->pow2) {
        c->R = 0;
    } else {
        /* floor(2^116 / B) by long division, 64 quotient bits after the leading 2^63 */
        uint64_t rem = (1ull << 63) % c->B, q = (1ull << 63) / c->B; /* 2^63 / B < 2^11 */
        for (int i = 0; i < 53; i++) {
            rem <<= 1;
            q <<= 1;
            if (rem >= c->B) {
                rem -= c->B;
                q |= 1;
            }
        }
        c->R = q;
    }
    return 0;
}

/* 1: subnormal dividends of kg_idiv stay on the integer pipes; 0: they take the hardware division */
#ifndef KG_IDIV_SUBN
#define KG_IDIV_SUBN 1
#endif

/*
 * sign | RN(Q 2^(e-1075)) for a quotient whose exact significand is Q = q + rem/B
 * (q in [2^52, 2^53), rem in [0, B)) and whose biased exponent e < 1: a
 * subnormal result (or zero), rounded once from the exact quotient.
 */
KG_HD double kg_round_subnormal(uint64_t sign, uint64_t q, uint64_t rem, int e)
{
    int s = 1 - e;
    if (s > 53)
        return kg_from_bits(sign);
    uint64_t low = q & ((1ull << s) - 1), half = 1ull << (s - 1), m = q >> s;
    m += (uint64_t)((low > half) | ((low == half) & ((rem != 0) | (int)(m & 1))));
    return kg_from_bits(sign | m);
}

KG_HD double kg_idiv(double a, const kg_idivc* c)
{
    uint64_t ua = kg_bits(a);
    uint64_t sign = ua & 0x8000000000000000ull;
    int ea = (int)((ua >> 52) & 0x7ff);
    if ((ua & 0x7fffffffffffffffull) == 0)
        return a;
    if (ea == 0x7ff)
        return kg_div_slow(a, c->b);
    uint64_t A;
#if KG_IDIV_SUBN == 0
    if (ea == 0)
        return kg_div_slow(a, c->b);
#endif
    if (ea == 0) { /* subnormal dividend: normalise its significand */
        int sh = kg_clz64(ua & 0x7fffffffffffffffull) - 11;
        A = (ua & 0x7fffffffffffffffull) << sh;
        ea = 1 - sh;
    } else {
        A = (ua & 0x000fffffffffffffull) | 0x0010000000000000ull;
    }
    if (c->pow2) {
        int e = ea - c->eb + 1023;
        if (e >= 1 && e <= 2046)
            return kg_from_bits(sign | ((uint64_t)e << 52) | (A & 0x000fffffffffffffull));
        if (e < 1)
            return kg_round_subnormal(sign, A, 0, e);
    } else {
        int shift = A < c->B;
        uint64_t Ap = A << shift;
        uint64_t q = kg_umulhi64(Ap, c->R);
        uint64_t rem = (Ap << 52) - q * c->B;
        if (rem >= c->B) {
            q += 1;
            rem -= c->B;
        }
        int e = ea - c->eb + 1023 - shift;
        if (e >= 1 && e <= 2046)
            return kg_from_bits(sign | (((uint64_t)(e - 1) << 52) + q + ((rem << 1) > c->B)));
        if (e < 1)
            return kg_round_subnormal(sign, q, rem, e);
    }
    return kg_div_slow(a, c->b);
}



/* RN(RN(2 s) + y), the reference's "2.0 * s + y", in one FMA.  2 s is exact
 * unless it overflows, so the two roundings reduce to the FMA's one.  The
 * exception is |s| >= 2^1023 (exponent field 2046), where RN(2 s) = +-inf;
 * that case is finished in integer arithmetic, with no FP64 instruction:
 * inf + y = inf, except NaN for y = NaN or y = -inf of the other sign. */
KG_HD double kg_twice_plus(double s, double y)
{
    uint64_t u = kg_bits(s);
    if ((u & 0x7ff0000000000000ull) != 0x7fe0000000000000ull)
        return kg_fma(2.0, s, y);
    uint64_t inf = (u & 0x8000000000000000ull) | 0x7ff0000000000000ull;
    uint64_t v = kg_bits(y);
    if ((v & 0x7fffffffffffffffull) > 0x7ff0000000000000ull)
        return kg_from_bits(v | 0x0008000000000000ull);
    if (v == (inf ^ 0x8000000000000000ull))
        return kg_from_bits(0x7ff8000000000000ull);
    return kg_from_bits(inf);
}

/* The largest |t| for which c - t rounds to c exactly, as a bit pattern of
 * |t| (compare (bits(t) & ~sign) <= bound): 2^(e-55) for c normal in
 * [2^e, 2^(e+1)), below half the spacing of the doubles next to c on either
 * side; only t = +-0 for c zero or subnormal. */
KG_HD uint64_t kg_absorb_bound(double c)
{
    uint64_t a = kg_bits(c) & 0x7fffffffffffffffull;
    int e = (int)(a >> 52); /* biased exponent of c */
    if (e == 0 || e == 0x7ff)
        return 0;
    int eb = e - 55; /* biased exponent of 2^(e-55) */
    if (eb >= 1)
        return (uint64_t)eb << 52;
    if (eb > -52)
        return 1ull << (51 + eb); /* a subnormal power of two */
    return 0;
}

/*
 * R ~ 2^116 / B for a significand B in (2^52, 2^53), within a few units: the
 * correctly rounded FP32 reciprocal of B's top 24 bits (relative error
 * < 2^-22) refined by two Newton steps R += R (2^116 - B R) / 2^116 in 64- and
 * 128-bit integer arithmetic (error < 2^-44, then a few units of R).
 */
KG_HD uint64_t kg_recip116(uint64_t B)
{
    /* seed: 1/(B >> 29) in FP32 (B >> 29 < 2^24 converts exactly), as R0 ~ 2^116 / B */
    uint32_t fy = kg_fbits(kg_rcp_f((float)(uint32_t)(B >> 29)));
    int fe = (int)(fy >> 23); /* 103 or 104: the reciprocal lies in (2^-24, 2^-23] */
    uint64_t R = fe >= 104 ? 0xffffffffffffffffull : ((uint64_t)((fy & 0x7fffff) | 0x800000)) << (fe - 63);
    for (int it = 0; it < 2; it++) {
        /* D = (2^116 - B R) / 2^52, from the 128-bit product B R */
        uint64_t phi = kg_umulhi64(B, R), plo = B * R;
        int64_t D = (int64_t)((0x0010000000000000ull - phi) << 12) - (int64_t)(plo >> 52);
        if (D >= 0)
            R += kg_umulhi64(R, (uint64_t)D);
        else
            R -= kg_umulhi64(R, (uint64_t)(-D));
    }
    return R;
}

/*
 * a / b with the bits of the IEEE division, for any divisor, on the integer
 * pipes.  With A, B the significands (hidden bit set) and A' = A or 2A so
 * that A'/B is in [1, 2):
 *   R ~ 2^116 / B (kg_recip116);
 *   q = floor(A' R / 2^64) is then within one of floor(A' 2^52 / B); the
 *     exact remainder A' 2^52 - q B (small, so it is computed modulo 2^64
 *     and read as signed) corrects q and gives the rounding bit.  A quotient
 *     of two 53-bit significands is never halfway between two doubles
 *     unless B is a power of two, which is an exponent shift here.
 * Zero dividends give a signed zero; subnormal operands are normalised and
 * subnormal quotients rounded once from the exact remainder; non-finite
 * operands, a zero divisor and overflowing quotients take the hardware
 * division.
 */
KG_HD double kg_gdiv(double a, double b)
{
    const uint64_t MANT = 0x000fffffffffffffull, HID = 0x0010000000000000ull;
    uint64_t ua = kg_bits(a), ub = kg_bits(b);
    uint64_t sign = (ua ^ ub) & 0x8000000000000000ull;
    int ea = (int)((ua >> 52) & 0x7ff), eb = (int)((ub >> 52) & 0x7ff);
    if (eb == 0x7ff || ea == 0x7ff || (ub & 0x7fffffffffffffffull) == 0)
        return kg_div_slow(a, b);
    if ((ua & 0x7fffffffffffffffull) == 0)
        return kg_from_bits(sign);
    uint64_t A, B;
    if (ea == 0) { /* subnormal operands: normalise the significands */
        int sh = kg_clz64(ua & 0x7fffffffffffffffull) - 11;
        A = (ua & 0x7fffffffffffffffull) << sh;
        ea = 1 - sh;
    } else {
        A = (ua & MANT) | HID;
    }
    if (eb == 0) {
        int sh = kg_clz64(ub & 0x7fffffffffffffffull) - 11;
        B = (ub & 0x7fffffffffffffffull) << sh;
        eb = 1 - sh;
    } else {
        B = (ub & MANT) | HID;
    }
    if (B == HID) {
        int e = ea - eb + 1023;
        if (e >= 1 && e <= 2046)
            return kg_from_bits(sign | ((uint64_t)e << 52) | (A & MANT));
        if (e < 1)
            return kg_round_subnormal(sign, A, 0, e);
        return kg_div_slow(a, b);
    }
    uint64_t R = kg_recip116(B);
    int shift = A < B;
    uint64_t Ap = A << shift;
    uint64_t q = kg_umulhi64(Ap, R);
    int64_t r = (int64_t)((Ap << 52) - q * B);
    if (r < 0) {
        q -= 1;
        r += (int64_t)B;
    }
    if (r >= (int64_t)B) {
        q += 1;
        r -= (int64_t)B;
    }
    int e = ea - eb + 1023 - shift;
    if (e >= 1 && e <= 2046)
        return kg_from_bits(sign | (((uint64_t)(e - 1) << 52) + q + ((uint64_t)r * 2 > B)));
    if (e < 1)
        return kg_round_subnormal(sign, q, (uint64_t)r, e);
    return kg_div_slow(a, b);
}

/* ---- elementary functions on the integer pipes (fixed point) ----
 *
 * Qn below means an integer holding value * 2^n.  Every step is integer
 * arithmetic with a fixed truncation, so host and device give the same bits.
 * Absolute errors stay near 2^-62; the results are faithful wherever the
 * result is not tiny (atan: everywhere, relative error < 2^-56; sin/cos:
 * |value| >= 2^-9, and absolute error < 2^-60 everywhere).
 */

/* high 64 bits of the signed 128-bit product */
KG_HD int64_t kg_smulhi64(int64_t a, int64_t b)
{
#if defined(__CUDA_ARCH__)
    return __mul64hi(a, b);
#else
    uint64_t h = kg_umulhi64((uint64_t)a, (uint64_t)b);
    if (a < 0)
        h -= (uint64_t)b;
    if (b < 0)
        h -= (uint64_t)a;
    return (int64_t)h;
#endif
}

/* RN(V 2^-s) for V > 0 whose value is a normal double; ties to even on V's bits */
KG_HD double kg_fix_to_double(uint64_t V, int s)
{
    int lz = kg_clz64(V);
    uint64_t N = V << lz;
    uint64_t m = N >> 11, rest = N & 0x7ff;
    m += (uint64_t)((rest > 0x400) | ((rest == 0x400) & (int)(m & 1)));
    return kg_from_bits(((uint64_t)(1022 + 63 - lz - s) << 52) + m);
}

/* a signed Q62 value as a double, its sign flipped by `flip` (0 or the sign bit) */
KG_HD double kg_q62_to_double(int64_t V, uint64_t flip)
{
    uint64_t sign = ((uint64_t)V & 0x8000000000000000ull) ^ flip;
    uint64_t m = V < 0 ? (uint64_t)0 - (uint64_t)V : (uint64_t)V;
    if (m == 0)
        return kg_from_bits(flip);
    return kg_from_bits(kg_bits(kg_fix_to_double(m, 62)) | sign);
}

/*
 * atan(x) on the integer pipes, for every double (NaN propagates).
 *   |x| < 2^-27: atan x rounds to x.  |x| > 2^64: +-pi/2 rounded.
 *   t = |x|, or 1/|x| (kg_recip116) with the result pi/2 - atan(t), as a
 *     64-bit significand Tm (top bit set) and scale: t = Tm 2^tq.
 *   t >= 2^-7: node k = nearest of 128 t, d = t - k/128 in Q64 (exact),
 *     atan(t) = A_k + d (a_1 + d (a_2 + ... + d a_7)), A_k in Q64 and the
 *     Taylor coefficients a_j in Q62 (Gal's accurate-tables method in fixed
 *     point; |d| <= 2^-8, so the truncated tail is below 2^-65).
 *   t < 2^-7: atan(t) = t (1 - z (1/3 - z (1/5 - z (1/7 - z/9)))), z = t^2,
 *     relative to t (Q78 for z), so small results keep their precision.
 */
KG_HD double kg_atan_x(double x)
{
    const uint64_t MANT = 0x000fffffffffffffull, HID = 0x0010000000000000ull;
    uint64_t ux = kg_bits(x), ua = ux & 0x7fffffffffffffffull;
    uint64_t sign = ux & 0x8000000000000000ull;
    if (ua > 0x43f0000000000000ull) { /* |x| > 2^64, inf or NaN */
        if (ua > 0x7ff0000000000000ull)
            return kg_add_slow(x, x);
        return kg_from_bits(sign | kg_bits(KG_PIO2_HI));
    }
    if (ua < 0x3e40000000000000ull) /* |x| < 2^-27 */
        return x;
    int ex = (int)(ua >> 52) - 1023; /* -27 .. 64 */
    uint64_t mx = (ua & MANT) | HID;
    int inv = ua > 0x3ff0000000000000ull; /* |x| > 1 */
    uint64_t Tm;
    int tq;
    if (!inv) {
        Tm = mx << 11;
        tq = ex - 63;
    } else if (mx == HID) {
        Tm = 0x8000000000000000ull; /* 1/2^ex */
        tq = -63 - ex;
    } else {
        Tm = kg_recip116(mx); /* 2^116/mx 2^(-64-ex) = 1/|x| */
        tq = -64 - ex;
    }
    double r;
    if (tq >= -70) { /* t >= 2^-7 */
        uint64_t T63 = Tm >> (-(tq + 63)); /* t in Q63 */
        int k = (int)((T63 + (1ull << 55)) >> 56);
        int64_t D = (int64_t)(T63 - ((uint64_t)k << 56)) * 2; /* d in Q64 */
        const int b = k * 8;
        int64_t p = (int64_t)kg_tab_atanx(b + 7);
        p = (int64_t)kg_tab_atanx(b + 6) + kg_smulhi64(D, p);
        p = (int64_t)kg_tab_atanx(b + 5) + kg_smulhi64(D, p);
        p = (int64_t)kg_tab_atanx(b + 4) + kg_smulhi64(D, p);
        p = (int64_t)kg_tab_atanx(b + 3) + kg_smulhi64(D, p);
        p = (int64_t)kg_tab_atanx(b + 2) + kg_smulhi64(D, p);
        p = (int64_t)kg_tab_atanx(b + 1) + kg_smulhi64(D, p);
        /* d p in Q64 from the 128-bit product (Q126) */
        uint64_t hi = (uint64_t)kg_smulhi64(D, p), lo = (uint64_t)D * (uint64_t)p;
        uint64_t A = kg_tab_atanx(b) + ((hi << 2) | (lo >> 62)); /* atan(t) in Q64 */
        r = inv ? kg_fix_to_double(KG_X_PIO2_62 - (A >> 2), 62) : kg_fix_to_double(A, 64);
    } else { /* t < 2^-7 */
        uint64_t z2 = kg_umulhi64(Tm, Tm); /* t^2 = z2 2^(2 tq + 64) */
        int sh = -(2 * tq + 142);          /* z in Q78 = z2 >> sh, sh >= 0 */
        uint64_t Z = sh < 64 ? z2 >> sh : 0;
        uint64_t u = KG_X_ATAN_I9;
        u = KG_X_ATAN_I7 - (kg_umulhi64(Z, u) >> 14);
        u = KG_X_ATAN_I5 - (kg_umulhi64(Z, u) >> 14);
        u = KG_X_ATAN_I3 - (kg_umulhi64(Z, u) >> 14);
        uint64_t zu = kg_umulhi64(Z, u) >> 14;     /* z u in Q64 */
        uint64_t V = Tm - kg_umulhi64(Tm, zu);      /* atan(t) = V 2^tq */
        if (!inv) {
            r = kg_fix_to_double(V, -tq);
        } else {
            int s2 = -tq - 62; /* atan(t) in Q62 = V >> s2 */
            r = kg_fix_to_double(KG_X_PIO2_62 - (s2 < 64 ? V >> s2 : 0), 62);
        }
    }
    return kg_from_bits(kg_bits(r) | sign);
}

/* kg_sincos_f64 out of line on the device (see kg_div_slow) */
#if defined(__CUDA_ARCH__) && KG_SLOW_NOINLINE
__device__ __noinline__ static void kg_sincos_slow_dev(double x, double* s, double* c) { kg_sincos_f64(x, s, c); }
#endif

KG_HD void kg_sincos_slow(double x, double* s_out, double* c_out)
{
#if defined(__CUDA_ARCH__) && KG_SLOW_NOINLINE
    kg_sincos_slow_dev(x, s_out, c_out);
#else
    kg_sincos_f64(x, s_out, c_out);
#endif
}

/*
 * sin(x) and cos(x) on the integer pipes for |x| < 64; larger |x| (and inf,
 * NaN) take kg_sincos_f64.
 *   |x| < 2^-27: sin x rounds to x, cos x to 1.
 *   |x| < 2^-5: sin x = x (1 + z H(z)), cos x = 1 - z G(z), z = x^2, relative
 *     to x's own significand.
 *   otherwise: y = |x| 128/pi from the exact 192-bit product of |x| (Q57) and
 *     128/pi (Q122) -- a Payne-Hanek style reduction, exact to 2^-115 --
 *     n = nearest integer to y, r = (y - n) pi/128 in Q68, |r| <= pi/256;
 *     sin|x| = S_n (1 - z G) + C_n r (1 + z H), cos|x| = C_n (1 - z G) -
 *     S_n r (1 + z H) with S_n, C_n = sin, cos(n pi/128) in Q62.
 * H(z) = -1/6 + z/120 - z^2/5040 + z^3/362880 and G(z) = 1/2 - z/24 + z^2/720
 * - z^3/40320 are the Taylor series of (sin r / r - 1)/z and (1 - cos r)/z.
 */
KG_HD void kg_sincos_x(double x, double* s_out, double* c_out)
{
    const uint64_t MANT = 0x000fffffffffffffull, HID = 0x0010000000000000ull;
    uint64_t ux = kg_bits(x), ua = ux & 0x7fffffffffffffffull;
    if (ua >= 0x4050000000000000ull) { /* |x| >= 64, inf, NaN */
        kg_sincos_slow(x, s_out, c_out);
        return;
    }
    if (ua < 0x3e40000000000000ull) { /* |x| < 2^-27 */
        *s_out = x;
        *c_out = 1.0;
        return;
    }
    uint64_t flip = ux & 0x8000000000000000ull; /* sin is odd, cos even */
    int ex = (int)(ua >> 52) - 1023;            /* -27 .. 5 */
    uint64_t mx = (ua & MANT) | HID;
    int64_t Z; /* z = r^2 (or x^2) in Q72 */
    int64_t R = 0, S = 0, C = 0;
    int small = ex < -5;
    if (small) {
        uint64_t M = mx << 11;                      /* |x| = M 2^(ex-63) */
        Z = (int64_t)(kg_umulhi64(M, M) >> (-(2 * ex + 10))); /* x^2 = umulhi(M, M) 2^(2 ex - 62) */
    } else {
        uint64_t X = mx << (ex + 5); /* |x| in Q57 */
        uint64_t h0 = kg_umulhi64(X, KG_X_INVH_LO);
        uint64_t l1 = X * KG_X_INVH_HI, h1 = kg_umulhi64(X, KG_X_INVH_HI);
        uint64_t p1 = l1 + h0;
        uint64_t p2 = h1 + (uint64_t)(p1 < l1); /* y 2^179 = p2 2^128 + p1 2^64 + (below) */
        uint64_t n = (p2 + (1ull << 50)) >> 51; /* nearest integer to y */
        int64_t F = (int64_t)((p2 - (n << 51)) << 13) + (int64_t)(p1 >> 51); /* y - n in Q64 */
        R = kg_smulhi64(F, (int64_t)KG_X_H68); /* r in Q68 */
        Z = kg_smulhi64(R, R);                 /* r^2 in Q72 */
        S = kg_tab_scx(2 * (int)(n & (KG_SC_N - 1)));
        C = kg_tab_scx(2 * (int)(n & (KG_SC_N - 1)) + 1);
    }
    int64_t H = KG_X_H3;
    H = KG_X_H2 + (kg_smulhi64(Z, H) >> 8);
    H = KG_X_H1 + (kg_smulhi64(Z, H) >> 8);
    H = KG_X_H0 + (kg_smulhi64(Z, H) >> 8); /* Q63 */
    int64_t G = KG_X_G3;
    G = KG_X_G2 + (kg_smulhi64(Z, G) >> 8);
    G = KG_X_G1 + (kg_smulhi64(Z, G) >> 8);
    G = KG_X_G0 + (kg_smulhi64(Z, G) >> 8); /* Q63 */
    int64_t ps = kg_smulhi64(Z, H);          /* sin(r)/r - 1 in Q71 (<= 0) */
    int64_t pc = kg_smulhi64(Z, G);          /* 1 - cos(r) in Q71 (>= 0) */
    if (small) {
        uint64_t M = mx << 11;
        uint64_t V = M - (kg_umulhi64(M, (uint64_t)(-ps)) >> 7); /* sin|x| = V 2^(ex-63) */
        *s_out = kg_from_bits(kg_bits(kg_fix_to_double(V, 63 - ex)) | flip);
        *c_out = kg_fix_to_double((1ull << 62) - (uint64_t)(pc >> 9), 62);
        return;
    }
    int64_t sr = R + (kg_smulhi64(R, ps) >> 7); /* sin(r) in Q68 */
    int64_t sn = S - (kg_smulhi64(S, pc) >> 7) + (kg_smulhi64(C, sr) >> 4);
    int64_t cs = C - (kg_smulhi64(C, pc) >> 7) - (kg_smulhi64(S, sr) >> 4);
    *s_out = kg_q62_to_double(sn, flip);
    *c_out = kg_q62_to_double(cs, 0);
}

/* the functions the step uses: the integer-pipe versions */
KG_HD double kg_atan(double x) { return kg_atan_x(x); }

KG_HD void kg_sincos(double x, double* s_out, double* c_out) { kg_sincos_x(x, s_out, c_out); }

#endif /* KG_MATH_H */

"""Generate kg_math_tables.h: the constant tables behind kg_atan and kg_sincos.

Every entry is computed with mpmath at 320-bit precision and rounded to the
nearest double through an exact rational (``fractions.Fraction.__float__`` is
correctly rounded), so the tables are a pure function of the mathematics and
regenerate bit-identically.

Methods (both published, written here from the mathematics):

* atan: table-driven Taylor expansion (Gal's "accurate tables" idea, as used by
  Tang for exp/log).  The reduced argument t in [0, 1] is split as
  t = c_k + d with c_k = k/128 and |d| <= 1/256; atan(c_k + d) is the degree-7
  Taylor polynomial of atan around c_k.  The value atan(c_k) (and pi/2 -
  atan(c_k) for the reciprocal branch) is stored as an unevaluated hi+lo pair.
* sin/cos: Cody-Waite additive reduction by h = pi/128 (three-part split of h),
  then sin(n h + r) = S_n cos r + C_n sin r with S_n, C_n stored as hi+lo
  pairs and Taylor polynomials for sin r, cos r on |r| <= pi/256.

Run:  python gen_kg_math_tables.py > kg_math_tables.h
"""
from fractions import Fraction
import mpmath as mp

mp.mp.prec = 320

ATAN_N = 128          # table spacing 1/ATAN_N on [0, 1]
ATAN_DEG = 7          # Taylor degree around each node
SC_N = 256            # sin/cos nodes per period: h = 2 pi / SC_N = pi/128
STRIDE = 16           # doubles per atan entry (one 128-byte line)


def exact(x):
    """Exact rational value of an mpf (sign, mantissa, exponent)."""
    if isinstance(x, Fraction):
        return x
    sign, man, exp, _ = mp.mpf(x)._mpf_
    v = Fraction(int(man)) * (Fraction(2) ** int(exp)) if exp >= 0 else Fraction(int(man), 2 ** int(-exp))
    return -v if sign else v


def rn(x):
    """Round an mpf (or Fraction) to the nearest double."""
    if isinstance(x, Fraction):
        return float(x)
    return float(exact(x))


def hilo(x):
    hi = rn(x)
    lo = float(exact(x) - Fraction(hi))
    return hi, lo


def fmt(v):
    return float.hex(float(v))


def atan_taylor(k, n_nodes, deg):
    """Exact Taylor coefficients a_1..a_deg of atan around c = k/n_nodes.

    atan'(c + d) = 1 / (A + B d + d^2) with A = 1 + c^2, B = 2c; its power
    series g_n obeys g_0 = 1/A, g_n = -(B g_{n-1} + g_{n-2}) / A, and
    a_n = g_{n-1} / n.  Everything is an exact rational."""
    c = Fraction(k, n_nodes)
    A, B = 1 + c * c, 2 * c
    g = [1 / A]
    for n in range(1, deg):
        g.append(-(B * g[n - 1] + (g[n - 2] if n >= 2 else 0)) / A)
    return [None] + [g[n - 1] / n for n in range(1, deg + 1)]


def main():
    out = []
    out.append("/* Generated by gen_kg_math_tables.py -- do not edit. */")
    out.append("#pragma once")
    out.append(f"#define KG_ATAN_N {ATAN_N}")
    out.append(f"#define KG_ATAN_STRIDE {STRIDE}")
    out.append("/* atan entry k: c_k, atan_hi, atan_lo, (pi/2-atan)_hi, (pi/2-atan)_lo, a1..a7, pad */")
    out.append("#define KG_ATAN_TAB_DATA { \\")
    pio2 = mp.pi / 2
    for k in range(ATAN_N + 1):
        c = mp.mpf(k) / ATAN_N
        a = atan_taylor(k, ATAN_N, ATAN_DEG)
        a0 = mp.atan(c)
        ahi, alo = hilo(a0)
        bhi, blo = hilo(pio2 - a0)
        row = [rn(c), ahi, alo, bhi, blo] + [rn(a[n]) for n in range(1, ATAN_DEG + 1)]
        row += [0.0] * (STRIDE - len(row))
        out.append("  " + ", ".join(fmt(v) for v in row) + ", \\")
    out.append("}")

    h = 2 * mp.pi / SC_N
    # three-part Cody-Waite split: H1, H2 keep 35 significant bits each so n*H1
    # and n*H2 are exact for |n| < 2^18; H3 is the rounded remainder
    hf = exact(h)
    e = int(mp.floor(mp.log(h, 2)))
    q1 = Fraction(2) ** (e - 34)
    h1 = Fraction(int(hf / q1)) * q1
    q2 = Fraction(2) ** (e - 34 - 35)
    h2 = Fraction(int((hf - h1) / q2)) * q2
    h3 = rn(hf - h1 - h2)
    h1, h2 = float(h1), float(h2)
    out.append(f"#define KG_SC_N {SC_N}")
    out.append(f"#define KG_SC_INV_H_F {float(rn(1 / h)):.9g}f   /* 128/pi, used in FP32 to pick n */")
    out.append(f"#define KG_SC_H1 {fmt(h1)}   /* pi/128, leading 35 bits */")
    out.append(f"#define KG_SC_H2 {fmt(h2)}   /* next 35 bits */")
    out.append(f"#define KG_SC_H3 {fmt(h3)}   /* pi/128 - H1 - H2, rounded */")
    out.append("/* sin/cos entry n: S_hi, S_lo, C_hi, C_lo with S = sin(n pi/128), C = cos(n pi/128) */")
    out.append("#define KG_SC_TAB_DATA { \\")
    for n in range(SC_N):
        s_hi, s_lo = hilo(mp.sin(n * h))
        c_hi, c_lo = hilo(mp.cos(n * h))
        out.append("  " + ", ".join(fmt(v) for v in (s_hi, s_lo, c_hi, c_lo)) + ", \\")
    out.append("}")
    # Taylor coefficients of sin r / r - 1 = z*(S3 + z*(S5 + z*S7)) and 1 - cos r = z*(C2 + z*(C4 + z*C6))
    out.append(f"#define KG_S3 {fmt(rn(mp.mpf(-1) / 6))}")
    out.append(f"#define KG_S5 {fmt(rn(mp.mpf(1) / 120))}")
    out.append(f"#define KG_S7 {fmt(rn(mp.mpf(-1) / 5040))}")
    out.append(f"#define KG_C2 {fmt(0.5)}")
    out.append(f"#define KG_C4 {fmt(rn(mp.mpf(-1) / 24))}")
    out.append(f"#define KG_C6 {fmt(rn(mp.mpf(1) / 720))}")
    pio2_hi, pio2_lo = hilo(pio2)
    out.append(f"#define KG_PIO2_HI {fmt(pio2_hi)}")
    out.append(f"#define KG_PI {fmt(rn(mp.pi))}")
    out += fixed_point_tables()
    print("\n".join(out))


def q(x, bits):
    """x * 2^bits rounded to the nearest integer (exact rational arithmetic)."""
    v = exact(x) * (Fraction(2) ** bits)
    return int(v + Fraction(1, 2)) if v >= 0 else -int(-v + Fraction(1, 2))


def u64(v):
    """a 64-bit literal for a value in [-2^63, 2^64) (negative values in two's complement)"""
    assert -(1 << 63) <= v < (1 << 64)
    return "0x%016xull" % (v & ((1 << 64) - 1))


def fixed_point_tables():
    """Tables of the integer-pipe atan and sin/cos (fixed point, Qn = value * 2^n).

    atan: for the node c_k = k/128 (k = 0..128), atan(c_k) in Q64 and the
    Taylor coefficients a_1..a_7 of atan around c_k in Q62 (signed).
    sin/cos: sin(n pi/128), cos(n pi/128) for n = 0..255 in Q62 (signed).
    Reduction: 128/pi in Q122 as two 64-bit words, pi/128 in Q68, pi/2 in Q62.
    Polynomials: atan(t)/t - 1 = -z (1/3 - z (1/5 - z (1/7 - z/9))), z = t^2,
    coefficients in Q64; sin(r)/r - 1 = z H(z), 1 - cos(r) = z G(z), z = r^2,
    H, G coefficients in Q63 (signed)."""
    out = []
    out.append("/* integer-pipe atan, entry k (8 words): atan(k/128) Q64, a1..a7 Q62 (signed) */")
    out.append("#define KG_ATANX_TAB_DATA { \\")
    for k in range(ATAN_N + 1):
        a = atan_taylor(k, ATAN_N, ATAN_DEG)
        row = [q(mp.atan(mp.mpf(k) / ATAN_N), 64)] + [q(a[n], 62) for n in range(1, ATAN_DEG + 1)]
        assert row[0] < (1 << 64) and all(-(1 << 63) <= v < (1 << 63) for v in row[1:])
        out.append("  " + ", ".join(u64(v) for v in row) + ", \\")
    out.append("}")
    out.append("/* integer-pipe sin/cos, entry n: sin(n pi/128), cos(n pi/128) in Q62 (signed) */")
    out.append("#define KG_SCX_TAB_DATA { \\")
    h = mp.pi / 128
    for n in range(SC_N):
        out.append("  " + u64(q(mp.sin(n * h), 62)) + ", " + u64(q(mp.cos(n * h), 62)) + ", \\")
    out.append("}")
    k = q(128 / mp.pi, 122)
    assert k < (1 << 128)
    out.append("#define KG_X_INVH_HI %s /* 128/pi in Q122, high word */" % u64(k >> 64))
    out.append("#define KG_X_INVH_LO %s /* low word */" % u64(k & ((1 << 64) - 1)))
    out.append("#define KG_X_H68 %s /* pi/128 in Q68 */" % u64(q(h, 68)))
    out.append("#define KG_X_PIO2_62 %s /* pi/2 in Q62 */" % u64(q(mp.pi / 2, 62)))
    for n in (3, 5, 7, 9):
        out.append("#define KG_X_ATAN_I%d %s /* 1/%d in Q64 */" % (n, u64(q(mp.mpf(1) / n, 64)), n))
    for name, v in (("H0", mp.mpf(-1) / 6), ("H1", mp.mpf(1) / 120), ("H2", mp.mpf(-1) / 5040),
                    ("H3", mp.mpf(1) / 362880), ("G0", mp.mpf(1) / 2), ("G1", mp.mpf(-1) / 24),
                    ("G2", mp.mpf(1) / 720), ("G3", mp.mpf(-1) / 40320)):
        out.append("#define KG_X_%s ((int64_t)%s) /* %s in Q63 */" % (name, u64(q(v, 63)), mp.nstr(v, 8)))
    return out


if __name__ == "__main__":
    main()

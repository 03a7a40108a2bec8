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
    print("\n".join(out))


if __name__ == "__main__":
    main()

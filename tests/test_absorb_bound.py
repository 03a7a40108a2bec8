"""The exponent bound behind the step's latent-heat shortcut (kg_stage2 in
crystalgrowth_gb300/csrc/kg_device.cuh, switch KG_ABSORB).

The reference updates T' = (T + lap_T dt) + K (phi' - phi) with phi' = phi + q
(src/Kobayashi.cpp:211-215).  Writing x = T + lap_T dt, the kernel returns x
without computing the last term wherever

    1 <= eb_x <= 2046  and  eb_K + M + 56 < eb_x,
    M = max(eb_q - 1022, max(eb_phi', 1) - 1076),

eb being a double's biased exponent field.  This test restates that predicate
(checking the source still has it), and on millions of adversarial IEEE
values (powers of two, subnormals, zeros of both signs, huge and tiny K, q
near half an ulp of phi, cancellation) checks that wherever it holds the full
expression x + K (phi' - phi), evaluated in IEEE double arithmetic with round
to nearest, gives x's bits exactly."""
import os

import numpy as np

SRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "crystalgrowth_gb300", "csrc",
                   "kg_device.cuh")


def eb(a):
    return ((a.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7ff)).astype(np.int64)


def predicate(x, q, new_phi, K):
    M = np.maximum(eb(q) - 1022, np.maximum(eb(new_phi), 1) - 1076)
    ebx = eb(x)
    return (ebx >= 1) & (ebx <= 2046) & (eb(K) + M + 56 < ebx)


def test_source_has_the_predicate():
    src = open(SRC).read()
    for s in ("const int M = max(ebq - 1022, ebn - 1076);", "if (ebx >= 1 && ebx <= 2046 && P.ebk + M + 56 < ebx)",
              "const int ebn = max((int)((kg_bits(new_phi) >> 52) & 0x7ff), 1);", "t = x + P.K * (new_phi - old_phi);"):
        assert s in src, s


def _cases(rng, n):
    def scaled(lo, hi, size):
        return rng.uniform(1, 2, size) * 2.0 ** rng.integers(lo, hi, size) * rng.choice([-1.0, 1.0], size)
    old_phi = np.concatenate([scaled(-1074, 2, n), rng.uniform(-0.1, 1.1, n), np.full(n // 8, 0.0),
                              np.full(n // 8, -0.0), scaled(-1074, -1000, n // 4)])
    m = old_phi.size
    # q relative to phi's ulp: from far below half an ulp (absorbed into phi') to far above
    rel = 2.0 ** rng.integers(-70, 5, m) * rng.uniform(0.25, 2.0, m) * rng.choice([-1.0, 1.0], m)
    q = old_phi * rel
    sub = rng.uniform(size=m) < 0.1
    q[sub] = rng.integers(-2 ** 40, 2 ** 40, sub.sum()) * 5e-324
    q[rng.uniform(size=m) < 0.02] = 0.0
    x = scaled(-1022, 1023, m)
    pw = rng.uniform(size=m) < 0.2
    x[pw] = np.sign(x[pw]) * 2.0 ** np.floor(np.log2(np.abs(x[pw])))   # exact powers of two
    K = scaled(-30, 30, m)
    K[rng.uniform(size=m) < 0.05] = 0.0
    # x near the term's size, where the predicate is decided by one exponent step
    near = rng.uniform(size=m) < 0.3
    with np.errstate(all="ignore"):
        approx = np.abs(K * q) * 2.0 ** rng.integers(50, 62, m)
    ok = near & np.isfinite(approx) & (approx > 2.0 ** -1000) & (approx < 2.0 ** 1000)
    x[ok] = approx[ok] * np.sign(x[ok])
    return x, q, old_phi, K


def test_absorbed_term_leaves_x_unchanged():
    rng = np.random.default_rng(2026)
    held = 0
    for _ in range(4):
        x, q, old_phi, K = _cases(rng, 1_000_000)
        with np.errstate(all="ignore"):
            new_phi = old_phi + q
            full = x + K * (new_phi - old_phi)
        p = predicate(x, q, new_phi, K)
        bad = p & (full.view(np.uint64) != x.view(np.uint64))
        assert not bad.any(), (x[bad][:3], q[bad][:3], old_phi[bad][:3], K[bad][:3])
        held += int(p.sum())
    assert held > 1_000_000  # the predicate holds often enough to matter


def test_predicate_is_tight_enough_to_be_useful():
    """a term one exponent step below the bound is absorbed, and the predicate accepts terms up to
    about 2^-56 of x (a few steps from the exact limit ulp(x)/4 = 2^-54 |x|)"""
    x = np.array([1.0, 1.5, 2.0 ** 100])
    q = x * 2.0 ** -60
    old_phi = np.zeros(3)
    K = np.ones(3)
    assert predicate(x, q, old_phi + q, K).all()
    assert not predicate(x, x * 2.0 ** -50, x * 2.0 ** -50, K).any()

"""Reverse-mode gradients on the GPU against the CPU tangent-linear model
(oracle/ko_oracle.c ko_tlm_run, written independently) and against central
finite differences of the forward rollout.

Tolerances: adjoint vs TLM 1e-8 relative (both are exact derivatives of the
same discrete map, they differ only in rounding); adjoint vs central finite
differences with relative step h = 1e-6 * |parameter|: 1e-6 relative.
"""
import numpy as np
import pytest

import ko_oracle
from crystalgrowth_gb300 import Adjoint, Kobayashi, configs

pytestmark = pytest.mark.gpu
PARAMS = ("delta", "K", "theta0", "tau", "gamma")


def bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float64).view(np.uint64), np.asarray(b, np.float64).view(np.uint64))


def setup(n, steps, seed=0, k=16):
    p = dict(configs.BASE)
    phi0, _, th0 = configs.initial_fields(n, n, [(n // 2, n // 2, 5)])
    T0 = np.random.default_rng(seed).normal(0, 0.01, (n, n))
    target = ko_oracle.port_run(phi0, T0, th0, dict(p, delta=0.04, K=1.8, theta0=0.5), steps, threads=8)[0]
    adj = Adjoint(n, n, p, steps, checkpoint_every=k)
    adj.set_initial(phi0, T0, th0)
    adj.set_target(target)
    return p, (phi0, T0, th0), target, adj


def test_forward_rollout_is_the_step_kernel():
    n, steps = 40, 70
    p, init, target, adj = setup(n, steps)
    loss, (phi, T, th) = adj.forward(want_state=True)
    ref = ko_oracle.port_run(*init, p, steps, threads=8)
    for x, y in zip((phi, T, th), ref):
        assert bits_equal(x, y)
    assert loss == pytest.approx(0.5 * np.sum((ref[0] - target) ** 2), rel=1e-14)
    adj.close()


@pytest.mark.parametrize("n,steps,k", [(40, 70, 16), (33, 50, 7), (64, 120, 64)])
def test_adjoint_matches_tangent_linear_model(n, steps, k):
    p, init, target, adj = setup(n, steps, k=k)
    g, dT0 = adj.gradient()
    z = np.zeros((n, n))
    for name in PARAMS:
        st, tg = ko_oracle.tlm_run(*init, z, z, z, p, {"d_" + name: 1.0}, steps, threads=8)
        dl = float(np.sum((st[0] - target) * tg[0]))
        assert g["d_" + name] == pytest.approx(dl, rel=1e-8, abs=1e-12 * abs(dl) + 1e-14), name
    v = np.random.default_rng(1).normal(0, 1, (n, n))
    st, tg = ko_oracle.tlm_run(*init, z, v, z, p, {}, steps, threads=8)
    dl = float(np.sum((st[0] - target) * tg[0]))
    assert float(np.sum(dT0 * v)) == pytest.approx(dl, rel=1e-8)
    adj.close()


def test_adjoint_matches_finite_differences():
    n, steps = 48, 150
    p, init, target, adj = setup(n, steps, k=32)
    g, dT0 = adj.gradient()

    def loss(pp, T0=init[1]):
        return 0.5 * float(np.sum((ko_oracle.port_run(init[0], T0, init[2], pp, steps, threads=8)[0] - target) ** 2))

    for name in PARAMS:
        h = 1e-6 * abs(p[name]) if p[name] != 0 else 1e-6
        fd = (loss(dict(p, **{name: p[name] + h})) - loss(dict(p, **{name: p[name] - h}))) / (2 * h)
        assert g["d_" + name] == pytest.approx(fd, rel=1e-6), name
    v = np.random.default_rng(2).normal(0, 1, (n, n))
    h = 1e-6
    fd = (loss(p, init[1] + h * v) - loss(p, init[1] - h * v)) / (2 * h)
    assert float(np.sum(dT0 * v)) == pytest.approx(fd, rel=1e-6)
    adj.close()


def test_gradient_is_deterministic():
    n, steps = 40, 60
    _, _, _, adj = setup(n, steps)
    g1, d1 = adj.gradient()
    g2, d2 = adj.gradient()
    assert g1 == g2 and bits_equal(d1, d2)
    adj.close()


def test_checkpoint_interval_does_not_change_the_gradient():
    n, steps = 36, 90
    res = []
    for k in (1, 10, 90):
        _, _, _, adj = setup(n, steps, k=k)
        res.append(adj.gradient())
        adj.close()
    for g, d in res[1:]:
        assert g == res[0][0] and bits_equal(d, res[0][1])


def _config4(steps=None):
    """the 512^2 adjoint case: target from delta=.04, K=1.8, theta0=.5; gradient at delta=.02, K=1.6,
    theta0=.2; T0 ~ N(0, 0.01^2); checkpoints every 64 steps"""
    cfg = configs.adjoint_512()
    n = cfg["nx"]
    steps = steps or cfg["steps"]
    phi0, _, th0 = configs.initial_fields(n, n, cfg["disks"])
    T0 = cfg["T0"]
    tgt = Adjoint(n, n, cfg["target_params"], steps, checkpoint_every=cfg["checkpoint_every"])
    tgt.set_initial(phi0, T0, th0)
    tgt.set_target(np.zeros((n, n)))
    _, (target, _, _) = tgt.forward(want_state=True)
    tgt.close()
    adj = Adjoint(n, n, cfg["params"], steps, checkpoint_every=cfg["checkpoint_every"])
    adj.set_initial(phi0, T0, th0)
    adj.set_target(target)
    return cfg["params"], (phi0, T0, th0), target, adj, steps


def test_adjoint_512_full_horizon_matches_tangent_linear_model():
    """512^2, 4000 steps: the gradient against the CPU tangent-linear model along one combined
    direction (all five parameters and a random T0 field at once).  Both are the exact derivative of
    the discrete map (branches differentiated piecewise), so the tolerance is 1e-10 relative."""
    import os
    p, init, target, adj, steps = _config4()
    g, dT0 = adj.gradient()
    rng = np.random.default_rng(44)
    w = dict(zip(PARAMS, rng.uniform(0.5, 1.5, len(PARAMS))))
    v = rng.normal(0, 1, init[1].shape)
    z = np.zeros_like(v)
    thr = max(1, min(16, os.cpu_count() or 1))
    st, tg = ko_oracle.tlm_run(*init, z, v, z, p, {"d_" + k: w[k] for k in PARAMS}, steps, threads=thr)
    tlm = float(np.sum((st[0] - target) * tg[0]))
    ours = sum(w[k] * g["d_" + k] for k in PARAMS) + float(np.sum(dT0 * v))
    assert ours == pytest.approx(tlm, rel=1e-10)
    adj.close()


def test_adjoint_512_finite_differences_1000_steps():
    """central finite differences on the 512^2 case over 1000 steps (the GPU forward rollout,
    bit-identical to the CPU oracle), steps h = 1e-6 |parameter| and h/2, h/4: 1e-6 relative for every
    parameter and a random T0 direction.  The loss is only piecewise smooth -- a cell whose gradient
    crosses the FLT_EPSILON dead-zone threshold (src/Kobayashi.cpp:154-167) under the perturbation
    changes its angle by a finite amount -- so a single difference can straddle such a jump; the
    median of the three differences is the estimate.  Over the full 4000 steps the jumps and the
    curvature are too large for any finite difference (design notes, adjoint section); the
    tangent-linear check above covers that horizon."""
    p, init, target, adj, steps = _config4(1000)
    g, dT0 = adj.gradient()

    def fd(setter, h):
        setter(+h)
        lp = adj.forward()
        setter(-h)
        lm = adj.forward()
        return (lp - lm) / (2 * h)

    for name in PARAMS:
        def setter(d, name=name):
            adj.set_params(dict(p, **{name: p[name] + d}))
        h = 1e-6 * abs(p[name])
        est = float(np.median([fd(setter, h / s) for s in (1, 2, 4)]))
        assert g["d_" + name] == pytest.approx(est, rel=1e-6), (name, g["d_" + name], est)
    adj.set_params(p)
    v = np.random.default_rng(4000).normal(0, 1, init[1].shape)

    def setter_t0(d):
        adj.set_initial(init[0], init[1] + d * v, init[2])
    est = float(np.median([fd(setter_t0, 1e-6 / s) for s in (1, 2, 4)]))
    assert float(np.sum(dT0 * v)) == pytest.approx(est, rel=1e-6)
    adj.close()

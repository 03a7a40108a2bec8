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


def test_adjoint_512_config_full():
    """The spec adjoint case: 512^2, 4000 steps, checkpoints every 64, target from
    delta=.04, K=1.8, theta0=.5, gradient at delta=.02, K=1.6, theta0=.2, T0 ~ N(0, 0.01^2).
    Finite differences use the GPU forward rollout, which is bit-identical to the CPU oracle
    (tests/test_gpu_step.py); the tangent-linear check runs on the CPU."""
    cfg = configs.adjoint_512()
    n, steps = cfg["nx"], cfg["steps"]
    phi0, _, th0 = configs.initial_fields(n, n, cfg["disks"])
    T0 = cfg["T0"]
    tgt = Adjoint(n, n, cfg["target_params"], steps, checkpoint_every=cfg["checkpoint_every"])
    tgt.set_initial(phi0, T0, th0)
    tgt.set_target(np.zeros((n, n)))
    _, (target, _, _) = tgt.forward(want_state=True)
    tgt.close()
    p = cfg["params"]
    adj = Adjoint(n, n, p, steps, checkpoint_every=cfg["checkpoint_every"])
    adj.set_initial(phi0, T0, th0)
    adj.set_target(target)
    g, dT0 = adj.gradient()
    assert g["loss"] > 0
    for name in PARAMS:
        h = 1e-6 * abs(p[name])
        adj.set_params(dict(p, **{name: p[name] + h}))
        lp = adj.forward()
        adj.set_params(dict(p, **{name: p[name] - h}))
        lm = adj.forward()
        fd = (lp - lm) / (2 * h)
        assert g["d_" + name] == pytest.approx(fd, rel=1e-6), (name, g["d_" + name], fd)
    adj.set_params(p)
    v = np.random.default_rng(4000).normal(0, 1, (n, n))
    h = 1e-6
    adj.set_initial(phi0, T0 + h * v, th0)
    lp = adj.forward()
    adj.set_initial(phi0, T0 - h * v, th0)
    lm = adj.forward()
    fd = (lp - lm) / (2 * h)
    assert float(np.sum(dT0 * v)) == pytest.approx(fd, rel=1e-6)
    # CPU tangent-linear model along the same T0 direction and along K
    z = np.zeros((n, n))
    import os
    thr = max(1, min(16, os.cpu_count() or 1))
    st, tg = ko_oracle.tlm_run(phi0, T0, th0, z, v, z, p, {"d_K": 1.0}, steps, threads=thr)
    dl = float(np.sum((st[0] - target) * tg[0]))
    assert float(np.sum(dT0 * v)) + g["d_K"] == pytest.approx(dl, rel=1e-8)
    adj.close()

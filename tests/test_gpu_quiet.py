"""The quiet-cell shortcut of the fused step, and the handle's time-out latch.

Quiet cells (a 3x3 phi neighbourhood of +0) skip the phi update and, with a
+0 T neighbourhood too, the T update; the results must equal the oracle's
full expressions bit for bit, including the signs of zeros.  The cases here
put -0 into phi and T, a negative K (so K * (+0) = -0 in the T update), a
non-zero angle inside a zero-phi region (not flat eps^2: the shortcut must not
apply) and T values whose update T + lap_T dt is exactly zero.

The latch: after a bounded wait has run out (injected on the host: the
handle's error flag is raised without any kernel), kg_sync reports
KG_ERR_TIMEOUT, kg_step refuses, and replacing the state clears it."""
import ctypes

import numpy as np
import pytest

import ko_oracle
from crystalgrowth_gb300 import Kobayashi, KgError, configs, _lib

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float64).view(np.uint64), np.asarray(b, np.float64).view(np.uint64))


def signed_zero_state(nx=160, ny=120, seed=1):
    rng = np.random.default_rng(seed)
    phi = np.zeros((ny, nx))
    T = np.zeros((ny, nx))
    th = np.zeros((ny, nx))
    phi[50:60, 40:52] = 1.0                               # a crystal
    phi[10:14, 100:110] = -0.0                            # negative zeros in a quiet region
    T[:, 120:] = rng.normal(0, 1e-3, (ny, nx - 120))      # T without phi: phi quiet, T not
    T[80:90, 120:130] = -0.0
    T[100:104, 10:14] = 1e-300                            # tiny T: lap_T dt underflows
    T[105, 20] = -5e-324
    th[20:24, 60:64] = 0.3                                # an angle where phi is zero: eps^2 not flat
    th[30, 140] = -0.0
    return phi, T, th


@pytest.mark.parametrize("K", [1.6, -1.3, 0.0])
@pytest.mark.parametrize("tblock", [1, 2])
def test_quiet_cells_signed_zeros(K, tblock):
    p = dict(configs.BASE, K=K)
    init = signed_zero_state()
    sim = Kobayashi(160, 120, p["dt"], params=p)
    sim.set_fields(*init)
    sim.set_tblock(tblock)
    sim.step(37)
    a = sim.fields()
    sim.close()
    b = ko_oracle.port_run(*init, p, 37, libm=False, threads=8)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


@pytest.mark.parametrize("nx", [260, 141])
def test_quiet_and_busy_regions_with_bulk_copies(nx):
    """even width: interior strips stage rows with bulk copies; odd: per-lane loads"""
    p = dict(configs.BASE, K=-0.7, theta0=0.3)
    rng = np.random.default_rng(3)
    phi = np.zeros((90, nx))
    phi[40:50, 30:45] = 1.0
    T = np.where(rng.uniform(size=(90, nx)) < 0.05, rng.normal(0, 1e-2, (90, nx)), 0.0)
    T[T == 0] = np.where(rng.uniform(size=(T == 0).sum()) < 0.5, -0.0, 0.0)
    th = np.zeros((90, nx))
    sim = Kobayashi(nx, 90, p["dt"], params=p)
    sim.set_fields(phi, T, th)
    sim.step(25)
    a = sim.fields()
    sim.close()
    b = ko_oracle.port_run(phi, T, th, p, 25, libm=False, threads=8)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


def test_timeout_latch():
    p = dict(configs.BASE)
    sim = Kobayashi(64, 48, p["dt"], params=p)
    sim.step(10)
    _lib.check(_lib.lib().kg_diag_inject_timeout(sim._h))
    with pytest.raises(KgError) as e:
        sim.sync()
    assert e.value.code == _lib.KG_ERR_TIMEOUT
    with pytest.raises(KgError) as e:
        sim.step(5)
    assert e.value.code == _lib.KG_ERR_TIMEOUT
    with pytest.raises(KgError):
        sim.fields()
    # replacing one field is not enough; the whole state is
    z = np.zeros((48, 64))
    sim.set_fields(phi=z)
    with pytest.raises(KgError):
        sim.step(1)
    sim.iResetSimulationState()
    sim.step(20)
    got = sim.fields()
    init = configs.initial_fields(64, 48, [(32, 24, 1)])
    ref = ko_oracle.port_run(*init, p, 20, libm=False)
    for x, y in zip(got, ref):
        assert bits_equal(x, y)
    # set_fields with all three fields clears it as well
    _lib.check(_lib.lib().kg_diag_inject_timeout(sim._h))
    with pytest.raises(KgError):
        sim.sync()
    sim.set_fields(*init)
    sim.step(3)
    sim.sync()
    sim.close()


def test_fp64_probe():
    lanes, per_clk = ctypes.c_double(), ctypes.c_double()
    for op in range(4):
        _lib.check(_lib.lib().kg_diag_fp64_probe(op, 8, 4, 256, ctypes.byref(lanes), ctypes.byref(per_clk)))
        assert 1e10 < lanes.value < 1e13
        assert 0.1 < per_clk.value < 64
    with pytest.raises(KgError):
        _lib.check(_lib.lib().kg_diag_fp64_probe(9, 8, 4, 256, ctypes.byref(lanes), None))

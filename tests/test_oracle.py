"""The CPU oracle, pinned against the reference's own code (CPU only).

oracle/ko_oracle.c restates src/Kobayashi.cpp:125-221 in C.  With the C
library's atan/sin/cos it must reproduce the reference -- compiled unmodified
in FP64 -- bit for bit; with kg_math's functions (what the GPU uses) it may
differ only by the measured noise floor.
"""
import json
import os
import platform

import numpy as np
import pytest

import ko_oracle
from crystalgrowth_gb300 import configs

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DEFAULT = dict(dx=0.03, dy=0.03, dt=1e-4, tau=3e-4, eps_bar=0.01, mu=1.0, K=1.6, delta=0.05, aniso=6.0, alpha=0.9,
               gamma=10.0, teq=1.0, theta0=0.0)


def bits_equal(a, b):
    return np.array_equal(np.asarray(a, dtype=np.float64).view(np.uint64), np.asarray(b, dtype=np.float64).view(np.uint64))


def nucleus(nx, ny):
    """the reference's _createNucleus(nx/2, ny/2) (src/Kobayashi.cpp:113-123)"""
    return configs.initial_fields(nx, ny, [(nx // 2, ny // 2, 1)])


def have_reference():
    try:
        ko_oracle.Reference(3, 3, 1e-4)
        return True
    except FileNotFoundError:
        return False


needs_ref = pytest.mark.skipif(not have_reference(), reason="reference sources not staged")


@needs_ref
@pytest.mark.parametrize("nx,ny,steps", [(3, 3, 25), (17, 13, 25), (64, 48, 200), (5, 40, 60)])
def test_port_libm_is_the_reference_bit_for_bit(nx, ny, steps):
    r = ko_oracle.Reference(nx, ny, 1e-4)
    r.set_params(DEFAULT)
    r.vector_init()
    r.step(steps)
    ref = r.get_state()
    out = ko_oracle.port_run(*nucleus(nx, ny), DEFAULT, steps, libm=True)
    for a, b in zip(ref, out):
        assert bits_equal(a, b)


@needs_ref
def test_reference_nucleus_matches_seed_disk():
    for nx, ny in ((3, 3), (17, 13), (64, 48)):
        r = ko_oracle.Reference(nx, ny, 1e-4)
        phi, t, th = r.get_state()
        p0, t0, h0 = nucleus(nx, ny)
        assert bits_equal(phi, p0) and not t.any() and not th.any()


@needs_ref
def test_iupdate_is_ten_steps():
    a = ko_oracle.Reference(40, 30, 1e-4)
    b = ko_oracle.Reference(40, 30, 1e-4)
    for r in (a, b):
        r.set_params(DEFAULT)
    a.update()
    b.step(10)
    assert a.frame() == 1
    for x, y in zip(a.get_state(), b.get_state()):
        assert bits_equal(x, y)


def _same_libm_as_fixtures():
    """the FP64 fixtures hold this container's C-library results; another libm differs in the last bits"""
    if not have_reference():
        return False
    fx = np.load(os.path.join(GOLD, "ref64_default_64x48.npz"))
    r = ko_oracle.Reference(64, 48, 1e-4)
    r.set_params(DEFAULT)
    for _ in range(20):
        r.update()
    return bits_equal(r.get_state()[0], fx["phi"])


def test_port_libm_reproduces_reference_fixture():
    fx = np.load(os.path.join(GOLD, "ref64_default_64x48.npz"))
    out = ko_oracle.port_run(*nucleus(64, 48), DEFAULT, 200, libm=True)
    if not bits_equal(out[0], fx["phi"]):
        if platform.machine() != "x86_64" or not _same_libm_as_fixtures():
            pytest.skip("fixture made with a different C library")
    assert bits_equal(out[0], fx["phi"]) and bits_equal(out[1], fx["T"]) and bits_equal(out[2], fx["theta"])


def test_port_libm_reproduces_grid300_hash():
    g = json.load(open(os.path.join(GOLD, "ref64_grid300.json")))
    init = configs.initial_fields(300, 300, g["disks"])
    phi, t, th = ko_oracle.port_run(*init, g["params"], g["steps"], libm=True, threads=8)
    import hashlib
    h = hashlib.sha256(phi.tobytes()).hexdigest()
    if h != g["sha_phi"] and platform.machine() != "x86_64":
        pytest.skip("fixture made with a different C library")
    assert h == g["sha_phi"]
    assert hashlib.sha256(t.tobytes()).hexdigest() == g["sha_T"]
    assert hashlib.sha256(th.tobytes()).hexdigest() == g["sha_theta"]


@pytest.mark.parametrize("tag", ["theta0_0", "theta0_02"])
def test_port_kgmath_grid300_hash_is_platform_independent(tag):
    """kg_math results are a fixed sequence of IEEE operations: the hash holds on any machine."""
    import hashlib
    g = json.load(open(os.path.join(GOLD, "kgm_grid300.json")))
    init = configs.initial_fields(300, 300, g["disks"])
    phi, t, th = ko_oracle.port_run(*init, g[tag]["params"], g["steps"], libm=False, threads=8)
    assert hashlib.sha256(phi.tobytes()).hexdigest() == g[tag]["sha_phi"]
    assert hashlib.sha256(t.tobytes()).hexdigest() == g[tag]["sha_T"]
    assert hashlib.sha256(th.tobytes()).hexdigest() == g[tag]["sha_theta"]


def test_noise_floor_kgmath_vs_libm():
    """kg_math vs the C library after 2000 steps on 300^2: the recorded floor (about 1e-12 on phi)."""
    g = json.load(open(os.path.join(GOLD, "kgm_grid300.json")))
    assert g["theta0_0"]["noise_floor_phi"] < 5e-12
    assert g["theta0_0"]["noise_floor_T"] < 5e-12
    init = configs.initial_fields(64, 64, [(32, 32, 5)])
    p = dict(configs.BASE)
    a = ko_oracle.port_run(*init, p, 300, libm=False)
    b = ko_oracle.port_run(*init, p, 300, libm=True)
    assert np.abs(a[0] - b[0]).max() / np.abs(b[0]).max() < 1e-13


def test_theta0_zero_is_bit_neutral():
    """aniso*(theta - 0) == aniso*theta for every double theta."""
    th = np.random.default_rng(3).standard_normal(100000) * 5
    assert bits_equal(6.0 * (th - 0.0), 6.0 * th)


def test_fp32_build_tracks_fp64():
    """the reference as shipped (FP32) stays near the FP64 restatement: the promotion changes rounding, not the model"""
    fx32 = np.load(os.path.join(GOLD, "ref32_default_64x48.npz"))
    fx64 = np.load(os.path.join(GOLD, "ref64_default_64x48.npz"))
    assert np.abs(fx32["phi"].astype(np.float64) - fx64["phi"]).max() < 1e-2
    assert np.abs(fx32["T"].astype(np.float64) - fx64["T"]).max() < 1e-2


def test_edge_fixture_small_grids():
    fx = np.load(os.path.join(GOLD, "ref64_edge.npz"))
    for nx, ny in ((3, 3), (17, 13)):
        out = ko_oracle.port_run(*nucleus(nx, ny), DEFAULT, 25, libm=True)
        ref = fx["phi_%dx%d" % (nx, ny)]
        if platform.machine() == "x86_64":
            assert bits_equal(out[0], ref)
        assert np.abs(out[0] - ref).max() < 1e-13

"""GPU parity of the fused step (libkobayashi_gpu.so through the C ABI) against
the CPU oracle, which follows src/Kobayashi.cpp:125-221 operation by
operation.  Integer/byte-exact bar: the FP64 fields must be identical bit for
bit (tolerance 0); the reference defaults fixture, computed with the C
library's atan/sin/cos, must agree within the measured noise floor.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import ko_oracle
from crystalgrowth_gb300 import Kobayashi, KgError, configs

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
THREADS = max(1, min(16, os.cpu_count() or 1))


def bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float64).view(np.uint64), np.asarray(b, np.float64).view(np.uint64))


def gpu_run(nx, ny, params, disks, steps, chunk=None):
    sim = Kobayashi(nx, ny, params["dt"], params=params)
    sim.seed_disks(disks)
    if chunk is not None:
        sim.set_graph_chunk(chunk)
    sim.step(steps)
    out = sim.fields()
    sim.close()
    return out


def oracle_run(nx, ny, params, disks, steps):
    return ko_oracle.port_run(*configs.initial_fields(nx, ny, disks), params, steps, libm=False, threads=THREADS)


@pytest.mark.parametrize("nx,ny,steps", [(1, 1, 5), (2, 3, 10), (3, 3, 25), (17, 13, 300), (64, 48, 200),
                                         (126, 64, 60), (127, 65, 60), (130, 70, 200), (253, 129, 100),
                                         (1000, 777, 40)])
def test_step_bitwise_small_and_ragged(nx, ny, steps):
    p = dict(configs.BASE)
    disks = [(nx // 2, ny // 2, max(1, min(nx, ny) // 6))]
    a = gpu_run(nx, ny, p, disks, steps)
    b = oracle_run(nx, ny, p, disks, steps)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


def test_grid300_2000_steps_matches_golden_hash():
    """configuration 0 in full: 300^2, 2000 steps, against hashes made on another machine by the oracle"""
    g = json.load(open(os.path.join(GOLD, "kgm_grid300.json")))
    for tag in ("theta0_0", "theta0_02"):
        phi, t, th = gpu_run(300, 300, g[tag]["params"], g["disks"], g["steps"])
        assert hashlib.sha256(phi.tobytes()).hexdigest() == g[tag]["sha_phi"]
        assert hashlib.sha256(t.tobytes()).hexdigest() == g[tag]["sha_T"]
        assert hashlib.sha256(th.tobytes()).hexdigest() == g[tag]["sha_theta"]


def test_reference_defaults_within_noise_floor():
    """the reference's own FP64 output (C-library atan/sin/cos) vs the GPU: 1e-12 relative max-norm"""
    fx = np.load(os.path.join(GOLD, "ref64_default_64x48.npz"))
    p = json.loads(str(fx["params"]))
    sim = Kobayashi(64, 48, p["dt"], params=p)  # kg_create seeds the reference nucleus
    for _ in range(20):
        sim.iUpdate()
    phi, t, th = sim.fields()
    assert sim.counters() == (200, 20)
    sim.close()
    assert np.abs(phi - fx["phi"]).max() / np.abs(fx["phi"]).max() <= 1e-12
    assert np.abs(t - fx["T"]).max() / np.abs(fx["T"]).max() <= 1e-12


@pytest.mark.parametrize("variant", [0, 13, 26, 40, 53])
def test_variants_2048_truncated(variant):
    """configuration 2 (anisotropy variants on 2048^2), truncated to 60 steps"""
    v = configs.variants_2048()[variant]
    a = gpu_run(v["nx"], v["ny"], v["params"], v["disks"], 60)
    b = oracle_run(v["nx"], v["ny"], v["params"], v["disks"], 60)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


def test_grid8192_truncated():
    """configuration 1 (8192^2, 64 disks), truncated to 12 steps (graph chunk 5 + remainder)"""
    cfg = configs.grid_8192()
    a = gpu_run(cfg["nx"], cfg["ny"], cfg["params"], cfg["disks"], 12, chunk=5)
    b = oracle_run(cfg["nx"], cfg["ny"], cfg["params"], cfg["disks"], 12)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


def test_graph_chunks_do_not_change_results():
    p = dict(configs.BASE)
    disks = [(40, 30, 4)]
    runs = [gpu_run(80, 60, p, disks, 230, chunk=c) for c in (0, 1, 7, 100)]
    for r in runs[1:]:
        for x, y in zip(runs[0], r):
            assert bits_equal(x, y)


@pytest.mark.parametrize("nx", [141, 260])
@pytest.mark.parametrize("nt,bh", [(32, 1), (32, 17), (64, 1), (64, 8), (64, 40), (128, 3), (128, 16), (128, 200),
                                   (256, 1), (256, 24), (256, 200)])
def test_strip_shape_does_not_change_results(nx, nt, bh):
    """odd width: every strip loads its columns lane by lane; even width (260): interior strips
    stage their rows with bulk copies, across strip heights that wrap each 8-row ring several times"""
    p = dict(configs.BASE)
    disks = [(70, 50, 6), (10, 90, 4), (nx - 20, 30, 5)]
    sim = Kobayashi(nx, 103, p["dt"], params=p)
    sim.seed_disks(disks)
    sim.set_tile(nt, bh)
    assert sim.tile() == (nt, min(bh, 103))
    sim.step(90)
    a = sim.fields()
    sim.close()
    b = oracle_run(nx, 103, p, disks, 90)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


@pytest.mark.parametrize("nt,nx", [(256, 2), (256, 3), (256, 254), (256, 255), (256, 256), (256, 510), (256, 512),
                                   (256, 766), (128, 126), (128, 252), (128, 254), (128, 380)])
def test_strip_edges_against_grid_width(nt, nx):
    """widths around the bulk-copy condition (an even width and a strip lying inside the grid: i0 >= 2,
    i0 + NT <= nx) and single strips that wrap a grid narrower than themselves"""
    p = dict(configs.BASE)
    disks = [(nx // 2, 18, 5), (nx // 5, 30, 3)]
    sim = Kobayashi(nx, 37, p["dt"], params=p)
    sim.seed_disks(disks)
    sim.set_tile(nt, 7)
    sim.step(40)
    a = sim.fields()
    sim.close()
    b = oracle_run(nx, 37, p, disks, 40)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


def test_default_strip_shapes():
    """the library's strip choice: the first of 256 x 24, 128 x 32, 128 x 16 that gives at least 8000
    CTAs (8192^2: 256 x 24; 4096^2: 128 x 16), one-warp strips of 4 rows for the 2048^2 and 512^2 cases"""
    for n, want in ((8192, (256, 24)), (4096, (128, 16)), (2048, (32, 4)), (512, (32, 4))):
        sim = Kobayashi(n, n, 1e-4)
        assert sim.tile() == want, (n, sim.tile())
        sim.close()


def test_translation_invariance_full_size():
    """periodic grid: shifting the nuclei shifts the solution exactly (every cell runs the same arithmetic)"""
    cfg = configs.grid_8192()
    n = cfg["nx"]
    di, dj = 1234, 567
    shifted = [((x + di) % n, (y + dj) % n, r) for x, y, r in cfg["disks"]]
    a = gpu_run(n, n, cfg["params"], cfg["disks"], 30)
    b = gpu_run(n, n, cfg["params"], shifted, 30)
    for x, y in zip(a, b):
        assert bits_equal(np.roll(x, (dj, di), axis=(0, 1)), y)


def test_determinism():
    p = dict(configs.BASE)
    a = gpu_run(512, 512, p, [(256, 256, 5)], 300)
    b = gpu_run(512, 512, p, [(256, 256, 5)], 300)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


def test_set_params_mid_run_and_reset():
    p = dict(configs.BASE)
    q = dict(p, delta=0.05, K=1.2, theta0=0.7)
    sim = Kobayashi(96, 80, p["dt"], params=p)
    sim.seed_disks([(48, 40, 6)])
    sim.step(150)
    sim.set_params(**{k: q[k] for k in ("delta", "K", "theta0")})
    sim.step(150)
    got = sim.fields()
    init = configs.initial_fields(96, 80, [(48, 40, 6)])
    mid = ko_oracle.port_run(*init, p, 150)
    ref = ko_oracle.port_run(*mid, q, 150)
    for x, y in zip(got, ref):
        assert bits_equal(x, y)
    sim.iResetSimulationState()
    phi, t, th = sim.fields()
    p0, _, _ = configs.initial_fields(96, 80, [(48, 40, 1)])
    assert bits_equal(phi, p0) and not t.any() and not th.any()
    assert sim.counters() == (0, 0)
    sim.close()


def test_set_fields_roundtrip_and_continue():
    p = dict(configs.BASE)
    rng = np.random.default_rng(5)
    phi = rng.uniform(0, 1, (50, 70))
    t = rng.normal(0, 0.1, (50, 70))
    th = rng.uniform(-1.5, 6.2, (50, 70))
    sim = Kobayashi(70, 50, p["dt"], params=p)
    sim.set_fields(phi, t, th)
    got = sim.fields()
    for x, y in zip(got, (phi, t, th)):
        assert bits_equal(x, y)
    sim.step(40)
    a = sim.fields()
    b = ko_oracle.port_run(phi, t, th, p, 40)
    for x, y in zip(a, b):
        assert bits_equal(x, y)
    sim.close()


def test_invalid_arguments_fail_cleanly():
    with pytest.raises(KgError):
        Kobayashi(0, 10, 1e-4)
    with pytest.raises(KgError):
        Kobayashi(10, 10, 1e-4, params=dict(tau=0.0))
    with pytest.raises(KgError):
        Kobayashi(10, 10, 1e-4, params=dict(aniso=2.5))
    sim = Kobayashi(10, 10, 1e-4)
    with pytest.raises(KgError):
        sim.step(-1)
    with pytest.raises(KgError):
        sim.set_params(dx=float("nan"))
    sim.step(3)  # still usable
    sim.close()


def test_variant_2048_full_length():
    """one anisotropy variant of the 2048^2 set (j=4, delta=0.05, K=2.0, theta0=pi/4) over its full
    5000 steps, against the CPU oracle, bit for bit"""
    v = [x for x in configs.variants_2048() if x["params"]["aniso"] == 4.0 and x["params"]["delta"] == 0.05
         and x["params"]["K"] == 2.0 and x["params"]["theta0"] > 0.7][0]
    a = gpu_run(v["nx"], v["ny"], v["params"], v["disks"], v["steps"])
    b = oracle_run(v["nx"], v["ny"], v["params"], v["disks"], v["steps"])
    for x, y in zip(a, b):
        assert bits_equal(x, y)


def test_translation_invariance_grid8192_1000_steps():
    """the 8192^2 workload over 1000 steps, nuclei shifted by (3001, 77): the solution shifts exactly"""
    cfg = configs.grid_8192()
    n = cfg["nx"]
    di, dj = 3001, 77
    shifted = [((x + di) % n, (y + dj) % n, r) for x, y, r in cfg["disks"]]
    a = gpu_run(n, n, cfg["params"], cfg["disks"], 1000)
    b = gpu_run(n, n, cfg["params"], shifted, 1000)
    assert np.abs(a[0]).max() > 0.5  # crystals have grown
    for x, y in zip(a, b):
        assert bits_equal(np.roll(x, (dj, di), axis=(0, 1)), y)


def test_device_out_of_memory_is_an_error_not_a_crash():
    """a grid larger than the GPU's memory: cudaMalloc fails, the call returns KG_ERR_NOMEM and the
    library (and the CUDA context) stay usable"""
    from crystalgrowth_gb300 import _lib
    with pytest.raises(KgError) as e:
        Kobayashi(131072, 131072, 1e-4)  # 2^34 cells: 824 GB of state
    assert e.value.code == _lib.KG_ERR_NOMEM
    sim = Kobayashi(32, 32, 1e-4)
    sim.step(5)
    sim.close()


def test_bulk_copy_wait_runs_out_and_context_survives():
    """the strip kernel's mbarrier wait is bounded: on a barrier nothing completes it gives up,
    raises the flag, and the context stays usable"""
    import ctypes
    from crystalgrowth_gb300 import _lib
    flag = ctypes.c_int(-1)
    _lib.check(_lib.lib().kg_diag_mbar_timeout(ctypes.byref(flag)))
    assert flag.value == 1
    sim = Kobayashi(64, 64, 1e-4)
    sim.step(3)
    sim.sync()
    sim.close()

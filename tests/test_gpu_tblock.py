"""Temporal blocking (two time steps per pass over HBM, kg_strip2) on the GPU
against the CPU oracle, bit for bit: the single-grid handle (kg_set_tblock)
on small, ragged and odd-sized grids, every strip width and several strip
heights, odd step counts (the last step then takes a one-step launch) and
odd CUDA-graph chunks; and the batched ensemble in both execution modes.
The k = 2 pass recomputes a 4-column, 3-row halo and keeps the intermediate
step in shared memory, so any slip in its ring indexing shows up here as a
bit difference."""
import numpy as np
import pytest

import ko_oracle
from crystalgrowth_gb300 import Batch, Kobayashi, configs
from crystalgrowth_gb300.batch import KG_BATCH_LAUNCH, KG_BATCH_PERSISTENT

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float64).view(np.uint64), np.asarray(b, np.float64).view(np.uint64))


def run_k2(nx, ny, params, disks, steps, tile=None, chunk=None):
    sim = Kobayashi(nx, ny, params["dt"], params=params)
    sim.seed_disks(disks)
    sim.set_tblock(2)
    assert sim.tblock() == 2
    if tile:
        sim.set_tile(*tile)
    if chunk is not None:
        sim.set_graph_chunk(chunk)
    sim.step(steps)
    out = sim.fields()
    assert sim.counters()[0] == steps
    sim.close()
    return out


def oracle(nx, ny, params, disks, steps):
    return ko_oracle.port_run(*configs.initial_fields(nx, ny, disks), params, steps, libm=False, threads=8)


@pytest.mark.parametrize("nx,ny,steps", [(1, 1, 5), (2, 3, 10), (3, 3, 25), (5, 40, 31), (17, 13, 300),
                                         (64, 48, 200), (122, 64, 61), (123, 65, 60), (253, 129, 101),
                                         (1000, 777, 40)])
def test_k2_bitwise_small_and_ragged(nx, ny, steps):
    p = dict(configs.BASE)
    disks = [(nx // 2, ny // 2, max(1, min(nx, ny) // 6))]
    a = run_k2(nx, ny, p, disks, steps)
    b = oracle(nx, ny, p, disks, steps)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


@pytest.mark.parametrize("nt,bh", [(32, 1), (32, 5), (64, 2), (64, 33), (128, 4), (128, 16), (128, 200), (256, 24)])
def test_k2_strip_shapes(nt, bh):
    """(256-thread strips: the two-step pass runs on 128-thread strips of the same height)"""
    p = dict(configs.BASE, delta=0.05, theta0=0.7)
    disks = [(70, 50, 6), (10, 90, 4), (120, 30, 5)]
    a = run_k2(141, 103, p, disks, 90, tile=(nt, bh))
    b = oracle(141, 103, p, disks, 90)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


@pytest.mark.parametrize("chunk", [0, 1, 7, 100])
def test_k2_graph_chunks(chunk):
    p = dict(configs.BASE)
    disks = [(40, 30, 4)]
    a = run_k2(80, 60, p, disks, 233, chunk=chunk)
    b = oracle(80, 60, p, disks, 233)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


def test_k1_k2_switch_mid_run():
    p = dict(configs.BASE)
    disks = [(100, 70, 7)]
    sim = Kobayashi(200, 150, p["dt"], params=p)
    sim.seed_disks(disks)
    sim.step(33)
    sim.set_tblock(2)
    sim.step(101)
    sim.set_tblock(1)
    sim.step(7)
    a = sim.fields()
    sim.close()
    b = oracle(200, 150, p, disks, 141)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


def test_k2_variant_2048_truncated():
    v = configs.variants_2048()[40]
    a = run_k2(v["nx"], v["ny"], v["params"], v["disks"], 80)
    b = oracle(v["nx"], v["ny"], v["params"], v["disks"], 80)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


def test_k2_invalid_factor():
    from crystalgrowth_gb300 import KgError
    sim = Kobayashi(16, 16, 1e-4)
    for k in (0, 3, -1):
        with pytest.raises(KgError):
            sim.set_tblock(k)
    assert sim.tblock() == 1
    sim.close()


def small_ensemble(count=20, seed=9, lo=5, hi=260):
    rng = configs.SplitMix64(seed)
    inst = []
    for _ in range(count):
        nx, ny = rng.randint(lo, hi), rng.randint(lo, hi)
        p = dict(configs.BASE, delta=rng.uniform(0.01, 0.06), aniso=float(4 if rng.next() & 1 else 6),
                 K=rng.uniform(1.2, 2.0), theta0=rng.uniform(0.0, 1.5), tau=rng.uniform(2e-4, 4e-4))
        inst.append(dict(nx=nx, ny=ny, params=p, disks=[(nx // 2, ny // 2, rng.randint(1, max(1, min(nx, ny) // 4)))]))
    return inst


@pytest.mark.parametrize("mode", [KG_BATCH_LAUNCH, KG_BATCH_PERSISTENT])
@pytest.mark.parametrize("nt,bh,chunk,streams", [(32, 8, 5, 1), (64, 16, 7, 4), (128, 32, 100, 1), (128, 4, 3, 8)])
def test_batch_k2_bitwise(mode, nt, bh, chunk, streams):
    inst = small_ensemble()
    steps = 43
    b = Batch([(i["nx"], i["ny"]) for i in inst], [i["params"] for i in inst])
    for k, i in enumerate(inst):
        b.seed_disks(k, i["disks"])
    b.set_tuning(nt=nt, bh=bh, mode=mode, chunk=chunk, streams=streams if mode == KG_BATCH_LAUNCH else 1, tblock=2)
    assert b.tuning()["tblock"] == 2
    b.step(steps)
    assert b.info()["steps"] == steps
    for k, i in enumerate(inst):
        ref = oracle(i["nx"], i["ny"], i["params"], i["disks"], steps)
        for x, y in zip(b.fields(k), ref):
            assert bits_equal(x, y), (k, i["nx"], i["ny"])
    b.close()


def test_batch_k2_rejects_wide_strips():
    from crystalgrowth_gb300 import KgError
    b = Batch([(40, 40)], [dict(configs.BASE)])
    with pytest.raises(KgError):
        b.set_tuning(nt=256, bh=16, tblock=2)
    b.close()

"""Batched ensemble (kg_batch_*): every instance bit-identical to the CPU
oracle run of the same grid and parameters, in both execution modes and for
every strip shape the autotuner may choose; the autotuner leaves the state as
it found it; the bounded grid barrier gives up instead of hanging."""
import ctypes

import numpy as np
import pytest

import ko_oracle
from crystalgrowth_gb300 import Batch, Kobayashi, configs, _lib
from crystalgrowth_gb300.batch import KG_BATCH_LAUNCH, KG_BATCH_PERSISTENT

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    return np.array_equal(np.asarray(a, np.float64).view(np.uint64), np.asarray(b, np.float64).view(np.uint64))


def small_ensemble(count=24, seed=7, lo=5, hi=300):
    rng = configs.SplitMix64(seed)
    inst = []
    for _ in range(count):
        nx = rng.randint(lo, hi)
        ny = rng.randint(lo, hi)
        p = dict(configs.BASE, delta=rng.uniform(0.01, 0.06), aniso=float(4 if rng.next() & 1 else 6),
                 K=rng.uniform(1.2, 2.0), theta0=rng.uniform(0.0, 1.5), tau=rng.uniform(2e-4, 4e-4))
        r = rng.randint(1, max(1, min(nx, ny) // 4))
        inst.append(dict(nx=nx, ny=ny, params=p, disks=[(nx // 2, ny // 2, r)]))
    return inst


def make_batch(inst):
    b = Batch([(i["nx"], i["ny"]) for i in inst], [i["params"] for i in inst])
    for k, i in enumerate(inst):
        b.seed_disks(k, i["disks"])
    return b


def oracle(inst, steps):
    return [ko_oracle.port_run(*configs.initial_fields(i["nx"], i["ny"], i["disks"]), i["params"], steps,
                               threads=8) for i in inst]


@pytest.mark.parametrize("mode", [KG_BATCH_LAUNCH, KG_BATCH_PERSISTENT])
@pytest.mark.parametrize("nt,bh,chunk", [(32, 8, 5), (64, 16, 7), (128, 64, 100), (256, 32, 3)])
def test_batch_bitwise_vs_oracle(mode, nt, bh, chunk):
    inst = small_ensemble()
    steps = 41
    b = make_batch(inst)
    b.set_tuning(nt=nt, bh=bh, mode=mode, chunk=chunk)
    b.step(steps)
    ref = oracle(inst, steps)
    for k in range(len(inst)):
        for x, y in zip(b.fields(k), ref[k]):
            assert bits_equal(x, y), (k, inst[k]["nx"], inst[k]["ny"])
    assert b.info()["steps"] == steps
    b.close()


def test_batch_equals_single_grid_runs():
    inst = small_ensemble(count=6, seed=11, lo=30, hi=200)
    b = make_batch(inst)
    b.step(60)
    for k, i in enumerate(inst):
        s = Kobayashi(i["nx"], i["ny"], i["params"]["dt"], params=i["params"])
        s.seed_disks(i["disks"])
        s.step(60)
        for x, y in zip(b.fields(k), s.fields()):
            assert bits_equal(x, y)
        s.close()
    b.close()


def test_autotune_restores_state_and_keeps_results():
    inst = small_ensemble(count=10, seed=3)
    b = make_batch(inst)
    b.step(5)
    before = [b.fields(k) for k in range(len(inst))]
    best, ms = b.autotune(trial_steps=3)
    assert best["nt"] in (32, 64, 128, 256) and ms > 0
    after = [b.fields(k) for k in range(len(inst))]
    for x, y in zip(before, after):
        for u, v in zip(x, y):
            assert bits_equal(u, v)
    assert b.info()["steps"] == 5
    b.step(20)
    ref = oracle(inst, 25)
    for k in range(len(inst)):
        for x, y in zip(b.fields(k), ref[k]):
            assert bits_equal(x, y)
    b.close()


def test_ensemble_512_config_truncated():
    """the 512-instance mixed-size ensemble: a sample of instances checked after 10 steps"""
    cfg = configs.ensemble_512()
    inst = cfg["instances"]
    b = make_batch(inst)
    b.step(10)
    for k in (0, 1, 100, 255, 511):
        ref = ko_oracle.port_run(*configs.initial_fields(inst[k]["nx"], inst[k]["ny"], inst[k]["disks"]),
                                 inst[k]["params"], 10, threads=8)
        for x, y in zip(b.fields(k), ref):
            assert bits_equal(x, y)
    b.close()


def test_barrier_wait_runs_out_and_context_survives():
    flag = ctypes.c_int(-1)
    _lib.check(_lib.lib().kg_diag_barrier_timeout(2, 20000, ctypes.byref(flag)))
    assert flag.value == 1
    s = Kobayashi(32, 32, 1e-4)  # the context is still usable
    s.step(3)
    s.sync()
    s.close()


def test_batch_rejects_bad_input():
    with pytest.raises(_lib.KgError):
        Batch([(0, 5)], [dict()])
    b = Batch([(8, 8)], [dict()])
    with pytest.raises(_lib.KgError):
        b.set_tuning(nt=100)
    with pytest.raises(_lib.KgError):
        b.set_tuning(streams=17)
    assert _lib.lib().kg_batch_get_fields(b._h, 3, None, None, None) == _lib.KG_ERR_INVALID
    assert b"out of range" in _lib.lib().kg_last_error()
    b.close()


def test_ensemble_512_full_length_sample():
    """the 512-instance ensemble over its full 3000 steps; six instances (smallest, largest and
    four others) checked against the CPU oracle bit for bit"""
    cfg = configs.ensemble_512()
    inst = cfg["instances"]
    b = make_batch(inst)
    best, _ = b.autotune(trial_steps=3)
    b.step(cfg["steps"])
    sides = [i["nx"] for i in inst]
    picks = sorted({sides.index(min(sides)), sides.index(max(sides)), 7, 128, 300, 509})
    for k in picks:
        ref = ko_oracle.port_run(*configs.initial_fields(inst[k]["nx"], inst[k]["ny"], inst[k]["disks"]),
                                 inst[k]["params"], cfg["steps"], threads=16)
        for x, y in zip(b.fields(k), ref):
            assert bits_equal(x, y), k
    b.close()


@pytest.mark.parametrize("streams,chunk", [(2, 7), (3, 100), (5, 4), (16, 1)])
def test_batch_group_streams_bitwise(streams, chunk):
    """instances split over several streams (each group steps on its own): same bits as the oracle"""
    inst = small_ensemble(count=17, seed=9)
    steps = 23
    b = make_batch(inst)
    b.set_tuning(nt=64, bh=8, mode=KG_BATCH_LAUNCH, chunk=chunk, streams=streams)
    b.step(steps)
    ref = oracle(inst, steps)
    for k in range(len(inst)):
        for x, y in zip(b.fields(k), ref[k]):
            assert bits_equal(x, y), k
    b.close()


def test_batch_timeout_latch():
    """after a grid-barrier wait ran out (injected on the host), kg_batch_step refuses until every
    instance's state has been replaced; then the batch steps on, bit-identical to the oracle"""
    inst = small_ensemble(count=3, seed=5, lo=20, hi=60)
    b = make_batch(inst)
    b.step(4)
    rc = _lib.lib().kg_diag_batch_inject_timeout(b._h)
    assert rc == _lib.KG_ERR_TIMEOUT
    with pytest.raises(_lib.KgError) as e:
        b.step(1)
    assert e.value.code == _lib.KG_ERR_TIMEOUT
    b.seed_disks(0, inst[0]["disks"])
    b.seed_disks(1, inst[1]["disks"])
    with pytest.raises(_lib.KgError):
        b.step(1)  # instance 2 still holds the unreliable state
    init = configs.initial_fields(inst[2]["nx"], inst[2]["ny"], inst[2]["disks"])
    b.set_fields(2, *init)
    b.step(9)
    ref = oracle(inst, 9)
    for k in range(len(inst)):
        for x, y in zip(b.fields(k), ref[k]):
            assert bits_equal(x, y)
    b.close()

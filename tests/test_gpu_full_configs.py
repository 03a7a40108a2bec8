"""The large workloads at their full length, bit for bit against the oracle.

tests/golden/full_configs.json holds SHA-256 hashes of the final fields that
the CPU oracle (oracle/ko_oracle.c with kg_math, the arithmetic the GPU
reproduces) computed for
  - the 8192^2 grid with 64 seeded disks at time steps 1000, 2000, 5000 and
    10,000 (the benchmark's trajectory);
  - all 54 anisotropy variants of the 2048^2 set at 5000 steps;
  - all 512 instances of the mixed-size ensemble at 3000 steps.
They were made by tests/golden/make_golden.py --full-configs (hours of CPU
time).  Each GPU run here takes seconds to a minute.  A part missing from the
fixture is skipped, not failed.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from crystalgrowth_gb300 import Batch, Kobayashi, configs
from crystalgrowth_gb300.batch import KG_BATCH_LAUNCH, KG_BATCH_PERSISTENT

pytestmark = pytest.mark.gpu
FULL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "full_configs.json")


def load():
    if not os.path.exists(FULL):
        pytest.skip("no full-length fixture")
    return json.load(open(FULL))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def check_fields(fields, want, what):
    got = dict(zip(("sha_phi", "sha_T", "sha_theta"), (sha(a) for a in fields)))
    bad = [k for k in got if got[k] != want[k]]
    assert not bad, "%s: %s differ from the oracle" % (what, ", ".join(bad))


def test_grid8192_full_trajectory():
    g = load().get("grid_8192", {}).get("at_step", {})
    marks = sorted(int(s) for s in g)
    if not marks:
        pytest.skip("8192^2 hashes not in the fixture")
    cfg = configs.grid_8192()
    sim = Kobayashi(cfg["nx"], cfg["ny"], cfg["params"]["dt"], params=cfg["params"])
    sim.seed_disks(cfg["disks"])
    at = 0
    for m in marks:
        sim.step(m - at)
        at = m
        check_fields(sim.fields(), g[str(m)], "grid_8192 at step %d" % m)
    sim.close()


VARIANT_CFG = {v["name"]: v for v in configs.variants_2048()}


@pytest.mark.parametrize("name", sorted(VARIANT_CFG))
def test_variant_2048_full_length(name):
    vd = load().get("variants_2048", {}).get("variants", {})
    if name not in vd:
        pytest.skip("variant not in the fixture yet")
    v = VARIANT_CFG[name]
    sim = Kobayashi(v["nx"], v["ny"], v["params"]["dt"], params=v["params"])
    sim.seed_disks(v["disks"])
    sim.step(v["steps"])
    check_fields(sim.fields(), vd[name], name)
    sim.close()


@pytest.mark.parametrize("tuning", [dict(nt=64, bh=32, mode=KG_BATCH_LAUNCH, chunk=100, streams=4, tblock=1),
                                    dict(nt=32, bh=8, mode=KG_BATCH_PERSISTENT, chunk=250, streams=1, tblock=2)])
def test_ensemble_512_full_length(tuning):
    ens = load().get("ensemble_512", {})
    hashes = ens.get("instances", {})
    cfg = configs.ensemble_512()
    if len(hashes) != len(cfg["instances"]):
        pytest.skip("ensemble hashes incomplete")
    inst = cfg["instances"]
    b = Batch([(i["nx"], i["ny"]) for i in inst], [i["params"] for i in inst])
    for k, i in enumerate(inst):
        b.seed_disks(k, i["disks"])
    b.set_tuning(**tuning)
    b.step(ens["steps"])
    bad = []
    for k in range(len(inst)):
        h = hashlib.sha256(b"".join(np.ascontiguousarray(a).tobytes() for a in b.fields(k))).hexdigest()
        if h != hashes[str(k)]:
            bad.append(k)
    b.close()
    assert not bad, "instances differing from the oracle: %s" % bad[:20]

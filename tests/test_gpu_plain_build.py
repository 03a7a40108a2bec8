"""The plain build -- every compile-time switch of the kernels in its other
setting (no bit-pattern move, hardware division for gy/gx, no far-field, FMA,
T-bound or quiet-cell shortcuts, hardware division for subnormal dividends,
fallbacks inlined, per-lane row loads) -- computes the same bits as the
oracle.  It is built into a temporary folder and run in a child process, so
the library the other tests load is not touched."""
import json
import os
import subprocess
import sys
import tempfile

import pytest

from crystalgrowth_gb300 import build as kbuild

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, %(root)r); sys.path.insert(0, %(oracle)r)
from crystalgrowth_gb300 import _lib
_lib.load(%(lib)r)
import ko_oracle
from crystalgrowth_gb300 import Kobayashi, configs
out = []
for nx, ny, steps, th0, tile in ((260, 103, 90, 0.2, (128, 16)), (141, 77, 120, 0.7, (64, 8)), (64, 48, 200, 0.0, (32, 4))):
    p = dict(configs.BASE, theta0=th0)
    disks = [(nx // 2, ny // 2, 6), (10, 20, 3)]
    sim = Kobayashi(nx, ny, p["dt"], params=p)
    sim.seed_disks(disks)
    sim.set_tile(*tile)
    sim.step(steps)
    a = sim.fields()
    sim.close()
    b = ko_oracle.port_run(*configs.initial_fields(nx, ny, disks), p, steps, libm=False, threads=8)
    out.append(all(np.array_equal(x.view(np.uint64), y.view(np.uint64)) for x, y in zip(a, b)))
print(json.dumps(out))
"""


@pytest.mark.timeout(900)
def test_plain_build_equals_oracle():
    with tempfile.TemporaryDirectory() as d:
        lib = kbuild.build_variant(os.path.join(d, "libkobayashi_plain.so"), kbuild.PLAIN)
        code = CHILD % dict(root=ROOT, oracle=os.path.join(ROOT, "oracle"), lib=lib)
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr[-3000:]
        assert json.loads(r.stdout.strip().splitlines()[-1]) == [True, True, True]

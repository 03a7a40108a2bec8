"""Every compile-time switch of the kernels, in each of its settings, still
compiles for sm_103a (no GPU needed: nvcc cross-compiles).  The switches are
kept for A/B measurements; the library ships with the measured winners
(crystalgrowth_gb300/build.py SWITCHES).  Every setting computes the same bits:
the plain build, with every switch in its other setting, is checked against
the oracle on the GPU in tests/test_gpu_plain_build.py."""
import concurrent.futures as cf
import os
import subprocess
import tempfile

import pytest

from crystalgrowth_gb300 import build as kbuild

SETTINGS = {"KG_BITS_ASM": [0], "KG_GDIV": [0], "KG_FAR": [0], "KG_FUSE": [0], "KG_QUIET": [0, 1, 2], "KG_ABSORB": [0],
            "KG_IDIV_SUBN": [0], "KG_SLOW_NOINLINE": [0], "KG_TMA": [0]}


def test_switch_table_matches_the_sources():
    """every switch named in the build's table is defined with that default in the sources"""
    src = ""
    for f in os.listdir(kbuild.CSRC):
        if f.endswith((".cu", ".cuh", ".h")):
            src += open(os.path.join(kbuild.CSRC, f)).read()
    for name, default in kbuild.SWITCHES.items():
        assert "#ifndef %s\n#define %s %d\n#endif" % (name, name, default) in src, name
    assert set(SETTINGS) == set(kbuild.SWITCHES) == set(kbuild.PLAIN)


def _compile(defines):
    with tempfile.TemporaryDirectory() as d:
        flags = ["-D%s=%s" % kv for kv in defines.items()]
        for src in ("kg_sim.cu", "kg_batch.cu", "kg_adjoint.cu"):
            r = subprocess.run([kbuild.nvcc()] + kbuild.cflags() + flags +
                               ["-c", os.path.join(kbuild.CSRC, src), "-o", os.path.join(d, src + ".o")],
                               capture_output=True, text=True)
            if r.returncode != 0:
                return "%s %s: %s" % (src, flags, r.stderr[-2000:])
    return None


@pytest.mark.timeout(900)
def test_every_setting_compiles():
    cases = [{k: v} for k, vals in SETTINGS.items() for v in vals] + [dict(kbuild.PLAIN)]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        errs = [e for e in ex.map(_compile, cases) if e]
    assert not errs, errs[0]

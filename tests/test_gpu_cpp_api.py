"""The header-only C++ class (include/kobayashi.hpp) as a reference caller
would use it (src/main.cpp:14-18: Kobayashi(250, 250, 0.0001f), then iUpdate
per frame): compiled with g++ against the library, its results must equal the
same run through the Python binding bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from crystalgrowth_gb300 import Kobayashi, _lib

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def fnv(arrays):
    h = 1469598103934665603
    for a in arrays:
        for b in np.ascontiguousarray(a, dtype=np.float64).tobytes():
            h ^= b
            h = (h * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def test_cpp_class_runs_like_the_reference_main(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "kobayashi_hpp_check"
    libdir = os.path.dirname(_lib.LIB_PATH)
    subprocess.run([gxx, "-std=c++14", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "kobayashi_hpp_check.cpp"), "-o", str(exe),
                    "-L", libdir, "-lkobayashi_gpu", "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    nx, ny, steps, frames, h = out[0].split()
    assert (int(nx), int(ny), int(steps), int(frames)) == (250, 250, 300, 30)
    sim = Kobayashi(250, 250, 0.0001)
    for _ in range(30):
        sim.iUpdate()
    assert int(h, 16) == fnv(sim.fields())
    sim.close()
    assert out[1] == "reset 0 0"
    assert out[2] == "invalid params rejected 1"
    assert out[3] == "tblock 2 same 1"

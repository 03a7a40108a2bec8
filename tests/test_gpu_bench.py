"""bench.py's own legs on small cases: the JSON line of the single-grid arm (the end-to-end leg replays
the timed window and must arrive at the same final state bit for bit), and the batched ensemble's
window mode (state saved at one time step and timed again from the file)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + list(args), capture_output=True,
                       text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-3000:]
    return json.loads(lines[0])


def test_bench_line_and_e2e_replay():
    d = run_bench("--grid", "1024", "--disks", "1", "--steps", "2", "--warmup", "3", "--no-cpu-baseline",
                  "--no-extras")
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "dtype", "config", "roofline", "e2e", "gpu_launches", "clocks"):
        assert key in d, key
    assert d["steps"] == 2 and d["gpu_launches"] == 200 and d["value"] > 0
    e = d["e2e"]
    assert e["value"] > 0 and e["h2d_bytes_per_step"] == e["d2h_bytes_per_step"] == 3 * 8 * 1024 * 1024
    assert e["breakdown"]["same_final_state"] is True
    assert "time step 0" in d["config"]["e2e_steps"]


def test_bench_ensemble_window(tmp_path):
    snap = str(tmp_path / "ens.npz")
    a = run_bench("--ensemble-at", "20", "--ensemble-save", snap, "--ensemble-tuning", "64,32,1", "--steps", "3",
                  "--warmup", "2")
    assert a["ensemble_window"] == "ensemble_512, time steps 22..25" and a["ms_per_step"] > 0
    b = run_bench("--ensemble-load", snap, "--ensemble-tuning", "128,16,2", "--steps", "3", "--warmup", "2")
    assert b["ensemble_window"] == "ensemble_512, time steps 22..25"
    assert b["tuning"] == {"nt": 128, "bh": 16, "mode": 0, "streams": 2, "tblock": 1}

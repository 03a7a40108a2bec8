"""Regenerate the golden fixtures in this folder from the reference's own code.

Runs jklae/CrystalGrowth's src/Kobayashi.cpp, compiled unmodified by
oracle/build_oracle.py (FP64 "float -> double" build and the FP32 build as
shipped), on small cases, and stores what it produced:

  ref64_default_64x48.npz   reference defaults (src/Kobayashi.cpp:61-63,76-84),
                            the reference's own nucleus (_vectorInit), 20 x iUpdate
                            = 200 steps; full phi, T, theta
  ref32_default_64x48.npz   the same with the FP32 build as shipped
  ref64_colors_64x64.npz    iUpdateConstantBuffer colours of every cell after
                            100 steps on a 64x64 grid (FP64 and FP32 builds)
  ref64_edge.npz            3x3 and 17x13 grids, 25 steps, reference nucleus
  ref64_grid300.json        300^2, delta=0.02, theta0=0 (the reference has no
                            theta0), disk r=5 at (150,150), 2000 steps: SHA-256
                            of the final phi/T/theta bytes plus summary numbers
  kgm_grid300.json          the same case through the oracle with kg_math's
                            atan/sin/cos and theta0=0.2: the GPU must reproduce
                            these hashes; also the measured noise floor between
                            kg_math and the C library after 2000 steps

Needs the reference checkout (only present where fixtures are made).
Run from the repository root:  python tests/golden/make_golden.py [--only-kgm]
(--only-kgm rewrites kgm_grid300.json alone, after a change to kg_math.h)
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import ko_oracle  # noqa: E402
from crystalgrowth_gb300 import configs  # noqa: E402

DEFAULT = dict(dx=0.03, dy=0.03, dt=1e-4, tau=3e-4, eps_bar=0.01, mu=1.0, K=1.6, delta=0.05, aniso=6.0, alpha=0.9,
               gamma=10.0, teq=1.0, theta0=0.0)


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def run_ref(nx, ny, params, steps, fp64=True, init=None, via_update=False):
    r = ko_oracle.Reference(nx, ny, params["dt"], fp64=fp64)
    r.set_params(params)
    if init is None:
        r.vector_init()
    else:
        r.set_state(*init)
    if via_update:
        assert steps % 10 == 0
        for _ in range(steps // 10):
            r.update()
    else:
        r.step(steps)
    return r


def main():
    ko_oracle.build()
    only_kgm = "--only-kgm" in sys.argv[1:]
    if only_kgm:
        write_kgm()
        return
    # 1, 2: reference defaults on 64x48 through iUpdate
    for fp64, name in ((True, "ref64_default_64x48.npz"), (False, "ref32_default_64x48.npz")):
        r = run_ref(64, 48, DEFAULT, 200, fp64=fp64, via_update=True)
        phi, t, th = r.get_state()
        dt = np.float64 if fp64 else np.float32
        np.savez_compressed(os.path.join(HERE, name), phi=phi.astype(dt), T=t.astype(dt), theta=th.astype(dt),
                            steps=200, frames=r.frame(), params=json.dumps(DEFAULT))
    # 3: colours
    cols = {}
    for fp64 in (True, False):
        r = run_ref(64, 64, DEFAULT, 100, fp64=fp64)
        phi, _, _ = r.get_state()
        cols["rgba64" if fp64 else "rgba32"] = r.colors()
        cols["phi64" if fp64 else "phi32"] = phi
    np.savez_compressed(os.path.join(HERE, "ref64_colors_64x64.npz"), **cols)
    # 4: small and ragged grids
    edge = {}
    for nx, ny in ((3, 3), (17, 13)):
        r = run_ref(nx, ny, DEFAULT, 25)
        phi, t, th = r.get_state()
        edge["phi_%dx%d" % (nx, ny)] = phi
        edge["T_%dx%d" % (nx, ny)] = t
        edge["theta_%dx%d" % (nx, ny)] = th
    np.savez_compressed(os.path.join(HERE, "ref64_edge.npz"), **edge)
    # 5: 300^2, 2000 steps, reference (theta0 = 0)
    cfg = configs.grid_300()
    p0 = dict(cfg["params"], theta0=0.0)
    init = configs.initial_fields(300, 300, cfg["disks"])
    r = run_ref(300, 300, p0, cfg["steps"], init=init)
    phi, t, th = r.get_state()
    ref = dict(params=p0, steps=cfg["steps"], disks=cfg["disks"], sha_phi=sha(phi), sha_T=sha(t), sha_theta=sha(th),
               max_phi=float(phi.max()), max_T=float(np.abs(t).max()), sum_phi=float(phi.sum()))
    with open(os.path.join(HERE, "ref64_grid300.json"), "w") as f:
        json.dump(ref, f, indent=1)
    write_kgm()
    print("fixtures written to", HERE)


def write_kgm():
    """6: the 300^2 case through kg_math (what the GPU computes), theta0 = 0 and 0.2, with the noise
    floor against the C library's functions"""
    cfg = configs.grid_300()
    p0 = dict(cfg["params"], theta0=0.0)
    init = configs.initial_fields(300, 300, cfg["disks"])
    out = dict(steps=cfg["steps"], disks=cfg["disks"])
    for tag, prm in (("theta0_0", p0), ("theta0_02", cfg["params"])):
        a = ko_oracle.port_run(*init, prm, cfg["steps"], libm=False, threads=8)
        b = ko_oracle.port_run(*init, prm, cfg["steps"], libm=True, threads=8)
        out[tag] = dict(params=prm, sha_phi=sha(a[0]), sha_T=sha(a[1]), sha_theta=sha(a[2]),
                        noise_floor_phi=float(np.abs(a[0] - b[0]).max() / np.abs(b[0]).max()),
                        noise_floor_T=float(np.abs(a[1] - b[1]).max() / np.abs(b[1]).max()))
    with open(os.path.join(HERE, "kgm_grid300.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()

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

  full_configs.json         the large workloads at full length through the oracle
                            with kg_math (what the GPU computes): SHA-256 of the
                            final fields of the 8192^2 grid (64 disks) at steps
                            1000, 2000, 5000 and 10,000; of all 54 anisotropy
                            variants on 2048^2 at 5000 steps; and of all 512
                            instances of the mixed-size ensemble at 3000 steps.
                            Written by --full-configs (hours of CPU time; each
                            finished part is saved at once, and a rerun skips
                            the parts already present)

Needs the reference checkout (only present where fixtures are made), except
for --only-kgm and --full-configs, which run the C restatement alone.
Run from the repository root:
  python tests/golden/make_golden.py [--only-kgm]
  python tests/golden/make_golden.py --full-configs [--threads N] [--part grid8192|variants|ensemble]
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
    if "--full-configs" in sys.argv[1:]:
        write_full_configs()
        return
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


FULL = os.path.join(HERE, "full_configs.json")


def _arg(name, default):
    a = sys.argv[1:]
    return a[a.index(name) + 1] if name in a else default


def _save_full(doc):
    tmp = FULL + ".tmp"
    with open(tmp, "w") as f:
        json.dump(doc, f, indent=1, sort_keys=True)
    os.replace(tmp, FULL)


def field_hashes(phi, t, th):
    return dict(sha_phi=sha(phi), sha_T=sha(t), sha_theta=sha(th))


def _variants_done(path):
    try:
        return json.load(open(path)).get("variants_2048", {}).get("variants", {})
    except (OSError, ValueError):
        return {}


def _variant_job(args):
    v, threads, path = args
    if v["name"] in _variants_done(path):  # another process finished it meanwhile
        return v["name"], None
    st = ko_oracle.port_run(*configs.initial_fields(v["nx"], v["ny"], v["disks"]), v["params"], v["steps"],
                            libm=False, threads=threads)
    return v["name"], field_hashes(*st)


def _merge_variants(path, steps, found):
    """adds `found` to the variants in `path` under a file lock (several processes may share the file)
    and returns everything the file then holds"""
    import fcntl
    with open(path + ".lock", "w") as lk:
        fcntl.flock(lk, fcntl.LOCK_EX)
        doc = json.load(open(path)) if os.path.exists(path) else {}
        vd = doc.setdefault("variants_2048", {"steps": steps, "variants": {}})
        vd["variants"].update(found)
        tmp = path + ".tmp%d" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(doc, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
        return dict(vd["variants"])


def _instance_job(args):
    k, inst, steps = args
    st = ko_oracle.port_run(*configs.initial_fields(inst["nx"], inst["ny"], inst["disks"]), inst["params"], steps,
                            libm=False, threads=1)
    return k, hashlib.sha256(b"".join(np.ascontiguousarray(a).tobytes() for a in st)).hexdigest()


def write_full_configs():
    """7: the large workloads at full length (see the module docstring)"""
    import concurrent.futures as cf
    import multiprocessing as mp
    import time
    threads = int(_arg("--threads", str(os.cpu_count() or 1)))
    part = _arg("--part", "all")
    doc = json.load(open(FULL)) if os.path.exists(FULL) else {}
    doc["note"] = ("oracle ko_run with kg_math (libm=0), the arithmetic the GPU reproduces; sha256 of the "
                   "float64 little-endian bytes of each [ny, nx] field")
    ctx = mp.get_context("spawn")
    if part in ("all", "ensemble"):
        cfg = configs.ensemble_512()
        ens = doc.setdefault("ensemble_512", {"steps": cfg["steps"], "instances": {}})
        todo = [(k, i, cfg["steps"]) for k, i in enumerate(cfg["instances"]) if str(k) not in ens["instances"]]
        # largest first, so the pool ends on small jobs
        todo.sort(key=lambda a: -a[1]["nx"] * a[1]["ny"])
        t0 = time.time()
        with cf.ProcessPoolExecutor(max_workers=threads, mp_context=ctx) as ex:
            for n, (k, h) in enumerate(ex.map(_instance_job, todo)):
                ens["instances"][str(k)] = h
                if n % 32 == 31:
                    _save_full(doc)
        ens["what"] = "per instance: sha256 of phi, T, theta bytes concatenated, after %d steps" % cfg["steps"]
        _save_full(doc)
        print("ensemble_512 done in %.0f s" % (time.time() - t0), flush=True)
    if part in ("all", "grid8192"):
        cfg = configs.grid_8192()
        g = doc.setdefault("grid_8192", {"disks_seed": 8192, "params": cfg["params"], "at_step": {}})
        marks = [1000, 2000, 5000, 10000]
        done = [int(s) for s in g["at_step"]]
        if not all(m in done for m in marks):
            st = configs.initial_fields(cfg["nx"], cfg["ny"], cfg["disks"])
            at = 0
            t0 = time.time()
            for m in marks:
                st = ko_oracle.port_run(*st, cfg["params"], m - at, libm=False, threads=threads)
                at = m
                g["at_step"][str(m)] = field_hashes(*st)
                _save_full(doc)
                print("grid_8192 step %d at %.0f s" % (m, time.time() - t0), flush=True)
    if part in ("all", "variants"):
        # written to `--out` (default: the fixture itself) with locked merges, so that several processes
        # can share the list: each skips the variants already present
        out = _arg("--out", FULL)
        vs = configs.variants_2048()
        if "--reverse" in sys.argv[1:]:
            vs = vs[::-1]
        found = dict(doc.get("variants_2048", {}).get("variants", {})) if out == FULL else {}
        found.update(_variants_done(out))
        todo = [(v, 1, out) for v in vs if v["name"] not in found]
        t0 = time.time()
        with cf.ProcessPoolExecutor(max_workers=threads, mp_context=ctx) as ex:
            for name, h in ex.map(_variant_job, todo):
                if h is None:
                    continue
                _merge_variants(out, vs[0]["steps"], {name: h})
                print("variant %s at %.0f s" % (name, time.time() - t0), flush=True)


if __name__ == "__main__":
    main()

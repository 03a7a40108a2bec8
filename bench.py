"""Benchmark of the fused Kobayashi step on GB300 (FP64 cell-updates/s).

Workload (the headline throughput case): one 8192 x 8192 FP64 grid, 64
seeded disks of radius 4..8, reference parameters with delta = 0.02 and
theta0 = 0.2, 10,000 explicit steps advanced in CUDA-graph chunks of 100.
One bench step = one chunk = 100 time steps = 6.71e9 cell-updates.  After W
warm-up chunks the state is re-seeded, and K chunks are timed from step 0:
the default K = 100 is the whole 10,000-step trajectory, over which the
crystals (and the costlier interface cells) grow.  The state is 3.2 GB (two
copies of phi, T, theta), far above the 129 MB L2, so no flush is needed
between timed chunks.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference's own CPU step (src/Kobayashi.cpp built
unmodified in FP64 by oracle/build_oracle.py; the restated oracle if that
build is absent) on the host, one time step of the same 8192^2 state per
bench step.  Under torchrun with N > 1 every rank runs an independent replica
(the grid is not sharded: one GPU per box), rank 0 prints.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CHUNK = 100
BYTES_PER_CELL = 48  # phi, T, theta: FP64, read once and written once


def dist_init(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if os.environ.get("KG_BENCH_BACKEND", "nccl") == "nccl" else "gloo"
        dist.init_process_group(backend=backend)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi samples of the SM clock and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.proc = None
        self.device = device

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        rows = []
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 7:
                try:
                    rows.append((float(f[0]), float(f[1]), f[3:7]))
                except ValueError:
                    pass
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for _, _, fl in rows for k, v in enumerate(fl) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes and FP64 thread-operations per launch of the step kernel on the 8192^2 workload,
    from the committed ncu summary (None if absent)."""
    try:
        with open(os.path.join(ROOT, "profiles", "kg_step_kernel_traffic.json")) as f:
            d = json.load(f)
        return d.get("bytes_per_launch_8192"), d
    except (OSError, ValueError):
        return None, {}


def fp64_peak():
    """FP64 lane-operations per second of this GPU, measured now: the best of kg_diag_fp64_peak's sweep
    (FMA, add, multiply and the step's add/multiply mix; 8 or 16 chains; 2-8 CTAs per SM), and the
    lanes per SM clock of the add/multiply mix (clock64 stamps, independent of the clock rate)."""
    import ctypes
    from crystalgrowth_gb300 import _lib
    v, a, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    _lib.check(_lib.lib().kg_diag_fp64_peak(ctypes.byref(v)))
    _lib.check(_lib.lib().kg_diag_fp64_probe(3, 8, 4, 256, ctypes.byref(a), ctypes.byref(c)))
    return v.value, c.value


def cpu_baseline_sample(cfg, seconds_budget=20.0):
    """The reference's own FP64 step on the host: 8192^2 state from the workload, whole time steps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import ko_oracle
    from crystalgrowth_gb300 import configs
    nx, ny = cfg["nx"], cfg["ny"]
    init = configs.initial_fields(nx, ny, cfg["disks"])
    p = dict(cfg["params"])
    try:
        r = ko_oracle.Reference(nx, ny, p["dt"], fp64=True)
        kind = "reference"
        p_ref = dict(p)  # the reference has no theta0; its step is timed with the same field sizes
        r.set_params(p_ref)
        r.set_state(*init)
        step = r.step
    except (FileNotFoundError, OSError):
        kind = "port"
        state = list(init)

        def step(n):
            state[:] = ko_oracle.port_run(*state, p, n, libm=True, threads=1)
    t0 = time.perf_counter()
    step(1)
    t1 = time.perf_counter()
    n_steps = 1
    per = t1 - t0
    extra = max(0, int(seconds_budget / max(per, 1e-3)) - 1)
    extra = min(extra, 4)
    if extra:
        t2 = time.perf_counter()
        step(extra)
        per = (time.perf_counter() - t2) / extra
        n_steps += extra
    out = {"value": nx * ny / per, "unit": "cell-updates/s", "cores": 1, "kind": kind,
           "sample": "%d time step(s) of the %dx%d FP64 state, single thread (the reference is single-threaded)"
                     % (n_steps, nx, ny)}
    # beside it: the reference as shipped (FP32, single thread), and the C restatement (FP64, C library
    # math) with OpenMP over all host cores -- two time steps each of the same state
    try:
        r32 = ko_oracle.Reference(nx, ny, p["dt"], fp64=False)
        r32.set_params(p)
        r32.set_state(*init)
        r32.step(1)
        t0 = time.perf_counter()
        r32.step(2)
        out["fp32_as_shipped"] = {"value": 2 * nx * ny / (time.perf_counter() - t0), "cores": 1,
                                  "kind": "reference", "sample": "2 time steps, FP32 build as shipped"}
        del r32
    except (FileNotFoundError, OSError):
        pass
    cores = os.cpu_count() or 1
    st = ko_oracle.port_run(*init, p, 1, libm=True, threads=cores)
    t0 = time.perf_counter()
    ko_oracle.port_run(*st, p, 2, libm=True, threads=cores)
    out["restatement_all_cores"] = {"value": 2 * nx * ny / (time.perf_counter() - t0), "cores": cores,
                                    "kind": "port", "sample": "2 time steps, FP64, OpenMP over rows"}
    return out


def measure_ensemble(steps=3000, trial_steps=10, tune_at=1500):
    """The mixed-size ensemble (512 instances, sides 64..512, per-instance parameters), timed over its
    whole 3000-step workload from the initial state three ways: the autotuned batched form (CUDA graphs
    of 100 steps); the 512 instances as single-grid handles run one after another on one stream (the
    looped baseline); and the same handles each on its own stream (concurrent single-grid runs).
    The autotuner runs on the ensemble's own state at step `tune_at`, the middle of the workload (its
    trials restore the state they start from), and the timed run starts again from the seeds."""
    import torch
    from crystalgrowth_gb300 import Batch, Kobayashi, configs
    cfg = configs.ensemble_512()
    inst = cfg["instances"]
    cells = sum(i["nx"] * i["ny"] for i in inst)
    b = Batch([(i["nx"], i["ny"]) for i in inst], [i["params"] for i in inst])

    def seed_batch():
        for k, i in enumerate(inst):
            b.seed_disks(k, i["disks"])
    seed_batch()
    b.step(tune_at)
    t0 = time.perf_counter()
    best, _ = b.autotune(trial_steps=trial_steps)
    tune_s = time.perf_counter() - t0
    seed_batch()
    b.set_tuning(**dict(best, chunk=CHUNK))
    b.step(CHUNK)  # warm-up (graph build)
    seed_batch()
    stream = torch.cuda.ExternalStream(b.stream())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    b.sync()
    e0.record(stream)
    b.step(steps)
    e1.record(stream)
    e1.synchronize()
    batched_s = e0.elapsed_time(e1) / 1e3
    b.close()

    sims = []
    for i in inst:
        s = Kobayashi(i["nx"], i["ny"], i["params"]["dt"], params=i["params"])
        s.set_graph_chunk(CHUNK)
        s.step(CHUNK)  # warm-up (graph build)
        sims.append(s)

    def run(sequential):
        for s, i in zip(sims, inst):
            s.seed_disks(i["disks"])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s in sims:
            s.step(steps)
            if sequential:
                s.sync()
        for s in sims:
            s.sync()
        return time.perf_counter() - t0
    looped_s = run(True)
    concurrent_s = run(False)
    for s in sims:
        s.close()
    work = cells * steps
    return {"workload": "ensemble_512: 512 instances, sides log-uniform 64..512, %d cells; time steps 0..%d"
                        % (cells, steps),
            "batched_cell_updates_per_s": work / batched_s, "looped_cell_updates_per_s": work / looped_s,
            "concurrent_streams_cell_updates_per_s": work / concurrent_s,
            "speedup_vs_looped": looped_s / batched_s, "speedup_vs_concurrent_streams": concurrent_s / batched_s,
            "tuning": best, "autotune_s": tune_s, "tuned_at_step": tune_at,
            "looped": "512 single-grid handles, one after another (each in CUDA graphs of %d steps)" % CHUNK,
            "concurrent_streams": "the same 512 handles, each on its own stream, all enqueued before waiting"}


def ensemble_window(args):
    """The batched ensemble's step time at one point of its trajectory, with one launch-mode tuning (no
    autotuning): the state comes from the seeds advanced --ensemble-at steps, or from a file written
    by --ensemble-save; W warm-up steps, then K timed steps (CUDA events).  For profiling the batched
    kernel at a later state without replaying the trajectory under a profiler."""
    import numpy as np
    import torch
    from crystalgrowth_gb300 import Batch, configs
    inst = configs.ensemble_512()["instances"]
    cells = sum(i["nx"] * i["ny"] for i in inst)
    b = Batch([(i["nx"], i["ny"]) for i in inst], [i["params"] for i in inst])
    if args.ensemble_load:
        snap = np.load(args.ensemble_load)
        start, flat = int(snap["step"]), snap["state"]
        off = 0
        for k, i in enumerate(inst):
            n = i["nx"] * i["ny"]
            b.set_fields(k, flat[off:off + n], flat[off + n:off + 2 * n], flat[off + 2 * n:off + 3 * n])
            off += 3 * n
    else:
        start = args.ensemble_at
        for k, i in enumerate(inst):
            b.seed_disks(k, i["disks"])
        b.set_tuning(nt=64, bh=64, mode=0, chunk=CHUNK, streams=4, tblock=1)
        b.step(start)
    if args.ensemble_save:
        b.sync()
        np.savez(args.ensemble_save, step=start,
                 state=np.concatenate([a.ravel() for k in range(len(inst)) for a in b.fields(k)]))
    nt, bh, streams = (int(v) for v in args.ensemble_tuning.split(","))
    b.set_tuning(nt=nt, bh=bh, mode=0, chunk=max(1, min(args.steps, CHUNK)), streams=streams, tblock=1)
    stream = torch.cuda.ExternalStream(b.stream())
    b.step(args.warmup)
    b.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.step(args.steps)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    b.close()
    print(json.dumps({"ensemble_window": "ensemble_512, time steps %d..%d" % (start + args.warmup,
                                                                             start + args.warmup + args.steps),
                      "ms_per_step": ms, "cell_updates_per_s": cells / ms * 1e3,
                      "tuning": {"nt": nt, "bh": bh, "mode": 0, "streams": streams, "tblock": 1}}), flush=True)
    return 0


def measure_adjoint():
    """Adjoint/forward cost on the 512^2, 4000-step rollout with checkpoints every 64 steps."""
    import numpy as np
    from crystalgrowth_gb300 import Adjoint, configs
    cfg = configs.adjoint_512()
    n, steps = cfg["nx"], cfg["steps"]
    phi0, _, th0 = configs.initial_fields(n, n, cfg["disks"])
    tgt = Adjoint(n, n, cfg["target_params"], steps, checkpoint_every=cfg["checkpoint_every"])
    tgt.set_initial(phi0, cfg["T0"], th0)
    tgt.set_target(np.zeros((n, n)))
    _, (target, _, _) = tgt.forward(want_state=True)
    tgt.close()
    adj = Adjoint(n, n, cfg["params"], steps, checkpoint_every=cfg["checkpoint_every"])
    adj.set_initial(phi0, cfg["T0"], th0)
    adj.set_target(target)
    adj.forward()
    adj.gradient()  # warm-up
    t0 = time.perf_counter()
    loss = adj.forward()
    t1 = time.perf_counter()
    g, _ = adj.gradient()
    t2 = time.perf_counter()
    adj.close()
    fwd, grad = t1 - t0, t2 - t1
    return {"workload": "adjoint_512: 512x512, 4000 steps, checkpoints every 64",
            "forward_s": fwd, "gradient_s": grad, "adjoint_forward_ratio": grad / fwd,
            "loss": loss, "gradient": {k: v for k, v in g.items() if k != "loss"},
            "note": "gradient_s includes its own forward rollout; ratio = gradient time / forward time"}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ko_oracle
    from crystalgrowth_gb300 import configs
    cfg = configs.grid_8192()
    nx, ny = cfg["nx"], cfg["ny"]
    init = configs.initial_fields(nx, ny, cfg["disks"])
    try:
        r = ko_oracle.Reference(nx, ny, cfg["params"]["dt"], fp64=True)
        r.set_params(cfg["params"])
        r.set_state(*init)
        step = r.step
        kind = "reference"
    except (FileNotFoundError, OSError):
        kind = "port"
        state = list(init)

        def step(n):
            state[:] = ko_oracle.port_run(*state, cfg["params"], n, libm=True, threads=1)
    for _ in range(args.warmup):
        step(1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step(1)
    dt = time.perf_counter() - t0
    value = nx * ny * args.steps / dt
    line = {"impl": "reference", "metric": "fp64_cell_updates_per_s", "value": value, "unit": "cell-updates/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "grid_%d: %dx%d FP64 Kobayashi step, %d seeded disks r=4..8, "
                                   "delta=0.02 theta0=0.2" % (nx, nx, ny, len(cfg["disks"])),
                       "bench_step": "1 time step on the host (reference CPU path)", "disks_seed": 8192,
                       "l2": "inputs larger than L2 (3.2 GB state)",
                       "note": "the reference's model has no theta0: it steps the same state with theta0 = 0 "
                               "(the cost per cell does not depend on theta0)"},
            "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": 1, "kind": kind,
                             "sample": "%d timed time steps of the 8192^2 state, single thread" % args.steps},
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, rank, world):
    import numpy as np
    import torch
    from crystalgrowth_gb300 import Kobayashi, configs

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    cfg = configs.grid_8192(n=args.grid, n_disks=args.disks)
    nx, ny = cfg["nx"], cfg["ny"]
    cells = nx * ny
    sim = Kobayashi(nx, ny, cfg["params"]["dt"], params=cfg["params"])
    sim.seed_disks(cfg["disks"])
    sim.set_graph_chunk(CHUNK)
    if args.tile:
        sim.set_tile(*(int(v) for v in args.tile.split(",")))
    if args.tblock != 1:
        sim.set_tblock(args.tblock)
    stream = torch.cuda.ExternalStream(sim.stream())

    # warm-up chunks (graph build, clocks), then the state is re-seeded: the timed chunks are time
    # steps 0 .. 100 K of the workload's trajectory (K = 100: the whole 10,000-step run)
    for _ in range(args.warmup):
        sim.step(CHUNK)

    def to_window_start():
        """the state at the first time step of the timed window; returns that step"""
        if args.load_snapshot:
            sim.load(args.load_snapshot)  # the timed window starts at the snapshot's step
            return sim.counters()[0]
        sim.seed_disks(cfg["disks"])
        if args.skip_to:
            sim.step(args.skip_to)  # untimed: the timed window starts later in the trajectory
        return args.skip_to

    start = to_window_start()
    if args.save_snapshot:
        sim.save(args.save_snapshot)
    sim.sync()

    # one event at every chunk boundary: the whole timed run, and the time of each 100-step chunk
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    clocks = Clocks(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    evs[0].record(stream)
    for k in range(args.steps):
        sim.step(CHUNK)
        evs[k + 1].record(stream)
    evs[-1].synchronize()
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()
    ms = evs[0].elapsed_time(evs[-1])
    chunk_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)]
    ms = max_over_ranks(ms, world)
    ms_per_step = ms / args.steps
    value = world * cells * CHUNK * args.steps / (ms / 1e3)
    launch_s = ms_per_step / 1e3 / CHUNK  # average duration of one step-kernel launch

    # end to end through the C ABI with host buffers, over the same time-step window as the timed run:
    # every chunk uploads the state, takes 100 steps and downloads the state
    e2e_steps = 0 if args.no_e2e else args.steps
    e2e_value = None
    e2e_parts = None
    if e2e_steps:
        pinned = [torch.empty((ny, nx), dtype=torch.float64, pin_memory=True) for _ in range(3)]
        host = [t.numpy() for t in pinned]
        final = [t.numpy() for t in (torch.empty((ny, nx), dtype=torch.float64, pin_memory=True) for _ in range(3))]
        sim.fields(out=final)  # the timed run's final state
        # the buffers are filled by a download, not by the CPU, then one untimed round trip: the first
        # device write into host lines the CPU holds dirty runs at a fraction of the link's speed
        to_window_start()
        sim.fields(out=host)
        sim.set_fields(*host)
        sim.fields(out=host)
        barrier(world)
        torch.cuda.synchronize()
        parts = [0.0, 0.0, 0.0]  # upload, steps, download (host clock; the steps' part ends at a sync)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ta = time.perf_counter()
            sim.set_fields(*host)
            tb = time.perf_counter()
            sim.step(CHUNK)
            sim.sync()
            tc = time.perf_counter()
            sim.fields(out=host)
            td = time.perf_counter()
            parts[0] += tb - ta
            parts[1] += tc - tb
            parts[2] += td - tc
        t1 = time.perf_counter()
        e2e_s = max_over_ranks(t1 - t0, world)
        e2e_value = world * cells * CHUNK * e2e_steps / e2e_s
        state_bytes = 3 * 8 * cells
        e2e_parts = {"upload_ms": 1e3 * parts[0] / e2e_steps, "steps_ms": 1e3 * parts[1] / e2e_steps,
                     "download_ms": 1e3 * parts[2] / e2e_steps,
                     "upload_gbs": state_bytes * e2e_steps / parts[0] / 1e9,
                     "download_gbs": state_bytes * e2e_steps / parts[2] / 1e9,
                     "same_final_state": all(np.array_equal(a.view(np.uint64), b.view(np.uint64))
                                             for a, b in zip(host, final))}
        del pinned, host, final

    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_CELL * cells / launch_s / 1e9
    traffic, prof = profile_traffic()
    # the FP64 pipe's share at the time steps whose FP64-pipe load ncu measured (per cell, on 4096^2
    # with the same disk density and strip shape): lane-slots = warp instructions on the FP64 pipe x 32,
    # against the probe's lane rate measured now; the time is that step's chunk, from the events
    fp64 = None
    samples = prof.get("fp64_lane_slots_per_cell_at_step", {}) if nx == 8192 and ny == 8192 else {}
    pts = []
    pk = None
    for step, opc in sorted((int(k), float(v)) for k, v in samples.items()):
        k = (step - start) // CHUNK
        if 0 <= k < len(chunk_ms):
            if pk is None:
                pk, per_clk = fp64_peak()
            t = chunk_ms[k] / 1e3 / CHUNK
            pts.append({"step": step, "lane_slots_per_cell_update": opc, "achieved": opc * cells / t / 1e9,
                        "frac": opc * cells / t / pk})
    if pts:
        # the nominal rate, 2 FP64 lanes per clock per SM at the highest SM clock sampled under load
        nominal = None
        if clk.get("sm_max_mhz"):
            nominal = 2 * torch.cuda.get_device_properties(local).multi_processor_count * clk["sm_max_mhz"] * 1e6
            for q in pts:
                q["frac_of_nominal"] = q["achieved"] * 1e9 / nominal
        fp64 = {"bound": "fp64 pipe", "unit": "G lane-slots/s", "peak": pk / 1e9,
                "peak_kind": "measured now (kg_diag_fp64_peak: best of FMA/add/multiply/mix dependency-chain "
                             "loops over chains and CTAs per SM)",
                "probe_lanes_per_sm_clock": per_clk,
                "nominal": nominal / 1e9 if nominal else None, "at_steps": pts,
                "ops_source": "ncu sm__inst_executed_pipe_fp64 x 32 per cell at those steps "
                              "(profiles/kg_step_kernel_traffic.json)"}
    line = {"metric": "fp64_cell_updates_per_s", "value": value, "unit": "cell-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "grid_%d: %dx%d FP64 Kobayashi step, %d seeded disks r=4..8, "
                                   "delta=0.02 theta0=0.2" % (nx, nx, ny, args.disks),
                       "bench_step": "one CUDA graph of %d time steps" % CHUNK,
                       "steps_timed": "time steps %d..%d of the trajectory from the seeded state (the "
                                      "workload is 10,000 steps)" % (start, start + args.steps * CHUNK),
                       "e2e_steps": "the timed window again (%d chunks from time step %d), after one untimed "
                                    "round trip; same_final_state: its downloaded final state equals the timed "
                                    "run's, bit for bit" % (e2e_steps, start),
                       "strips": "%d threads x %d rows" % sim.tile(),
                       "tblock": sim.tblock(),
                       "l2": "inputs larger than L2 (3.2 GB state)", "parallelism": "replicas" if world > 1 else "1 GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                         "note": "48 B/cell algorithmic; the kernel is FP64-pipe bound on GB300"},
            "fp64_roofline": fp64,
            "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": 3 * 8 * cells,
                    "d2h_bytes_per_step": 3 * 8 * cells, "breakdown": e2e_parts},
            "gpu_launches": args.steps * CHUNK,
            "chunk_ms": {"first": chunk_ms[0], "median": statistics.median(chunk_ms), "last": chunk_ms[-1],
                         "mean_per_1000_steps": [statistics.mean(chunk_ms[k:k + 10])
                                                 for k in range(0, len(chunk_ms), 10)]},
            "clocks": clk}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(cfg)
    if rank == 0 and not args.no_extras:
        line["ensemble"] = measure_ensemble()
        line["adjoint"] = measure_adjoint()
    sim.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100,
                    help="chunks of 100 time steps to time, from the seeded state (100: the whole 10,000-step run)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the ensemble and adjoint side measurements")
    ap.add_argument("--grid", type=int, default=8192, help="side of the square grid (8192 = the benchmark workload)")
    ap.add_argument("--disks", type=int, default=64)
    ap.add_argument("--tile", default="", help="strip shape NT,BH (default: the library's choice for the grid)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (short profiling runs)")
    ap.add_argument("--skip-to", type=int, default=0,
                    help="advance this many time steps untimed before the timed window (profiling of later windows)")
    ap.add_argument("--save-snapshot", default="", help="write the state at the start of the timed window to this "
                    "file (kg_save), for profiling a later window without replaying the trajectory")
    ap.add_argument("--load-snapshot", default="", help="start the timed window from this snapshot (kg_load) "
                    "instead of the seeds")
    ap.add_argument("--tblock", type=int, default=1, help="time steps per pass over HBM (1, or 2: temporal blocking)")
    ap.add_argument("--ensemble-at", type=int, default=-1, help="time only the batched ensemble, K steps after "
                    "W warm-up steps from this time step (profiling of the batched kernel)")
    ap.add_argument("--ensemble-save", default="", help="with --ensemble-at: write the state at that step here (.npz)")
    ap.add_argument("--ensemble-load", default="", help="time only the batched ensemble, from a state written by "
                    "--ensemble-save")
    ap.add_argument("--ensemble-tuning", default="64,64,1", help="NT,BH,STREAMS of the ensemble window (launch mode)")
    args = ap.parse_args()
    if args.ensemble_at >= 0 or args.ensemble_load:
        return ensemble_window(args)
    rank, world = dist_init(args.gpus)
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world)


if __name__ == "__main__":
    sys.exit(main())

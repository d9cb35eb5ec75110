"""Benchmark of the Barnes-Hut step (and the naive pair kernels) on GB300.

Default workload (the headline configuration): plain Barnes-Hut in FP64, theta = 0.5, the
reference's per-body opening rule, N = 1,048,576 bodies of the seeded heliocentric disc, dt = 1 h.
One step = leapfrog part 1 + octree build (AABB, keys, sort, cells, centre of mass) + traversal +
leapfrog part 2, i.e. one iteration of BarnesHutAlgorithm::startSimulation's loop.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints ONE JSON line on rank 0. `value` is device-resident throughput (steps/s summed over
ranks); `e2e` times the same step through the C ABI with the state in pinned host memory,
copied in and out every step. Multi-GPU: independent replicas (one per rank, no collective on
the data path), `scaling: weak`. `--impl reference` times the CPU restatement of the reference
(OpenMP, all host cores) on the same workload.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "n-body-simulation_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

N_BODIES = 1 << 20
THETA = 0.5
DT = 1.0 / 24
EPS2 = 1e-22
SEED = 1
def launches_per_step(n: int) -> int:
    """Kernels of ours launched per step: kick_drift 1, build (aabb 1, keys 1, radix 10 (one
    histogram of all digits, their offsets, 8 look-back passes), runs 1, splits 1, count 1, scan 3,
    emit 1, centre of mass: leaves 1, chunks of 4,096 bodies 1, one tier per factor of 64 above
    the chunk until one block spans all bodies), walk order from the last walk lengths 1,
    traversal 1, kick 1."""
    tiers, span = 0, 4096
    while True:
        tiers += 1
        span *= 64
        if span >= n:
            break
    return 4 + 21 + tiers
# algorithmic FLOP of the traversal (Nyland's 20 per pair interaction for an accepted cell; an
# opened cell costs its distance test: 3 sub, 3 mul, 2 add, 1 rsqrt, 1 mul = 10)
FLOP_ACCEPTED, FLOP_OPENED = 20, 10
TRAVERSAL_KERNEL = "bh_theta_lane_kernel"


from nbody.replicas import dist_env, job_throughput, max_over_ranks  # noqa: E402


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-i", str(self.device), "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [c.strip() for c in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_traffic(name):
    """(bytes per launch, source) of a kernel from the committed ncu summary, or (None, None)."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            e = json.load(f).get(name)
        return (e["bytes_per_launch"], e["source"]) if e else (None, None)
    except (OSError, ValueError, KeyError):
        return None, None


def measured_hbm_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def headline_config(ws: int) -> dict:
    """The workload both arms (ours and --impl reference) report, as one dict."""
    return {"workload": f"barnes-hut fp64 theta={THETA}, {N_BODIES:,}-body heliocentric disc "
                        f"(seed {SEED}), dt=1h, per-body opening rule (the reference's), "
                        "leapfrog + build + traversal per step",
            "bodies": N_BODIES, "theta": THETA, "dt_days": DT, "eps2": EPS2,
            "l2": "GPU arm: 256 MB buffer written before every timed step (L2 is 129 MB)",
            "parallelism": f"replicas x{ws}"}


# ---------------------------------------------------------------------------------------------
# CPU baseline (the oracle: C++/OpenMP restatement of the reference, timed on the host cores)
# ---------------------------------------------------------------------------------------------
def cpu_bh_step_seconds(d, sample_fraction: float):
    """One BH step of the restated reference on all host cores: leapfrog, full tree build and the
    traversal of an evenly strided sample of the bodies (scaled to all bodies)."""
    import numpy as np

    import oracle
    n = len(d["m"])
    x, y, z = d["x"].copy(), d["y"].copy(), d["z"].copy()
    v = [d["vx"].copy(), d["vy"].copy(), d["vz"].copy()]
    a = [np.zeros(n), np.zeros(n), np.zeros(n)]
    stride = max(1, int(round(1.0 / sample_fraction)))
    targets = np.arange(0, n, stride, dtype=np.uint32)
    t0 = time.perf_counter()
    vh = oracle.leapfrog_part1(v, [x, y, z], a, DT)
    t1 = time.perf_counter()
    tree = oracle.build_subtrees(d["m"], x, y, z)
    t2 = time.perf_counter()
    oracle.bh_accel_subset(tree, x, y, z, targets, d["G"], EPS2, THETA)
    t3 = time.perf_counter()
    oracle.leapfrog_part2(v, vh, a, DT)
    t4 = time.perf_counter()
    trav = (t3 - t2) * (n / len(targets))
    return (t1 - t0) + (t2 - t1) + trav + (t4 - t3), {"build_s": t2 - t1, "traversal_s": trav,
                                                       "traversal_sample_bodies": len(targets)}


def cpu_other_configs():
    """The restated reference (OpenMP, all host cores) on bounded samples of the other
    configurations, reported beside the GPU figures as baselines."""
    import numpy as np

    import oracle
    from nbody import generators
    out = {"cores": os.cpu_count(), "kind": "port"}
    # naive FP64, 16,384-body disc: one full evaluation (the reference's CPU-path configuration)
    d = generators.heliocentric_disc(16384, 1)
    t0 = time.perf_counter()
    oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], d["G"], EPS2)
    t = time.perf_counter() - t0
    out["naive_f64_disc_16384"] = {"gpairs_per_s": 16384.0 ** 2 / t / 1e9, "s_per_eval": t,
                                   "sample": "one full evaluation"}
    # naive FP64, 262,144-body Plummer: 2,048 evenly strided targets against all sources
    n = 262144
    p = generators.plummer(n, 1)
    tg = np.arange(0, n, n // 2048, dtype=np.uint32)
    t0 = time.perf_counter()
    oracle.naive_accel_subset(p["m"], p["x"], p["y"], p["z"], tg, 1.0, 1e-6)
    t = time.perf_counter() - t0
    out["naive_f64_plummer_262144"] = {"gpairs_per_s": len(tg) * float(n) / t / 1e9,
                                       "sample": f"{len(tg)} strided targets x {n} sources"}
    # Barnes-Hut theta = 0.5 on the 1,048,576-body disc + Plummer mix: full build, every 64th
    # body traversed, scaled to all bodies
    try:
        mix = generators.disc_plummer_mix(1 << 20, seed=21)
        n = len(mix["m"])
        t0 = time.perf_counter()
        tree = oracle.build_subtrees(mix["m"], mix["x"], mix["y"], mix["z"], storage_param=32)
        t1 = time.perf_counter()
        tg = np.arange(0, n, 64, dtype=np.uint32)
        oracle.bh_accel_subset(tree, mix["x"], mix["y"], mix["z"], tg, mix["G"], EPS2, THETA)
        t2 = time.perf_counter()
        step = (t1 - t0) + (t2 - t1) * n / len(tg)
        out["bh_theta0.5_mix_1M"] = {"steps_per_s": 1.0 / step, "build_s": t1 - t0,
                                     "sample": "full build + every 64th body traversed, scaled"}
    except Exception as e:  # reported, not fatal: the GPU figures do not depend on it
        out["bh_theta0.5_mix_1M"] = {"error": str(e)}
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from nbody import generators

    d = generators.heliocentric_disc(N_BODIES, SEED)
    cores = os.cpu_count()
    # size the per-step traversal sample so that warmup + steps stay within ~2.5 minutes
    probe_t, parts = cpu_bh_step_seconds(d, 1.0 / 64)
    fixed = probe_t - parts["traversal_s"]
    total_steps = args.steps + args.warmup
    frac = 1.0
    while frac > 1.0 / 64 and total_steps * (fixed + parts["traversal_s"] * frac) > 150:
        frac /= 2
    for _ in range(args.warmup):
        cpu_bh_step_seconds(d, frac)
    times = []
    for _ in range(args.steps):
        t, parts = cpu_bh_step_seconds(d, frac)
        times.append(t)
    t_step = sum(times) / len(times)
    value = 1.0 / t_step
    sample = (f"each step: leapfrog + full octree build of {N_BODIES} bodies + traversal of "
              f"1/{int(round(1 / frac))} of the bodies (strided) scaled to all bodies; every "
              f"step starts from the initial state (not advanced between timed steps) with zero "
              f"accelerations in its leapfrog")
    line = {"impl": "reference", "metric": "bh_steps_per_s_1M_fp64_theta0.5", "value": value,
            "unit": "steps/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": headline_config(ws),
            "cpu_baseline": {"value": value, "unit": "steps/s", "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------------
# ours
# ---------------------------------------------------------------------------------------------
def run_ours(args):
    import numpy as np
    import torch

    from nbody import generators
    from nbody.lib import REC_FP64, BHTree, Context, fma_peak

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    ctx = Context(local)
    d = generators.heliocentric_disc(N_BODIES, SEED)
    n = N_BODIES
    G = d["G"]
    f64 = dict(dtype=torch.float64, device="cuda")
    m = torch.as_tensor(d["m"], **f64)
    pos = [torch.as_tensor(d[k], **f64) for k in ("x", "y", "z")]
    vel = [torch.as_tensor(d[k], **f64) for k in ("vx", "vy", "vz")]
    acc = [torch.zeros(n, **f64) for _ in range(3)]
    vh = [torch.zeros(n, **f64) for _ in range(3)]
    tree = BHTree(ctx, n, theta=THETA)
    tree.set_records(REC_FP64)  # the node records the FP64 per-body rule reads
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    trav_ev = []

    def step(record_traversal=False):
        ctx.kick_drift(vh, vel, pos, acc, DT)
        tree.build(m, *pos, G)
        if record_traversal:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
        tree.accel(*pos, *acc, G, EPS2, "theta", "f64")
        if record_traversal:
            e1.record()
            trav_ev.append((e0, e1))
        ctx.kick(vel, vh, acc, DT)

    # initial accelerations (the reference's step 0)
    tree.build(m, *pos, G)
    tree.accel(*pos, *acc, G, EPS2, "theta", "f64")
    for _ in range(args.warmup):
        step()
    ctx.sync()

    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    step_ms = []
    for _ in range(args.steps):
        flush.zero_()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record()
        step(record_traversal=True)
        s1.record()
        step_ms.append((s0, s1))
    barrier()
    clk = clocks.stop()
    ctx.sync()
    t_local = sum(a.elapsed_time(b) for a, b in step_ms) / 1e3
    value = job_throughput(args.steps, t_local, ws, device="cuda")
    t_total = ws * args.steps / value  # the slowest rank's time
    ms_per_step = t_total / args.steps * 1e3
    trav_ms = sum(a.elapsed_time(b) for a, b in trav_ev) / len(trav_ev)

    # work model of the traversal on the current state
    accepted, opened = tree.count_interactions(*pos, "theta")
    flop = FLOP_ACCEPTED * accepted + FLOP_OPENED * opened
    fp64_peak = fma_peak(ctx, fp64=True)
    stats = tree.stats()

    # build passes against HBM, per phase (CUDA events between the phases of nb_bh_build):
    # algorithmic bytes per body / per node of each phase
    nodes = stats["node_count"]
    phase_bytes = {
        "aabb": 24 * n,                                  # read x, y, z
        "keys": 24 * n + 12 * n,                         # read x, y, z; write key + id
        "sort": 8 * 24 * n + 8 * n,                      # 8 passes: read + write key + id; histogram
        "cells": 16 * n + 29 * n + 12 * n + 8 * n + 24 * nodes,  # runs, splits, counts, scan,
                                                         # emit (node level/first/last/skip/...)
        "centre_of_mass": 64 * n + 192 * nodes,          # body m, x, y, z read, leaf sums
                                                         # written; per node: child sums read (40),
                                                         # sums (40) and child list (32) written,
                                                         # the FP64 record set (FP64 + FP32
                                                         # records: 80)
    }
    tree.set_phase_timing(True)
    phase_runs = []
    build_ev = []
    for _ in range(3):
        flush.zero_()
        b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        b0.record()
        tree.build(m, *pos, G)
        b1.record()
        build_ev.append((b0, b1))
        phase_runs.append(tree.build_phase_ms())
    tree.set_phase_timing(False)
    torch.cuda.synchronize()
    build_ms = min(a.elapsed_time(b) for a, b in build_ev)
    phase_ms = [min(r[k] for r in phase_runs) for k in range(5)]
    build_bytes = sum(phase_bytes.values())
    hbm_peak, hbm_src = measured_hbm_peak()

    # e2e: same step through the C ABI with the state in pinned host memory
    host = {k: torch.as_tensor(d[k], dtype=torch.float64).pin_memory()
            for k in ("m", "x", "y", "z", "vx", "vy", "vz")}
    host_acc = [torch.zeros(n, dtype=torch.float64).pin_memory() for _ in range(3)]
    h2d_arrays = [host["m"], host["x"], host["y"], host["z"], host["vx"], host["vy"], host["vz"]]
    h2d_arrays += host_acc
    dev_in = [m] + pos + vel + acc
    e2e_steps = max(3, min(args.steps, 10))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for dv, hv in zip(dev_in, h2d_arrays):
            dv.copy_(hv, non_blocking=True)
        step()
        for hv, dv in zip([host["x"], host["y"], host["z"], host["vx"], host["vy"], host["vz"]]
                          + host_acc, pos + vel + acc):
            hv.copy_(dv, non_blocking=True)
        torch.cuda.synchronize()
    t_e2e = max_over_ranks(time.perf_counter() - t0, device="cuda")
    ctx.sync()
    e2e_value = ws * e2e_steps / t_e2e

    also = {}
    if rank == 0 and ws == 1 and not args.quick:  # one GPU only: replicas runs stay short
        also = secondary_measurements(ctx, tree, m, pos, acc, G,
                                      with_cpu=not args.no_cpu_baseline,
                                      bench_ms_per_step=ms_per_step)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline and not args.quick:
        also["cpu_baselines_other_configs"] = cpu_other_configs()
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        t_cpu, parts = cpu_bh_step_seconds(d, 1.0 / 16)
        cpu = {"value": 1.0 / t_cpu, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "one step: leapfrog + full octree build of 1,048,576 bodies + traversal of "
                         "every 16th body scaled x16 (restated reference, OpenMP, all host cores)",
               "build_s": parts["build_s"], "traversal_s": parts["traversal_s"]}

    if rank == 0:
        achieved = flop / (trav_ms * 1e-3)
        line = {
            "metric": "bh_steps_per_s_1M_fp64_theta0.5", "value": value, "unit": "steps/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": headline_config(ws),
            "e2e": {"value": e2e_value, "unit": "steps/s",
                    "h2d_bytes_per_step": 8 * n * len(h2d_arrays),
                    "d2h_bytes_per_step": 8 * n * 9},
            "gpu_launches": launches_per_step(n) * args.steps,
            "roofline": {"kernel": TRAVERSAL_KERNEL + " (traversal)", "bound": "fp64",
                         "achieved": achieved / 1e12, "peak": fp64_peak / 1e12,
                         "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                         "traffic": load_traffic(TRAVERSAL_KERNEL)[0],
                         "traffic_source": load_traffic(TRAVERSAL_KERNEL)[1],
                         "peak_source": "FP64 FMA throughput measured in this run "
                                        "(nb_util_fma_peak)",
                         "work": {"accepted_cells": accepted, "opened_cells": opened,
                                  "flop_per_launch": flop, "ms_per_launch": trav_ms}},
            "roofline_build": {"bound": "hbm", "achieved": build_bytes / (build_ms * 1e-3) / 1e9,
                               "peak": hbm_peak, "unit": "GB/s",
                               "frac": build_bytes / (build_ms * 1e-3) / 1e9 / hbm_peak,
                               "peak_source": f"{hbm_src} (MEASURED_PEAKS.json hbm_gbs)",
                               "ms_per_build": build_ms, "algorithmic_bytes": build_bytes,
                               "traffic": load_traffic("bh_build")[0],
                               "phases": {name: {"ms": ms, "algorithmic_bytes": b,
                                                 "gbs": b / (ms * 1e-3) / 1e9,
                                                 "frac": b / (ms * 1e-3) / 1e9 / hbm_peak}
                                          for (name, b), ms in zip(phase_bytes.items(),
                                                                   phase_ms)}},
            "tree": {"nodes": nodes, "max_depth": stats["max_depth"],
                     "reference_layout_nodes": stats["ref_node_count"]},
            "clocks": clk,
            "cpu_baseline": cpu,
            "also": also,
        }
        print(json.dumps(line), flush=True)
    tree.close()
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def config1_cli_run(with_cpu: bool):
    """The reference's CPU-path configuration end to end through the reference's surface: the
    host driver nbody_sim, naive FP64 (opt_stage 2, block size 128) on the seeded 16,384-body
    heliocentric disc written as the reference's CSV, dt = 1 h, t_end = 10 d (240 leapfrog steps
    after the initial evaluation), energies on, output every 10 days. Wall time of the process
    (CSV parsing, CUDA context, upload, the run, output files) and the device time of its phases
    from its times.json; beside it the restated reference's full run of the same loop on the
    host cores (OpenMP), as the baseline."""
    import shutil
    import tempfile

    import numpy as np

    from nbody import generators
    exe = os.path.join(PKG, "_build", "nbody_sim")
    d = generators.heliocentric_disc(16384, 1)
    work = tempfile.mkdtemp(prefix="nbody_cfg1_")
    try:
        csv = os.path.join(work, "disc16384.csv")
        generators.write_csv(csv, d)
        out = os.path.join(work, "out")
        cmd = [exe, f"--file={csv}", "--dt=1h", "--t_end=10d", "--vs=10d", f"--vs_dir={out}",
               "--algorithm=naive", "--opt_stage=2", "--block_size=128", "--energy=true"]
        t0 = time.perf_counter()
        r = subprocess.run(cmd, capture_output=True, text=True)
        wall = time.perf_counter() - t0
        if r.returncode != 0:
            return {"error": r.stderr[-500:]}
        run_dir = os.path.join(out, os.listdir(out)[0])
        with open(os.path.join(run_dir, "times.json")) as f:
            times = json.load(f)
        res = {"command": "nbody_sim --file=disc16384.csv --dt=1h --t_end=10d --vs=10d "
                          "--algorithm=naive --opt_stage=2 --block_size=128 --energy=true",
               "steps": 240, "evaluations": 241, "cli_wall_s": wall,
               "device_s": {k: sum(v) / 1e3 for k, v in times.items() if isinstance(v, list)},
               "gpairs_per_s_over_wall": 241 * 16384.0 ** 2 / wall / 1e9}
        if with_cpu:
            import oracle
            x, y, z = d["x"].copy(), d["y"].copy(), d["z"].copy()
            v = [d["vx"].copy(), d["vy"].copy(), d["vz"].copy()]
            t0 = time.perf_counter()
            a = list(oracle.naive_accel(d["m"], x, y, z, d["G"], EPS2))
            for _ in range(240):
                vh = oracle.leapfrog_part1(v, [x, y, z], a, DT)
                a = list(oracle.naive_accel(d["m"], x, y, z, d["G"], EPS2))
                oracle.leapfrog_part2(v, vh, a, DT)
            cpu = time.perf_counter() - t0
            rows = np.loadtxt(os.path.join(run_dir, "lastState.csv"), delimiter=",", skiprows=1)
            dev_ = max(float(np.max(np.abs(rows[:, c] - o) / (np.abs(o) + 1e-9)))
                       for c, o in enumerate((x, y, z)))
            res["cpu_baseline"] = {"kind": "port", "cores": os.cpu_count(), "run_s": cpu,
                                   "sample": "the full run: 241 naive FP64 evaluations and 240 "
                                             "leapfrog steps (restated reference, OpenMP)",
                                   "speedup_cli_wall": cpu / wall}
            res["last_state_max_rel_diff_vs_cpu"] = dev_
        return res
    finally:
        shutil.rmtree(work, ignore_errors=True)


def config2_cli_run(bench_ms_per_step: float, steps: int = 10):
    """The headline configuration through the reference's surface: nbody_sim on the seeded
    1,048,576-body disc written as the reference's CSV, Barnes-Hut FP64, theta = 0.5, dt = 1 h,
    `steps` steps, output of the first and the last step only. The driver enqueues the whole run
    on one stream and times its phases with CUDA events (times.json); the per-step sum of its
    phases is compared with the bench's device-timed step."""
    import shutil
    import tempfile

    from nbody import generators
    exe = os.path.join(PKG, "_build", "nbody_sim")
    d = generators.heliocentric_disc(N_BODIES, SEED)
    work = tempfile.mkdtemp(prefix="nbody_cfg2_")
    try:
        csv = os.path.join(work, "disc.csv")
        generators.write_csv(csv, d)
        out = os.path.join(work, "out")
        cmd = [exe, f"--file={csv}", "--dt=1h", f"--t_end={steps}h", f"--vs={steps}h",
               f"--vs_dir={out}", "--algorithm=BarnesHut", f"--theta={THETA}"]
        t0 = time.perf_counter()
        r = subprocess.run(cmd, capture_output=True, text=True)
        wall = time.perf_counter() - t0
        if r.returncode != 0:
            return {"error": r.stderr[-500:]}
        run_dir = os.path.join(out, os.listdir(out)[0])
        with open(os.path.join(run_dir, "times.json")) as f:
            t = json.load(f)
        # steps after the initial evaluation: leapfrog part 1, build + traversal, part 2
        per_step = [a + b + c for a, b, c in zip(t["Leapfrog Part 1"], t["Total Time"][1:],
                                                  t["Leapfrog Part 2"])]
        ms = sum(per_step) / len(per_step)
        return {"command": f"nbody_sim --file=disc.csv --dt=1h --t_end={steps}h --vs={steps}h "
                           f"--algorithm=BarnesHut --theta={THETA}",
                "steps": len(per_step), "ms_per_step_device": ms,
                "bench_ms_per_step": bench_ms_per_step,
                "ratio_to_bench_step": ms / bench_ms_per_step, "process_wall_s": wall,
                "note": "process wall time includes parsing the 1M-row CSV, the CUDA context and "
                        "two ASCII .vtp files of 1M bodies"}
    finally:
        shutil.rmtree(work, ignore_errors=True)


def secondary_measurements(ctx, tree, m, pos, acc, G, with_cpu=True, bench_ms_per_step=None):
    """The other workloads on the same GPU: the FP32-pair group-rule step on the headline state,
    the reference's CPU-path configuration (naive FP64, 16,384-body disc), and the precision,
    batched and learned forms of the method (nbody/workloads.py)."""
    import torch

    from nbody import generators, workloads
    from nbody.lib import (REC_DF, REC_FP64, SYM_AUTO, SYM_NEVER, build_mask_for, fma_peak,
                           set_naive_symmetric)

    out = {}

    def timed(fn, reps):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        ctx.sync()
        return e0.elapsed_time(e1) / reps

    # FP32-pair Barnes-Hut (group rule) step at 1M on the same state
    def bh32():
        tree.build(m, *pos, G)
        tree.accel(*pos, *acc, G, EPS2, "group", "f32c")
    tree.set_records(build_mask_for("group", "f32c"))  # FP32 records, quantized keys
    ms = timed(bh32, 10)
    tree.set_records(REC_FP64)
    out["bh_f32c_group_theta0.5_1M"] = {"build_plus_traversal_ms": ms, "steps_per_s": 1e3 / ms}
    # the headline step with the double-float traversal (NB_DF64: same accepted cells, monopoles
    # in FP32-pair arithmetic) on a copy of the state, and its force difference to FP64
    pos2 = [p.clone() for p in pos]
    acc64 = [a.clone() for a in acc]
    acc2 = [torch.zeros_like(a) for a in acc]
    tree.set_records(REC_FP64 | REC_DF)  # the double-float traversal also reads the DF records
    tree.build(m, *pos2, G)
    tree.accel(*pos2, *acc64, G, EPS2, "theta", "f64")
    tree.accel(*pos2, *acc2, G, EPS2, "theta", "df64")
    torch.cuda.synchronize()
    num = torch.sqrt(sum((u - v) ** 2 for u, v in zip(acc2, acc64)))
    rel = (num / torch.sqrt(sum(u * u for u in acc64))).cpu()

    def bh_df():
        tree.build(m, *pos2, G)
        tree.accel(*pos2, *acc2, G, EPS2, "theta", "df64")
    ms = timed(bh_df, 10)
    ms_tr = timed(lambda: tree.accel(*pos2, *acc2, G, EPS2, "theta", "df64"), 10)
    tree.set_records(REC_FP64)
    out["bh_df64_theta0.5_1M"] = {
        "build_plus_traversal_ms": ms, "traversal_ms": ms_tr,
        "steps_per_s_excluding_leapfrog": 1e3 / ms,
        "rel_diff_vs_f64": {"median": float(rel.median()), "p99": float(rel.quantile(0.99)),
                            "max": float(rel.max())},
        "arithmetic": "double-float (FP32 pairs, ~2^-46 per pair term) for the accepted "
                      "monopoles; FP64 for positions, opening decisions and the output"}
    # the headline step replayed from a captured CUDA graph (one launch per step instead of 54
    # kernel launches), on copies of the state
    vel2 = [torch.zeros_like(p) for p in pos]
    vh2 = [torch.zeros_like(p) for p in pos]
    acc3 = [a.clone() for a in acc64]
    g = tree.graph(m, pos2, vel2, vh2, acc3, G, EPS2, DT, 1, "theta", "f64")
    ms = timed(g.launch, 10)
    g.close()
    out["bh_f64_theta0.5_1M_graph_step"] = {"ms_per_step": ms, "steps_per_s": 1e3 / ms}
    # naive FP64 on the reference's CPU-path configuration (16,384-body disc)
    n = 16384
    dd = generators.heliocentric_disc(n, 1)
    t = {k: torch.as_tensor(dd[k], device="cuda") for k in ("m", "x", "y", "z")}
    a = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    ms = timed(lambda: ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *a, dd["G"], EPS2, "f64"), 5)
    gp = n * n / (ms * 1e-3) / 1e9
    set_naive_symmetric(SYM_NEVER)
    ms1 = timed(lambda: ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *a, dd["G"], EPS2, "f64"),
                3)
    set_naive_symmetric(SYM_AUTO)
    gp1 = n * n / (ms1 * 1e-3) / 1e9
    peak64 = fma_peak(ctx, fp64=True)
    out["naive_f64_disc_16384"] = {
        "kernel": "pair_sym_kernel<double> (each unordered pair once, added to both bodies: 20 "
                  "FP64 operations per unordered pair = 10 per ordered pair)",
        "ms_per_eval": ms, "gpairs_per_s": gp,
        "frac_of_measured_fp64_fma_peak": gp * 20e9 / peak64,
        "executed_fp64_ops_frac_of_measured_peak": gp * 10e9 / (peak64 / 2),
        "one_sided": {"kernel": "naive_f64_kernel (16 FP64 operations per ordered pair)",
                      "ms_per_eval": ms1, "gpairs_per_s": gp1,
                      "frac_of_measured_fp64_fma_peak": gp1 * 20e9 / peak64}}
    ms = timed(lambda: ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *a, dd["G"], EPS2, "df64"),
               5)
    out["naive_df64_disc_16384"] = {
        "kernel": "pair_sym_df_kernel (each unordered pair once, added to both bodies)",
        "ms_per_eval": ms, "gpairs_per_s": n * n / (ms * 1e-3) / 1e9,
        "arithmetic": "double-float (FP32 pairs) on the FP32 pipe, FP64-accurate to ~1e-14"}
    if bench_ms_per_step:
        out["config2_bh_cli_disc_1M_10_steps"] = config2_cli_run(bench_ms_per_step)
    t0 = time.perf_counter()
    out["config1_naive_cli_disc_16384_10d"] = config1_cli_run(with_cpu)
    out["config1_naive_cli_disc_16384_10d"]["bench_wall_s"] = time.perf_counter() - t0
    for name, fn in (("precision_form_naive_f32c_plummer_262144", workloads.precision_form),
                     ("batched_ensemble_512_plummer", workloads.batched_ensemble),
                     ("learned_opening_bh_mix_1M", workloads.learned_form)):
        t0 = time.perf_counter()
        out[name] = fn(ctx)
        out[name]["wall_s"] = time.perf_counter() - t0
    return out


# ---------------------------------------------------------------------------------------------
# profiling cases (--case): small, self-contained runs of single kernels for ncu captures
# ---------------------------------------------------------------------------------------------
def pair_case(n: int = 262144, config: int = 0, symmetric: bool = False):
    import torch

    from nbody import generators, learned
    from nbody.lib import (SYM_ALWAYS, SYM_NEVER, Context, set_naive_pair_config,
                           set_naive_symmetric)
    ctx = Context(0)
    if symmetric:
        set_naive_symmetric(SYM_ALWAYS, config)
    else:
        set_naive_symmetric(SYM_NEVER, 0)
        set_naive_pair_config(config)
    t = learned.device_system(generators.plummer(n, 1))
    acc = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    for _ in range(3):
        ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *acc, 1.0, 1e-6, "f32c")
    ctx.sync()


def sym64_case(n: int = 65536, config: int = 0):
    import torch

    from nbody import generators, learned
    from nbody.lib import SYM_ALWAYS, Context, set_naive_symmetric
    ctx = Context(0)
    set_naive_symmetric(SYM_ALWAYS, 0, config)
    d = generators.heliocentric_disc(n, 1)
    t = learned.device_system(d)
    acc = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    for _ in range(3):
        ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *acc, d["G"], learned.EPS2, "f64")
    ctx.sync()


def learned_case(n: int = 262144, log10_tau: float = -4.25, pairs: int = 2_000_000):
    import torch

    from nbody import generators, learned
    from nbody.lib import BHTree, Context
    ctx = Context(0)
    X, Y = learned.training_set(ctx, n, pairs)
    params, _ = learned.train(ctx, X, Y, epochs=4)
    d = generators.disc_plummer_mix(n, seed=21)
    t = learned.device_system(d)
    tree = BHTree(ctx, n, theta=0.4)
    tree.build(t["m"], t["x"], t["y"], t["z"], d["G"])
    acc = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    tree.accel(t["x"], t["y"], t["z"], *acc, d["G"], learned.EPS2, "group", "f32c")
    tree.set_policy(params, log10_tau, 0.3, learned.NO_CAP)
    for _ in range(3):
        tree.accel(t["x"], t["y"], t["z"], *acc, d["G"], learned.EPS2, "learned", "f32c")
    ctx.sync()


def df64_case(n: int = 262144):
    import torch

    from nbody import generators, learned
    from nbody.lib import BHTree, Context
    ctx = Context(0)
    d = generators.heliocentric_disc(n, 1)
    t = learned.device_system(d)
    tree = BHTree(ctx, n, theta=0.5)
    tree.build(t["m"], t["x"], t["y"], t["z"], d["G"])
    acc = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    for _ in range(3):
        tree.accel(t["x"], t["y"], t["z"], *acc, d["G"], learned.EPS2, "theta", "df64")
    ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *acc, d["G"], learned.EPS2, "df64")
    ctx.sync()


def batch_case(systems: int = 512, config: int = -1):
    """The 512-system Plummer ensemble (N log-uniform in [256, 16384], seed 3): batch pair
    kernel in tile configuration `config` (-1: the autotuner's choice), three evaluations."""
    import numpy as np
    import torch

    from nbody import generators, learned, workloads
    from nbody.lib import Batch, Context
    ctx = Context(0)
    counts = workloads._ensemble_counts(systems, 256, 16384, 3)
    parts = [generators.plummer(int(c), seed=3 * 100003 + s) for s, c in enumerate(counts)]
    cat = {k: np.concatenate([p[k] for p in parts]) for k in ("m", "x", "y", "z", "vx", "vy", "vz")}
    t = learned.device_system(cat)
    n = len(cat["m"])
    acc = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    b = Batch(ctx, counts)
    if config < 0:
        b.autotune(t["m"], t["x"], t["y"], t["z"], *acc, 1.0, 1e-6, reps=2)
    else:
        b.set_config(config)
    for _ in range(3):
        b.accel(t["m"], t["x"], t["y"], t["z"], *acc, 1.0, 1e-6)
    ctx.sync()
    b.close()


def build_case(n: int = 1 << 20, mask: str = "fp64"):
    """Three octree builds of the seeded heliocentric disc with the node record set of a
    traversal: "fp64" (the headline's), "learned" (learned policy, quantized keys) or "all"."""
    from nbody import generators, learned
    from nbody.lib import BUILD_QUANTIZED_KEYS, REC_ALL, REC_FP64, REC_LEARNED, BHTree, Context
    masks = {"fp64": REC_FP64, "learned": REC_LEARNED | BUILD_QUANTIZED_KEYS, "all": REC_ALL}
    ctx = Context(0)
    d = generators.heliocentric_disc(n, 1)
    t = learned.device_system(d)
    tree = BHTree(ctx, n, theta=0.5)
    tree.set_records(masks[mask])
    for _ in range(3):
        tree.build(t["m"], t["x"], t["y"], t["z"], d["G"])
    ctx.sync()
    tree.close()


def leapfrog_case(n: int = 1 << 20, n_energy: int = 16384):
    """The leapfrog kernels on the seeded 1,048,576-body disc (HBM-bound: 120 and 72 bytes per
    body) and the energy (an O(N^2) FP64 pair sum, like the naive kernel) on its first 16,384
    bodies: three calls each."""
    import torch

    from nbody import generators, learned
    from nbody.lib import Context
    ctx = Context(0)
    d = generators.heliocentric_disc(n, 1)
    t = learned.device_system(d)
    pos = [t[k] for k in ("x", "y", "z")]
    vel = [t[k] for k in ("vx", "vy", "vz")]
    acc = [torch.full((n,), 1e-3, dtype=torch.float64, device="cuda") for _ in range(3)]
    vh = [torch.zeros_like(a) for a in acc]
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    ke = min(n, n_energy)
    for _ in range(3):
        ctx.kick_drift(vh, vel, pos, acc, DT)
        ctx.kick(vel, vh, acc, DT)
    for _ in range(3):
        ctx.energy(t["m"][:ke], *[a[:ke] for a in pos], *[v[:ke] for v in vel], d["G"], out)
    ctx.sync()


CASES = {
    "pair": lambda a: pair_case(int(a[0]) if a else 262144, int(a[1]) if len(a) > 1 else 0),
    "sym": lambda a: pair_case(int(a[0]) if a else 262144, int(a[1]) if len(a) > 1 else 0, True),
    "sym64": lambda a: sym64_case(int(a[0]) if a else 65536, int(a[1]) if len(a) > 1 else 0),
    "learned": lambda a: learned_case(int(a[0]) if a else 262144,
                                      float(a[1]) if len(a) > 1 else -4.25,
                                      int(a[2]) if len(a) > 2 else 2_000_000),
    "df64": lambda a: df64_case(int(a[0]) if a else 262144),
    "batch": lambda a: batch_case(int(a[0]) if a else 512, int(a[1]) if len(a) > 1 else -1),
    "build": lambda a: build_case(int(a[0]) if a else 1 << 20, a[1] if len(a) > 1 else "fp64"),
    "leapfrog": lambda a: leapfrog_case(int(a[0]) if a else 1 << 20),
}


def main():
    global N_BODIES
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--quick", action="store_true", help="skip the secondary measurements")
    ap.add_argument("--bodies", type=int, default=N_BODIES,
                    help="bodies of the disc (default 1,048,576; smaller only for profiling)")
    ap.add_argument("--case", nargs="+", metavar=("NAME", "ARG"),
                    help="run one profiling case instead of the benchmark: pair [N] [config], "
                         "sym [N] [config], sym64 [N] [config], learned [N] [log10_tau] [pairs], "
                         "df64 [N], batch [systems] [config], build [N] [fp64|learned|all]")
    args = ap.parse_args()
    if args.case:
        if args.case[0] not in CASES:
            ap.error(f"unknown case {args.case[0]!r}; one of {', '.join(CASES)}")
        CASES[args.case[0]](args.case[1:])
        print("ok")
        return 0
    if args.warmup < 3:
        args.warmup = 3
    N_BODIES = args.bodies
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

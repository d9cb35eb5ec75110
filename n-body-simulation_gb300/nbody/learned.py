"""Training and evaluation of the learned opening policy (driver code over the C ABI).

Pipeline (all compute in libnbody_cuda.so kernels):
  1. labelled pairs: for seeded systems, FP32-naive reference accelerations, a tree build, and
     nb_bh_generate_pairs (a theta-rule walk samples (32-body group, cell) pairs; each gets 8
     features and the label log10(worst relative error of the cell's monopole)/5);
  2. training: Adam on the mean-squared error with nb_mlp_loss_grad / nb_mlp_adam;
  3. evaluation: force errors of a traversal against FP64 naive accelerations of sampled bodies
     (nb_naive_accel_targets), and a sweep of the acceptance threshold (or of theta for the
     group rule) to compare both at matched error.
"""

from __future__ import annotations

import math
import time

import numpy as np

from . import generators
from .lib import (BUILD_QUANTIZED_KEYS, REC_LEARNED, BHTree, Context, MLP_PARAMS, build_mask_for,
                  mlp_adam, mlp_loss_grad)

EPS2 = 1e-22


def _dev(a, dtype=None):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda", dtype=dtype)


def reference_accelerations(ctx: Context, t: dict, G: float):
    """FP32-compensated naive accelerations (|a| reference for labels and the first step)."""
    import torch
    n = t["m"].numel()
    a = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *a, G, EPS2, "f32c")
    return a


def make_pairs(ctx: Context, d: dict, max_pairs: int, theta_gen: float = 0.3, seed: int = 0,
               count_cap: int = 8192):
    """Labelled (features, labels) pairs of one system on the device."""
    t = {k: _dev(d[k]) for k in ("m", "x", "y", "z")}
    n = t["m"].numel()
    a = reference_accelerations(ctx, t, d["G"])
    tree = BHTree(ctx, n, theta=0.5)
    tree.build(t["m"], t["x"], t["y"], t["z"], d["G"])
    # count candidates with a tiny buffer, then sample the wanted number
    _, _, _, found = tree.generate_pairs(t["m"], t["x"], t["y"], t["z"], *a, d["G"], EPS2,
                                         theta_gen, 1.0, seed, count_cap, 1)
    frac = min(1.0, max_pairs / max(found, 1))
    X, Y, _, _ = tree.generate_pairs(t["m"], t["x"], t["y"], t["z"], *a, d["G"], EPS2, theta_gen,
                                     frac, seed, count_cap, max_pairs)
    ctx.sync()
    tree.close()
    return X.clone(), Y.clone(), found


def init_params(seed: int = 0):
    rng = np.random.default_rng(seed)
    p = []
    for fan_in, fan_out in ((8, 32), (32, 32)):
        lim = math.sqrt(6.0 / (fan_in + fan_out))
        p.append(rng.uniform(-lim, lim, size=(fan_in, fan_out)).ravel())
        p.append(np.zeros(fan_out))
    lim = math.sqrt(6.0 / 33)
    p.append(rng.uniform(-lim, lim, size=32))
    p.append(np.array([-1.0]))
    return np.concatenate(p).astype(np.float32)


def train(ctx: Context, X, Y, epochs: int = 4, batch: int = 8192, lr: float = 2e-3, seed: int = 0,
          log=None):
    """Adam on the device; returns (params [1377] float32 cuda tensor, per-epoch mean losses)."""
    import torch
    n = X.shape[0]
    params = _dev(init_params(seed))
    m = torch.zeros(MLP_PARAMS, dtype=torch.float32, device="cuda")
    v = torch.zeros_like(m)
    grad = torch.zeros_like(m)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    step = 0
    history = []
    for ep in range(epochs):
        perm = torch.randperm(n, device="cuda", generator=gen).to(torch.int32)
        tot = torch.zeros(1, dtype=torch.float32, device="cuda")
        nb = 0
        for b0 in range(0, n, batch):
            idx = perm[b0:b0 + batch]
            mlp_loss_grad(ctx, params, X, Y, idx, idx.numel(), grad, loss)
            step += 1
            lr_t = lr * (0.5 * (1 + math.cos(math.pi * step / (epochs * math.ceil(n / batch)))))
            mlp_adam(ctx, params, m, v, grad, max(lr_t, lr * 0.02), 0.9, 0.999, 1e-8, step)
            tot += loss
            nb += 1
        history.append(float(tot.item()) / nb)
        if log:
            log(f"epoch {ep}: mse {history[-1]:.5f}")
    return params, history


def sample_targets(n: int, k: int, seed: int = 7):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(n, size=min(k, n), replace=False)).astype(np.uint32)


def fp64_reference(ctx: Context, t: dict, G: float, targets):
    import torch
    tg = _dev(targets.view(np.int32))
    k = len(targets)
    a = [torch.zeros(k, dtype=torch.float64, device="cuda") for _ in range(3)]
    ctx.naive_accel_targets(t["m"], t["x"], t["y"], t["z"], tg, *a, G, EPS2)
    ctx.sync()
    return [v.cpu().numpy() for v in a]


def errors(acc, ref, targets):
    ax, ay, az = (a.cpu().numpy()[targets] for a in acc)
    rx, ry, rz = ref
    num = np.sqrt((ax - rx) ** 2 + (ay - ry) ** 2 + (az - rz) ** 2)
    e = num / np.sqrt(rx * rx + ry * ry + rz * rz)
    return float(np.median(e)), float(np.percentile(e, 99))


def timed(fn, reps=3):
    import torch
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


NO_CAP = 2 ** 31 - 1  # count cap that keeps every cell in the network's range


def device_system(d: dict):
    return {k: _dev(d[k]) for k in ("m", "x", "y", "z", "vx", "vy", "vz")}


def training_set(ctx: Context, n: int, n_pairs: int, seeds=(11, 12), theta_gen: float = 0.3,
                 count_cap: int = NO_CAP, log=None):
    """Labelled pairs from seeded disc + Plummer mixes of n bodies, n_pairs in total."""
    import torch
    Xs, Ys = [], []
    for s in seeds:
        d = generators.disc_plummer_mix(n, seed=s)
        X, Y, found = make_pairs(ctx, d, n_pairs // len(seeds), theta_gen=theta_gen, seed=s,
                                 count_cap=count_cap)
        Xs.append(X)
        Ys.append(Y)
        if log:
            log(f"seed {s}: {found} candidate pairs, kept {X.shape[0]}")
    return torch.cat(Xs), torch.cat(Ys)


def sweep(ctx: Context, t: dict, G: float, targets, ref, params, taus, thetas,
          theta_fallback: float = 0.3, count_cap: int = NO_CAP, eps2: float = EPS2,
          net_only_taus=()):
    """Force error (median, p99 over the targets) and time of one traversal for each threshold
    (learned policy: analytic-bound acceptance, then the network), each theta (the same walk with
    the group theta rule instead: the method without the network) and each of net_only_taus (the
    network alone, no bound acceptance). Rows: dict(kind, param, ms, median, p99, interactions,
    cells, decisions)."""
    import torch
    n = t["m"].numel()
    tree = BHTree(ctx, n, theta=0.5)
    tree.set_records(REC_LEARNED | BUILD_QUANTIZED_KEYS)  # the timed learned steps' build
    tree.build(t["m"], t["x"], t["y"], t["z"], G)
    prev = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    tree.accel(t["x"], t["y"], t["z"], *prev, G, eps2, "group", "f32c")  # |a| of a previous step
    acc = [torch.zeros_like(v) for v in prev]
    rows = []
    cases = ([("theta-walk", th) for th in thetas] + [("learned", lt) for lt in taus]
             + [("learned-net-only", lt) for lt in net_only_taus])
    for kind, q in cases:
        if kind == "theta-walk":
            tree.set_policy(None, 0.0, q, count_cap)
        else:
            tree.set_policy(params, q, theta_fallback, count_cap, bound_accept=(kind == "learned"))

        def run():
            for a_, b_ in zip(acc, prev):
                a_.copy_(b_)
            tree.accel(t["x"], t["y"], t["z"], *acc, G, eps2, "learned", "f32c")

        ms_copy = timed(lambda: [a_.copy_(b_) for a_, b_ in zip(acc, prev)])
        ms = timed(run) - ms_copy
        med, p99 = errors(acc, ref, targets)  # acc holds the last run's result
        for a_, b_ in zip(acc, prev):
            a_.copy_(b_)
        inter, dec, cells, _ = tree.accel_learned_counted(t["x"], t["y"], t["z"], *acc, eps2)
        rows.append({"kind": kind, "param": q, "ms": ms, "median": med, "p99": p99,
                     "interactions": inter, "cells": cells, "decisions": dec})
    tree.close()
    return rows


def best_within(rows, kind, median_max=1e-4, p99_max=1e-3, key="ms"):
    """The row of a kind with the smallest `key` (time, or "interactions") whose error is within
    both bounds (None if there is none)."""
    ok = [r for r in rows if r["kind"] == kind and r["median"] <= median_max and r["p99"] <= p99_max]
    return min(ok, key=lambda r: r[key]) if ok else None


def time_steps(ctx: Context, t: dict, G: float, steps: int, opening: str, precision: str,
               theta: float = 0.5, policy=None, dt: float = 1.0 / 24, eps2: float = EPS2,
               warmup: int = 3):
    """ms per leapfrog step (kick + drift, octree build, traversal, kick) of a state copy.
    policy = (params or None, log10_tau, theta_fallback, count_cap) for opening "learned"."""
    import torch
    n = t["m"].numel()
    pos = [t[k].clone() for k in ("x", "y", "z")]
    vel = [t[k].clone() for k in ("vx", "vy", "vz")]
    acc = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    vh = [torch.zeros_like(a) for a in acc]
    tree = BHTree(ctx, n, theta=theta)
    tree.set_records(build_mask_for(opening, precision))  # only what the traversal reads
    tree.build(t["m"], *pos, G)
    tree.accel(*pos, *acc, G, eps2, "group", "f32c")  # step 0 accelerations
    if policy is not None:
        tree.set_policy(*policy)

    def step():
        ctx.kick_drift(vh, vel, pos, acc, dt)
        tree.build(t["m"], *pos, G)
        tree.accel(*pos, *acc, G, eps2, opening, precision)
        ctx.kick(vel, vh, acc, dt)

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    ctx.sync()
    tree.close()
    return e0.elapsed_time(e1) / steps


def error_over_steps(ctx: Context, t: dict, G: float, steps: int, checkpoints, targets,
                     opening: str, precision: str, theta: float = 0.5, policy=None,
                     dt: float = 1.0 / 24, eps2: float = EPS2):
    """Leapfrog run of a state copy (kick + drift, octree build, traversal, kick per step) with
    the force error of the step's traversal measured at the given step numbers (0 = the initial
    evaluation): median and p99 relative error of the sampled targets against FP64 naive sums at
    that step's positions. Returns [{step, median, p99}]."""
    import torch
    n = t["m"].numel()
    pos = [t[k].clone() for k in ("x", "y", "z")]
    vel = [t[k].clone() for k in ("vx", "vy", "vz")]
    acc = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    vh = [torch.zeros_like(a) for a in acc]
    tree = BHTree(ctx, n, theta=theta)
    tree.set_records(build_mask_for(opening, precision))
    tree.build(t["m"], *pos, G)
    tree.accel(*pos, *acc, G, eps2, "group", "f32c")  # a first |a| for the learned policy
    if policy is not None:
        tree.set_policy(*policy)
    tree.accel(*pos, *acc, G, eps2, opening, precision)
    out = []
    cur = {"m": t["m"], "x": pos[0], "y": pos[1], "z": pos[2]}

    def measure(step):
        ref = fp64_reference(ctx, cur, G, targets)
        med, p99 = errors(acc, ref, targets)
        out.append({"step": step, "median": med, "p99": p99})

    marks = set(checkpoints)
    if 0 in marks:
        measure(0)
    for k in range(1, steps + 1):
        ctx.kick_drift(vh, vel, pos, acc, dt)
        tree.build(t["m"], *pos, G)
        tree.accel(*pos, *acc, G, eps2, opening, precision)
        ctx.kick(vel, vh, acc, dt)
        if k in marks:
            measure(k)
    ctx.sync()
    tree.close()
    return out

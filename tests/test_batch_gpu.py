"""Batched ensembles (nb_batch_*): independent systems of uneven size in one persistent launch,
every tile configuration, the autotuner and CUDA-graph replay. Tolerances as the naive FP32C
tests: per-body relative error vs the FP64 oracle median <= 1e-5, max <= 1e-3."""

import numpy as np
import pytest

import oracle
from helpers import dev, host, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from nbody.lib import Context
    c = Context(0)
    yield c
    c.close()


def ensemble(counts, seed=0):
    from nbody import generators
    parts = []
    for s, n in enumerate(counts):
        if n == 0:
            continue
        d = generators.plummer(n, seed=seed + s) if n >= 4 else {
            k: np.random.default_rng(s).normal(size=n) for k in ("x", "y", "z", "vx", "vy", "vz")}
        if n < 4:
            d["m"] = np.full(n, 1.0 / n)
        shift = 10.0 * s  # systems far apart: any cross-talk would show
        d["x"] = d["x"] + shift
        parts.append(d)
    cat = {k: np.concatenate([p[k] for p in parts]) for k in ("m", "x", "y", "z", "vx", "vy", "vz")}
    return cat


def run_batch(ctx, b, cat, eps2=1e-6):
    import torch
    t = {k: dev(cat[k]) for k in ("m", "x", "y", "z")}
    n = len(cat["m"])
    a = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    b.accel(t["m"], t["x"], t["y"], t["z"], *a, 1.0, eps2)
    ctx.sync()
    return [host(v) for v in a]


COUNTS = [1, 2, 3, 0, 300, 1023, 1024, 1025, 2500, 7000, 5]


@pytest.mark.parametrize("config", [0, 8])
def test_batch_matches_oracle_per_system(ctx, config):
    """Configuration 0: the one-sided kernel; 8: the symmetric kernel's default shape."""
    from nbody.lib import Batch
    cat = ensemble(COUNTS)
    b = Batch(ctx, COUNTS)
    assert b.info()["n_total"] == sum(COUNTS)
    b.set_config(config)
    got = run_batch(ctx, b, cat)
    off = 0
    for n in COUNTS:
        if n == 0:
            continue
        sl = slice(off, off + n)
        ref = oracle.naive_accel(cat["m"][sl], cat["x"][sl], cat["y"][sl], cat["z"][sl], 1.0, 1e-6)
        if n >= 3:
            err = rel_err(*[g[sl] for g in got], *ref)
            assert np.median(err) <= 1e-5 and err.max() <= 1e-3, (n, np.median(err), err.max())
        elif n == 1:
            assert all(np.all(g[sl] == 0) for g in got)
        off += n


@pytest.mark.parametrize("config", range(16))
def test_every_configuration(ctx, config):
    """Every shape of both kernels (0-7 one-sided, 8-15 symmetric) against configuration 0, and
    the single-system entry point with the same shape against the oracle."""
    from nbody.lib import (PAIR_CONFIGS, SYM_ALWAYS, SYM_AUTO, Batch, set_naive_pair_config,
                           set_naive_symmetric)
    cat = ensemble(COUNTS, seed=3)
    b = Batch(ctx, COUNTS)
    b.set_config(config)
    assert b.info()["config"] == config
    got = run_batch(ctx, b, cat)
    b.set_config(0)
    base = run_batch(ctx, b, cat)
    e = rel_err(*got, *base)
    e = e[np.isfinite(e)]
    assert np.median(e) <= 1e-6 and e.max() <= 1e-3, (np.median(e), e.max())
    # the single-system entry point with the same configuration
    import torch
    from nbody import generators
    d = generators.plummer(5000, seed=9)
    t = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    a = [torch.zeros(5000, dtype=torch.float64, device="cuda") for _ in range(3)]
    try:
        if config < PAIR_CONFIGS:
            set_naive_pair_config(config)
        else:
            set_naive_symmetric(SYM_ALWAYS, config - PAIR_CONFIGS)
        ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *a, 1.0, 1e-6, "f32c")
        ctx.sync()
    finally:
        set_naive_pair_config(0)
        set_naive_symmetric(SYM_AUTO, 0)
    err = rel_err(*[host(v) for v in a], *oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], 1.0, 1e-6))
    assert np.median(err) <= 1e-5 and err.max() <= 1e-3


def test_autotune_picks_a_configuration(ctx):
    import torch
    from nbody.lib import Batch
    counts = [4096, 300, 9000, 64]
    cat = ensemble(counts, seed=5)
    b = Batch(ctx, counts)
    t = {k: dev(cat[k]) for k in ("m", "x", "y", "z")}
    a = [torch.zeros(len(cat["m"]), dtype=torch.float64, device="cuda") for _ in range(3)]
    chosen, ms = b.autotune(t["m"], t["x"], t["y"], t["z"], *a, 1.0, 1e-6, reps=2)
    assert 0 <= chosen < 16 and len(ms) == 16 and all(v > 0 for v in ms)
    assert ms[chosen] == min(ms)
    assert b.info()["config"] == chosen


@pytest.mark.parametrize("config", [0, 8])
def test_graph_replay_equals_stepwise_calls(ctx, config):
    import torch
    from nbody.lib import Batch
    counts = [500, 1200, 77, 3000]
    cat = ensemble(counts, seed=11)
    n = len(cat["m"])
    b = Batch(ctx, counts)
    b.set_config(config)

    def state():
        s = {k: dev(cat[k]) for k in ("m", "x", "y", "z", "vx", "vy", "vz")}
        s["acc"] = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
        s["vh"] = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
        return s

    dt, steps = 1e-3, 4
    A, B = state(), state()
    for s in (A, B):
        b.accel(s["m"], s["x"], s["y"], s["z"], *s["acc"], 1.0, 1e-6)
    for _ in range(steps):  # stepwise
        pos, vel = [A["x"], A["y"], A["z"]], [A["vx"], A["vy"], A["vz"]]
        ctx.kick_drift(A["vh"], vel, pos, A["acc"], dt)
        b.accel(A["m"], *pos, *A["acc"], 1.0, 1e-6)
        ctx.kick(vel, A["vh"], A["acc"], dt)
    g = b.graph(B["m"], [B["x"], B["y"], B["z"]], [B["vx"], B["vy"], B["vz"]], B["vh"], B["acc"],
                1.0, 1e-6, dt, steps)
    g.launch()
    ctx.sync()
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        np.testing.assert_array_equal(host(A[k]), host(B[k]))

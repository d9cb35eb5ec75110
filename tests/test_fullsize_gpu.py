"""Parity at the configurations' full sizes, through sampled bodies and size-independent checks.

* 1,048,576-body heliocentric disc, Barnes-Hut theta = 0.5 (the headline configuration): the
  reference-rule traversal in NB_F64_IEEE is bit-identical to the oracle's traversal
  (BarnesHutAlgorithm.cpp:319-393 over the oracle's ParallelOctreeTopDownSubtrees build) on 4,096
  sampled bodies; NB_F64 is within 1e-12 of it for every body; against FP64 naive sums of the
  sampled bodies the theta = 0.5 approximation error stays at median <= 1e-4, p99 <= 1e-2 (the
  method's error, the same for the reference).
* 262,144-body Plummer sphere, naive FP32C (symmetric kernel): sampled bodies against FP64 sums,
  median <= 1e-5, max <= 1e-3.
* 512 Plummer spheres of 256..16,384 bodies in one batch (autotuned): eight systems against the
  oracle's naive sums, median <= 1e-5, max <= 1e-3 per system.
"""

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


def _targets_fp64(ctx, t, targets, G, eps2):
    import torch
    tg = torch.as_tensor(targets.astype(np.uint32).view(np.int32), device="cuda")
    ref = [torch.zeros(len(targets), dtype=torch.float64, device="cuda") for _ in range(3)]
    ctx.naive_accel_targets(t["m"], t["x"], t["y"], t["z"], tg, *ref, G, eps2)
    ctx.sync()
    return [host(v) for v in ref]


def test_barnes_hut_1m_disc(ctx):
    import torch
    from nbody import generators
    from nbody.lib import BHTree
    n = 1 << 20
    d = generators.heliocentric_disc(n, 1)
    G, eps2, theta = d["G"], 1e-22, 0.5
    t = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    tree = BHTree(ctx, n, theta=theta)
    tree.build(t["m"], t["x"], t["y"], t["z"], G)
    acc = {}
    for prec in ("f64_ieee", "f64"):
        a = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
        tree.accel(t["x"], t["y"], t["z"], *a, G, eps2, "theta", prec)
        ctx.sync()
        acc[prec] = [host(v) for v in a]
    tree.close()
    targets = np.sort(np.random.default_rng(5).choice(n, 4096, replace=False))
    otree = oracle.build_subtrees(d["m"], d["x"], d["y"], d["z"])
    ref = oracle.bh_accel_subset(otree, d["x"], d["y"], d["z"], targets, G, eps2, theta)
    for g, r in zip(acc["f64_ieee"], ref):
        np.testing.assert_array_equal(g[targets], r)
    assert rel_err(*acc["f64"], *acc["f64_ieee"]).max() <= 1e-12
    exact = _targets_fp64(ctx, t, targets, G, eps2)
    err = rel_err(*(v[targets] for v in acc["f64"]), *exact)
    assert np.median(err) <= 1e-4 and np.percentile(err, 99) <= 1e-2, (np.median(err),
                                                                       np.percentile(err, 99))


def test_naive_f32c_262k_plummer(ctx):
    import torch
    from nbody import generators
    n = 262144
    d = generators.plummer(n, 1)
    t = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    a = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *a, 1.0, 1e-6, "f32c")
    ctx.sync()
    got = [host(v) for v in a]
    targets = np.sort(np.random.default_rng(6).choice(n, 4096, replace=False))
    exact = _targets_fp64(ctx, t, targets, 1.0, 1e-6)
    err = rel_err(*(v[targets] for v in got), *exact)
    assert np.median(err) <= 1e-5 and err.max() <= 1e-3, (np.median(err), err.max())


def test_ensemble_512_systems(ctx):
    import math

    import torch
    from nbody import generators
    from nbody.lib import Batch
    rng = np.random.default_rng(3)
    counts = np.exp(rng.uniform(math.log(256), math.log(16384), 512)).astype(np.int64)
    parts = [generators.plummer(int(c), seed=300009 + s) for s, c in enumerate(counts)]
    cat = {k: np.concatenate([p[k] for p in parts]) for k in ("m", "x", "y", "z")}
    n = len(cat["m"])
    t = {k: dev(cat[k]) for k in ("m", "x", "y", "z")}
    a = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    b = Batch(ctx, counts)
    b.autotune(t["m"], t["x"], t["y"], t["z"], *a, 1.0, 1e-6, reps=1)
    b.accel(t["m"], t["x"], t["y"], t["z"], *a, 1.0, 1e-6)
    ctx.sync()
    got = [host(v) for v in a]
    b.close()
    off = np.concatenate([[0], np.cumsum(counts)])
    check = sorted({int(np.argmax(counts)), int(np.argmin(counts))}
                   | set(rng.choice(512, 6, replace=False).tolist()))
    for s in check:
        sl = slice(off[s], off[s + 1])
        ref = oracle.naive_accel(cat["m"][sl], cat["x"][sl], cat["y"][sl], cat["z"][sl], 1.0, 1e-6)
        err = rel_err(*(g[sl] for g in got), *ref)
        assert np.median(err) <= 1e-5 and err.max() <= 1e-3, (s, np.median(err), err.max())

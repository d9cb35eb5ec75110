"""Failure detection on the GPU without a GPU fault: the bounded device-side waits and the learned
traversal's stack check, driven to their limits through the context's test hooks
(nb_ctx_set_fault_hooks), report their status to the host, and the context keeps working.

* Pair kernels (one-sided, symmetric, batched): a tile wait limit of 0 makes every CTA give up at
  its first j-tile; each CTA still drains its own bulk copies before it leaves. nb_sync returns
  NB_ERR_TIMEOUT, and the next evaluation on the same context (hooks reset) matches the oracle.
* Radix look-back: the first tile's published count is withheld (a message the test drops), so
  the tiles after it wait for a word nothing writes until their short limit runs out.
* Learned traversal: a stack capacity of 8 cells cannot hold the root's children plus one step
  of pushes; the walk stops and sets the stack bit (NB_ERR_STACK_OVERFLOW).

The reference leaves these unchecked: its spin loops (BarnesHutOctree.cpp:263-384) wait without
bound and its traversal stack (BarnesHutAlgorithm.cpp:340-388) has no overflow check.
"""

import numpy as np
import pytest

import oracle
from helpers import bodies, dev, host, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture()
def ctx():
    from nbody.lib import Context
    c = Context(0)
    yield c
    c.close()


def _naive(ctx, d, prec="f32c"):
    import torch
    n = len(d["m"])
    t = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    a = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *a, d["G"], 1e-6, prec)
    return a


@pytest.mark.parametrize("symmetric", [False, True])
def test_pair_tile_wait_timeout_is_reported_and_the_context_recovers(ctx, symmetric):
    from nbody.lib import SYM_ALWAYS, SYM_AUTO, SYM_NEVER, NBodyError, set_naive_symmetric
    d = bodies("plummer", 20000, seed=5)
    set_naive_symmetric(SYM_ALWAYS if symmetric else SYM_NEVER)
    try:
        ctx.set_fault_hooks(wait_limit=0)
        _naive(ctx, d)
        with pytest.raises(NBodyError, match="TIMEOUT"):
            ctx.sync()
        ctx.set_fault_hooks()  # default limit
        a = _naive(ctx, d)
        ctx.sync()
    finally:
        set_naive_symmetric(SYM_AUTO)
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], d["G"], 1e-6)
    assert np.median(rel_err(*[host(v) for v in a], *ref)) <= 1e-5


def test_batch_tile_wait_timeout_then_recovery(ctx):
    import torch
    from nbody.lib import Batch, NBodyError
    counts = np.array([300, 5000, 1200], dtype=np.int64)
    parts = [bodies("plummer", int(c), seed=20 + s) for s, c in enumerate(counts)]
    cat = {k: np.concatenate([p[k] for p in parts]) for k in ("m", "x", "y", "z")}
    t = {k: dev(cat[k]) for k in cat}
    n = int(counts.sum())
    a = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    b = Batch(ctx, counts)
    for cfg in (0, 8):  # a one-sided and a symmetric tile configuration
        b.set_config(cfg)
        ctx.set_fault_hooks(wait_limit=0)
        b.accel(t["m"], t["x"], t["y"], t["z"], *a, 1.0, 1e-6)
        with pytest.raises(NBodyError, match="TIMEOUT"):
            ctx.sync()
        ctx.set_fault_hooks()
        b.accel(t["m"], t["x"], t["y"], t["z"], *a, 1.0, 1e-6)
        ctx.sync()
        got = [host(v) for v in a]
        off = 0
        for p, c in zip(parts, counts):
            ref = oracle.naive_accel(p["m"], p["x"], p["y"], p["z"], 1.0, 1e-6)
            e = rel_err(*[g[off:off + c] for g in got], *ref)
            assert np.median(e) <= 1e-5, (cfg, np.median(e))
            off += c
    b.close()


def test_radix_lookback_timeout_is_reported_and_the_sort_recovers(ctx):
    import torch
    from nbody.lib import FAULT_DROP_LOOKBACK, NBodyError, util_radix_sort_pairs
    n = 100000
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 1 << 62, size=n, dtype=np.uint64)
    vals = np.arange(n, dtype=np.uint32)

    def sort():
        tk = torch.as_tensor(keys.view(np.int64), device="cuda")
        tv = torch.as_tensor(vals.view(np.int32), device="cuda")
        util_radix_sort_pairs(ctx, tk, tv, 0, 64)
        return tk, tv

    ctx.set_fault_hooks(wait_limit=1000, flags=FAULT_DROP_LOOKBACK)
    sort()
    with pytest.raises(NBodyError, match="TIMEOUT"):
        ctx.sync()
    ctx.set_fault_hooks()
    tk, tv = sort()
    ctx.sync()
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(tk.cpu().numpy().view(np.uint64), keys[order])
    np.testing.assert_array_equal(tv.cpu().numpy().view(np.uint32), vals[order])


def test_learned_stack_overflow_is_reported_and_the_walk_recovers(ctx):
    import torch
    from nbody.lib import REC_LEARNED, BHTree, NBodyError
    d = bodies("disc", 6000, seed=10)
    t = BHTree(ctx, len(d["m"]), theta=0.5)
    t.set_records(REC_LEARNED)
    dd = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    t.build(dd["m"], dd["x"], dd["y"], dd["z"], d["G"])
    t.set_policy(None, 0.0, 0.4, 2 ** 31 - 1)  # the learned walk with the group theta rule
    n = len(d["m"])
    a = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    ctx.set_fault_hooks(learned_stack_cap=8)
    t.accel(dd["x"], dd["y"], dd["z"], *a, d["G"], 1e-22, "learned", "f32c")
    with pytest.raises(NBodyError, match="STACK"):
        ctx.sync()
    with pytest.raises(NBodyError, match="INVALID_ARG"):
        ctx.set_fault_hooks(learned_stack_cap=1025)
    ctx.set_fault_hooks()
    t.accel(dd["x"], dd["y"], dd["z"], *a, d["G"], 1e-22, "learned", "f32c")
    ctx.sync()
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], d["G"], 1e-22)
    assert np.median(rel_err(*[host(v) for v in a], *ref)) <= 1e-3
    t.close()


def test_a_fresh_context_after_a_timeout_works():
    from nbody.lib import Context, NBodyError
    d = bodies("plummer", 5000, seed=8)
    c = Context(0)
    c.set_fault_hooks(wait_limit=0)
    _naive(c, d)
    with pytest.raises(NBodyError, match="TIMEOUT"):
        c.sync()
    c.close()
    c2 = Context(0)
    a = _naive(c2, d, "f64")
    c2.sync()
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], d["G"], 1e-6)
    assert np.median(rel_err(*[host(v) for v in a], *ref)) <= 1e-12
    c2.close()

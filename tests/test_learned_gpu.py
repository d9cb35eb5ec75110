"""Learned opening policy: the training kernels' gradients and Adam step against the CPU oracle
(oracle/mlp.py, float64), the BF16 tensor-core inference against the FP32 forward pass, and the
label generator against a CPU direct sum over the cell's bodies."""

import numpy as np
import pytest

import oracle.mlp as omlp
from helpers import dev

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from nbody.lib import Context
    c = Context(0)
    yield c
    c.close()


def _rand(seed, n):
    rng = np.random.default_rng(seed)
    p = (rng.normal(size=omlp.COUNT) * 0.2).astype(np.float32)
    X = rng.normal(size=(n, 8)).astype(np.float32)
    Y = rng.normal(size=n).astype(np.float32)
    return p, X, Y


@pytest.mark.parametrize("n,use_idx", [(1000, False), (777, True), (64, False)])
def test_mlp_gradient_matches_cpu_oracle(ctx, n, use_idx):
    import torch
    from nbody.lib import mlp_loss_grad
    p, X, Y = _rand(n, n + 50)
    rows = np.random.default_rng(3).permutation(n + 50)[:n].astype(np.int32) if use_idx else None
    grad = torch.zeros(omlp.COUNT, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    tp, tX, tY = (torch.as_tensor(a, device="cuda") for a in (p, X, Y))
    tidx = torch.as_tensor(rows, device="cuda") if use_idx else None
    mlp_loss_grad(ctx, tp, tX, tY, tidx, n, grad, loss)
    ctx.sync()
    sel = rows if use_idx else np.arange(n)
    l_ref, g_ref = omlp.loss_grad(p.astype(np.float64), X[sel], Y[sel])
    assert loss.item() == pytest.approx(l_ref, rel=1e-4)
    g = grad.cpu().numpy().astype(np.float64)
    scale = np.abs(g_ref).max()
    assert np.max(np.abs(g - g_ref)) <= 1e-4 * scale, np.max(np.abs(g - g_ref)) / scale


def test_adam_matches_cpu_oracle(ctx):
    import torch
    from nbody.lib import mlp_adam
    rng = np.random.default_rng(5)
    p = rng.normal(size=omlp.COUNT).astype(np.float32)
    m = (rng.normal(size=omlp.COUNT) * 0.01).astype(np.float32)
    v = (rng.uniform(size=omlp.COUNT) * 0.01).astype(np.float32)
    g = rng.normal(size=omlp.COUNT).astype(np.float32)
    tp, tm, tv, tg = (torch.as_tensor(a.copy(), device="cuda") for a in (p, m, v, g))
    mlp_adam(ctx, tp, tm, tv, tg, 1e-3, 0.9, 0.999, 1e-8, 7)
    ctx.sync()
    f32 = lambda v: float(np.float32(v))  # the kernel's hyperparameters are FP32
    p2, m2, v2 = omlp.adam_step(p.astype(np.float64), m.astype(np.float64), v.astype(np.float64),
                                g.astype(np.float64), f32(1e-3), f32(0.9), f32(0.999), f32(1e-8), 7)
    np.testing.assert_allclose(tp.cpu().numpy(), p2, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(tm.cpu().numpy(), m2, rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(tv.cpu().numpy(), v2, rtol=1e-5, atol=1e-9)


def test_bf16_tensor_core_inference_matches_fp32(ctx):
    import torch
    from nbody.lib import mlp_predict
    p, X, _ = _rand(11, 5003)
    tp, tX = torch.as_tensor(p, device="cuda"), torch.as_tensor(X, device="cuda")
    o32 = torch.zeros(len(X), dtype=torch.float32, device="cuda")
    o16 = torch.zeros_like(o32)
    mlp_predict(ctx, tp, tX, o32, bf16=False)
    mlp_predict(ctx, tp, tX, o16, bf16=True)
    ctx.sync()
    ref, _ = omlp.forward(p.astype(np.float64), X.astype(np.float64))
    np.testing.assert_allclose(o32.cpu().numpy(), ref, rtol=1e-4, atol=1e-4)
    err = np.abs(o16.cpu().numpy() - ref)
    # BF16 inputs/weights/activations (8-bit mantissa) with FP32 accumulation
    assert np.median(err) <= 0.02 * np.median(np.abs(ref)) + 1e-3 and err.max() <= 0.15


def test_labels_match_cpu_direct_sum(ctx):
    import torch
    from nbody import generators
    from nbody.lib import BHTree
    d = generators.disc_plummer_mix(8192, seed=4)
    t = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    n = len(d["m"])
    a = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *a, d["G"], 1e-22, "f64")
    tree = BHTree(ctx, n, theta=0.5)
    tree.build(t["m"], t["x"], t["y"], t["z"], d["G"])
    X, Y, ids, found = tree.generate_pairs(t["m"], t["x"], t["y"], t["z"], *a, d["G"], 1e-22, 0.3,
                                           0.05, 1, 8192, 4000, with_ids=True)
    assert found > 0 and X.shape[0] == min(found, 4000)
    order, _ = tree.export_order(n)
    nodes = tree.export_node_ranges()
    aa = np.sqrt(sum(v.cpu().numpy() ** 2 for v in a))
    Yh, ids = Y.cpu().numpy(), ids.cpu().numpy()
    G = d["G"]
    checked = 0
    for q in range(0, len(Yh), max(1, len(Yh) // 40)):
        g, k = int(ids[q, 0]), int(ids[q, 1])
        grp = order[g * 32: min(n, g * 32 + 32)]
        cell = order[nodes["first"][k]: nodes["first"][k] + nodes["count"][k]]
        M = d["m"][cell].sum()
        com = np.array([np.dot(d["m"][cell], d[c][cell]) / M for c in ("x", "y", "z")])
        worst = 0.0
        for b in grp:
            p = np.array([d["x"][b], d["y"][b], d["z"][b]])
            r = np.stack([d[c][cell] for c in ("x", "y", "z")], axis=1) - p
            exact = G * (d["m"][cell][:, None] * r / ((r * r).sum(1) + 1e-22)[:, None] ** 1.5).sum(0)
            rm = com - p
            mono = G * M * rm / ((rm @ rm) + 1e-22) ** 1.5
            worst = max(worst, np.linalg.norm(exact - mono) / aa[b])
        ref = np.clip(np.log10(max(worst, 1e-30)), -12, 2) / 5
        if ref > -9 / 5:  # below ~1e-9 the FP32 label reaches its rounding floor
            assert abs(Yh[q] - ref) <= 0.05, (q, Yh[q] * 5, ref * 5)
            checked += 1
    assert checked >= 10


def test_trained_policy_gain_over_theta_walk(ctx):
    """What the trained network gains: on a held-out disc + Plummer mix, the learned policy's
    cheapest setting within 1e-4 median / 1e-3 p99 relative force error (against FP64 naive sums
    of sampled bodies) needs fewer body-cell interactions than the same walk with the group theta
    rule at its cheapest setting within the same bounds."""
    from nbody import generators, learned
    n = 65536
    X, Y = learned.training_set(ctx, n, 400_000, seeds=(31, 32))
    params, hist = learned.train(ctx, X, Y, epochs=3, batch=8192, lr=2e-3)
    assert hist[-1] < hist[0]
    d = generators.disc_plummer_mix(n, seed=41)
    t = learned.device_system(d)
    targets = learned.sample_targets(n, 4096)
    ref = learned.fp64_reference(ctx, t, d["G"], targets)
    rows = learned.sweep(ctx, t, d["G"], targets, ref, params,
                         taus=(-5.0, -4.75, -4.5, -4.25, -4.0, -3.75, -3.5),
                         thetas=(0.25, 0.3, 0.35, 0.4, 0.45, 0.5))
    bl = learned.best_within(rows, "learned", key="interactions")
    bt = learned.best_within(rows, "theta-walk", key="interactions")
    assert bl is not None and bt is not None, rows
    print(f"\nlearned tau 1e{bl['param']}: {bl['interactions'] / n:.0f} interactions/body, "
          f"p99 {bl['p99']:.2e}, {bl['ms']:.3f} ms; theta-walk {bt['param']}: "
          f"{bt['interactions'] / n:.0f} interactions/body, p99 {bt['p99']:.2e}, {bt['ms']:.3f} ms")
    assert bl["interactions"] <= 0.8 * bt["interactions"]


def test_trained_policy_holds_on_held_out_seeds(ctx):
    """The gain holds on systems the threshold was not tuned on: tau is chosen once on a
    validation mix (the cheapest setting within 80% of the 1e-4 median / 1e-3 p99 relative force
    error bounds against FP64 naive sums), then on three held-out mixes the learned policy at that fixed tau
    stays within the bounds and needs at most 0.8x the body-cell interactions of the same walk
    with the group theta rule at each system's own cheapest theta within the bounds."""
    from nbody import generators, learned
    n = 65536
    X, Y = learned.training_set(ctx, n, 400_000, seeds=(31, 32))
    params, _ = learned.train(ctx, X, Y, epochs=3, batch=8192, lr=2e-3)
    targets = learned.sample_targets(n, 4096)

    def rows_for(seed, taus, thetas):
        d = generators.disc_plummer_mix(n, seed=seed)
        t = learned.device_system(d)
        ref = learned.fp64_reference(ctx, t, d["G"], targets)
        return learned.sweep(ctx, t, d["G"], targets, ref, params, taus=taus, thetas=thetas)

    val = rows_for(40, (-5.0, -4.75, -4.5, -4.25, -4.0, -3.75), ())
    # a 20% margin below the bounds on the validation system: the held-out systems must then
    # stay within the bounds themselves
    chosen = learned.best_within(val, "learned", median_max=0.8e-4, p99_max=0.8e-3,
                                 key="interactions")
    assert chosen is not None, val
    for seed in (41, 42, 43):
        rows = rows_for(seed, (chosen["param"],), (0.25, 0.3, 0.35, 0.4, 0.45, 0.5))
        lr = [r for r in rows if r["kind"] == "learned"][0]
        bt = learned.best_within(rows, "theta-walk", key="interactions")
        assert bt is not None, rows
        print(f"\nseed {seed}: learned tau 1e{chosen['param']}: {lr['interactions'] / n:.0f} "
              f"interactions/body, median {lr['median']:.1e} p99 {lr['p99']:.2e}, "
              f"{lr['ms']:.3f} ms; theta-walk {bt['param']}: {bt['interactions'] / n:.0f}, "
              f"{bt['ms']:.3f} ms")
        assert lr["median"] <= 1e-4 and lr["p99"] <= 1e-3, lr
        assert lr["interactions"] <= 0.8 * bt["interactions"], (lr, bt)


@pytest.mark.parametrize("n", [65536, 4000])
def test_group_order_does_not_change_the_result(ctx, n):
    """Each learned traversal records a cost per group, and the next one walks the groups
    costliest first: the accelerations stay bit-identical to the first call's (tree order), for
    the network and for the theta rule on the same walk, and after a rebuild with fewer bodies (a
    stale order is not used)."""
    import torch
    from nbody import generators, learned
    from nbody.lib import BHTree, BUILD_QUANTIZED_KEYS, REC_LEARNED
    rng = np.random.default_rng(5)
    p = torch.as_tensor((rng.normal(size=omlp.COUNT) * 0.2).astype(np.float32), device="cuda")
    d = generators.disc_plummer_mix(n, seed=44)
    t = learned.device_system(d)
    tree = BHTree(ctx, n, theta=0.5)
    tree.set_records(REC_LEARNED | BUILD_QUANTIZED_KEYS)
    tree.build(t["m"], t["x"], t["y"], t["z"], d["G"])
    prev = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    tree.accel(t["x"], t["y"], t["z"], *prev, d["G"], learned.EPS2, "group", "f32c")

    def run():
        acc = [v.clone() for v in prev]
        tree.accel(t["x"], t["y"], t["z"], *acc, d["G"], learned.EPS2, "learned", "f32c")
        ctx.sync()
        return [v.cpu().numpy() for v in acc]

    for policy in ((p, -4.0, 0.3, learned.NO_CAP), (None, 0.0, 0.4, learned.NO_CAP)):
        tree.set_policy(*policy)
        first = run()
        for _ in range(2):
            again = run()
            for a, b in zip(first, again):
                np.testing.assert_array_equal(a, b)
    # fewer bodies in the same tree: the order built for the larger system must not be used
    m = n // 2 + 17
    tree.build(t["m"][:m], t["x"][:m], t["y"][:m], t["z"][:m], d["G"])
    small = [v[:m].clone() for v in prev]
    res = []
    for _ in range(2):
        acc = [v.clone() for v in small]
        tree.accel(t["x"][:m], t["y"][:m], t["z"][:m], *acc, d["G"], learned.EPS2, "learned", "f32c")
        ctx.sync()
        res.append([v.cpu().numpy() for v in acc])
        assert all(np.all(np.isfinite(v)) for v in res[-1])
    for a, b in zip(*res):
        np.testing.assert_array_equal(a, b)
    tree.close()

"""Parity of the Barnes-Hut path against the CPU oracle restating the reference
(ParallelOctreeTopDownSubtrees.cpp, BarnesHutOctree.cpp, BarnesHutAlgorithm.cpp:280-401),
through the C ABI.

* radix sort / scan building blocks: exact vs numpy.
* tree: the reference's known answers, and cell-by-cell equality (octants, cell corners, edge,
  FP64 mass and centre-of-mass sums, body counts, in-order body sort) with the oracle's tree.
* accelerations, reference rule: NB_F64_IEEE bit-identical to the oracle's traversal; NB_F64
  within 1e-12 relative per body.
* group rule / FP32: within stated bounds of the naive FP64 oracle.
"""

import numpy as np
import pytest

import oracle
from helpers import bodies, canonical_compare, dev, host, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from nbody.lib import Context
    c = Context(0)
    yield c
    c.close()


def build(ctx, d, **params):
    from nbody.lib import BHTree
    t = BHTree(ctx, len(d["m"]), **params)
    dd = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    t.build(dd["m"], dd["x"], dd["y"], dd["z"], d["G"])
    ctx.sync()
    return t, dd


def accel(ctx, t, dd, G, eps2, opening, precision):
    import torch
    n = dd["x"].numel()
    a = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    t.accel(dd["x"], dd["y"], dd["z"], *a, G, eps2, opening, precision)
    ctx.sync()
    return [host(v) for v in a]


# -- building blocks ----------------------------------------------------------------------------
@pytest.mark.parametrize("n", [1, 2, 2047, 2048, 2049, 100000])
def test_radix_sort_stable(ctx, n):
    import torch
    from nbody.lib import util_radix_sort_pairs
    rng = np.random.default_rng(n)
    keys = rng.integers(0, 1 << 20, size=n, dtype=np.uint64) << np.uint64(40)
    keys |= rng.integers(0, 4, size=n, dtype=np.uint64)  # many duplicates
    vals = np.arange(n, dtype=np.uint32)
    tk = torch.as_tensor(keys.view(np.int64), device="cuda")
    tv = torch.as_tensor(vals.view(np.int32), device="cuda")
    util_radix_sort_pairs(ctx, tk, tv, 0, 63)
    ctx.sync()
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(tk.cpu().numpy().view(np.uint64), keys[order])
    np.testing.assert_array_equal(tv.cpu().numpy().view(np.uint32), vals[order])


@pytest.mark.parametrize("n", [1, 1023, 4096, 4097, 1 << 20])
def test_exclusive_scan(ctx, n):
    import torch
    from nbody.lib import util_exclusive_scan_u32
    rng = np.random.default_rng(n)
    a = rng.integers(0, 9, size=n, dtype=np.uint32)
    tin = torch.as_tensor(a.view(np.int32), device="cuda")
    tout = torch.zeros(n + 1, dtype=torch.int32, device="cuda")
    util_exclusive_scan_u32(ctx, tin, tout)
    ctx.sync()
    ref = np.concatenate([[0], np.cumsum(a, dtype=np.uint64)]).astype(np.uint32)
    np.testing.assert_array_equal(tout.cpu().numpy().view(np.uint32), ref)


# -- tree ---------------------------------------------------------------------------------------
def test_reference_known_answers(ctx, kats):
    t = [t for t in kats["BarnesHutTest.cpp"] if t["name"] == "buildOctreeSubtreesTest"][0]
    v = t["vectors"]
    d = {"m": np.array(v["masses"], float), "x": np.array(v["x_positions"], float),
         "y": np.array(v["y_positions"], float), "z": np.array(v["z_positions"], float), "G": 1.0}
    tree, _ = build(ctx, d, max_build_level=1)
    lay = tree.export_ref_layout(3)
    assert lay["node_count"] == 9
    for e in t["expects"]:
        arr = {"BODY_OF_NODE": "body_of_node", "SUM_MASSES": "sum_masses",
               "SORTED_BODIES": "sorted_bodies"}[e["array"]]
        assert lay[arr][e["index"]] == pytest.approx(e["value"]), e


def _clustered(n, seed):
    """Tight clumps with near-coincident pairs: forces leaves below 21 levels (second key word)."""
    rng = np.random.default_rng(seed)
    c = rng.normal(size=(3, n // 4))
    pts = np.repeat(c, 4, axis=1)
    pts[:, 1::4] += 1e-8 * rng.normal(size=(3, n // 4))
    pts[:, 2::4] += 1e-5 * rng.normal(size=(3, n // 4))
    pts[:, 3::4] += 1e-10 * rng.normal(size=(3, n // 4))
    return {"m": rng.uniform(1, 2, n // 4 * 4), "x": pts[0].copy(), "y": pts[1].copy(),
            "z": pts[2].copy(), "G": 1.0}


def _midpoints(n, seed):
    """Bodies on the FP64 midpoints of the reference's key recurrence (random cells of levels
    0..20 per axis, nudged by -2..2 ulps) mixed with uniform bodies, in a box fixed by two
    corners: the keys kernel must take the recurrence itself for the first kind (their digits
    depend on its rounding) and the fixed-point digits for the second, in the same warps."""
    rng = np.random.default_rng(seed)
    lo, hi = -1.37, 2.11
    box = oracle.aabb(np.array([lo, hi]), np.array([lo, hi]), np.array([lo, hi]))
    e = box["edge"]
    cols = []
    for a in ("x", "y", "z"):
        mn, ce = np.full(n, box["min_" + a]), e
        stop, v = rng.integers(0, 21, size=n), np.zeros(n)
        for level in range(21):
            ce = ce / 2
            mid = mn + ce
            v[stop == level] = mid[stop == level]
            mn = np.where(rng.random(n) < 0.5, mid, mn)
        cols.append(v)
    p = np.unique(np.stack(cols, axis=1), axis=0)  # distinct cells: no near-coincident bodies
    k = rng.integers(-2, 3, size=p.shape)
    for s in (1, 2):
        p[k >= s] = np.nextafter(p[k >= s], np.inf)
        p[k <= -s] = np.nextafter(p[k <= -s], -np.inf)
    p = np.concatenate([p, rng.uniform(lo, hi, size=(n // 3, 3))])
    p = np.clip(rng.permutation(p), lo, hi)
    x, y, z = (np.concatenate([[lo, hi], p[:, a]]) for a in range(3))
    return {"m": rng.uniform(1, 2, len(x)), "x": x, "y": y, "z": z, "G": 1.0}


@pytest.mark.parametrize("case", ["disc-2000", "plummer-5000", "disc-1", "disc-2", "plummer-3",
                                  "clustered-4000", "shifted-3000", "midpoints-3000"])
def test_tree_matches_oracle_cell_by_cell(ctx, case):
    kind, n = case.split("-")
    n = int(n)
    if kind == "clustered":
        d = _clustered(n, 3)
    elif kind == "midpoints":
        d = _midpoints(n, 4)
    elif kind == "shifted":
        d = bodies("plummer", n, seed=9)
        d["x"] = d["x"] + 25.0  # box must still contain the origin (reference convention)
    else:
        d = bodies(kind, n, seed=5)
    # deep clumps need more than the reference's default 16*N node slots (each level of a
    # single-child chain costs 8 slots there)
    storage = 256 if kind in ("clustered", "midpoints") else 16
    ot = oracle.build_subtrees(d["m"], d["x"], d["y"], d["z"], max_level=7, threads=4,
                               storage_param=storage)
    tree, _ = build(ctx, d)
    st = tree.stats()
    assert st["ref_node_count"] == ot.node_count
    assert st["node_count"] <= 2 * len(d["m"]) - 1
    np.testing.assert_array_equal(np.array(st["aabb"]), ot.aabb)
    lay = tree.export_ref_layout(len(d["m"]))
    cells = canonical_compare(ot, lay, len(d["m"]))
    assert cells == ot.node_count
    if kind == "clustered":
        assert st["max_depth"] > 21  # exercised the second key word


@pytest.mark.parametrize("precision", ["f64_ieee", "f64"])
def test_walk_order_from_the_last_walk_lengths_is_bit_identical(ctx, precision):
    """The per-body FP64 traversal groups its bodies by the walk lengths of the tree's previous
    traversal (within windows of 1,024 sorted positions): a repeated call, and a call after the
    bodies moved and the tree was rebuilt, equal a fresh tree's first call (tree order) bit for
    bit, and the first call matches the oracle's traversal."""
    import torch
    from nbody.lib import BHTree
    d = bodies("disc", 5000, seed=8)
    tree, dd = build(ctx, d, theta=0.5)
    a1 = accel(ctx, tree, dd, d["G"], 1e-22, "theta", precision)
    a2 = accel(ctx, tree, dd, d["G"], 1e-22, "theta", precision)
    for u, v in zip(a1, a2):
        np.testing.assert_array_equal(u, v)
    if precision == "f64_ieee":
        ot = oracle.build_subtrees(d["m"], d["x"], d["y"], d["z"], max_level=7, threads=4)
        ref = oracle.bh_accel(ot, d["x"], d["y"], d["z"], d["G"], 1e-22, 0.5, threads=4)
        for u, v in zip(a1, ref):
            np.testing.assert_array_equal(u, v)
    # moved bodies, same tree (history from the previous positions) vs a fresh tree
    rng = np.random.default_rng(3)
    for k in ("x", "y", "z"):
        d[k] = d[k] * (1 + 1e-3 * rng.standard_normal(len(d[k])))
    dd2 = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    tree.build(dd2["m"], dd2["x"], dd2["y"], dd2["z"], d["G"])
    ctx.sync()
    b1 = accel(ctx, tree, dd2, d["G"], 1e-22, "theta", precision)
    fresh, _ = build(ctx, d, theta=0.5)
    b2 = accel(ctx, fresh, dd2, d["G"], 1e-22, "theta", precision)
    for u, v in zip(b1, b2):
        np.testing.assert_array_equal(u, v)
    tree.close()
    fresh.close()


def test_coincident_bodies_report_depth_overflow(ctx):
    from nbody.lib import NBodyError, BHTree
    d = bodies("plummer", 100, seed=1)
    d["x"][7], d["y"][7], d["z"][7] = d["x"][3], d["y"][3], d["z"][3]
    t = BHTree(ctx, 100)
    dd = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    t.build(dd["m"], dd["x"], dd["y"], dd["z"], 1.0)
    with pytest.raises(NBodyError, match="DEPTH"):
        ctx.sync()
    ctx.sync()  # error word cleared; context still usable
    d2 = bodies("plummer", 100, seed=2)
    t.build(*[dev(d2[k]) for k in ("m", "x", "y", "z")], 1.0)
    ctx.sync()


# -- accelerations ------------------------------------------------------------------------------
def _check_df64(got, ref, median_rel=1e-12, typical_rel=1e-11):
    """Per-body error relative to max(|a|, median |a|): a body's own |a| can be a tiny remainder
    of large cancelling terms, where any arithmetic's error is large relative to |a|."""
    e = rel_err(*got, *ref)
    diff = np.sqrt(sum((g - r) ** 2 for g, r in zip(got, ref)))
    mag = np.sqrt(sum(r * r for r in ref))
    scale = np.maximum(mag, np.median(mag))
    assert np.median(e) <= median_rel, np.median(e)
    assert (diff / scale).max() <= typical_rel, (diff / scale).max()


@pytest.mark.parametrize("kind,n,theta", [("disc", 3000, 0.5), ("disc", 3000, 1.05),
                                          ("plummer", 4000, 0.5), ("plummer", 2, 0.5),
                                          ("plummer", 1, 0.5), ("clustered", 2000, 0.7),
                                          ("plummer", 1500, 0.0)])
def test_accel_theta_ieee_bit_identical(ctx, kind, n, theta):
    d = _clustered(n, 4) if kind == "clustered" else bodies(kind, n, seed=8)
    eps2 = 1e-22 if kind == "disc" else 1e-6
    ot = oracle.build_subtrees(d["m"], d["x"], d["y"], d["z"], threads=4,
                               storage_param=256 if kind == "clustered" else 16)
    ref = oracle.bh_accel(ot, d["x"], d["y"], d["z"], d["G"], eps2, theta, threads=4)
    tree, dd = build(ctx, d, theta=theta)
    got = accel(ctx, tree, dd, d["G"], eps2, "theta", "f64_ieee")
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)
    fast = accel(ctx, tree, dd, d["G"], eps2, "theta", "f64")
    if n > 1:
        assert rel_err(*fast, *ref).max() <= 1e-12
    # double-float monopoles on the FP32 pipe: same accepted cells; each pair term carries
    # ~2^-46 relative error (FP64: ~2^-52), so the error is bounded against the typical
    # acceleration, not against a body's own |a| (which can be a tiny remainder of large terms)
    df = accel(ctx, tree, dd, d["G"], eps2, "theta", "df64")
    if n > 1:
        _check_df64(df, ref)


def test_theta_zero_equals_direct_sum(ctx):
    d = bodies("plummer", 700, seed=12)
    tree, dd = build(ctx, d, theta=0.0)
    got = accel(ctx, tree, dd, 1.0, 1e-6, "theta", "f64")
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], 1.0, 1e-6)
    assert rel_err(*got, *ref).max() <= 1e-12
    _check_df64(accel(ctx, tree, dd, 1.0, 1e-6, "theta", "df64"), ref)


def test_df64_matches_f64_on_a_large_disc(ctx):
    """The headline distribution (disc, masses in kg, G in AU^3 kg^-1 d^-2, eps^2 = 1e-22):
    double-float monopoles against the FP64 traversal of the same tree."""
    d = bodies("disc", 100000, seed=23)
    tree, dd = build(ctx, d, theta=0.5)
    a64 = accel(ctx, tree, dd, d["G"], 1e-22, "theta", "f64")
    adf = accel(ctx, tree, dd, d["G"], 1e-22, "theta", "df64")
    _check_df64(adf, a64)
    # another G than the build's scales the result
    adf2 = accel(ctx, tree, dd, 2.0 * d["G"], 1e-22, "theta", "df64")
    np.testing.assert_allclose(adf2[0], 2.0 * adf[0], rtol=1e-15)


@pytest.mark.parametrize("kind,n", [("disc", 20000), ("plummer", 20000)])
def test_group_rule_and_f32(ctx, kind, n):
    d = bodies(kind, n, seed=21)
    eps2 = 1e-22 if kind == "disc" else 1e-6
    naive = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], d["G"], eps2)
    tree, dd = build(ctx, d, theta=0.5)
    e_theta = rel_err(*accel(ctx, tree, dd, d["G"], eps2, "theta", "f64"), *naive)
    e_group = rel_err(*accel(ctx, tree, dd, d["G"], eps2, "group", "f64"), *naive)
    e_group32 = rel_err(*accel(ctx, tree, dd, d["G"], eps2, "group", "f32c"), *naive)
    e_theta32 = rel_err(*accel(ctx, tree, dd, d["G"], eps2, "theta", "f32c"), *naive)
    # the group rule opens a superset of cells: never less accurate in the median
    assert np.median(e_group) <= np.median(e_theta) * 1.0001
    assert np.median(e_theta) <= 5e-3
    # FP32 pair math adds ~1e-6 on top of the approximation error
    assert abs(np.median(e_group32) - np.median(e_group)) <= 1e-5 + 0.05 * np.median(e_group)
    assert abs(np.median(e_theta32) - np.median(e_theta)) <= 1e-5 + 0.05 * np.median(e_theta)
    assert np.all(np.isfinite(e_group32))


def test_accel_before_build_is_rejected(ctx):
    import torch
    from nbody.lib import BHTree, NBodyError
    t = BHTree(ctx, 10)
    z = torch.zeros(10, dtype=torch.float64, device="cuda")
    with pytest.raises(NBodyError, match="NOT_BUILT"):
        t.accel(z, z, z, z, z, z, 1.0, 0.0)


@pytest.mark.parametrize("precision", ["f64_ieee", "f64"])
def test_lane_and_lockstep_schedules_agree_bitwise(ctx, precision):
    from nbody.lib import set_bh_schedule
    d = bodies("disc", 30000, seed=17)
    tree, dd = build(ctx, d, theta=0.5)
    try:
        set_bh_schedule(lockstep=True)
        a = accel(ctx, tree, dd, d["G"], 1e-22, "theta", precision)
    finally:
        set_bh_schedule(lockstep=False)
    b = accel(ctx, tree, dd, d["G"], 1e-22, "theta", precision)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)


def test_build_phase_timing(ctx):
    import torch
    d = bodies("disc", 50000, seed=3)
    tree, dd = build(ctx, d, theta=0.5)
    tree.set_phase_timing(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    tree.build(dd["m"], dd["x"], dd["y"], dd["z"], d["G"])
    e1.record()
    ms = tree.build_phase_ms()
    ctx.sync()
    total = e0.elapsed_time(e1)
    assert len(ms) == 5 and all(v > 0 for v in ms)
    assert sum(ms) <= total * 1.05 + 0.05
    tree.set_phase_timing(False)


@pytest.mark.parametrize("precision", ["f64_ieee", "f64"])
def test_graph_replay_equals_stepwise_steps(ctx, precision):
    """A captured graph of K Barnes-Hut leapfrog steps gives the stepwise calls' state bit for
    bit."""
    import torch
    from nbody.lib import BHTree
    d = bodies("disc", 5000, seed=31)
    n, dt, steps = 5000, 1.0 / 24, 3

    def state():
        s = {k: dev(d[k]) for k in ("m", "x", "y", "z", "vx", "vy", "vz")}
        s["acc"] = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
        s["vh"] = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
        return s

    A, B = state(), state()
    ta, tb = BHTree(ctx, n, theta=0.5), BHTree(ctx, n, theta=0.5)
    for s, t in ((A, ta), (B, tb)):
        t.build(s["m"], s["x"], s["y"], s["z"], d["G"])
        t.accel(s["x"], s["y"], s["z"], *s["acc"], d["G"], 1e-22, "theta", precision)
    posA, velA = [A["x"], A["y"], A["z"]], [A["vx"], A["vy"], A["vz"]]
    for _ in range(steps):
        ctx.kick_drift(A["vh"], velA, posA, A["acc"], dt)
        ta.build(A["m"], *posA, d["G"])
        ta.accel(*posA, *A["acc"], d["G"], 1e-22, "theta", precision)
        ctx.kick(velA, A["vh"], A["acc"], dt)
    g = tb.graph(B["m"], [B["x"], B["y"], B["z"]], [B["vx"], B["vy"], B["vz"]], B["vh"],
                 B["acc"], d["G"], 1e-22, dt, steps, "theta", precision)
    g.launch()
    ctx.sync()
    for k in ("x", "y", "z", "vx", "vy", "vz"):
        np.testing.assert_array_equal(host(A[k]), host(B[k]))
    g.close()


def test_graph_create_rejects_phase_timing_and_bad_steps(ctx):
    import torch
    from nbody.lib import BHTree, NBodyError
    d = bodies("plummer", 500, seed=3)
    n = 500
    t = BHTree(ctx, n, theta=0.5)
    s = {k: dev(d[k]) for k in ("m", "x", "y", "z", "vx", "vy", "vz")}
    z = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(6)]
    args = (s["m"], [s["x"], s["y"], s["z"]], [s["vx"], s["vy"], s["vz"]], z[:3], z[3:], 1.0,
            1e-6, 1e-3)
    with pytest.raises(NBodyError, match="INVALID_ARG"):
        t.graph(*args, 0)
    t.set_phase_timing(True)
    with pytest.raises(NBodyError, match="phase timing"):
        t.graph(*args, 1)
    t.set_phase_timing(False)
    g = t.graph(*args, 2, "theta", "df64")
    g.launch()
    ctx.sync()
    g.close()
    t.close()


# -- node record sets -------------------------------------------------------------------------------
@pytest.mark.parametrize("opening,precision", [("theta", "f64_ieee"), ("theta", "f64"),
                                               ("theta", "df64"), ("group", "f64"),
                                               ("theta", "f32c"), ("group", "f32c")])
def test_record_sets_give_the_same_forces(ctx, opening, precision):
    """A build with only the records a traversal reads (records_for) gives that traversal the
    forces of a build with all records: bit for bit for the FP64 rules (the FP64 centres are the
    same IEEE quotients), within FP32 rounding of the centres for f32c (which then rounds a
    reciprocal-based centre)."""
    from nbody.lib import REC_ALL, records_for
    d = bodies("disc", 6000, seed=8)
    full, dd = build(ctx, d, theta=0.5)
    ref = accel(ctx, full, dd, d["G"], 1e-22, opening, precision)
    lean, _ = build(ctx, d, theta=0.5)
    lean.set_records(records_for(opening, precision))
    lean.build(dd["m"], dd["x"], dd["y"], dd["z"], d["G"])
    got = accel(ctx, lean, dd, d["G"], 1e-22, opening, precision)
    if precision == "f32c":
        assert np.median(rel_err(*got, *ref)) <= 1e-6
    else:
        for g, r in zip(got, ref):
            np.testing.assert_array_equal(g, r)
    assert records_for(opening, precision) != REC_ALL
    full.close()
    lean.close()


def test_missing_records_are_rejected(ctx):
    """Traversals that read records the last build did not compute fail with INVALID_ARG."""
    import torch
    from nbody.lib import REC_FP64, NBodyError
    d = bodies("plummer", 3000, seed=9)
    t, dd = build(ctx, d, theta=0.5)
    t.set_records(0)
    t.build(dd["m"], dd["x"], dd["y"], dd["z"], d["G"])
    a = [torch.zeros(3000, dtype=torch.float64, device="cuda") for _ in range(3)]
    for opening, precision in (("theta", "f64"), ("theta", "f64_ieee"), ("theta", "df64"),
                               ("group", "f64"), ("learned", "f32c")):
        with pytest.raises(NBodyError, match="INVALID_ARG"):
            t.accel(dd["x"], dd["y"], dd["z"], *a, d["G"], 1e-6, opening, precision)
    with pytest.raises(NBodyError, match="INVALID_ARG"):
        t.count_interactions(dd["x"], dd["y"], dd["z"], "theta")
    t.accel(dd["x"], dd["y"], dd["z"], *a, d["G"], 1e-6, "group", "f32c")  # FP32 records only
    t.set_records(REC_FP64)
    t.build(dd["m"], dd["x"], dd["y"], dd["z"], d["G"])
    t.accel(dd["x"], dd["y"], dd["z"], *a, d["G"], 1e-6, "theta", "f64")
    ctx.sync()
    with pytest.raises(NBodyError, match="INVALID_ARG"):
        t.set_records(16)
    t.close()


def test_learned_walk_on_learned_records(ctx):
    """The learned traversal's walk (group theta rule in place of the network) on a build with
    only the learned records agrees with a build with all records to FP32 rounding."""
    from nbody.lib import REC_LEARNED
    d = bodies("disc", 6000, seed=10)
    res = []
    for mask in (None, REC_LEARNED):
        t, dd = build(ctx, d, theta=0.5)
        if mask is not None:
            t.set_records(mask)
            t.build(dd["m"], dd["x"], dd["y"], dd["z"], d["G"])
        t.set_policy(None, 0.0, 0.4, 2 ** 31 - 1)
        res.append(accel(ctx, t, dd, d["G"], 1e-22, "learned", "f32c"))
        t.close()
    assert np.median(rel_err(*res[1], *res[0])) <= 1e-6


def test_quantized_keys_build_the_same_tree(ctx):
    """Quantized keys place random bodies in the reference's cells (no body lies within FP64
    rounding of a midpoint here): same node count and bit-identical FP32 forces."""
    from nbody.lib import BUILD_QUANTIZED_KEYS
    d = bodies("disc", 20000, seed=12)
    out = []
    for mask in (0, BUILD_QUANTIZED_KEYS):
        t, dd = build(ctx, d, theta=0.5)
        t.set_records(mask)
        t.build(dd["m"], dd["x"], dd["y"], dd["z"], d["G"])
        nodes = t.stats()["node_count"]
        out.append((nodes, accel(ctx, t, dd, d["G"], 1e-22, "group", "f32c")))
        t.close()
    assert out[0][0] == out[1][0]
    for g, r in zip(out[1][1], out[0][1]):
        np.testing.assert_array_equal(g, r)

"""Parity of the naive path (nb_naive_accel) against the CPU oracle restating
NaiveAlgorithm.cpp:262-360, through the C ABI.

Tolerances: NB_F64_IEEE bit-identical; NB_F64 per-body relative error <= 1e-12; NB_DF64 median
relative error <= 1e-12; NB_F32C per-body relative error median <= 1e-5 and max <= 1e-3
(Plummer, eps = 1e-3) / median <= 1e-4 (disc).
"""

import numpy as np
import pytest

import oracle
from helpers import bodies, dev, host, rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import torch
    from nbody.lib import Context
    assert torch.cuda.is_available()
    c = Context(0)
    yield c
    c.close()


def run_naive(ctx, d, eps2, precision):
    import torch
    t = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    n = len(d["m"])
    ax, ay, az = (torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(3))
    ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], ax, ay, az, d["G"], eps2, precision)
    ctx.sync()
    return host(ax), host(ay), host(az)


@pytest.mark.parametrize("n", [1, 2, 3, 63, 64, 65, 127, 128, 129, 1000, 4099])
def test_f64_ieee_bit_identical(ctx, n):
    d = bodies("disc", n, seed=n)
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], d["G"], 1e-22)
    got = run_naive(ctx, d, 1e-22, "f64_ieee")
    for g, r in zip(got, ref):
        np.testing.assert_array_equal(g, r)


@pytest.mark.parametrize("kind,n,eps2", [("disc", 16384, 1e-22), ("plummer", 5000, 1e-6),
                                         ("disc", 777, 1e-22)])
def test_f64_fast_within_1e12(ctx, kind, n, eps2):
    d = bodies(kind, n, seed=3)
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], d["G"], eps2)
    got = run_naive(ctx, d, eps2, "f64")
    err = rel_err(*got, *ref)
    assert err.max() <= 1e-12, err.max()


@pytest.mark.parametrize("kind,n,eps2", [("disc", 16384, 1e-22), ("plummer", 5000, 1e-6),
                                         ("disc", 1, 1e-22), ("plummer", 129, 1e-6)])
def test_df64_fp64_accurate(ctx, kind, n, eps2):
    """Double-float pair math: per-body error against the FP64 oracle relative to
    max(|a|, median |a|) <= 1e-11 and median relative error <= 1e-12 (each pair term carries
    ~2^-46 against FP64's ~2^-52)."""
    d = bodies(kind, n, seed=4)
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], d["G"], eps2)
    got = run_naive(ctx, d, eps2, "df64")
    if n == 1:
        assert all(np.all(g == 0) for g in got)  # the self pair alone contributes exactly 0
        return
    diff = np.sqrt(sum((g - r) ** 2 for g, r in zip(got, ref)))
    mag = np.sqrt(sum(r * r for r in ref))
    assert np.median(rel_err(*got, *ref)) <= 1e-12
    assert (diff / np.maximum(mag, np.median(mag))).max() <= 1e-11


@pytest.mark.parametrize("n", [1, 100, 1023, 1024, 1025, 3000, 20000])
def test_f32c_plummer(ctx, n):
    d = bodies("plummer", n, seed=7)
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], 1.0, 1e-6)
    got = run_naive(ctx, d, 1e-6, "f32c")
    err = rel_err(*got, *ref)
    if n == 1:
        assert np.all(np.array(got) == 0)
        return
    assert np.median(err) <= 1e-5 and err.max() <= 1e-3, (np.median(err), err.max())


def test_f32c_disc(ctx):
    d = bodies("disc", 5000, seed=11)
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], d["G"], 1e-22)
    got = run_naive(ctx, d, 1e-22, "f32c")
    err = rel_err(*got, *ref)
    assert np.median(err) <= 1e-4, np.median(err)
    assert np.all(np.isfinite(np.array(got)))


def test_range_matches_full(ctx):
    import torch
    d = bodies("plummer", 3000, seed=2)
    t = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    for prec in ("f64_ieee", "f32c", "df64"):
        full = run_naive(ctx, d, 1e-6, prec)
        ax, ay, az = (torch.zeros(3000, dtype=torch.float64, device="cuda") for _ in range(3))
        ctx.naive_accel_range(t["m"], t["x"], t["y"], t["z"], ax, ay, az, 1000, 2100, 1.0, 1e-6,
                              prec)
        ctx.sync()
        part = host(ax)
        if prec == "f64_ieee":
            np.testing.assert_array_equal(part[1000:2100], full[0][1000:2100])
        elif prec == "df64":
            np.testing.assert_allclose(part[1000:2100], full[0][1000:2100], rtol=1e-12, atol=1e-15)
        else:
            np.testing.assert_allclose(part[1000:2100], full[0][1000:2100], rtol=1e-5, atol=1e-9)
        assert np.all(part[:1000] == 0) and np.all(part[2100:] == 0)


@pytest.mark.parametrize("ws", [2, 3])
def test_target_shards_gather_to_the_full_result(ctx, ws):
    """The replica logic's target split (nbody.replicas.target_range) on the GPU hook: every
    rank's shard computed by nb_naive_accel_range and gathered equals the single call bit for bit
    (NB_F64_IEEE), as the ranks of a sharded run would produce it."""
    import torch
    from nbody.replicas import target_range
    n = 2501
    d = bodies("plummer", n, seed=4)
    t = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    full = run_naive(ctx, d, 1e-6, "f64_ieee")
    gathered = [np.zeros(n) for _ in range(3)]
    for rank in range(ws):
        b, e = target_range(n, rank, ws)
        acc = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
        ctx.naive_accel_range(t["m"], t["x"], t["y"], t["z"], *acc, b, e, 1.0, 1e-6, "f64_ieee")
        ctx.sync()
        for g, a in zip(gathered, acc):
            g[b:e] = host(a)[b:e]
    for g, f in zip(gathered, full):
        np.testing.assert_array_equal(g, f)


def test_invalid_arguments_are_reported(ctx):
    import torch
    from nbody.lib import NBodyError
    x = torch.zeros(4, dtype=torch.float64, device="cuda")
    with pytest.raises(NBodyError, match="INVALID_ARG"):
        ctx.naive_accel(x, x, x, x, x, x, x, 1.0, 0.0, "f64", block_size=-1)
    ctx.naive_accel(x[:0], x[:0], x[:0], x[:0], x[:0], x[:0], x[:0], 1.0, 0.0, "f64")  # n = 0


def test_momentum_conservation_f64(ctx):
    d = bodies("plummer", 2048, seed=5)
    ax, ay, az = run_naive(ctx, d, 1e-6, "f64")
    m = d["m"]
    for a in (ax, ay, az):
        assert abs(np.sum(m * a)) <= 1e-12 * np.sum(m * np.abs(a))

"""Parity of the symmetric FP32 pair kernel (nb_naive_accel NB_F32C over all bodies, each
unordered pair evaluated once and added to both bodies) against the CPU oracle restating
NaiveAlgorithm.cpp:262-360, through the C ABI.

Tolerances (those of the one-sided kernels): NB_F32C per-body relative error median <= 1e-5 and
max <= 1e-3 on Plummer spheres (eps = 1e-3), median <= 1e-4 on the heliocentric disc; NB_F64
per-body relative error <= 1e-12; NB_DF64 median relative error <= 1e-12 and per-body error
<= 1e-11 of max(|a|, median |a|); repeated calls bit-identical (fixed combine order).
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


def run_f32c(ctx, d, eps2, mode, config=0, precision="f32c", config_f64=0, config_df=0):
    import torch
    from nbody.lib import SYM_AUTO, set_naive_symmetric
    t = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    n = len(d["m"])
    a = [torch.full((n,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(3)]
    try:
        set_naive_symmetric(mode, config, config_f64, config_df)
        ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *a, d["G"], eps2, precision)
        ctx.sync()
    finally:
        set_naive_symmetric(SYM_AUTO, 0, 0, 0)
    return tuple(host(v) for v in a)


@pytest.mark.parametrize("config", list(range(8)))
@pytest.mark.parametrize("n", [1, 100, 1023, 2048, 3000, 20000])
def test_symmetric_plummer(ctx, n, config):
    from nbody.lib import SYM_ALWAYS
    if config and n in (1, 100, 1023):
        pytest.skip("small sizes run with the default configuration only")
    d = bodies("plummer", n, seed=17)
    got = run_f32c(ctx, d, 1e-6, SYM_ALWAYS, config)
    if n == 1:
        assert all(np.all(g == 0) for g in got)  # the self pair alone contributes exactly 0
        return
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], 1.0, 1e-6)
    err = rel_err(*got, *ref)
    assert np.median(err) <= 1e-5 and err.max() <= 1e-3, (np.median(err), err.max())


def test_symmetric_disc(ctx):
    from nbody.lib import SYM_ALWAYS
    d = bodies("disc", 5000, seed=11)
    got = run_f32c(ctx, d, 1e-22, SYM_ALWAYS)
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], d["G"], 1e-22)
    assert np.all(np.isfinite(np.array(got)))
    assert np.median(rel_err(*got, *ref)) <= 1e-4


def test_symmetric_deterministic(ctx):
    from nbody.lib import SYM_ALWAYS
    d = bodies("plummer", 20000, seed=5)
    first = run_f32c(ctx, d, 1e-6, SYM_ALWAYS)
    second = run_f32c(ctx, d, 1e-6, SYM_ALWAYS)
    for f, s in zip(first, second):
        np.testing.assert_array_equal(f, s)


def test_automatic_selection_large(ctx):
    """At 131,072 bodies the automatic mode takes the symmetric kernel; it agrees with the
    one-sided kernel and with FP64 sums of 2,048 sampled bodies (nb_naive_accel_targets)."""
    import torch
    from nbody.lib import SYM_AUTO, SYM_NEVER
    n = 131072
    d = bodies("plummer", n, seed=23)
    sym = run_f32c(ctx, d, 1e-6, SYM_AUTO)
    one = run_f32c(ctx, d, 1e-6, SYM_NEVER)
    e = rel_err(*sym, *one)
    assert np.median(e) <= 1e-5 and e.max() <= 1e-3, (np.median(e), e.max())
    targets = np.random.default_rng(3).choice(n, 2048, replace=False).astype(np.uint32)
    t = {k: dev(d[k]) for k in ("m", "x", "y", "z")}
    tg = torch.as_tensor(targets.view(np.int32), device="cuda")
    ref = [torch.zeros(len(targets), dtype=torch.float64, device="cuda") for _ in range(3)]
    ctx.naive_accel_targets(t["m"], t["x"], t["y"], t["z"], tg, *ref, 1.0, 1e-6)
    ctx.sync()
    ref = [host(v) for v in ref]
    err = rel_err(*(v[targets] for v in sym), *ref)
    assert np.median(err) <= 1e-5 and err.max() <= 1e-3, (np.median(err), err.max())


@pytest.mark.parametrize("config_f64", [0, 1, 2, 3])
@pytest.mark.parametrize("kind,n,eps2", [("disc", 16384, 1e-22), ("plummer", 3000, 1e-6),
                                         ("disc", 1, 1e-22), ("plummer", 129, 1e-6),
                                         ("disc", 777, 1e-22)])
def test_symmetric_f64_within_1e12(ctx, kind, n, eps2, config_f64):
    from nbody.lib import SYM_ALWAYS
    if config_f64 and n != 3000:
        pytest.skip("other sizes run with the default FP64 shape only")
    d = bodies(kind, n, seed=31)
    got = run_f32c(ctx, d, eps2, SYM_ALWAYS, precision="f64", config_f64=config_f64)
    if n == 1:
        assert all(np.all(g == 0) for g in got)
        return
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], d["G"], eps2)
    err = rel_err(*got, *ref)
    assert err.max() <= 1e-12, err.max()


def test_symmetric_f64_deterministic_and_selected(ctx):
    """At 16,384 bodies the automatic mode takes the FP64 symmetric kernel (its result equals the
    forced one bit for bit, and differs from the one-sided kernel's by rounding only)."""
    from nbody.lib import SYM_ALWAYS, SYM_AUTO, SYM_NEVER
    d = bodies("disc", 16384, seed=2)
    auto = run_f32c(ctx, d, 1e-22, SYM_AUTO, precision="f64")
    forced = run_f32c(ctx, d, 1e-22, SYM_ALWAYS, precision="f64")
    one = run_f32c(ctx, d, 1e-22, SYM_NEVER, precision="f64")
    for a, f in zip(auto, forced):
        np.testing.assert_array_equal(a, f)
    assert rel_err(*auto, *one).max() <= 2e-12


@pytest.mark.parametrize("config_df", [0, 1])
@pytest.mark.parametrize("kind,n,eps2", [("disc", 16384, 1e-22), ("plummer", 5000, 1e-6),
                                         ("disc", 1, 1e-22), ("plummer", 129, 1e-6)])
def test_symmetric_df64_fp64_accurate(ctx, kind, n, eps2, config_df):
    """The double-float form against the FP64 oracle with the one-sided double-float bounds."""
    from nbody.lib import SYM_ALWAYS
    if config_df and n != 5000:
        pytest.skip("other sizes run with the default double-float shape only")
    d = bodies(kind, n, seed=4)
    got = run_f32c(ctx, d, eps2, SYM_ALWAYS, precision="df64", config_df=config_df)
    if n == 1:
        assert all(np.all(g == 0) for g in got)
        return
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], d["G"], eps2)
    diff = np.sqrt(sum((g - r) ** 2 for g, r in zip(got, ref)))
    mag = np.sqrt(sum(r * r for r in ref))
    assert np.median(rel_err(*got, *ref)) <= 1e-12
    assert (diff / np.maximum(mag, np.median(mag))).max() <= 1e-11


def test_symmetric_df64_selected_and_deterministic(ctx):
    """At 16,384 bodies the automatic mode takes the double-float symmetric kernel; repeated
    calls agree bit for bit and differ from the one-sided double-float kernel by rounding only."""
    from nbody.lib import SYM_AUTO, SYM_NEVER
    d = bodies("disc", 16384, seed=6)
    first = run_f32c(ctx, d, 1e-22, SYM_AUTO, precision="df64")
    second = run_f32c(ctx, d, 1e-22, SYM_AUTO, precision="df64")
    one = run_f32c(ctx, d, 1e-22, SYM_NEVER, precision="df64")
    for f, s in zip(first, second):
        np.testing.assert_array_equal(f, s)
    mag = np.sqrt(sum(r * r for r in one))
    diff = np.sqrt(sum((f - o) ** 2 for f, o in zip(first, one)))
    assert (diff / np.maximum(mag, np.median(mag))).max() <= 1e-11
    assert any(np.any(f != o) for f, o in zip(first, one))  # a different kernel ran

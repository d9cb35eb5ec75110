"""The margin argument behind the fixed-point octree keys (nb_bh.cu, keys_kernel), checked on the
CPU: a restatement of the reference's FP64 midpoint recurrence (mid = min + edge/2, strict
compares, ParallelOctreeTopDownSubtrees.cpp:95-434; the edge halvings are exact) against the
digits read off U = floor((v - min) * 2^52 / edge) wherever U is more than
m = 10.5 (|min| + edge) / edge + 4 units from every multiple of 2^31. Outside that margin the two
must agree on every one of the 21 levels, for strict and non-strict compares alike (x and y use
>, z uses >=), on random data and on bodies placed on the recurrence's own midpoints and moved by
up to 80 ulps. The GPU test of the kernel itself is the cell-by-cell tree comparison with the
oracle in tests/test_bh_gpu.py (its "midpoints" case)."""

import numpy as np
import pytest

LEVELS = 21


def recurrence_digits(v, mn, edge, upper_ge):
    out = np.zeros(v.shape, dtype=np.int64)
    lo = np.full(v.shape, mn)
    half = edge
    for _ in range(LEVELS):
        half = half / 2
        mid = lo + half
        up = (v >= mid) if upper_ge else (v > mid)
        out = out * 2 + up
        lo = np.where(up, mid, lo)
    return out


def fixed_digits(v, mn, edge):
    """The kernel's rule: the 21 digits, or -1 where the body is within the margin."""
    scale = 4503599627370496.0 / edge
    m = int(10.5 * (abs(mn) * (scale * 2.0 ** -52) + 1.0) * (1 + 2.0 ** -30) + 4.0) + 1
    u = (v - mn) * scale
    ok = (u >= 0) & (u <= 4503599627370496.0)
    U = np.where(ok, u, 0).astype(np.int64)
    hi, lo = (U + m) >> 31, (U - m - 1) >> 31
    return np.where(ok & (hi == lo), hi, -1)


def on_midpoints(rng, n, mn, edge, ulps):
    """Bodies on the recurrence's computed midpoints (random cells and levels), moved by up to
    `ulps` units in the last place."""
    lo = np.full(n, mn)
    half = edge
    stop = rng.integers(0, LEVELS, size=n)
    out = np.zeros(n)
    for level in range(LEVELS):
        half = half / 2
        mid = lo + half
        out[stop == level] = mid[stop == level]
        lo = np.where(rng.random(n) < 0.5, mid, lo)
    steps = rng.integers(-ulps, ulps + 1, size=n)
    for s in range(ulps):
        sel = np.abs(steps) > s
        out[sel] = np.nextafter(out[sel], np.where(steps[sel] > 0, np.inf, -np.inf))
    return out


def _check(v, mn, edge):
    fx = fixed_digits(v, mn, edge)
    good = fx >= 0
    for upper_ge in (False, True):
        ref = recurrence_digits(v, mn, edge, upper_ge)
        bad = np.flatnonzero(good & (ref != fx))
        assert bad.size == 0, (upper_ge, v[bad[:5]], ref[bad[:5]], fx[bad[:5]])
    return int(np.count_nonzero(~good))


@pytest.mark.parametrize("seed", range(6))
def test_fixed_point_digits_match_the_recurrence_on_random_data(seed):
    rng = np.random.default_rng(seed)
    n = 50_000
    v = rng.normal(size=n) * 10.0 ** rng.uniform(-6, 12)
    if seed % 2:
        v = v + 1e3 * np.abs(v).max()  # a box far from the origin: a wide margin
    mn = min(v.min(), 0.0)  # the box contains the origin (the reference's AABB)
    edge = max(v.max(), 0.0) - mn
    fallbacks = _check(v, mn, edge)
    assert fallbacks <= 16  # only bodies on the box faces (or a rare near-midpoint one)


@pytest.mark.parametrize("seed", range(6))
def test_fixed_point_digits_match_the_recurrence_next_to_its_midpoints(seed):
    rng = np.random.default_rng(100 + seed)
    scale = 10.0 ** rng.uniform(-6, 12)
    mn, mx = (0.0, scale) if seed % 2 else (-rng.random() * scale, rng.random() * scale)
    edge = mx - mn
    for ulps in (0, 2, 80):
        v = np.clip(on_midpoints(rng, 40_000, mn, edge, ulps), mn, mx)
        fallbacks = _check(v, mn, edge)
        if ulps <= 2:
            assert fallbacks == len(v)  # every such body takes the recurrence itself
        else:
            assert 0 < fallbacks < len(v)  # both rules run, and agree where the fast one does

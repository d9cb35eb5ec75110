"""Parity of leapfrog (bit-identical), energy (<= 1e-12 relative) and AABB (bit-identical)
against the CPU oracle, through the C ABI."""

import numpy as np
import pytest

import oracle
from helpers import bodies, dev, host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from nbody.lib import Context
    c = Context(0)
    yield c
    c.close()


def test_leapfrog_bit_identical(ctx):
    import torch
    rng = np.random.default_rng(1)
    n = 10007
    v = [rng.normal(size=n) for _ in range(3)]
    p = [rng.normal(size=n) * 10 for _ in range(3)]
    a = [rng.normal(size=n) * 1e-3 for _ in range(3)]
    dt = 1.0 / 24
    # oracle: part 1 then part 2 then part 1 again
    po = [q.copy() for q in p]
    vh = oracle.leapfrog_part1(v, po, a, dt)
    vo = [q.copy() for q in v]
    oracle.leapfrog_part2(vo, vh, a, dt)
    vh2 = oracle.leapfrog_part1(vo, po, a, dt)
    # GPU
    V, P, A = [dev(q) for q in v], [dev(q) for q in p], [dev(q) for q in a]
    VH = [torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    ctx.kick_drift(VH, V, P, A, dt)
    P2 = [q.clone() for q in P]
    VH2 = [q.clone() for q in VH]
    V2 = [q.clone() for q in V]
    ctx.kick(V, VH, A, dt)
    ctx.kick_drift(VH, V, P, A, dt)
    ctx.kick_kick_drift(V2, VH2, P2, A, dt)  # fused: same result as kick + kick_drift
    ctx.sync()
    for k in range(3):
        np.testing.assert_array_equal(host(P[k]), po[k])
        np.testing.assert_array_equal(host(V[k]), vo[k])
        np.testing.assert_array_equal(host(VH[k]), vh2[k])
        np.testing.assert_array_equal(host(P2[k]), po[k])
        np.testing.assert_array_equal(host(V2[k]), vo[k])
        np.testing.assert_array_equal(host(VH2[k]), vh2[k])


@pytest.mark.parametrize("kind,n", [("plummer", 1), ("plummer", 2), ("plummer", 3001),
                                    ("disc", 5000)])
def test_energy(ctx, kind, n):
    import torch
    d = bodies(kind, n, seed=4)
    ref = oracle.energy(d["m"], d["x"], d["y"], d["z"], d["vx"], d["vy"], d["vz"], d["G"])
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    ctx.energy(*[dev(d[k]) for k in ("m", "x", "y", "z", "vx", "vy", "vz")], d["G"], out)
    ctx.sync()
    got = host(out)
    names = ("kinetic", "potential", "total", "virial")
    for g, k in zip(got, names):
        r = ref[k]
        if n == 1 and k in ("potential", "virial"):
            continue  # no pairs: U = 0 and the virial ratio divides by zero in both
        assert abs(g - r) <= 1e-12 * max(abs(r), abs(ref["kinetic"])), (k, g, r)


@pytest.mark.parametrize("n,shift", [(3, 0.0), (1000, 0.0), (100003, 0.0), (5000, 7.5),
                                     (4096, -3.0)])
def test_aabb_bit_identical(ctx, n, shift):
    import torch
    rng = np.random.default_rng(n)
    x, y, z = rng.normal(size=(3, n)) + shift
    z = z * 3.0
    ref = oracle.aabb(x, y, z)
    out = torch.zeros(7, dtype=torch.float64, device="cuda")
    ctx.aabb(dev(x), dev(y), dev(z), out)
    ctx.sync()
    got = host(out)
    keys = ("min_x", "min_y", "min_z", "max_x", "max_y", "max_z", "edge")
    for g, k in zip(got, keys):
        assert g == ref[k], (k, g, ref[k])


def test_aabb_reference_known_answer(ctx, kats):
    import torch
    t = [t for t in kats["BarnesHutTest.cpp"] if t["name"] == "AABB_creation"][0]
    v = t["vectors"]
    out = torch.zeros(7, dtype=torch.float64, device="cuda")
    ctx.aabb(dev(v["x_positions"]), dev(v["y_positions"]), dev(v["z_positions"]), out)
    ctx.sync()
    got = dict(zip(("octree.min_x", "octree.min_y", "octree.min_z", "octree.max_x",
                    "octree.max_y", "octree.max_z", "octree.AABB_EdgeLength"), host(out)))
    for e in t["expects"]:
        assert got[e["expr"]] == e["value"], e

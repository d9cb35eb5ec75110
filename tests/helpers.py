"""Shared helpers for the parity tests (device arrays via torch, data via the generators)."""

import numpy as np

from nbody import generators


def bodies(kind: str, n: int, seed: int = 1):
    if kind == "disc":
        return generators.heliocentric_disc(max(n, 9), seed) if n >= 9 else _tiny(n, seed)
    if kind == "plummer":
        return generators.plummer(n, seed)
    raise ValueError(kind)


def _tiny(n, seed):
    rng = np.random.default_rng(seed)
    d = {k: rng.normal(size=n) for k in ("x", "y", "z", "vx", "vy", "vz")}
    d["m"] = rng.uniform(1e20, 1e25, size=n)
    d["G"] = generators.reference_G()
    return d


def dev(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def host(t):
    return t.detach().cpu().numpy()


def rel_err(ax, ay, az, bx, by, bz):
    """Per-body |a - b| / |b| (b = reference)."""
    num = np.sqrt((ax - bx) ** 2 + (ay - by) ** 2 + (az - bz) ** 2)
    den = np.sqrt(bx ** 2 + by ** 2 + bz ** 2)
    return num / np.where(den > 0, den, 1.0)


def as_layout(tree):
    """Reference-layout dict from an oracle.OracleTree or a BHTree export dict."""
    if isinstance(tree, dict):
        return tree
    keys = ("octants", "edge", "min_x", "min_y", "min_z", "body_of_node", "node_is_leaf",
            "sum_masses", "com_x", "com_y", "com_z", "body_count", "sorted_bodies")
    d = {k: getattr(tree, k) for k in keys}
    d["node_count"] = tree.node_count
    return d


def canonical_compare(a, b, n):
    """Walks two reference-layout octrees from the root, pairing children by octant, and asserts
    that every cell holds the same record (exact equality, including FP64 sums). Node ids may
    differ. Returns the number of cells compared."""
    a, b = as_layout(a), as_layout(b)
    assert a["node_count"] == b["node_count"], (a["node_count"], b["node_count"])
    fields_f = ("edge", "min_x", "min_y", "min_z", "sum_masses", "com_x", "com_y", "com_z")
    fields_i = ("body_of_node", "node_is_leaf", "body_count")
    stack = [(0, 0)]
    seen = 0
    while stack:
        ia, ib = stack.pop()
        seen += 1
        for f in fields_i:
            assert int(a[f][ia]) == int(b[f][ib]), (f, ia, ib, a[f][ia], b[f][ib])
        for f in fields_f:
            assert a[f][ia] == b[f][ib], (f, ia, ib, a[f][ia], b[f][ib])
        if not a["node_is_leaf"][ia]:
            for o in range(8):
                stack.append((int(a["octants"][o][ia]), int(b["octants"][o][ib])))
    assert seen == a["node_count"]
    np.testing.assert_array_equal(a["sorted_bodies"][:n], b["sorted_bodies"][:n])
    return seen

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

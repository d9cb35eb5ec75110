"""Small, self-contained GPU cases of the hot kernels, for profiling runs.

    python n-body-simulation_gb300/nbody/cases.py pair [N] [config]
        seeded Plummer sphere (G = M = a = 1, softening 1e-3), three FP32-compensated naive
        evaluations with the one-sided kernel (pair_f32c_kernel), tile configuration `config`
    python n-body-simulation_gb300/nbody/cases.py sym [N] [config]
        the same three evaluations with the symmetric kernel (pair_sym_kernel), configuration
        `config`
    python n-body-simulation_gb300/nbody/cases.py sym64 [N] [config]
        seeded heliocentric disc, three FP64 naive evaluations (NB_F64) with the FP64 form of the
        symmetric kernel, FP64 configuration `config`
    python n-body-simulation_gb300/nbody/cases.py learned [N] [log10_tau] [pairs]
        seeded disc + Plummer mix: labelled pairs and a short training of the opening network,
        then three learned traversals (bh_learned_kernel) at threshold tau
    python n-body-simulation_gb300/nbody/cases.py df64 [N]
        seeded heliocentric disc: three double-float Barnes-Hut traversals (bh_theta_df_kernel,
        theta = 0.5) and one double-float naive evaluation (naive_df_kernel)

Each case prints "ok" when its launches finished without a device error. The headline FP64
traversal is profiled through bench.py itself (`--bodies`, `--quick`).
"""

from __future__ import annotations

import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def pair_case(n: int = 262144, config: int = 0, symmetric: bool = False):
    import torch

    from nbody import generators, learned
    from nbody.lib import (SYM_ALWAYS, SYM_NEVER, Context, set_naive_pair_config,
                           set_naive_symmetric)
    ctx = Context(0)
    if symmetric:
        set_naive_symmetric(SYM_ALWAYS, config)
    else:
        set_naive_symmetric(SYM_NEVER, 0)
        set_naive_pair_config(config)
    t = learned.device_system(generators.plummer(n, 1))
    acc = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    for _ in range(3):
        ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *acc, 1.0, 1e-6, "f32c")
    ctx.sync()


def sym64_case(n: int = 65536, config: int = 0):
    import torch

    from nbody import generators, learned
    from nbody.lib import SYM_ALWAYS, Context, set_naive_symmetric
    ctx = Context(0)
    set_naive_symmetric(SYM_ALWAYS, 0, config)
    d = generators.heliocentric_disc(n, 1)
    t = learned.device_system(d)
    acc = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    for _ in range(3):
        ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *acc, d["G"], learned.EPS2, "f64")
    ctx.sync()


def learned_case(n: int = 262144, log10_tau: float = -4.25, pairs: int = 2_000_000):
    import torch

    from nbody import generators, learned
    from nbody.lib import BHTree, Context
    ctx = Context(0)
    X, Y = learned.training_set(ctx, n, pairs)
    params, _ = learned.train(ctx, X, Y, epochs=4)
    d = generators.disc_plummer_mix(n, seed=21)
    t = learned.device_system(d)
    tree = BHTree(ctx, n, theta=0.4)
    tree.build(t["m"], t["x"], t["y"], t["z"], d["G"])
    acc = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    tree.accel(t["x"], t["y"], t["z"], *acc, d["G"], learned.EPS2, "group", "f32c")
    tree.set_policy(params, log10_tau, 0.3, learned.NO_CAP)
    for _ in range(3):
        tree.accel(t["x"], t["y"], t["z"], *acc, d["G"], learned.EPS2, "learned", "f32c")
    ctx.sync()


def df64_case(n: int = 262144):
    import torch

    from nbody import generators, learned
    from nbody.lib import BHTree, Context
    ctx = Context(0)
    d = generators.heliocentric_disc(n, 1)
    t = learned.device_system(d)
    tree = BHTree(ctx, n, theta=0.5)
    tree.build(t["m"], t["x"], t["y"], t["z"], d["G"])
    acc = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    for _ in range(3):
        tree.accel(t["x"], t["y"], t["z"], *acc, d["G"], learned.EPS2, "theta", "df64")
    ctx.naive_accel(t["m"], t["x"], t["y"], t["z"], *acc, d["G"], learned.EPS2, "df64")
    ctx.sync()


def main(argv):
    if not argv or argv[0] not in ("pair", "sym", "sym64", "learned", "df64"):
        print(__doc__)
        return 2
    args = argv[1:]
    if argv[0] in ("pair", "sym"):
        pair_case(int(args[0]) if args else 262144, int(args[1]) if len(args) > 1 else 0,
                  argv[0] == "sym")
    elif argv[0] == "sym64":
        sym64_case(int(args[0]) if args else 65536, int(args[1]) if len(args) > 1 else 0)
    elif argv[0] == "df64":
        df64_case(int(args[0]) if args else 262144)
    else:
        learned_case(int(args[0]) if args else 262144, float(args[1]) if len(args) > 1 else -4.25,
                     int(args[2]) if len(args) > 2 else 2_000_000)
    print("ok")
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))

"""The C++ driver end to end on the GPU: the reference's command line on a CSV, checked against
the oracle's simulation of the same loop (BarnesHutAlgorithm / NaiveAlgorithm::startSimulation):
lastState.csv (6 significant digits, the reference's stream format), the ParaView files and
times.json."""

import json
import os
import subprocess

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EXE = os.path.join(ROOT, "n-body-simulation_gb300", "_build", "nbody_sim")


def oracle_simulation(d, dt, t_end, vs, algorithm, theta=1.05, energies=None):
    """Positions of the last visualised step, following NaiveAlgorithm.cpp:131-259 (and
    BarnesHutAlgorithm.cpp:149-277); with `energies` (a list) also the total energy
    (nBodyAlgorithm.cpp:11-86) of every visualised step, step 0 first."""
    G, eps2 = d["G"], 1e-22
    x, y, z = d["x"].copy(), d["y"].copy(), d["z"].copy()
    v = [d["vx"].copy(), d["vy"].copy(), d["vz"].copy()]

    def accel():
        if algorithm == "naive":
            return list(oracle.naive_accel(d["m"], x, y, z, G, eps2))
        t = oracle.build_subtrees(d["m"], x, y, z)
        return list(oracle.bh_accel(t, x, y, z, G, eps2, theta))

    def energy():
        if energies is not None:
            energies.append(oracle.energy(d["m"], x, y, z, *v, G)["total"])

    a = accel()
    energy()
    last = (x.copy(), y.copy(), z.copy())
    steps = 0
    time, since = dt, dt
    while time <= t_end + 1e-6:
        vis = abs(since - vs) < 1e-6
        vh = oracle.leapfrog_part1(v, [x, y, z], a, dt)
        a = accel()
        oracle.leapfrog_part2(v, vh, a, dt)
        if vis:
            last = (x.copy(), y.copy(), z.copy())
            energy()
            steps += 1
            since = 0.0
        time += dt
        since += dt
    return last, steps


def _run_dir(out):
    run_dirs = [os.path.join(out, p) for p in os.listdir(out)]
    assert len(run_dirs) == 1
    return run_dirs[0]


def _vtp_array(path, name):
    """Values of one ASCII DataArray of a .vtp file (the reference's output layout)."""
    text = open(path).read()
    head = text.index(f'Name="{name}"')
    start = text.index(">", head) + 1
    return np.array(text[start:text.index("</DataArray>", start)].split(), dtype=float)


@pytest.mark.parametrize("algorithm,extra", [("naive", ["--precision=f64_ieee"]),
                                             ("BarnesHut", ["--theta=0.5"]),
                                             ("BarnesHut", ["--theta=0.5", "--graph"]),
                                             ("naive", ["--block_size=128", "--opt_stage=2"])])
def test_driver_matches_oracle(tmp_path, algorithm, extra):
    from nbody import generators
    d = generators.heliocentric_disc(600, seed=13)
    csv = tmp_path / "bodies.csv"
    generators.write_csv(str(csv), d)
    out = tmp_path / "out"
    cmd = [EXE, f"--file={csv}", "--dt=1h", "--t_end=1d", "--vs=12h", f"--vs_dir={out}",
           f"--algorithm={algorithm}", "--energy=true"] + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rd = _run_dir(out)
    (ox, oy, oz), vis_steps = oracle_simulation(d, 1 / 24, 1.0, 0.5, algorithm, theta=0.5)
    assert vis_steps == 2
    rows = np.loadtxt(os.path.join(rd, "lastState.csv"), delimiter=",", skiprows=1)
    np.testing.assert_allclose(rows[:, 0], ox, rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(rows[:, 1], oy, rtol=1e-5, atol=1e-9)
    np.testing.assert_allclose(rows[:, 2], oz, rtol=1e-5, atol=1e-9)
    files = sorted(os.listdir(rd))
    assert {"simulation.pvd", "simulation_step0.vtp", "simulation_step1.vtp",
            "simulation_step2.vtp", "times.json", "lastState.csv"} <= set(files)
    pvd = open(os.path.join(rd, "simulation.pvd")).read()
    assert pvd.count("<DataSet") == 3
    vtp = open(os.path.join(rd, "simulation_step2.vtp")).read()
    assert 'NumberOfPoints="600"' in vtp and 'Name="kinetic energy"' in vtp
    t = json.load(open(os.path.join(rd, "times.json")))
    assert t["body count"] == 600
    assert t["algorithm"] == ("Naive Algorithm" if algorithm == "naive" else "Barnes-Hut Algorithm")
    if "--graph" in extra:  # steps between visualised ones replayed from the captured graph
        assert len(t["Acceleration Kernel Time"]) == 3  # initial evaluation + 2 visualised steps
        assert len(t["Leapfrog step (CUDA graph)"]) == 22
    else:
        assert len(t["Acceleration Kernel Time"]) == 25  # initial evaluation + 24 steps
        assert len(t["Leapfrog Part 1"]) == 24


def test_config1_naive_cli_run_matches_the_oracle_run(tmp_path):
    """The reference's CPU-path configuration through the reference's surface: naive FP64
    (opt_stage 2, block size 128) on the seeded 16,384-body heliocentric disc, dt = 1 h,
    t_end = 10 d (240 leapfrog steps after the initial evaluation), energies on, every day
    visualised. lastState.csv and every visualised step's total energy agree with the oracle's
    run of the same loop to the 6 significant digits of the reference's output format."""
    from nbody import generators
    d = generators.heliocentric_disc(16384, seed=1)
    csv = tmp_path / "disc16384.csv"
    generators.write_csv(str(csv), d)
    out = tmp_path / "out"
    cmd = [EXE, f"--file={csv}", "--dt=1h", "--t_end=10d", "--vs=1d", f"--vs_dir={out}",
           "--algorithm=naive", "--opt_stage=2", "--block_size=128", "--energy=true"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rd = _run_dir(out)
    energies = []
    (ox, oy, oz), vis_steps = oracle_simulation(d, 1 / 24, 10.0, 1.0, "naive", energies=energies)
    assert vis_steps == 10 and len(energies) == 11
    rows = np.loadtxt(os.path.join(rd, "lastState.csv"), delimiter=",", skiprows=1)
    for c, o in enumerate((ox, oy, oz)):
        np.testing.assert_allclose(rows[:, c], o, rtol=1e-5, atol=1e-9)
    for k, e in enumerate(energies):
        got = _vtp_array(os.path.join(rd, f"simulation_step{k}.vtp"), "total energy")
        assert got.size == 1 and abs(got[0] - e) <= 1e-5 * abs(e), (k, got, e)
    t = json.load(open(os.path.join(rd, "times.json")))
    assert t["block size"] == 128 and t["optimization stage"] == 2
    assert len(t["Acceleration Kernel Time"]) == 241
    assert len(t["Leapfrog Part 1"]) == 240 and len(t["Leapfrog Part 2"]) == 240


def test_learned_opening_cli_run(tmp_path):
    """--opening=learned --policy=<file>: a network trained by the library's own kernels and
    saved with nb_policy_save drives a Barnes-Hut run of the disc + Plummer mix from a CSV.
    The initial evaluation's |a| (step-0 .vtp, the reference's output) is within the learned
    form's error bounds of the oracle's FP64 naive sums (median 1e-4, p99 1e-3), and the run's
    last state, with the steps between visualised ones replayed from a CUDA graph, agrees with the
    oracle's naive FP64 run to the output's 6 significant digits."""
    from nbody import generators, learned
    from nbody.lib import POLICY_BOUND_ACCEPT, Context, policy_save
    ctx = Context(0)
    X, Y = learned.training_set(ctx, 262144, 2_000_000)
    params, hist = learned.train(ctx, X, Y, epochs=4, batch=8192, lr=2e-3)
    ctx.sync()
    ctx.close()
    assert hist[-1] < hist[0]
    policy = tmp_path / "policy.txt"
    policy_save(str(policy), params, -4.5, 0.3, 2 ** 31 - 1, POLICY_BOUND_ACCEPT)
    n = 65536
    d = generators.disc_plummer_mix(n, seed=21)
    csv = tmp_path / "mix.csv"
    generators.write_csv(str(csv), d)
    out = tmp_path / "out"
    cmd = [EXE, f"--file={csv}", "--dt=1h", "--t_end=3h", "--vs=3h", f"--vs_dir={out}",
           "--algorithm=BarnesHut", "--theta=0.4", "--precision=f32c", "--opening=learned",
           f"--policy={policy}", "--graph"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rd = _run_dir(out)
    ref = oracle.naive_accel(d["m"], d["x"], d["y"], d["z"], d["G"], 1e-22)
    a_ref = np.sqrt(sum(c * c for c in ref))
    a0 = _vtp_array(os.path.join(rd, "simulation_step0.vtp"), "acceleration")
    e = np.abs(a0 - a_ref) / a_ref
    assert np.median(e) <= 1e-4 and np.percentile(e, 99) <= 1e-3, (np.median(e),
                                                                     np.percentile(e, 99))
    (ox, oy, oz), vis_steps = oracle_simulation(d, 1 / 24, 0.125, 0.125, "naive")
    assert vis_steps == 1
    rows = np.loadtxt(os.path.join(rd, "lastState.csv"), delimiter=",", skiprows=1)
    for c, o in enumerate((ox, oy, oz)):
        np.testing.assert_allclose(rows[:, c], o, rtol=1e-5, atol=1e-9)
    t = json.load(open(os.path.join(rd, "times.json")))
    assert len(t["Leapfrog step (CUDA graph)"]) == 2


def test_learned_opening_needs_a_policy_file(tmp_path):
    from nbody import generators
    d = generators.heliocentric_disc(100, seed=3)
    csv = tmp_path / "b.csv"
    generators.write_csv(str(csv), d)
    base = [EXE, f"--file={csv}", "--dt=1h", "--t_end=1h", "--vs=1h",
            f"--vs_dir={tmp_path / 'o'}", "--algorithm=BarnesHut", "--opening=learned"]
    r = subprocess.run(base, capture_output=True, text=True)
    assert r.returncode != 0 and "--policy" in r.stderr
    bad = tmp_path / "bad.txt"
    bad.write_text("not a policy\n")
    r = subprocess.run(base + [f"--policy={bad}", "--precision=f32c"], capture_output=True,
                       text=True)
    assert r.returncode != 0 and "nb_policy_load" in r.stderr
    r = subprocess.run(base + [f"--policy={bad}"], capture_output=True, text=True)
    assert r.returncode != 0

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


def oracle_simulation(d, dt, t_end, vs, algorithm, theta=1.05):
    """Positions of the last visualised step, following NaiveAlgorithm.cpp:131-259."""
    G, eps2 = d["G"], 1e-22
    x, y, z = d["x"].copy(), d["y"].copy(), d["z"].copy()
    v = [d["vx"].copy(), d["vy"].copy(), d["vz"].copy()]

    def accel():
        if algorithm == "naive":
            return list(oracle.naive_accel(d["m"], x, y, z, G, eps2))
        t = oracle.build_subtrees(d["m"], x, y, z)
        return list(oracle.bh_accel(t, x, y, z, G, eps2, theta))

    a = accel()
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
            steps += 1
            since = 0.0
        time += dt
        since += dt
    return last, steps


@pytest.mark.parametrize("algorithm,extra", [("naive", ["--precision=f64_ieee"]),
                                             ("BarnesHut", ["--theta=0.5"]),
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
    run_dirs = [os.path.join(out, p) for p in os.listdir(out)]
    assert len(run_dirs) == 1
    rd = run_dirs[0]
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
    assert len(t["Acceleration Kernel Time"]) == 25  # initial evaluation + 24 steps
    assert len(t["Leapfrog Part 1"]) == 24

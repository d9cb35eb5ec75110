"""The synthetic disc's orbital-element conversion (nbody.generators.kepler_to_state) against a
scalar restatement of the reference's dataset converter (dataset_converter/src/conversion.cpp:
13-89, in oracle/conversion.py), element by element, and against the two-body invariants every
Keplerian state must satisfy: specific orbital energy -mu / (2a), specific angular momentum
sqrt(mu a (1 - e^2)), and the orbit's inclination and ascending node recovered from the angular
momentum vector."""

import math

import numpy as np
import pytest

from nbody import generators
from oracle import conversion

MU = generators.reference_G() * generators.MSUN_KG  # AU^3 / d^2 of the 1 Msun central body


def _elements(n, seed, e_fixed=None):
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.4, 30.0, n)
    e = np.full(n, e_fixed) if e_fixed is not None else rng.uniform(0.0, 0.2, n)
    inc = np.deg2rad(rng.uniform(0.0, 10.0, n))
    node, peri, ma = (rng.uniform(0.0, 2 * np.pi, n) for _ in range(3))
    return a, e, inc, node, peri, ma


@pytest.mark.parametrize("e_fixed", [0.0, 0.2, None])
def test_kepler_to_state_matches_scalar_converter(e_fixed):
    a, e, inc, node, peri, ma = _elements(500, seed=5, e_fixed=e_fixed)
    got = generators.kepler_to_state(a, e, inc, node, peri, ma, MU)
    for k in range(len(a)):
        want = conversion.orbital_element_to_state_vector(a[k], e[k], inc[k], node[k], peri[k],
                                                          ma[k], MU)
        pos_scale = a[k] * (1 + e[k])
        vel_scale = math.sqrt(MU / a[k] * (1 + e[k]) / max(1 - e[k], 1e-12))
        for c in range(3):
            assert abs(got[c][k] - want[c]) <= 1e-13 * pos_scale, (k, c, got[c][k], want[c])
            assert abs(got[3 + c][k] - want[3 + c]) <= 1e-13 * vel_scale, (k, c)


@pytest.mark.parametrize("e_fixed", [0.0, 0.2, None])
def test_kepler_states_keep_two_body_invariants(e_fixed):
    a, e, inc, node, peri, ma = _elements(2000, seed=6, e_fixed=e_fixed)
    x, y, z, vx, vy, vz = generators.kepler_to_state(a, e, inc, node, peri, ma, MU)
    r = np.sqrt(x * x + y * y + z * z)
    v2 = vx * vx + vy * vy + vz * vz
    energy = 0.5 * v2 - MU / r
    np.testing.assert_allclose(energy, -MU / (2 * a), rtol=1e-12)
    hx, hy, hz = y * vz - z * vy, z * vx - x * vz, x * vy - y * vx
    h = np.sqrt(hx * hx + hy * hy + hz * hz)
    np.testing.assert_allclose(h, np.sqrt(MU * a * (1 - e * e)), rtol=1e-12)
    # inclination and ascending node of the angular momentum vector
    np.testing.assert_allclose(np.arccos(hz / h), inc, atol=1e-10)
    tilted = inc > 1e-3
    node_got = np.mod(np.arctan2(hx, -hy), 2 * np.pi)
    d = np.abs(node_got - node)[tilted]
    assert np.all(np.minimum(d, 2 * np.pi - d) < 1e-8)
    # eccentricity vector: magnitude e and (for e > 0) direction of the periapsis
    ex = (vy * hz - vz * hy) / MU - x / r
    ey = (vz * hx - vx * hz) / MU - y / r
    ez = (vx * hy - vy * hx) / MU - z / r
    np.testing.assert_allclose(np.sqrt(ex * ex + ey * ey + ez * ez), e, atol=1e-11)


def test_disc_bodies_follow_the_converter():
    """heliocentric_disc draws its small bodies' elements and converts them with
    kepler_to_state; re-drawing the same elements from the same seed reproduces its states."""
    n, seed = 64, 9
    d = generators.heliocentric_disc(n, seed)
    rng = np.random.default_rng(seed)
    a_p = rng.uniform(0.4, 30.0, size=8)
    rng.uniform(size=8)  # planet masses (log-uniform draw)
    ma_p = rng.uniform(0, 2 * np.pi, 8)
    for k in range(8):
        want = conversion.orbital_element_to_state_vector(a_p[k], 0.0, 0.0, 0.0, 0.0, ma_p[k], MU)
        got = [d[c][1 + k] for c in ("x", "y", "z", "vx", "vy", "vz")]
        np.testing.assert_allclose(got, want, rtol=1e-13, atol=1e-15)
    ns = n - 9
    a = rng.uniform(2.1, 3.3, ns)
    e = rng.uniform(0.0, 0.2, ns)
    inc = np.deg2rad(rng.uniform(0.0, 10.0, ns))
    node, peri, ma = (rng.uniform(0, 2 * np.pi, ns) for _ in range(3))
    for k in range(ns):
        want = conversion.orbital_element_to_state_vector(a[k], e[k], inc[k], node[k], peri[k],
                                                          ma[k], MU)
        got = [d[c][9 + k] for c in ("x", "y", "z", "vx", "vy", "vz")]
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-14)
    assert d["m"][0] == generators.MSUN_KG and d["x"][0] == 0.0 and d["vx"][0] == 0.0

"""Scalar restatement of the reference's orbital-element -> state-vector conversion -- TEST
INFRASTRUCTURE ONLY (the parity reference of ``nbody.generators.kepler_to_state``).

Follows dataset_converter/src/conversion.cpp:13-89 (orbital_element_to_state_vector) one body at
a time with the ``math`` module: the mean anomaly advanced by (t - t0) * sqrt(mu / a^3)
(:23-26), 30 Newton-Raphson iterations on E - e sin E = M started at E = M (:28-33), the true
anomaly from atan2 of the half-angle terms (:35-36), the distance r_c = a (1 - e cos E) (:39),
the orbital-frame position and velocity (:42-49), the rotation by the argument of periapsis w,
the inclination i and the longitude of the ascending node om into the heliocentric frame
(:53-74), and the central body's position and velocity added (:77-85). Only tests import it.
"""

from __future__ import annotations

import math


def orbital_element_to_state_vector(a, e, i, om, w, ma, mu, t=0.0, t0=0.0,
                                    central=(0.0, 0.0, 0.0, 0.0, 0.0, 0.0)):
    """(x, y, z, vx, vy, vz) of one body with semi-major axis a, eccentricity e, inclination i,
    ascending node om, argument of periapsis w and mean anomaly ma (radians) about a central body
    with gravitational parameter mu at state `central`."""
    m_t = ma + (t - t0) * math.sqrt(mu / a ** 3)
    E = m_t
    for _ in range(30):
        E = E - (E - e * math.sin(E) - m_t) / (1.0 - e * math.cos(E))
    v_t = 2.0 * math.atan2(math.sqrt(1.0 + e) * math.sin(E / 2.0),
                           math.sqrt(1.0 - e) * math.cos(E / 2.0))
    r_c = a * (1.0 - e * math.cos(E))
    ox, oy = r_c * math.cos(v_t), r_c * math.sin(v_t)
    ovx = (math.sqrt(mu * a) / r_c) * -math.sin(E)
    ovy = (math.sqrt(mu * a) / r_c) * (math.sqrt(1.0 - e ** 2) * math.cos(E))
    cw, sw = math.cos(w), math.sin(w)
    co, so = math.cos(om), math.sin(om)
    ci, si = math.cos(i), math.sin(i)
    x = ox * (cw * co - sw * ci * so) - oy * (sw * co + cw * ci * so)
    y = ox * (cw * so + sw * ci * co) + oy * (cw * ci * co - sw * so)
    z = ox * (sw * si) + oy * (cw * si)
    vx = ovx * (cw * co - sw * ci * so) - ovy * (sw * co + cw * ci * so)
    vy = ovx * (cw * so + sw * ci * co) + ovy * (cw * ci * co - sw * so)
    vz = ovx * (sw * si) + ovy * (cw * si)
    cx, cy, cz, cvx, cvy, cvz = central
    return x + cx, y + cy, z + cz, vx + cvx, vy + cvy, vz + cvz

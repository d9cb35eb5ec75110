"""Seeded synthetic inputs in the reference's units and CSV layout.

* ``heliocentric_disc``: one 1.0 Msun central body at rest at the origin, 8 planets on circular
  coplanar orbits (a ~ U[0.4, 30] AU, m log-uniform in [1.6e-7, 1e-3] Msun) and N-9 small bodies
  (a ~ U[2.1, 3.3] AU, e ~ U[0, 0.2], i ~ U[0, 10] deg, node, periapsis and mean anomaly
  ~ U[0, 2pi), m log-uniform in [1e-15, 1e-10] Msun) on Keplerian orbits about the central body.
  Masses are written in kg (1 Msun = 1.98847e30 kg, dataset_converter/src/conversion.cpp:96-97)
  so the reference's G in AU^3 kg^-1 d^-2 (nBodyAlgorithm.hpp:55-61) applies unchanged.
  Orbital elements -> state vectors follows the procedure of dataset_converter/src/conversion.cpp:
  13-89 (Newton-Raphson Kepler solve, true anomaly, orbital-frame state, rotation by the
  argument of periapsis, inclination and node), vectorised over bodies.
* ``plummer``: G = M = a = 1, equal masses, positions and speeds by the Aarseth-Henon-Wielen
  (1974) sampling of the Plummer distribution function (cumulative-mass inversion for r,
  von Neumann rejection on q^2 (1-q^2)^(7/2) for v/v_esc), isotropic directions, radius cut off
  at 10 scale radii, shifted to the centre-of-mass frame.
"""

from __future__ import annotations

import numpy as np

MSUN_KG = 1.98847e30
G_SI = 6.67428e-11
AU_M = 1.49597870691e11
DAY_S = 86400.0


def reference_G() -> float:
    """G in AU^3 kg^-1 d^-2 computed the way nBodyAlgorithm.hpp:55-61 does."""
    G = 6.67428 * 10.0 ** -11
    meter_AU = 1.0 / (1.49597870691 * 10.0 ** 11)
    second_days = 1.0 / 86400
    return G * (meter_AU ** 3 / second_days ** 2)


def _loguniform(rng, lo, hi, n):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), size=n))


def kepler_to_state(a, e, inc, node, peri, mean_anom, mu):
    """Vectorised orbital elements -> heliocentric state vectors about a central mass at rest."""
    E = mean_anom.copy()
    for _ in range(30):  # Newton-Raphson on E - e sin E = M
        E = E - (E - e * np.sin(E) - mean_anom) / (1.0 - e * np.cos(E))
    nu = 2.0 * np.arctan2(np.sqrt(1.0 + e) * np.sin(E / 2.0), np.sqrt(1.0 - e) * np.cos(E / 2.0))
    rc = a * (1.0 - e * np.cos(E))
    ox, oy = rc * np.cos(nu), rc * np.sin(nu)
    k = np.sqrt(mu * a) / rc
    ovx, ovy = -k * np.sin(E), k * np.sqrt(1.0 - e * e) * np.cos(E)
    cw, sw, cO, sO, ci, si = np.cos(peri), np.sin(peri), np.cos(node), np.sin(node), np.cos(inc), np.sin(inc)
    r11, r12 = cw * cO - sw * ci * sO, -(sw * cO + cw * ci * sO)
    r21, r22 = cw * sO + sw * ci * cO, cw * ci * cO - sw * sO
    r31, r32 = sw * si, cw * si
    x, y, z = ox * r11 + oy * r12, ox * r21 + oy * r22, ox * r31 + oy * r32
    vx, vy, vz = ovx * r11 + ovy * r12, ovx * r21 + ovy * r22, ovx * r31 + ovy * r32
    return x, y, z, vx, vy, vz


def heliocentric_disc(n: int, seed: int = 1):
    """Returns dict of float64 arrays m (kg), x, y, z (AU), vx, vy, vz (AU/d) plus names/classes."""
    if n < 9:
        raise ValueError("the disc needs at least 9 bodies (central body + 8 planets)")
    rng = np.random.default_rng(seed)
    G = reference_G()
    mu = G * MSUN_KG
    n_small = n - 9
    m = np.empty(n)
    pos = np.zeros((3, n))
    vel = np.zeros((3, n))
    m[0] = MSUN_KG
    # planets: circular, coplanar
    a_p = rng.uniform(0.4, 30.0, size=8)
    m[1:9] = _loguniform(rng, 1.6e-7, 1e-3, 8) * MSUN_KG
    zeros = np.zeros(8)
    st = kepler_to_state(a_p, zeros, zeros, zeros, zeros, rng.uniform(0, 2 * np.pi, 8), mu)
    pos[:, 1:9] = st[:3]
    vel[:, 1:9] = st[3:]
    # small bodies
    a = rng.uniform(2.1, 3.3, n_small)
    e = rng.uniform(0.0, 0.2, n_small)
    inc = np.deg2rad(rng.uniform(0.0, 10.0, n_small))
    node, peri, ma = (rng.uniform(0, 2 * np.pi, n_small) for _ in range(3))
    m[9:] = _loguniform(rng, 1e-15, 1e-10, n_small) * MSUN_KG
    st = kepler_to_state(a, e, inc, node, peri, ma, mu)
    pos[:, 9:] = st[:3]
    vel[:, 9:] = st[3:]
    names = ["Sun"] + [f"planet{k}" for k in range(1, 9)] + [f"body{k}" for k in range(9, n)]
    classes = ["STA"] + ["PLA"] * 8 + ["MBA"] * n_small
    return {"m": m, "x": pos[0].copy(), "y": pos[1].copy(), "z": pos[2].copy(),
            "vx": vel[0].copy(), "vy": vel[1].copy(), "vz": vel[2].copy(),
            "names": names, "classes": classes, "G": G}


def plummer(n: int, seed: int = 1, r_cut: float = 10.0):
    """Plummer sphere, G = M = a = 1 (Henon units), equal masses 1/n."""
    rng = np.random.default_rng(seed)
    r = np.empty(0)
    while r.size < n:
        X = rng.uniform(0.0, 1.0, size=2 * n)
        rr = 1.0 / np.sqrt(X ** (-2.0 / 3.0) - 1.0)
        r = np.concatenate([r, rr[rr <= r_cut]])
    r = r[:n]

    def iso(k):
        cz = rng.uniform(-1.0, 1.0, k)
        ph = rng.uniform(0.0, 2 * np.pi, k)
        s = np.sqrt(1.0 - cz * cz)
        return np.stack([s * np.cos(ph), s * np.sin(ph), cz])

    pos = iso(n) * r
    q = np.empty(0)
    while q.size < n:
        qq = rng.uniform(0.0, 1.0, 4 * n)
        g = rng.uniform(0.0, 0.1, 4 * n)
        q = np.concatenate([q, qq[g < qq * qq * (1.0 - qq * qq) ** 3.5]])
    q = q[:n]
    vesc = np.sqrt(2.0) * (1.0 + r * r) ** -0.25
    vel = iso(n) * (q * vesc)
    pos -= pos.mean(axis=1, keepdims=True)
    vel -= vel.mean(axis=1, keepdims=True)
    m = np.full(n, 1.0 / n)
    return {"m": m, "x": pos[0].copy(), "y": pos[1].copy(), "z": pos[2].copy(),
            "vx": vel[0].copy(), "vy": vel[1].copy(), "vz": vel[2].copy(),
            "names": [f"p{k}" for k in range(n)], "classes": ["AST"] * n, "G": 1.0}


def write_csv(path: str, bodies: dict):
    """Writes the reference's input CSV (InputParser.cpp:7-32 column order)."""
    with open(path, "w") as f:
        f.write("id,name,class,mass,pos_x,pos_y,pos_z,vel_x,vel_y,vel_z\n")
        cols = [bodies[k] for k in ("m", "x", "y", "z", "vx", "vy", "vz")]
        for i in range(len(bodies["m"])):
            vals = ",".join(repr(float(c[i])) for c in cols)
            f.write(f"{i},{bodies['names'][i]},{bodies['classes'][i]},{vals}\n")


def disc_plummer_mix(n: int, seed: int = 1, plummer_mass_msun: float = 1e-3,
                     plummer_radius_au: float = 0.05, plummer_distance_au: float = 5.0):
    """Half heliocentric disc, half Plummer sphere (total mass 1e-3 Msun, scale radius 0.05 AU)
    centred 5 AU from the central body on a circular heliocentric orbit (bulk velocity along +y),
    with internal velocities from the Plummer distribution function. Masses in kg."""
    n_disc = n // 2
    d = heliocentric_disc(n_disc, seed)
    pl = plummer(n - n_disc, seed + 1000003)
    G = d["G"]
    m_pl = plummer_mass_msun * MSUN_KG
    a = plummer_radius_au
    vscale = np.sqrt(G * m_pl / a)  # Henon velocity unit for (G, M, a)
    vc = np.sqrt(G * MSUN_KG / plummer_distance_au)
    out = {"m": np.concatenate([d["m"], pl["m"] * m_pl]),
           "x": np.concatenate([d["x"], pl["x"] * a + plummer_distance_au]),
           "y": np.concatenate([d["y"], pl["y"] * a]),
           "z": np.concatenate([d["z"], pl["z"] * a]),
           "vx": np.concatenate([d["vx"], pl["vx"] * vscale]),
           "vy": np.concatenate([d["vy"], pl["vy"] * vscale + vc]),
           "vz": np.concatenate([d["vz"], pl["vz"] * vscale]),
           "names": d["names"] + [f"cluster{k}" for k in range(n - n_disc)],
           "classes": d["classes"] + ["AST"] * (n - n_disc), "G": G}
    return out

"""Seeded particle sources (host side; the same arrays feed the GPU and the oracle).

The reference spawns particles from point or surface sources with
theta = theta0 + U(-1,1)*expansion and a fixed phi
(include/Particle/PhysicsCore/ParticleDynamicUtils.hpp:52-97), then shifts
each one 0.05 mesh units along its direction, normalised by its largest
component (src/Particle/ParticleDisplacer.cpp:20-35). The workloads use the
distributions the benchmark configurations name instead: a uniform disk or
plate, a uniform cone or a cosine law about the normal, and monoenergetic or
Thompson energies, with the same displacement rule.
"""
from __future__ import annotations

import numpy as np

EV_J = 1.60217733000001e-19  # Constants.hpp eV_J
DISPLACEMENT = 0.05e-3  # 0.05 mesh units (mm) in metres


def _frame(normal):
    n = np.asarray(normal, float)
    n = n / np.linalg.norm(n)
    t = np.array([1.0, 0.0, 0.0]) if abs(n[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    e1 = np.cross(n, t)
    e1 /= np.linalg.norm(e1)
    e2 = np.cross(n, e1)
    return e1, e2, n


def disk_points(rng, n, centre, radius, normal=(0, 0, 1)):
    """Uniform over a disk: r = R sqrt(u), psi = 2 pi u'."""
    e1, e2, _ = _frame(normal)
    r = radius * np.sqrt(rng.random(n))
    psi = 2.0 * np.pi * rng.random(n)
    return np.asarray(centre, float) + (r * np.cos(psi))[:, None] * e1 + (r * np.sin(psi))[:, None] * e2


def rect_points(rng, n, xlim, ylim, z):
    x = xlim[0] + (xlim[1] - xlim[0]) * rng.random(n)
    y = ylim[0] + (ylim[1] - ylim[0]) * rng.random(n)
    return np.stack([x, y, np.full(n, float(z))], axis=1)


def cone_directions(rng, n, half_angle, normal=(0, 0, 1)):
    """Uniform in solid angle inside a cone: cos(theta) = 1 - u (1 - cos(half_angle))."""
    e1, e2, nn = _frame(normal)
    ct = 1.0 - rng.random(n) * (1.0 - np.cos(half_angle))
    st = np.sqrt(np.maximum(0.0, 1.0 - ct * ct))
    ph = 2.0 * np.pi * rng.random(n)
    return (st * np.cos(ph))[:, None] * e1 + (st * np.sin(ph))[:, None] * e2 + ct[:, None] * nn


def cosine_directions(rng, n, normal=(0, 0, 1)):
    """Lambert (cosine) law about the normal: sin(theta) = sqrt(u)."""
    e1, e2, nn = _frame(normal)
    st = np.sqrt(rng.random(n))
    ct = np.sqrt(np.maximum(0.0, 1.0 - st * st))
    ph = 2.0 * np.pi * rng.random(n)
    return (st * np.cos(ph))[:, None] * e1 + (st * np.sin(ph))[:, None] * e2 + ct[:, None] * nn


def thompson_energies(rng, n, binding_ev, emax_ev):
    """f(E) ~ E/(E+U)^3 truncated at E_max, by inverse CDF:
    CDF = (E/(E+U))^2 / (Emax/(Emax+U))^2, so E = U s/(1-s) with
    s = sqrt(u) Emax/(Emax+U). Returns joules."""
    U, Em = float(binding_ev), float(emax_ev)
    s = np.sqrt(rng.random(n)) * (Em / (Em + U))
    return U * s / (1.0 - s) * EV_J


def displace(pos, dirs, amount=DISPLACEMENT):
    """ParticleDisplacer rule: shift by dir / max|dir_k| * amount."""
    m = np.max(np.abs(dirs), axis=1, keepdims=True)
    m = np.where(m < np.finfo(float).eps, np.inf, m)
    return pos + dirs / m * amount


def make_particles(seed, n, mass, *, source="disk", centre=(0, 0, 0), radius=0.02, xlim=None, ylim=None, z=0.0,
                   normal=(0, 0, 1), directions="cone", half_angle=np.deg2rad(30.0), energy="mono",
                   energy_ev=1.0, binding_ev=4.9, emax_ev=50.0):
    """Positions (n,3) and velocities (n,3) in SI units."""
    rng = np.random.default_rng(seed)
    if source == "disk":
        pos = disk_points(rng, n, centre, radius, normal)
    elif source == "plate":
        pos = rect_points(rng, n, xlim, ylim, z)
    else:
        raise ValueError(source)
    if directions == "cone":
        d = cone_directions(rng, n, half_angle, normal)
    elif directions == "cosine":
        d = cosine_directions(rng, n, normal)
    else:
        raise ValueError(directions)
    if energy == "mono":
        E = np.full(n, energy_ev * EV_J)
    elif energy == "thompson":
        E = thompson_energies(rng, n, binding_ev, emax_ev)
    else:
        raise ValueError(energy)
    speed = np.sqrt(2.0 * E / mass)
    pos = displace(pos, d)
    return np.ascontiguousarray(pos), np.ascontiguousarray(d * speed[:, None])

"""Particle sources sampled on the device (spg_generate_particles) against
the sampling laws of the host sources (start_gb300/sources.py): the two draw
different random streams, so the laws are checked with Kolmogorov-Smirnov
tests (p > 1e-3 on 2e5 particles) and the displacement rule exactly.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EV_J = 1.60217733000001e-19
TI_MASS = 7.95e-26


def _engine(cells=10):
    from start_gb300 import StartPIC
    from start_gb300.workloads import workload0

    w = workload0(n_particles=10, cells=cells)
    return StartPIC(w.mesh, w.params)


def _undisplace(pos, d, amount):
    m = np.max(np.abs(d), axis=1, keepdims=True)
    return pos - d / m * amount


def test_disk_cone_mono(built):
    from scipy import stats

    e = _engine()
    n, R, alpha = 200_000, 0.02, np.deg2rad(30.0)
    c = np.array([0.05, 0.05, 0.0])
    e.generate_particles(n, shape="disk", directions="cone", energy="mono", centre=c, radius=R, half_angle=alpha,
                         energy_ev=1.0, seed=7)
    p = e.particles()
    v = p["vel"]
    speed = np.linalg.norm(v, axis=1)
    assert np.allclose(speed, np.sqrt(2 * EV_J / TI_MASS), rtol=1e-12)
    d = v / speed[:, None]
    x0 = _undisplace(p["pos"], d, 0.05e-3)
    assert np.abs(x0[:, 2]).max() <= 1e-15  # the disk lies in z = 0
    r2 = ((x0[:, 0] - c[0]) ** 2 + (x0[:, 1] - c[1]) ** 2) / R**2
    assert r2.max() <= 1.0 + 1e-12
    assert stats.kstest(r2, "uniform").pvalue > 1e-3  # r = R sqrt(u)
    psi = np.arctan2(x0[:, 1] - c[1], x0[:, 0] - c[0])
    assert stats.kstest((psi + np.pi) / (2 * np.pi), "uniform").pvalue > 1e-3
    ct = d[:, 2]
    lo = np.cos(alpha)
    assert ct.min() >= lo - 1e-12
    assert stats.kstest((ct - lo) / (1 - lo), "uniform").pvalue > 1e-3  # uniform in solid angle
    assert (p["tet"] >= 0).all() and not (p["flags"] & 2).any()
    e.close()


def test_rect_cosine_thompson(built):
    from scipy import stats

    e = _engine()
    n, U, Em = 200_000, 4.9, 50.0
    e.generate_particles(n, shape="rect", directions="cosine", energy="thompson", xlim=(0.02, 0.08),
                         ylim=(0.03, 0.07), z=0.0, binding_ev=U, emax_ev=Em, seed=11)
    p = e.particles()
    v = p["vel"]
    speed = np.linalg.norm(v, axis=1)
    d = v / speed[:, None]
    x0 = _undisplace(p["pos"], d, 0.05e-3)
    assert stats.kstest((x0[:, 0] - 0.02) / 0.06, "uniform").pvalue > 1e-3
    assert stats.kstest((x0[:, 1] - 0.03) / 0.04, "uniform").pvalue > 1e-3
    st2 = 1.0 - d[:, 2] ** 2
    assert stats.kstest(st2, "uniform").pvalue > 1e-3  # Lambert: sin^2(theta) uniform
    E = 0.5 * TI_MASS * speed**2 / EV_J
    assert E.max() <= Em * (1 + 1e-9)
    smax = Em / (Em + U)
    cdf = (E / (E + U)) ** 2 / smax**2
    assert stats.kstest(cdf, "uniform").pvalue > 1e-3
    e.close()


def test_generation_is_reproducible_and_runs(built):
    e = _engine()
    e.generate_particles(50_000, seed=3)
    a = e.particles()
    e.generate_particles(50_000, seed=3)
    b = e.particles()
    e.generate_particles(50_000, seed=4)
    c = e.particles()
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])
    assert not np.array_equal(a["pos"], c["pos"])
    st = e.run(20)
    assert st["particle_steps"] > 0
    e.close()


def test_generated_particles_match_the_oracle_run(built):
    """Device-sampled particles, run on the GPU and (copied) on the oracle:
    the collisionless run agrees bit for bit, as for host-given inputs."""
    import oracle

    from start_gb300.workloads import workload0

    w = workload0(n_particles=10, cells=10, collisions=False)
    w.params["cg_rtol"] = 1e-12
    from start_gb300 import StartPIC

    g = StartPIC(w.mesh, w.params)
    g.generate_particles(4000, seed=5)
    p0 = g.particles()
    o = oracle.Oracle(w.mesh, w.params)
    o.set_particles(p0["pos"], p0["vel"])
    g.run(100)
    o.run(100)
    pg, po = g.particles(), o.particles()
    assert np.array_equal(pg["tet"], po["tet"])
    assert np.array_equal(pg["flags"], po["flags"])
    assert np.array_equal(g.triangle_counts(), o.triangle_counts())
    g.close()
    o.close()

"""The reference's own particle sources on the device and continuous
injection (spg_generate_particles / spg_inject_particles):

* a point source with the fan law (ParticleDynamicUtils::calculateVelocityFromEnergy_eV):
  every particle at the centre plus the displacement, azimuth fixed at the
  normal's, polar angle uniform in theta0 +- expansion (KS test, p > 1e-3);
* a surface-cell source (ParticleGenerator::fromSurfaceSource): the count
  split evenly over the cells, the remainder one each, each particle at its
  cell's centre moving along the cell normal (expansion 0);
* injection mid-run (ModelingMainDriver::_spawnParticles): the set grows with
  the next ids, the earlier particles are untouched by the injection, a run
  repeats bit for bit, and tracking continues for the tracked ids."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EV_J = 1.60217733000001e-19
TI_MASS = 7.95e-26


def _engine(precision=0, collisions=False):
    from start_gb300 import StartPIC
    from start_gb300.workloads import workload0

    w = workload0(n_particles=10, cells=10, collisions=collisions)
    w.params.update(precision=precision)
    return StartPIC(w.mesh, w.params)


def test_point_source_fan_law(built):
    from scipy import stats

    e = _engine()
    c = np.array([0.05, 0.05, 0.02])
    th0, ex = np.deg2rad(30.0), np.deg2rad(10.0)
    phi0 = np.deg2rad(40.0)
    nrm = [np.sin(th0) * np.cos(phi0), np.sin(th0) * np.sin(phi0), np.cos(th0)]
    n = 100_000
    e.generate_particles(n, shape="point", directions="fan", centre=c, normal=nrm, expansion=ex, energy_ev=2.0,
                         seed=9)
    p = e.particles()
    v = p["vel"]
    speed = np.linalg.norm(v, axis=1)
    assert np.allclose(speed, np.sqrt(2 * 2.0 * EV_J / TI_MASS), rtol=1e-12)
    d = v / speed[:, None]
    theta = np.arccos(np.clip(d[:, 2], -1, 1))
    phi = np.arctan2(d[:, 1], d[:, 0])
    assert np.allclose(phi, phi0, atol=1e-12)
    assert theta.min() >= th0 - ex - 1e-12 and theta.max() <= th0 + ex + 1e-12
    assert stats.kstest((theta - (th0 - ex)) / (2 * ex), "uniform").pvalue > 1e-3
    m = np.max(np.abs(d), axis=1, keepdims=True)
    x0 = p["pos"] - d / m * 0.05e-3
    assert np.abs(x0 - c).max() <= 1e-15
    e.close()


def test_surface_cells_source(built):
    e = _engine()
    cells = np.array([[0.02, 0.03, 0.0, 0, 0, 1], [0.07, 0.05, 0.0, 0, 0, 2], [0.05, 0.08, 0.0, 1, 0, 1]], float)
    n = 10_001
    e.generate_particles(n, shape="cells", directions="fan", cells=cells, expansion=0.0, energy_ev=1.0, seed=3)
    p = e.particles()
    v = p["vel"]
    d = v / np.linalg.norm(v, axis=1)[:, None]
    m = np.max(np.abs(d), axis=1, keepdims=True)
    x0 = p["pos"] - d / m * 0.05e-3
    counts = []
    for c in cells:
        at = np.all(np.abs(x0 - c[:3]) <= 1e-15, axis=1)
        nrm = c[3:] / np.linalg.norm(c[3:])
        assert np.abs(d[at] - nrm).max() <= 1e-12
        counts.append(int(at.sum()))
    assert sum(counts) == n
    assert sorted(counts) == [3333, 3334, 3334]
    e.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_injection_mid_run(built, precision):
    out = []
    for _ in range(2):
        e = _engine(precision)
        e.generate_particles(5000, seed=5, centre=(0.05, 0.05, 0.0))
        e.track([0, 7], capacity=100)
        e.run(12)
        before = e.particles()
        e.inject_particles(2000, shape="point", directions="fan", centre=(0.05, 0.05, 0.01), normal=(0, 0, 1),
                           expansion=0.3, seed=11)
        assert e.n_particles == 7000
        mid = e.particles()
        assert np.array_equal(mid["pos"][:5000], before["pos"])
        assert np.array_equal(mid["vel"][:5000], before["vel"])
        e.run(12)
        after = e.particles()
        assert not np.array_equal(after["pos"][5000:], mid["pos"][5000:])
        assert e.stats()["n_particles"] == 7000
        tr = e.tracks()
        assert len(tr[0]) >= 20 or (after["flags"][0] & 3)
        out.append(after)
        e.close()
    assert np.array_equal(out[0]["pos"], out[1]["pos"]) and np.array_equal(out[0]["vel"], out[1]["vel"])

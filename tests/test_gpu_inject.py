"""The reference's own particle sources on the device and continuous
injection (spg_generate_particles / spg_inject_particles):

* a point source with the fan law (ParticleDynamicUtils::calculateVelocityFromEnergy_eV):
  azimuth fixed at the normal's, polar angle uniform in theta0 +- expansion
  (KS test, p > 1e-3); every particle at the centre plus one shift along the
  source's direction (ParticleDisplacer::displaceParticlesFromPointSources),
  whatever its own direction;
* a surface-cell source (ParticleGenerator::fromSurfaceSource): the count
  split evenly over the cells, the remainder one each, each particle at its
  cell's centre plus the cell's shift along its normal, bit for bit
  (displaceParticlesFromSurfaceSources), moving along the cell normal
  (expansion 0), or spread about it (expansion > 0) with the same shift;
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
    # one shift for the whole source, along its direction (theta0, phi0)
    assert (p["pos"] == p["pos"][0]).all()
    s = p["pos"][0] - c
    dir0 = np.array([np.sin(th0) * np.cos(phi0), np.sin(th0) * np.sin(phi0), np.cos(th0)])
    assert np.allclose(s, dir0 / np.abs(dir0).max() * 0.05e-3, rtol=1e-12, atol=1e-18)
    # the particles' own directions spread by +-10 deg: a per-particle shift would differ
    own = d / np.max(np.abs(d), axis=1, keepdims=True) * 0.05e-3
    assert np.abs(own - s).max() > 1e-6
    e.close()


def test_surface_cells_source(built):
    e = _engine()
    cells = np.array([[0.02, 0.03, 0.0, 0, 0, 1], [0.07, 0.05, 0.0, 0, 0, 2], [0.05, 0.08, 0.0, 1, 0, 1]], float)
    n = 10_001
    for ex in (0.0, np.deg2rad(20.0)):
        e.generate_particles(n, shape="cells", directions="fan", cells=cells, expansion=ex, energy_ev=1.0, seed=3)
        p = e.particles()
        v = p["vel"]
        d = v / np.linalg.norm(v, axis=1)[:, None]
        counts = []
        for c in cells:
            # ParticleDisplacer: the cell's normal as given over its largest
            # component, times 0.05 mm, added to the centre
            at = np.all(p["pos"] == c[:3] + (c[3:] / np.abs(c[3:]).max()) * 0.05e-3, axis=1)
            nrm = c[3:] / np.linalg.norm(c[3:])
            if ex == 0.0:
                assert np.abs(d[at] - nrm).max() <= 1e-12
            else:
                assert np.abs(d[at] - nrm).max() > 0.1  # spread about the normal, same shift
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

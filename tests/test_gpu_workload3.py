"""Workload 3 (jittered box with two internal plate electrodes) against the
CPU oracle, at a reduced size: 40 x 40 x 20 Kuhn cells jittered by +-0.2 h
(192,000 tets), plates at z = 20 mm (0 V) and 80 mm (-300 V), Ti+ from the
lower plate.

* FP64, no gas: every tet id and flag identical, positions within 1e-9
  relative, triangle counters identical (the plates are internal surfaces:
  a particle settles on the face of whichever tet it leaves through).
* FP64 with VSS argon: surface histograms agree (chi-square, p > 0.01).
* The mixed form against the FP64 form with VSS on the same Philox streams:
  L1 surface-histogram error below 1 %.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _w3(n, precision=0, collisions=True, gas_scale=1.0, **kw):
    from start_gb300.workloads import workload3

    w = workload3(n_particles=n, cells=(40, 40, 20), steps=1000)
    w.params.update(precision=precision, cg_rtol=1e-12, **kw)
    if not collisions:
        w.params["collision_model"] = 0
    w.params["gas_concentration"] *= gas_scale
    return w


def _bins(w):
    """Coarse surface bins: tag x 8 x 8 patches in the plane of the surface."""
    cen = w.mesh.triangle_centroids()
    ij = np.floor(cen / 0.025).astype(int).clip(0, 7)
    key = w.mesh.tri_tag * 1000 + (ij * np.array([64, 8, 1])).sum(1)
    return np.unique(key, return_inverse=True)[1]


def _chi2_p(a, b):
    from scipy import stats

    keep = (a + b) > 0
    a, b = a[keep], b[keep]
    k1, k2 = np.sqrt(b.sum() / a.sum()), np.sqrt(a.sum() / b.sum())
    chi2 = np.sum((k1 * a - k2 * b) ** 2 / (a + b))
    return stats.chi2.sf(chi2, len(a) - 1)


def test_w3_collisionless_bit_exact(built):
    import oracle
    from start_gb300 import StartPIC

    w = _w3(5000, collisions=False)
    g, o = StartPIC(w.mesh, w.params), oracle.Oracle(w.mesh, w.params)
    for e in (g, o):
        e.set_particles(w.pos, w.vel)
    sg, so = g.run(800), o.run(800)
    pg, po = g.particles(), o.particles()
    assert np.array_equal(pg["tet"], po["tet"])
    assert np.array_equal(pg["flags"], po["flags"])
    rel = np.abs(pg["pos"] - po["pos"]) / np.maximum(np.abs(po["pos"]), 1e-3)
    assert rel.max() <= 1e-9
    cg, co = g.triangle_counts(), o.triangle_counts()
    assert np.array_equal(cg, co)
    plate_hi = w.mesh.tri_tag == 8
    assert cg[plate_hi].sum() > 1000  # most ions land on the -300 V plate
    assert sg["particle_steps"] == so["particle_steps"]
    g.close()
    o.close()


def test_w3_vss_histogram(built):
    import oracle
    from start_gb300 import StartPIC

    w = _w3(20000)  # argon 2 Pa: about two collisions per ion
    g, o = StartPIC(w.mesh, w.params), oracle.Oracle(w.mesh, w.params)
    for e in (g, o):
        e.set_particles(w.pos, w.vel)
    sg, so = g.run(1000), o.run(1000)
    assert sg["collisions"] > 20000 and sg["n_settled"] > 10000
    assert abs(sg["collisions"] - so["collisions"]) <= 0.05 * so["collisions"]
    inv = _bins(w)
    a = np.bincount(inv, weights=g.triangle_counts().astype(float))
    b = np.bincount(inv, weights=o.triangle_counts().astype(float))
    assert _chi2_p(a, b) > 0.01
    g.close()
    o.close()


@pytest.mark.parametrize("precond", [0, 1])
def test_w3_mixed_vs_fp64(built, precond):
    from start_gb300 import StartPIC

    counts = []
    for precision in (0, 1):
        w = _w3(20000, precision=precision, preconditioner=precond)
        e = StartPIC(w.mesh, w.params)
        e.set_particles(w.pos, w.vel)
        e.run(1000)
        counts.append(e.triangle_counts().astype(float))
        e.close()
    c64, c32 = counts
    l1 = np.abs(c32 - c64).sum() / c64.sum()
    assert c64.sum() > 10000 and l1 <= 0.01, l1

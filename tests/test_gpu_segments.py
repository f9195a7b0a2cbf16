"""Segmented steps of the mixed form (spg_set_step_segments) against one
launch per step.

A segment runs every step between two events of the time loop (a solve, a
re-sort, the end of the call) with each particle in registers until a move
needs the exact walk; the walk runs batched and the particle resumes from
the next step. The operations per particle and step are those of the single
step, so the bar is identity: every position, velocity, tet id and flag,
every triangle counter and every cumulative counter equal, bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

VHS = 2


def _pair(w, seg):
    from start_gb300 import StartPIC

    out = []
    for m in (1, seg):
        g = StartPIC(w.mesh, dict(w.params, precision=1))
        g.set_step_segments(m)
        g.set_particles(w.pos, w.vel)
        out.append(g)
    return out


def _same(a, b, stats_a, stats_b):
    pa, pb = a.particles(), b.particles()
    for k in ("pos", "vel", "tet", "flags"):
        assert np.array_equal(pa[k], pb[k]), k
    assert np.array_equal(a.triangle_counts(), b.triangle_counts())
    for k in ("step", "n_alive", "n_settled", "n_lost", "particle_steps", "collisions", "crossings", "cg_iters_total"):
        assert stats_a[k] == stats_b[k], (k, stats_a[k], stats_b[k])


@pytest.mark.parametrize("model", [0, 1, 3], ids=["collisionless", "hs", "vss"])
def test_run_segments_identical_w0(built, model):
    """Workload 0 geometry, 200 steps (solve every 10, re-sort every 20)."""
    from start_gb300.workloads import workload0

    collisions = model != 0
    w = workload0(n_particles=20000, collisions=collisions, steps=200)
    w.params.update(cg_rtol=1e-12, resort_every=20)
    if collisions:
        w.params.update(collision_model=model)
        w.params["gas_concentration"] *= 50.0
    a, b = _pair(w, 32)
    sa, sb = a.run(200), b.run(200)
    assert sa["crossings"] > 2000 and sa["n_settled"] > 1000, sa
    if collisions:
        assert sa["collisions"] > 10000
    _same(a, b, sa, sb)
    a.close()
    b.close()


@pytest.mark.parametrize("seg", [3, 32])
def test_run_segments_identical_vhs_reduced_w1(built, seg):
    """Thompson energies, cosine directions, VHS argon (x10): 300 steps;
    segments of 3 split every 10-step span into 3 + 3 + 3 + 1."""
    from start_gb300.workloads import workload1

    w = workload1(n_particles=100000, cells=20, steps=300)
    w.params.update(cg_rtol=1e-12, collision_model=VHS)
    w.params["gas_concentration"] *= 10.0
    a, b = _pair(w, seg)
    sa, sb = a.run(150), b.run(150)
    _same(a, b, sa, sb)
    sa, sb = a.run(150), b.run(150)
    assert sa["collisions"] > 1000 and sa["crossings"] > 100000, sa
    _same(a, b, sa, sb)
    a.close()
    b.close()


def test_process_segments_identical(built):
    """spg_process over re-sort boundaries, from a given potential (no solve):
    47 steps with re-sorts every 20 steps (segments 20, 20, 7 after the
    first step's own)."""
    from start_gb300.workloads import workload0

    w = workload0(n_particles=30000, collisions=True, steps=47)
    w.params.update(resort_every=20)
    w.params["gas_concentration"] *= 50.0
    a, b = _pair(w, 32)
    phi = np.random.default_rng(5).uniform(-300.0, 300.0, a.n_nodes)
    for g in (a, b):
        g.set_potential(phi)
    a.process(1)
    b.process(1)
    sa, sb = a.process(46), b.process(46)
    assert sa["crossings"] > 1000
    _same(a, b, sa, sb)
    a.close()
    b.close()


def test_segment_setting_checked(built):
    from start_gb300 import StartPIC
    from start_gb300.engine import PICBaseException
    from start_gb300.workloads import workload0

    w = workload0(n_particles=10, collisions=False, steps=1)
    g = StartPIC(w.mesh, dict(w.params, precision=1))
    for bad in (0, -3, 65):
        with pytest.raises(PICBaseException):
            g.set_step_segments(bad)
    g.set_step_segments(64)
    g.close()


def test_box_inside_mesh(built):
    """A modelling box inside the mesh (bbox_expansion 0.8: [0.01, 0.09]^3 of the
    0.1 m cube). Tets that reach outside it carry no interior flag, so the
    mixed step runs the per-step box test there; particles that leave the box
    stop. Segments stay identical to one launch per step, and the particles
    stopped outside the box are those the FP64 oracle stops."""
    import oracle
    from start_gb300 import StartPIC
    from start_gb300.workloads import workload0

    w = workload0(n_particles=10, collisions=False, steps=100)
    w.params.update(bbox_expansion=0.8, cg_rtol=1e-12)
    rng = np.random.default_rng(9)
    n = 20000
    pos = rng.uniform(0.02, 0.08, size=(n, 3))
    d = rng.normal(size=(n, 3))
    vel = 1.5e4 * d / np.linalg.norm(d, axis=1, keepdims=True)
    runs = []
    for m in (1, 32):
        g = StartPIC(w.mesh, dict(w.params, precision=1))
        g.set_step_segments(m)
        g.set_particles(pos, vel)
        runs.append((g, g.run(100)))
    (a, sa), (b, sb) = runs
    _same(a, b, sa, sb)
    o = oracle.Oracle(w.mesh, dict(w.params, precision=0))
    o.set_particles(pos, vel)
    o.run(100)

    def stopped(p):
        alive = (p["flags"] & 3) == 0
        out = ((p["pos"] < 0.01) | (p["pos"] > 0.09)).any(axis=1)
        return alive & out

    sm, so = stopped(a.particles()), stopped(o.particles())
    assert so.sum() > 500, so.sum()
    assert (sm ^ so).sum() <= 0.005 * so.sum() + 2, ((sm ^ so).sum(), so.sum())
    a.close()
    b.close()

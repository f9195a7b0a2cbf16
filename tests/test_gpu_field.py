"""The per-tet field of the run solves: after a solve inside a run only the
tets holding particles are computed (the deposit lists them), and a walk
computes a tet when a particle enters it. The field read back after a run
(which completes the other tets) must equal the field of a full update from
the same potential bit for bit, for both forms; the push of every particle
used the same values, which the collisionless parity runs check against the
oracle (tests/test_gpu_parity.py)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_lazy_field_equals_full_update(built, precision):
    from start_gb300 import StartPIC
    from start_gb300.workloads import workload0

    w = workload0(n_particles=20000, cells=20, collisions=False)
    w.params.update(precision=precision, preconditioner=2, cg_rtol=1e-12)
    g = StartPIC(w.mesh, w.params)
    g.set_particles(w.pos, w.vel)
    g.run(45)
    e_run = g.efield()
    phi = g.potential()
    g.close()
    f = StartPIC(w.mesh, w.params)
    f.set_particles(w.pos, w.vel)
    f.set_potential(phi)
    e_full = f.efield()
    f.close()
    assert np.array_equal(e_run, e_full)
    assert np.abs(e_full).max() > 0.0


def test_run_after_field_readback_continues_identically(built):
    """Reading the field back mid-run (which completes every tet) does not
    change the run: the completed tets get the values the walks would give."""
    from start_gb300 import StartPIC
    from start_gb300.workloads import workload0

    w = workload0(n_particles=20000, cells=20, collisions=False)
    w.params.update(preconditioner=2, cg_rtol=1e-12)
    out = []
    for read in (False, True):
        g = StartPIC(w.mesh, w.params)
        g.set_particles(w.pos, w.vel)
        g.run(25)
        if read:
            g.efield()
        g.run(30)
        out.append(g.particles())
        g.close()
    a, b = out
    assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["tet"], b["tet"])

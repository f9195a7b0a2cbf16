"""Solves inside spg_run do not wait for the host: their scalars are read when
the call ends. A run whose solves hit cg_max_iter still runs every step and
then reports SPG_E_NOT_CONVERGED (the reference's loop logs the failure and
goes on: src/FiniteElementMethod/Solvers/MatrixEquationSolver.cpp:405-412),
with the statistics of every solve; a converging run reports them too.
"""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
@pytest.mark.parametrize("precond", [1, 2], ids=["amg", "amg32"])
def test_run_reports_capped_solves_at_the_end(built, precond, precision):
    from start_gb300 import StartPIC
    from start_gb300 import _native as N
    from start_gb300.engine import PICBaseException
    from start_gb300.workloads import workload0

    w = workload0(n_particles=5000, collisions=False, steps=25)
    # a tolerance no FP64 residual reaches, so every solve stops at the cap (on this
    # small mesh the AMG-preconditioned solves reach 1e-14 in one iteration)
    w.params.update(preconditioner=precond, precision=precision, cg_max_iter=1, cg_rtol=1e-30)
    g = StartPIC(w.mesh, w.params)
    g.set_particles(w.pos, w.vel)
    with pytest.raises(PICBaseException) as e:
        g.run(25)
    assert e.value.code == N.SPG_E_NOT_CONVERGED
    assert "did not converge" in str(e.value)
    st = g.stats()
    assert st["step"] == 25 and st["cg_solves"] == 3, st
    g.close()

    w.params.update(cg_max_iter=20000, cg_rtol=1e-10)
    g = StartPIC(w.mesh, w.params)
    g.set_particles(w.pos, w.vel)
    st = g.run(25)
    assert st["step"] == 25 and st["cg_solves"] == 3 and st["cg_iters_total"] >= 3, st
    assert 0.0 < st["cg_relres_last"] <= 1e-10, st
    g.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_run_with_more_solves_than_held_records(built, precision):
    """A solve every step for 70 steps: more solves than the run holds back
    (64), so the records are read in the middle of the run as well; every
    solve is counted once."""
    from start_gb300 import StartPIC
    from start_gb300.workloads import workload0

    w = workload0(n_particles=2000, collisions=False, steps=70)
    w.params.update(preconditioner=2, precision=precision, poisson_every=1, cg_rtol=1e-10)
    g = StartPIC(w.mesh, w.params)
    g.set_particles(w.pos, w.vel)
    st = g.run(70)
    assert st["step"] == 70 and st["cg_solves"] == 70, st
    assert st["cg_iters_total"] >= 70 and 0.0 < st["cg_relres_last"] <= 1e-10, st
    g.close()

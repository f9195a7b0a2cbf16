"""The smoothed-aggregation AMG preconditioner (SPG_PRECOND_AMG) of the FP64
Poisson PCG against the Jacobi-preconditioned solve and the CPU oracle.

Tolerances: both solves run to ||r|| <= 1e-13 ||b||; their potentials then
agree within 1e-8 of max|phi|, and the oracle's (Jacobi PCG) likewise. A
collisionless run with the AMG solve keeps every particle's tet and flags of
the oracle run and its positions within 1e-7 relative (the potentials differ
at the solver tolerance, not bit for bit).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _w(cells, n, collisions=False, precond=1, rtol=1e-13, **kw):
    from start_gb300.workloads import workload0

    w = workload0(n_particles=n, collisions=collisions, cells=cells)
    w.params.update(cg_rtol=rtol, preconditioner=precond, **kw)
    return w


def _solve_after_gather(w):
    from start_gb300 import StartPIC

    e = StartPIC(w.mesh, w.params)
    e.set_particles(w.pos, w.vel)
    rho = e.gather()
    phi = e.solve(rho)
    st = e.stats()
    return e, phi, st


@pytest.mark.parametrize("cells", [10, 40])
def test_amg_solution_matches_jacobi(built, cells):
    wa = _w(cells, 20000, precond=1)
    wj = _w(cells, 20000, precond=0)
    ea, pa, sa = _solve_after_gather(wa)
    ej, pj, sj = _solve_after_gather(wj)
    scale = np.abs(pj).max()
    assert np.abs(pa - pj).max() <= 1e-8 * scale
    assert sa["cg_relres_last"] <= 1e-13 and sj["cg_relres_last"] <= 1e-13
    # cold solves: the V-cycle needs a small fraction of the Jacobi iterations
    assert sa["cg_iters_last"] * 5 <= sj["cg_iters_last"], (sa["cg_iters_last"], sj["cg_iters_last"])
    ea.close()
    ej.close()


def test_amg_iterations_do_not_grow_with_the_mesh(built):
    its = []
    for cells in (20, 40, 80):
        w = _w(cells, 20000, rtol=1e-10)
        e, phi, st = _solve_after_gather(w)
        its.append(st["cg_iters_last"])
        e.close()
    assert max(its) <= 30 and its[-1] <= its[0] + 8, its


def test_amg_potential_matches_oracle(built):
    import oracle

    w = _w(10, 5000)
    e, phi, st = _solve_after_gather(w)
    o = oracle.Oracle(w.mesh, w.params)
    o.set_particles(w.pos, w.vel)
    rho_o = o.gather()
    phi_o, _, _ = o.solve(rho_o)
    assert np.abs(phi - phi_o).max() <= 1e-8 * np.abs(phi_o).max()
    e.close()
    o.close()


def test_amg_collisionless_run_matches_oracle(built):
    import oracle
    from start_gb300 import StartPIC

    w = _w(10, 4000, rtol=1e-12)
    g = StartPIC(w.mesh, w.params)
    o = oracle.Oracle(w.mesh, w.params)
    g.set_particles(w.pos, w.vel)
    o.set_particles(w.pos, w.vel)
    g.run(60)
    o.run(60)
    pg, po = g.particles(), o.particles()
    assert np.array_equal(pg["tet"], po["tet"])
    assert np.array_equal(pg["flags"], po["flags"])
    rel = np.abs(pg["pos"] - po["pos"]) / np.maximum(np.abs(po["pos"]), 1e-3)
    assert rel.max() <= 1e-7
    g.close()
    o.close()


def test_amg_adjoint_cg_matches_jacobi(built):
    from start_gb300.adjoint import LandingProblem

    V = np.array([0.0, 0.0, 0.0, 0.0, 0.0, 500.0])
    a0 = np.deg2rad(30.0)
    out = []
    for precond in (0, 1):
        p = LandingProblem(n_particles=3000, steps=400, collisions=False, cg_rtol=1e-13, preconditioner=precond)
        p.target = np.array([0.05, 0.05, 0.0])
        J = p.forward(V, a0)
        dV, da, iters = p.backward()
        out.append((J, dV, da, iters))
        p.close()
    (Jj, dVj, daj, itj), (Ja, dVa, daa, ita) = out
    assert abs(Ja - Jj) <= 1e-9 * Jj
    assert np.abs(dVa - dVj).max() <= 1e-6 * np.abs(dVj).max()
    assert abs(daa - daj) <= 1e-6 * abs(daj)
    assert ita * 5 <= itj

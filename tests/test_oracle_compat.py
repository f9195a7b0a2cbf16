"""The oracle's reference-behaviour switches (CPU). Each reproduces one
behaviour of the reference's own time loop that the build changes on purpose,
and each test pins the switch to the behaviour of the reference code it cites:

  PUSH_NEVER        src/Particle/Particle.cpp:113-155 (copies get new ids) and
                    src/Geometry/Mesh/Cubic/CubicGrid.cpp:149-158 (lookup by id)
  E_SIGN_SCALE      src/Geometry/Mesh/Volumetric/VolumetricMesh.cpp:371-375,398
  RHS_RAW_RHO       src/ParticleInCellEngine/ChargeDensityEquationSolver.cpp:17-29,
                    src/FiniteElementMethod/Solvers/MatrixEquationSolver.cpp:5-11
  DEPOSIT_VOLAVG    src/ParticleInCellEngine/NodeChargeDensityProcessor.cpp:25-113
  CLOSED_TETS       src/Geometry/Mesh/Volumetric/VolumetricMesh.cpp:23-33,
                    NodeChargeDensityProcessor.cpp:52-55
  SOLVE_EVERY_STEP  src/ModelingMainDriver.cpp:146-161
  MIXED_UNITS       src/Particle/Particle.cpp:157-165

The last test runs workload 0 with every switch on (the reference's own loop)
beside the build's loop and checks the differences the switches imply.
"""
import numpy as np
import pytest

import oracle
from start_gb300 import mesh as M
from start_gb300.workloads import workload0


def _w(n=4000, collisions=False, **kw):
    w = workload0(n_particles=n, collisions=collisions, steps=200)
    w.params.update(cg_rtol=1e-12, **kw)
    return w


def _engine(w, flags=0, **kw):
    o = oracle.Oracle(w.mesh, w.params)
    if flags:
        o.set_ref_compat(flags, **kw)
    return o


def test_unknown_flag_rejected():
    o = _engine(_w(10))
    with pytest.raises(ValueError):
        o.set_ref_compat(1 << 12)
    with pytest.raises(ValueError):
        o.set_ref_compat(oracle.E_SIGN_SCALE, cubature_w0=0.0)


def test_push_never_moves_ballistically():
    """In a strong field the reference's step still moves every ion along its
    unchanged velocity: the push is skipped because no tracker entry carries
    the particle's id."""
    w = _w()
    phi = np.random.default_rng(1).uniform(-2e3, 2e3, w.mesh.n_nodes)
    a, b = _engine(w), _engine(w, oracle.PUSH_NEVER)
    for o in (a, b):
        o.set_particles(w.pos, w.vel)
        o.set_potential(phi)
        o.process(1)
    pa, pb = a.particles(), b.particles()
    alive = pb["flags"] == 0
    assert alive.mean() > 0.99
    assert np.array_equal(pb["vel"][alive], w.vel[alive])
    assert np.array_equal(pb["pos"][alive], w.pos[alive] + w.vel[alive] * w.params["dt"])
    assert not np.array_equal(pa["vel"], w.vel)  # the build pushes


@pytest.mark.parametrize("w0", [1.0 / 6.0, 1.0 / 24.0])
def test_e_sign_scale(w0):
    """E = + sum phi_i grad N_i, each gradient weighted by the cubature
    measure |det J| w0 of point 0: the build's field negated and scaled by
    6 V w0 per tet (V for the one-point rule, V/4 for the four-point rule)."""
    w = _w(10)
    phi = np.random.default_rng(2).uniform(-50, 50, w.mesh.n_nodes)
    a, b = _engine(w), _engine(w, oracle.E_SIGN_SCALE, cubature_w0=w0)
    for o in (a, b):
        o.set_potential(phi)
    Ea, Eb = a.efield(), b.efield()
    meas = (6.0 * np.abs(w.mesh.volumes())) * w0
    assert np.allclose(Eb, -Ea * meas[:, None], rtol=1e-13, atol=0)


def _residual(o, phi, b):
    rp, ci, av, _ = o.matrix()
    Ax = np.array([np.dot(av[rp[i]:rp[i + 1]], phi[ci[rp[i]:rp[i + 1]]]) for i in range(len(phi))])
    return np.linalg.norm(Ax - b) / np.linalg.norm(b)


def test_rhs_raw_rho_and_cold_start():
    """The reference puts the nodal density itself into b at the free nodes
    (no eps0, no dual volume) and starts every solve from x = 0."""
    w = _w(10)
    rng = np.random.default_rng(3)
    rho = rng.uniform(0.0, 1e-6, w.mesh.n_nodes)
    a, b = _engine(w), _engine(w, oracle.RHS_RAW_RHO)
    _, _, lift = a.matrix()[0], None, a.matrix()[3]
    isd = np.zeros(w.mesh.n_nodes, bool)
    isd[w.mesh.dirichlet_nodes] = True
    g = np.zeros(w.mesh.n_nodes)
    g[w.mesh.dirichlet_nodes] = w.mesh.dirichlet_values
    dv = a.dual_volumes()
    pa, ita, _ = a.solve(rho)
    pb, itb, _ = b.solve(rho)
    assert _residual(a, pa, np.where(isd, g, rho * dv / w.params["epsilon0"] - lift)) <= 1e-10
    assert _residual(b, pb, np.where(isd, g, rho - lift)) <= 1e-10
    assert not np.allclose(pa, pb)
    # a second solve of the same density: the build starts from its solution,
    # the reference from zero
    _, ita2, _ = a.solve(rho)
    _, itb2, _ = b.solve(rho)
    assert ita2 == 0
    assert itb2 == itb and itb > 10


def _volavg_expected(w, tets, charge, prev=None):
    """NodeChargeDensityProcessor.cpp:58-93 in numpy: per-tet density q/V,
    then per node the volume average over its occupied tets; nodes without
    one keep `prev` (the map persists) or stay absent (nan)."""
    vol = np.abs(w.mesh.volumes())
    nt = w.mesh.n_tets
    q = np.bincount(tets, minlength=nt) * charge
    occ = q > 0
    rho_t = np.where(occ, q / vol, 0.0)
    num = np.zeros(w.mesh.n_nodes)
    den = np.zeros(w.mesh.n_nodes)
    for k in range(4):
        np.add.at(num, w.mesh.tets[occ, k], (rho_t * vol)[occ])
        np.add.at(den, w.mesh.tets[occ, k], vol[occ])
    out = np.full(w.mesh.n_nodes, np.nan) if prev is None else prev.copy()
    has = den > 0
    out[has] = num[has] / den[has]
    return out


def test_deposit_volavg_with_persistent_map():
    w = _w(3000)
    o = _engine(w, oracle.DEPOSIT_VOLAVG)
    wq = w.params["weight"] * w.params["charge"]
    # stage 1: the disk source's ions (lower part of the cube)
    o.set_particles(w.pos, w.vel)
    r1 = o.gather()
    e1 = _volavg_expected(w, o.particles()["tet"], wq)
    has1 = ~np.isnan(e1)
    assert has1.sum() > 20
    assert np.allclose(r1[has1], e1[has1], rtol=1e-12, atol=0)
    assert not r1[~has1].any()
    # stage 2: ions only near the top; nodes near the disk keep their density
    top = w.pos.copy()
    top[:, 2] = 0.085 + 0.01 * np.random.default_rng(4).random(len(top))
    o.set_particles(top, w.vel)
    r2 = o.gather()
    e2 = _volavg_expected(w, o.particles()["tet"], wq, prev=np.where(has1, e1, 0.0))
    assert np.allclose(r2, e2, rtol=1e-12, atol=0)
    kept = has1 & (r2 == r1)
    assert kept.sum() == has1.sum()  # the two regions share no tet here
    # the build's P1 deposit conserves charge; the volume average does not
    b = _engine(w)
    b.set_particles(w.pos, w.vel)
    dv = b.dual_volumes()
    total = wq * len(w.pos)
    assert abs(np.dot(b.gather(), dv) - total) <= 1e-12 * total
    assert abs(np.dot(np.nan_to_num(e1), dv) - total) > 1e-3 * total


def test_closed_tets_counts_shared_points():
    """A point on a vertex lies in every tet around it (the boundary counts
    as inside). On a dyadic lattice (h = 1/8) the barycentrics of a vertex are
    exact, so the closed test sees all of them."""
    m = M.kuhn_box((8, 8, 8), (1.0, 1.0, 1.0))
    w = _w(10)
    w.mesh = m
    node = int(np.argmin(np.sum((m.nodes - 0.5) ** 2, axis=1)))
    assert np.array_equal(m.nodes[node], [0.5, 0.5, 0.5])
    around = np.nonzero((m.tets == node).any(axis=1))[0]
    assert len(around) > 6
    pos = m.nodes[node][None, :].copy()
    vel = np.array([[100.0, 0.0, 0.0]])
    wq = w.params["weight"] * w.params["charge"]
    res = {}
    for flags in (oracle.DEPOSIT_VOLAVG, oracle.DEPOSIT_VOLAVG | oracle.CLOSED_TETS):
        o = oracle.Oracle(m, w.params)
        o.set_ref_compat(flags)
        o.set_particles(pos, vel)
        res[flags] = o.gather()
    vol = np.abs(m.volumes())
    closed = res[oracle.DEPOSIT_VOLAVG | oracle.CLOSED_TETS]
    # every tet around the node holds the ion: rho = k q / sum V over them
    assert closed[node] == pytest.approx(len(around) * wq / vol[around].sum(), rel=1e-12)
    open_ = res[oracle.DEPOSIT_VOLAVG]
    own = o.particles()["tet"][0]
    assert open_[node] == pytest.approx(wq / vol[own], rel=1e-12)


def test_solve_every_step():
    w = _w(500)
    a, b = _engine(w), _engine(w, oracle.SOLVE_EVERY_STEP)
    for o in (a, b):
        o.set_particles(w.pos, w.vel)
    assert a.run(10)["cg_solves"] == 1
    assert b.run(10)["cg_solves"] == 10


def test_mixed_units_moves_a_thousandth():
    w = _w()
    o = _engine(w, oracle.MIXED_UNITS | oracle.PUSH_NEVER)
    o.set_particles(w.pos, w.vel)
    o.process(1)
    p = o.particles()
    assert np.array_equal(p["pos"], w.pos + w.vel * (w.params["dt"] * 1e-3))


def test_reference_loop_against_the_build():
    """Workload 0 (HS argon, 200 steps, 1e4 ions) with every switch on is the
    reference's own loop. Without the push the ions never turn back to the
    source plane, and with metres added to millimetres they move a thousandth
    of their flight: none settles, while the build settles nearly all. The
    collisions, which do not depend on the push, run at the same rate per
    alive ion-step at their launch speed (the build's field slows them, so
    they collide less often per step); the solves run every step from zero."""
    w = workload0(n_particles=10000, collisions=True, steps=200)
    a, b = _engine(w), _engine(w, oracle.REFERENCE_LOOP)
    for o in (a, b):
        o.set_particles(w.pos, w.vel)
    sa, sb = a.run(200), b.run(200)
    assert sa["n_settled"] > 0.99 * len(w.pos)
    assert sb["n_settled"] == 0 and sb["n_lost"] == 0
    assert sb["cg_solves"] == 200 and sa["cg_solves"] == 20
    # collision rate per processed ion-step: the HS probability grows with |v|,
    # which only collisions change in the reference loop
    ra, rb = sa["collisions"] / sa["particle_steps"], sb["collisions"] / sb["particle_steps"]
    p0 = oracle.collision_probability(w.params, w.vel[0])
    assert rb == pytest.approx(p0, rel=0.1)
    assert ra < rb
    zb = b.particles()["pos"][:, 2]
    assert zb.max() < 1e-3  # 0.05 mm start + at most 200 x 20 nm

"""Pins of the CPU oracle (CPU only).

The reference has no golden vectors for the PIC loop, so the oracle is pinned
by (1) the reference's own known-answer unit tests for the primitives on this
path, restated here with the same inputs and expectations, (2) published
known answers (Philox4x32-10 test vectors), and (3) analytic known answers of
the discretisation (P1 exactness, constant-field ballistics, conservation,
scattering-angle laws).
"""
import numpy as np
import pytest

import oracle as O
from start_gb300 import workloads as W
from start_gb300.mesh import kuhn_box

E_CHARGE = 1.602176565e-19
EV_J = 1.60217733000001e-19
# Constants.hpp masses and radii of the species the reference tests use
MASS = dict(Ti=7.9485017e-26, Ar=6.6335209e-26, Ag=1.7911901e-25, Ne=3.3509177e-26, Au=3.2707137e-25,
            He=6.6464731e-27)
RADIUS = dict(Ti=140e-12, Ar=71e-12, Ag=160e-12, Ne=160e-12, Au=135e-12, He=120e-12)
VTI = dict(Ar=np.float32(0.81), Ne=np.float32(0.66), He=np.float32(0.66))  # stored as float in Constants.hpp
VSS_ALPHA = dict(Ar=np.float32(1.40), Ne=np.float32(1.31), He=np.float32(1.26))


@pytest.fixture(scope="module", autouse=True)
def _oracle(built):
    O.load()


def test_philox_known_answers():
    # Random123 kat_vectors for philox4x32-10
    assert O.philox([0, 0, 0, 0], [0, 0]).tolist() == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert O.philox([0xffffffff] * 4, [0xffffffff] * 2).tolist() == [0x408f276d, 0x41c83b0e, 0xa20bc7c6,
                                                                       0x6d5451fd]
    assert O.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]).tolist() == [
        0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_update_position_reference_kat():
    # tests/Particle/ParticleTests.cpp:99-108
    assert O.update_position([0.0, 0.0, 0.0], [1.0, 2.0, 3.0], 1.0).tolist() == [1.0, 2.0, 3.0]


TRI_Z = ([-1, 1, 0.5], [1, 1, 0.5], [0, -1, 0.5])
TRI_X = ([0.5, 1, 1], [0.5, -1, 1], [0.5, 0, -1])


@pytest.mark.parametrize("seg,tri,hit", [
    (([0, 0, 0], [0, 0, 1]), TRI_Z, True),
    (([1, 0, 0], [1, 0, 1]), TRI_Z, False),
    (([-1, 0, 0], [-1, 0, 1]), TRI_Z, False),
    (([0, 0, 0], [1, 0, 0]), TRI_X, True),
    (([-1, 0, 0], [1, -1, 0]), TRI_X, False),
    (([-1, 0, 0], [1, 1, 0]), TRI_X, False),
])
def test_segment_triangle_reference_kat(seg, tri, hit):
    # tests/Geometry/SegmentTriangleIntersectionTests.cpp:6-25
    assert (O.segment_triangle(*seg, *tri) is not None) == hit


def test_segment_triangle_point_reference_kat():
    # tests/Geometry/SegmentTriangleIntersectionTests.cpp:27-44 (tolerance 1e-5)
    p = O.segment_triangle([0, 0, 0], [0, 0, 1], *TRI_Z)
    assert np.allclose(p, [0, 0, 0.5], atol=1e-5)
    p = O.segment_triangle([0, 0, 0], [1, 0, 0], *TRI_X)
    assert np.allclose(p, [0.5, 0, 0], atol=1e-5)


def _species_params(model, proj, gas):
    d = RADIUS[proj] + RADIUS[gas]
    return dict(collision_model=model, mass=MASS[proj], gas_mass=MASS[gas], hs_diameter=d, vhs_dref=d,
                omega=float(VTI[gas]), alpha=float(VSS_ALPHA[gas]), kT_ref=297.0 * 1.380658e-23)


@pytest.mark.parametrize("model,proj,gas", [(1, "Ti", "Ar"), (2, "Ag", "Ne"), (3, "Au", "He")])
def test_collision_extremes_reference_kat(model, proj, gas):
    # tests/Particle/ParticleTests.cpp:155-183: 1 eV projectile collides at
    # n = 1e20, dt = 0.01 and does not at n = 1, dt = 1.
    v = np.array([0.0, 0.0, np.sqrt(2 * EV_J / MASS[proj])])
    p = _species_params(model, proj, gas)
    hi = dict(p, gas_concentration=1e20, dt=0.01)
    lo = dict(p, gas_concentration=1.0, dt=1.0)
    assert O.collision_probability(hi, v) > 1.0
    assert O.collision_probability(lo, v) < 1e-12
    for u0 in (0.0, 0.5, 1.0 - 2.0 ** -53):
        assert O.collide_with(hi, v, u0, 0.3, 0.7)[0]
        assert not O.collide_with(lo, v, u0 + 1e-9, 0.3, 0.7)[0]


def test_gas_concentration_formula():
    # util::calculateConcentration: (P / (R T)) N_A
    assert O.gas_concentration(1.0, 300.0) == (1.0 / (8.314 * 300.0)) * 6.02214076e23
    assert W.gas_concentration(0.5, 300.0) == O.gas_concentration(0.5, 300.0)


@pytest.mark.parametrize("model", [1, 2, 3])
def test_scattering_laws(model):
    """cos(chi) of the emitted direction: HS uniform on [-1, 1), VHS uniform on
    [0, 1) (the reference's forward-hemisphere law), VSS 2 u^(1/alpha) - 1."""
    from scipy import stats

    p = dict(_species_params(model, "Ti", "Ar"), gas_concentration=1e30, dt=1.0)
    v = np.array([300.0, -200.0, 2000.0])
    rng = np.random.default_rng(1)
    mcp = p["mass"] / (p["gas_mass"] + p["mass"])
    mct = p["gas_mass"] / (p["gas_mass"] + p["mass"])
    cosines = []
    for u1, u2 in rng.random((4000, 2)):
        hit, vn = O.collide_with(p, v, 0.0, u1, u2)
        assert hit
        rel = vn - mcp * v
        assert np.isclose(np.linalg.norm(rel), mct * np.linalg.norm(v), rtol=1e-12)
        n = rel / np.linalg.norm(rel)
        if model == 3:  # VSS rotates the direction into the frame of the relative velocity
            axis = v / np.linalg.norm(v)
            cosines.append(np.dot(n, axis))
        else:
            cosines.append(n[2])
    c = np.array(cosines)
    if model == 1:
        cdf = lambda x: (x + 1) / 2  # noqa: E731
    elif model == 2:
        cdf = lambda x: np.clip(x, 0, 1)  # noqa: E731
    else:
        a = p["alpha"]
        cdf = lambda x: ((x + 1) / 2) ** a  # noqa: E731
    assert stats.kstest(c, cdf).pvalue > 1e-3


def test_tet_map_inverts_edges():
    x = [np.array(v, float) for v in ([0.1, 0.2, 0.3], [1.1, 0.25, 0.3], [0.2, 1.3, 0.35], [0.15, 0.2, 1.4])]
    det, M = O.tet_map(*x)
    assert det > 0
    for k in range(3):
        e = np.zeros(3)
        e[k] = 1
        assert np.allclose(M @ (x[k + 1] - x[0]), e, atol=1e-14)


def test_reference_tet_fixture():
    """tests/meshes/TetrahedronTestMesh.msh.gtest: the 100 mm cube, 24 tets."""
    from pathlib import Path

    from start_gb300.mesh import TetMesh

    d = np.load(Path(__file__).parent / "golden" / "ref_meshes.npz")
    m = TetMesh(nodes=d["TetrahedronTestMesh_nodes"] * 1e-3, tets=d["TetrahedronTestMesh_tets"],
                triangles=d["TetrahedronTestMesh_triangles"], tri_tag=d["TetrahedronTestMesh_tri_tag"])
    assert m.n_tets == 24 and m.n_nodes == 14 and m.n_triangles == 24
    v = m.volumes()
    assert (v > 0).all() and np.isclose(v.sum(), 1e-3, rtol=1e-12)
    o = O.Oracle(m, dict(dt=1e-8))
    assert o.n_boundary_faces == 24  # every boundary face carries a surface triangle
    # a particle walks across the cube and settles on the x = 100 mm face
    o.set_particles([[0.01, 0.05, 0.05]], [[1e6, 0.0, 0.0]])
    o.process(20)
    p = o.particles()
    assert p["flags"][0] == 1
    assert np.isclose(p["pos"][0][0], 0.1, atol=1e-15)
    assert m.tri_tag[np.nonzero(o.triangle_counts())[0][0]] in set(m.tri_tag.tolist())


def _box(cells=6, L=0.1):
    return kuhn_box((cells,) * 3, (L,) * 3)


def test_dirichlet_rows_are_identity_and_rhs_is_value():
    # MatrixBoundaryConditionsTests.cpp:96-105, VectorBoundaryConditionsTests.cpp:46-56
    m = _box()
    dn = np.array([1, 2, 40], np.int32)
    m.with_dirichlet(dn, [1.0, 0.0, 3.5])
    o = O.Oracle(m, dict(dt=1e-8))
    rp, ci, av, lift = o.matrix()
    for n in dn:
        assert rp[n + 1] - rp[n] == 1 and ci[rp[n]] == n and av[rp[n]] == 1.0
        assert lift[n] == 0.0
    # Dirichlet columns moved to the right-hand side: no free row references them
    free_rows = np.setdiff1d(np.arange(m.n_nodes), dn)
    cols = np.concatenate([ci[rp[i]:rp[i + 1]] for i in free_rows])
    assert not np.isin(dn, cols).any()
    phi, _, _ = o.solve(np.zeros(m.n_nodes))
    assert phi[1] == 1.0 and phi[2] == 0.0 and phi[40] == 3.5


def test_out_of_range_dirichlet_rejected():
    # MatrixBoundaryConditionsTests.cpp:131-142 (OutOfBoundsNodeID)
    m = _box(cells=2)
    m.with_dirichlet([10_000], [1.0])
    with pytest.raises(RuntimeError):
        O.Oracle(m, dict(dt=1e-8))


def test_matrix_is_symmetric_with_zero_row_sums():
    m = _box()
    o = O.Oracle(m, dict(dt=1e-8))  # no Dirichlet nodes: pure stiffness
    rp, ci, av, _ = o.matrix()
    import scipy.sparse as sp

    K = sp.csr_matrix((av, ci, rp), shape=(m.n_nodes, m.n_nodes))
    assert abs(K - K.T).max() <= 1e-14 * abs(K).max()
    assert np.abs(K @ np.ones(m.n_nodes)).max() <= 1e-13 * abs(K).max()


def _linear_field_mesh(cells=6, L=0.1, grad=(120.0, -80.0, 300.0), c0=5.0):
    m = _box(cells, L)
    lo, hi = m.nodes.min(0), m.nodes.max(0)
    on = np.any((m.nodes <= lo + 1e-12) | (m.nodes >= hi - 1e-12), axis=1)
    dn = np.nonzero(on)[0].astype(np.int32)
    g = np.asarray(grad)
    m.with_dirichlet(dn, m.nodes[dn] @ g + c0)
    return m, g, c0


def test_p1_reproduces_linear_potential():
    m, g, c0 = _linear_field_mesh()
    o = O.Oracle(m, dict(dt=1e-8, cg_rtol=1e-14))
    phi, it, rr = o.solve(np.zeros(m.n_nodes))
    assert np.max(np.abs(phi - (m.nodes @ g + c0))) <= 1e-10 * np.max(np.abs(phi))
    E = o.efield()
    assert np.allclose(E, -g, rtol=1e-9, atol=1e-9 * np.abs(g).max())


def test_constant_field_ballistics_closed_form():
    m, g, c0 = _linear_field_mesh(grad=(0.0, 0.0, 400.0))
    p = dict(dt=1e-8, charge=E_CHARGE, mass=W.TI_MASS)
    o = O.Oracle(m, p)
    x0 = np.array([[0.05, 0.05, 0.05], [0.03, 0.06, 0.04]])
    v0 = np.array([[500.0, -300.0, 2000.0], [0.0, 100.0, -50.0]])
    o.set_particles(x0, v0)  # resets the field
    o.set_potential(m.nodes @ g + c0)
    N = 50
    o.process(N)
    a = E_CHARGE * (-g) / W.TI_MASS
    dt = p["dt"]
    x_exact = x0 + N * v0 * dt + a * dt * dt * N * (N + 1) / 2
    v_exact = v0 + N * a * dt
    q = o.particles()
    assert np.allclose(q["vel"], v_exact, rtol=1e-12, atol=1e-9)
    assert np.allclose(q["pos"], x_exact, rtol=1e-12, atol=1e-15)


def test_walk_agrees_with_point_location():
    w = W.workload0(n_particles=3000, collisions=False, steps=30)
    w.params["cg_rtol"] = 1e-12
    o = O.Oracle(w.mesh, w.params)
    o.set_particles(w.pos, w.vel)
    phi = np.random.default_rng(2).uniform(-3e3, 3e3, o.n_nodes)
    o.set_potential(phi)
    o.process(30)
    p = o.particles()
    alive = p["flags"] == 0
    assert alive.sum() > 100
    loc = o.locate(p["pos"][alive])
    assert np.array_equal(loc, p["tet"][alive])


def test_deposit_conserves_charge():
    w = W.workload0(n_particles=5000, collisions=False)
    o = O.Oracle(w.mesh, w.params)
    o.set_particles(w.pos, w.vel)
    rho = o.gather()
    total = w.params["weight"] * w.params["charge"] * 5000
    assert abs(np.dot(rho, o.dual_volumes()) - total) <= 1e-13 * total
    assert (rho >= -1e-30).all()


def _golden(name):
    from pathlib import Path

    return np.load(Path(__file__).parent / "golden" / f"oracle_w0_{name}.npz")


def test_oracle_reproduces_committed_golden_collisionless():
    g = _golden("collisionless")
    w = W.workload0(n_particles=2000, collisions=False, steps=int(g["steps"]))
    w.params["cg_rtol"] = 1e-12
    o = O.Oracle(w.mesh, w.params)
    o.set_particles(g["pos0"], g["vel0"])
    st = o.run(w.steps)
    p = o.particles()
    assert np.array_equal(p["tet"], g["tet"]) and np.array_equal(p["flags"], g["flags"])
    assert np.max(np.abs(p["pos"] - g["pos"])) <= 1e-12
    assert np.array_equal(o.triangle_counts(), g["tri_count"])
    assert st["particle_steps"] == int(g["particle_steps"])


def test_oracle_reproduces_committed_golden_hs():
    import platform

    g = _golden("hs")
    w = W.workload0(n_particles=2000, collisions=True, steps=int(g["steps"]))
    w.params["cg_rtol"] = 1e-12
    w.params["gas_concentration"] = float(g["gas_concentration"])
    o = O.Oracle(w.mesh, w.params)
    o.set_particles(g["pos0"], g["vel0"])
    st = o.run(w.steps)
    if platform.machine() == str(g["machine"]):
        assert st["collisions"] == int(g["collisions"])
        assert np.array_equal(o.triangle_counts(), g["tri_count"])
    else:  # libm may round transcendental results differently on another ISA
        assert abs(st["collisions"] - int(g["collisions"])) <= 0.05 * int(g["collisions"])

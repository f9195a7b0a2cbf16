"""The FEM set-up on the GPU (kernels_fem.cu) against the CPU oracle's
assembly: element maps, orientation and volumes, the node -> tet incidence
with the dual volumes, and the CSR stiffness with its Dirichlet elimination
(row structure, values, lifting) must agree bit for bit, on the Kuhn cube,
on the jittered box with internal electrodes, and on a mesh given with half
of its tets inverted (the set-up swaps two nodes of those)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _compare(w):
    import oracle
    from start_gb300 import StartPIC

    g = StartPIC(w.mesh, w.params)
    o = oracle.Oracle(w.mesh, w.params)
    rp, col, val, lift, dual = g.matrix()
    orp, ocol, oval, olift = o.matrix()
    assert np.array_equal(rp, orp)
    assert np.array_equal(col, ocol)
    assert np.array_equal(val, oval)
    assert np.array_equal(lift, olift)
    assert np.array_equal(dual, o.dual_volumes())
    phi = np.random.default_rng(1).uniform(-20, 20, g.n_nodes)
    g.set_potential(phi)
    o.set_potential(phi)
    assert np.array_equal(g.efield(), o.efield())  # the element maps, through E
    t = g.setup_times()
    assert min(t.values()) >= 0.0
    assert t["create"] >= t["fem_elements_gpu"] + t["fem_stiffness_gpu"] + t["mesh_host"]
    g.close()
    o.close()


def test_fem_kuhn_cube(built):
    from start_gb300.workloads import workload0

    _compare(workload0(n_particles=10, cells=12))


def test_fem_jittered_box(built):
    from start_gb300.workloads import workload3

    _compare(workload3(n_particles=10, cells=(20, 20, 10), steps=10))


def test_fem_inverted_tets(built):
    from start_gb300.workloads import workload0

    w = workload0(n_particles=10, cells=8)
    tets = np.array(w.mesh.tets, np.int32).copy()
    tets[::2, [2, 3]] = tets[::2, [3, 2]]
    w.mesh.tets = tets
    _compare(w)


def test_fem_degenerate_tet_is_reported(built):
    from start_gb300 import StartPIC
    from start_gb300.engine import PICBaseException
    from start_gb300.workloads import workload0

    w = workload0(n_particles=10, cells=6)
    tets = np.array(w.mesh.tets, np.int32).copy()
    tets[37, 3] = tets[37, 2]  # zero volume
    tets[90, 1] = tets[90, 0]
    w.mesh.tets = tets
    with pytest.raises(PICBaseException, match="tet 37 has a bad node index or zero volume"):
        StartPIC(w.mesh, w.params)

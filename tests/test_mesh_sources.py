"""Mesh generator, Gmsh reader and particle sources (CPU only)."""
from pathlib import Path

import numpy as np
import pytest

from start_gb300 import mesh as M
from start_gb300 import sources as S
from start_gb300 import workloads as W


def test_kuhn_box_counts_and_volume():
    m = M.kuhn_box((10, 10, 10), (0.1, 0.1, 0.1))
    assert (m.n_tets, m.n_nodes, m.n_triangles) == (6000, 1331, 1200)
    v = m.volumes()
    assert (v > 0).all()
    assert np.isclose(v.sum(), 1e-3, rtol=1e-12)
    assert np.isclose(m.triangle_areas().sum(), 6 * 0.01, rtol=1e-12)


def test_kuhn_box_is_conforming_and_triangles_are_faces(built):
    import oracle

    m = M.kuhn_box((4, 3, 5), (0.04, 0.03, 0.05))
    o = oracle.Oracle(m, dict(dt=1e-8))  # rejects non-manifold faces and stray triangles
    assert o.n_boundary_faces == m.n_triangles


def test_kuhn_box_morton_order():
    m = M.kuhn_box((8, 8, 8), (1.0, 1.0, 1.0))
    cen = m.nodes[m.tets].mean(1)
    cell = np.floor(cen * 8).astype(int)
    codes = M._morton3(cell[:, 0], cell[:, 1], cell[:, 2])
    assert (np.diff(codes.astype(np.int64)) >= 0).all()


def test_workload_sizes():
    w = W.workload0()
    assert w.mesh.n_tets == 6000 and len(w.pos) == 10_000 and w.steps == 200
    assert w.params["weight"] == 1e6 and w.params["collision_model"] == 1
    assert np.isclose(w.params["gas_concentration"], 2.414e20, rtol=1e-3)
    w1 = W.workload1(n_particles=1000, cells=10)
    assert w1.params["collision_model"] == 2 and w1.params["dt"] == 5e-9


def test_plates_and_jitter(built):
    import oracle

    m = M.kuhn_box((10, 10, 5), (0.2, 0.2, 0.1))
    low = M.add_plate(m, 0.02, (0.06, 0.14), (0.06, 0.14), tag=7)
    assert len(low) == 5 * 5 and (m.tri_tag == 7).sum() == 2 * 4 * 4
    v0 = m.volumes()
    M.jitter(m, 0.2, seed=3, frozen=low)
    assert (m.volumes() > 0.05 * v0).all()
    assert np.allclose(m.nodes[low, 2], 0.02)
    o = oracle.Oracle(m, dict(dt=1e-8))
    # plate triangles are internal: each sits on two tet faces
    assert o.n_boundary_faces == (m.tri_tag <= 6).sum()


def test_disk_source_and_displacement():
    rng = np.random.default_rng(0)
    p = S.disk_points(rng, 20000, (0.05, 0.05, 0.0), 0.02)
    r = np.hypot(p[:, 0] - 0.05, p[:, 1] - 0.05)
    assert r.max() <= 0.02 and np.all(p[:, 2] == 0.0)
    assert abs(np.mean(r ** 2) / 0.02 ** 2 - 0.5) < 0.01  # uniform in area
    d = S.cone_directions(rng, 20000, np.deg2rad(30))
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0)
    assert d[:, 2].min() >= np.cos(np.deg2rad(30)) - 1e-12
    q = S.displace(p, d)
    shift = (q - p) / S.DISPLACEMENT
    assert np.allclose(np.max(np.abs(shift), axis=1), 1.0)


def test_thompson_and_cosine_distributions():
    from scipy import stats

    rng = np.random.default_rng(1)
    U, Em = 4.9, 50.0
    E = S.thompson_energies(rng, 20000, U, Em) / S.EV_J
    assert E.max() <= Em * (1 + 1e-12)
    cdf = lambda e: (e / (e + U)) ** 2 / (Em / (Em + U)) ** 2  # noqa: E731
    assert stats.kstest(E, cdf).pvalue > 1e-3
    d = S.cosine_directions(rng, 20000)
    st = np.sqrt(1 - d[:, 2] ** 2)
    assert stats.kstest(st ** 2, "uniform").pvalue > 1e-3


def test_msh41_reader_on_reference_fixture():
    d = np.load(Path(__file__).parent / "golden" / "ref_meshes.npz")
    nodes = d["TetrahedronTestMesh_nodes"]
    assert nodes.min() == 0.0 and nodes.max() == 100.0  # millimetres, tag - 1 indexing
    assert set(d["TetrahedronTestMesh_tri_tag"].tolist()) == {1, 2, 3, 4, 5, 6}
    assert d["BoxMeshTest_triangles"].shape == (2076, 3)


def test_msh41_reader_roundtrip(tmp_path):
    """Writes a small msh 4.1 file and reads it back."""
    txt = """$MeshFormat
4.1 0 8
$EndMeshFormat
$Nodes
1 4 1 4
3 1 0 4
1
2
3
4
0 0 0
1 0 0
0 1 0
0 0 1
$EndNodes
$Elements
2 2 1 2
2 5 2 1
1 1 2 3
3 1 4 1
2 1 3 2 4
$EndElements
"""
    p = tmp_path / "t.msh"
    p.write_text(txt)
    m = M.read_msh41(p, scale=1e-3)
    assert m.tets.tolist() == [[0, 2, 3, 1]]  # tags 1 3 2 4, re-oriented to positive volume
    assert m.volumes()[0] > 0
    assert m.triangles.tolist() == [[0, 1, 2]] and m.tri_tag.tolist() == [5]
    assert np.allclose(m.nodes[3], [0, 0, 1e-3])


def test_triangle_count_writer_roundtrip(tmp_path):
    from start_gb300 import mesh as M
    from start_gb300 import output

    m = M.kuhn_box((3, 3, 3), (0.03, 0.03, 0.03))
    tris = np.asarray(m.triangles).reshape(-1, 3)
    counts = np.arange(len(tris), dtype=np.uint32) % 7
    p = tmp_path / "tri.npz"
    output.write_triangle_counts(p, m.nodes, tris, counts, length_scale=1e3)
    d = output.read(p)
    assert d["Coordinates"].shape == (len(tris), 9)
    assert np.array_equal(d["Counter"], counts.astype(np.uint64))
    # each boundary face of the 30 mm cube is 900 mm^2, split into 2*9 triangles
    assert np.isclose(d["Area"].sum(), 6 * 900.0)
    assert np.allclose(d["Area"], 50.0)
    pos = np.random.default_rng(0).random((10, 3))
    flags = np.array([1, 0, 1, 2, 0, 1, 0, 0, 3, 0], np.uint32)
    output.write_settled_particles(tmp_path / "s.npz", pos, flags)
    s = output.read(tmp_path / "s.npz")
    assert np.array_equal(s["positions"], pos[(flags & 1) != 0])

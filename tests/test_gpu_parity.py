"""GPU parity: libstart_gpu.so (through its C ABI) against the CPU oracle.

Tolerances (FP64 form):
  * collisionless runs: per-particle tet ids and flags identical, positions
    within 1e-9 relative, triangle counters identical;
  * E from a given potential, and the push/walk from a given E: bit-identical;
  * nodal charge density: 1e-12 relative (max-norm); potential: 1e-9 relative
    (two PCG runs to 1e-12 differ only in reduction order);
  * runs with collisions: surface histograms agree under a chi-square
    two-sample test at p > 0.01.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def libs(built):
    return built


def _pair(w):
    import oracle
    from start_gb300 import StartPIC

    return StartPIC(w.mesh, w.params), oracle.Oracle(w.mesh, w.params)


def _w0(n=4000, collisions=False, steps=200, cells=10, **kw):
    from start_gb300.workloads import workload0

    w = workload0(n_particles=n, collisions=collisions, steps=steps, cells=cells)
    w.params["cg_rtol"] = 1e-12
    w.params.update(kw)
    return w


def _relerr(a, b, floor):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


def test_mesh_tables_match(libs):
    w = _w0(n=10)
    g, o = _pair(w)
    assert (g.n_nodes, g.n_tets, g.n_triangles) == (1331, 6000, 1200)
    assert g.n_boundary_faces == o.n_boundary_faces == 1200
    assert g.nnz == o.nnz
    assert g.n_dirichlet == o.n_dirichlet == 242


def test_locate_matches_oracle(libs):
    w = _w0(n=10)
    g, o = _pair(w)
    rng = np.random.default_rng(3)
    pts = rng.uniform(1e-4, 0.1 - 1e-4, size=(20000, 3))
    tg, to = g.locate(pts), o.locate(pts)
    assert np.array_equal(tg, to)
    out = np.array([[0.2, 0.05, 0.05], [-0.01, 0.05, 0.05], [np.nan, 0.0, 0.0]])
    assert (g.locate(out) == -1).all()


def test_deposit_matches_oracle(libs):
    w = _w0(n=20000)
    g, o = _pair(w)
    for e in (g, o):
        e.set_particles(w.pos, w.vel)
    rg, ro = g.gather(), o.gather()
    assert np.max(np.abs(rg - ro)) <= 1e-12 * np.max(np.abs(ro))
    # charge conservation: sum rho_n V_n = N w q
    dv = o.dual_volumes()
    total = w.params["weight"] * w.params["charge"] * len(w.pos)
    assert abs(np.dot(rg, dv) - total) <= 1e-12 * total


def test_efield_from_given_potential_bit_exact(libs):
    w = _w0(n=10)
    g, o = _pair(w)
    phi = np.random.default_rng(5).uniform(-50, 50, g.n_nodes)
    g.set_potential(phi)
    o.set_potential(phi)
    assert np.array_equal(g.efield(), o.efield())


def test_solve_matches_oracle(libs):
    w = _w0(n=20000)
    g, o = _pair(w)
    for e in (g, o):
        e.set_particles(w.pos, w.vel)
        e.gather(want_rho=False)
    pg, itg, rrg = g.solve()
    po, ito, rro = o.solve()
    assert rrg <= 1e-12 and rro <= 1e-12
    assert abs(itg - ito) <= max(3, ito // 10)
    assert _relerr(pg, po, 1.0) <= 1e-9


def test_push_walk_bit_exact_given_field(libs):
    """Same E on both sides -> identical IEEE operations -> identical state."""
    w = _w0(n=5000)
    g, o = _pair(w)
    for e in (g, o):
        e.set_particles(w.pos, w.vel)
    phi = np.random.default_rng(7).uniform(-2e3, 2e3, g.n_nodes)
    g.set_potential(phi)
    o.set_potential(phi)
    for _ in range(4):
        g.process(10)
        o.process(10)
        pg, po = g.particles(), o.particles()
        assert np.array_equal(pg["tet"], po["tet"])
        assert np.array_equal(pg["flags"], po["flags"])
        assert np.array_equal(pg["pos"], po["pos"])
        assert np.array_equal(pg["vel"], po["vel"])
    assert np.array_equal(g.triangle_counts(), o.triangle_counts())
    sg, so = g.stats(), o.stats()
    for k in ("particle_steps", "crossings", "n_settled", "n_lost"):
        assert sg[k] == so[k], k


def test_full_run_collisionless(libs):
    """Workload 0 without gas: 200 steps, Poisson every 10, re-sort every 20."""
    w = _w0(n=10000, steps=200)
    g, o = _pair(w)
    for e in (g, o):
        e.set_particles(w.pos, w.vel)
    sg, so = g.run(w.steps), o.run(w.steps)
    pg, po = g.particles(), o.particles()
    assert np.array_equal(pg["tet"], po["tet"])
    assert np.array_equal(pg["flags"], po["flags"])
    assert _relerr(pg["pos"], po["pos"], 1e-3) <= 1e-9
    assert np.array_equal(g.triangle_counts(), o.triangle_counts())
    assert sg["particle_steps"] == so["particle_steps"]
    assert sg["n_settled"] == so["n_settled"] > 0


def _chi2_two_sample(a, b):
    from scipy import stats

    a = np.asarray(a, float)
    b = np.asarray(b, float)
    keep = (a + b) > 0
    a, b = a[keep], b[keep]
    Na, Nb = a.sum(), b.sum()
    k1, k2 = np.sqrt(Nb / Na), np.sqrt(Na / Nb)
    chi2 = np.sum((k1 * a - k2 * b) ** 2 / (a + b))
    dof = len(a) - 1
    return chi2, stats.chi2.sf(chi2, dof)


def test_full_run_with_collisions_histogram(libs):
    """HS collisions (Ar, 1 Pa): libm and CUDA transcendental results differ
    in the last bit, so trajectories may part; the surface histograms must
    agree statistically."""
    w = _w0(n=10000, steps=200, collisions=True)
    w.params["gas_concentration"] *= 200.0  # many collisions per particle
    g, o = _pair(w)
    for e in (g, o):
        e.set_particles(w.pos, w.vel)
    sg, so = g.run(w.steps), o.run(w.steps)
    assert sg["collisions"] > 1000
    assert abs(sg["collisions"] - so["collisions"]) <= 0.05 * so["collisions"]
    cg, co = g.triangle_counts(), o.triangle_counts()
    # group triangles into coarse surface bins (box faces x 4x4 patches)
    cen = w.mesh.triangle_centroids()
    tag = w.mesh.tri_tag
    ij = np.floor(cen / 0.025).astype(int).clip(0, 3)
    key = tag * 100 + ij[:, 0] * 0 + (ij * np.array([16, 4, 1])).sum(1)
    _, inv = np.unique(key, return_inverse=True)
    hg = np.bincount(inv, weights=cg.astype(float))
    ho = np.bincount(inv, weights=co.astype(float))
    _, p = _chi2_two_sample(hg, ho)
    assert p > 0.01
    same = np.mean(g.particles()["tet"] == o.particles()["tet"])
    assert same > 0.9


def test_resort_does_not_change_results(libs):
    w = _w0(n=6000, steps=60)
    w.params["resort_every"] = 0
    from start_gb300 import StartPIC

    a = StartPIC(w.mesh, w.params)
    w2 = _w0(n=6000, steps=60)
    w2.params["resort_every"] = 3
    b = StartPIC(w2.mesh, w2.params)
    for e in (a, b):
        e.set_particles(w.pos, w.vel)
        e.run(60)
    pa, pb = a.particles(), b.particles()
    assert np.array_equal(pa["tet"], pb["tet"])
    assert np.array_equal(pa["flags"], pb["flags"])
    assert _relerr(pa["pos"], pb["pos"], 1e-3) <= 1e-9
    assert np.array_equal(a.triangle_counts(), b.triangle_counts())


@pytest.mark.parametrize("precision", [0, 1])
def test_resort_is_a_permutation_of_crowded_tets(libs, precision):
    """The re-sort merges equal tets per block before its atomics: with
    hundreds of particles per tet (a 4-cell cube) and settled particles among
    them, every particle keeps its state through repeated re-sorts."""
    from start_gb300 import StartPIC

    w = _w0(n=60000, cells=4, collisions=True, precision=precision)
    vel = w.vel.copy()
    vel[::3, 2] = -np.abs(vel[::3, 2])  # a third head into the source plane and settle there
    g = StartPIC(w.mesh, w.params)
    g.set_particles(w.pos, vel)
    g.run(12)
    a = g.particles()
    assert (a["flags"] != 0).any()
    for _ in range(3):
        g.resort()
    b = g.particles()
    for k in a:
        assert np.array_equal(a[k], b[k])
    g.close()


@pytest.mark.parametrize("precond", [0, 2])
def test_checkpoint_restore_is_exact(libs, precond):
    """With AMG the run solves start from an extrapolation of the previous
    potentials; the checkpoint carries them, so the restored run repeats the
    original bit for bit (poisson_every 10: solves at steps 40-70 use the
    history of the solves before the checkpoint)."""
    w = _w0(n=5000, steps=80, collisions=True, preconditioner=precond)
    from start_gb300 import StartPIC

    g = StartPIC(w.mesh, w.params)
    g.set_particles(w.pos, w.vel)
    g.run(40)
    blob = g.checkpoint()
    g.run(40)
    a = g.particles()
    ca = g.triangle_counts()
    g.restore(blob)
    g.run(40)
    b = g.particles()
    assert np.array_equal(a["pos"], b["pos"])
    assert np.array_equal(a["vel"], b["vel"])
    assert np.array_equal(a["tet"], b["tet"])
    assert np.array_equal(ca, g.triangle_counts())


@pytest.mark.parametrize("precision", [0, 1])
def test_restore_refuses_corrupt_particles(libs, precision):
    """A checkpoint whose particle ids are not a permutation of 0..np-1, or
    whose tets are out of range, is refused before anything is copied: the
    handle keeps its state and a good blob still restores."""
    from start_gb300 import StartPIC
    from start_gb300.engine import PICBaseException

    w = _w0(n=3000, steps=10, precision=precision)
    g = StartPIC(w.mesh, w.params)
    g.set_particles(w.pos, w.vel)
    g.run(5)
    blob = g.checkpoint()
    before = g.particles()
    n, es, hdr = 3000, (4 if precision else 8), 104  # CkptHeader: 13 words of 8 B
    tet_off = hdr + 6 * es * n
    idf_off = tet_off + 4 * n
    ids = np.frombuffer(blob, np.uint32, n, idf_off)
    dup = bytearray(blob)
    dup[idf_off + 4 * 7: idf_off + 4 * 8] = ids[3:4].tobytes()  # two particles with one id
    big = bytearray(blob)
    big[idf_off: idf_off + 4] = np.uint32(n + 5).tobytes()  # id beyond np
    bad_tet = bytearray(blob)
    bad_tet[tet_off: tet_off + 4] = np.int32(g.n_tets).tobytes()
    for b in (dup, big, bad_tet):
        with pytest.raises(PICBaseException):
            g.restore(bytes(b))
    after = g.particles()
    for k in before:
        assert np.array_equal(before[k], after[k])
    g.restore(blob)
    g.run(5)
    g.close()


def test_edge_cases(libs):
    from start_gb300 import StartPIC
    from start_gb300.engine import PICBaseException

    w = _w0(n=4)
    g = StartPIC(w.mesh, w.params)
    with pytest.raises(PICBaseException):
        g.process(1)  # no particles yet
    # empty population
    g.set_particles(np.zeros((0, 3)), np.zeros((0, 3)))
    st = g.run(3)
    assert st["particle_steps"] == 0
    # outside the mesh -> lost at set; slow particle does not move; NaN -> lost
    pos = np.array([[0.05, 0.05, 0.05], [0.5, 0.5, 0.5], [0.05, 0.05, 0.06], [0.05, 0.05, 0.07]])
    vel = np.array([[1e3, 0, 0], [1e3, 0, 0], [5.0, 0, 0], [np.nan, 0, 0]])
    g.set_particles(pos, vel)
    st = g.stats()
    assert st["n_lost"] == 1
    g.process(1)
    p = g.particles()
    assert p["flags"][1] == 2
    assert np.array_equal(p["pos"][2], pos[2])
    assert np.array_equal(p["pos"][0], pos[0] + vel[0] * w.params["dt"])
    # the NaN particle is skipped like the reference (|v| is NaN, not < 10,
    # so it moves to NaN and is flagged lost)
    assert p["flags"][3] == 2


def test_walk_cap_flags_lost(libs):
    from start_gb300 import StartPIC

    w = _w0(n=4)
    w.params["max_crossings"] = 1
    g = StartPIC(w.mesh, w.params)
    pos = np.array([[0.0123, 0.0456, 0.05]])
    vel = np.array([[7e6, 0, 0]])  # 7 cm per step: many crossings
    g.set_particles(pos, vel)
    g.process(1)
    assert g.particles()["flags"][0] == 2


@pytest.mark.parametrize("precision", [0, 1])
def test_particles_into_caller_arrays(libs, precision):
    """The staged host copies (set / get / locate reuse one device buffer):
    a read into caller arrays equals a plain read, a smaller second particle
    set reads back exactly, and a wrongly typed output is refused."""
    from start_gb300 import StartPIC

    w = _w0(n=3000, precision=precision)
    g = StartPIC(w.mesh, w.params)
    g.set_particles(w.pos, w.vel)
    g.run(5)
    a = g.particles()
    out = {"pos": np.empty((3000, 3)), "vel": np.empty((3000, 3)), "tet": np.empty(3000, np.int32),
           "flags": np.empty(3000, np.uint32)}
    b = g.particles(out=out)
    for k in a:
        assert b[k] is out[k]
        assert np.array_equal(a[k], b[k])
    assert np.array_equal(g.locate(w.pos[:700]), g.locate(w.pos)[:700])
    g.set_particles(w.pos[:1000], w.vel[:1000])
    c = g.particles()
    assert np.allclose(c["pos"], w.pos[:1000], rtol=0, atol=0.0 if precision == 0 else 2e-9)  # FP32 local offsets
    assert np.array_equal(c["tet"], g.locate(w.pos[:1000]))
    with pytest.raises(ValueError):
        g.particles(out={"pos": np.empty((1000, 3), np.float32)})
    g.close()


@pytest.mark.parametrize("precision", [0, 1])
def test_direct_and_staged_host_copies_agree(libs, precision):
    """Caller arrays the GPU can reach (pinned memory; pageable memory where the
    device walks the host page tables) are read by the upload kernel where they
    lie and, when pinned, written by the download kernel directly; other arrays
    go through the staging buffer. Both routes give the same state bit for bit:
    uploads with and without given tets (the staged route), downloads into
    pinned and into pageable arrays."""
    import torch

    from start_gb300 import StartPIC

    w = _w0(n=20000, precision=precision)
    pos = w.pos.copy()
    pos[7] = [0.5, 0.5, 0.5]  # outside the mesh: lost at upload on both routes
    a, b = StartPIC(w.mesh, w.params), StartPIC(w.mesh, w.params)
    pin = lambda x: torch.from_numpy(np.ascontiguousarray(x)).pin_memory().numpy()
    a.set_particles(pin(pos), pin(w.vel))
    b.set_particles(pos, w.vel, tet=a.locate(pos))
    assert a.stats()["n_lost"] == b.stats()["n_lost"] == 1
    for e in (a, b):
        e.run(30)
    n = len(pos)
    out = {"pos": pin(np.empty((n, 3))), "vel": pin(np.empty((n, 3))), "tet": pin(np.empty(n, np.int32)),
           "flags": pin(np.empty(n, np.int32)).view(np.uint32)}
    pa = a.particles(out=out)
    pb = b.particles()
    for k in pa:
        assert np.array_equal(pa[k], pb[k]), k
    assert np.array_equal(a.triangle_counts(), b.triangle_counts())
    a.close()
    b.close()

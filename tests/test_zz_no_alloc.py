"""spg_pcg_solve_noalloc against spg_solve, through the C ABI.

The allocation-free solve is for callers that cannot call cudaMalloc: a
program whose device memory is all held by its own pool (PyTorch's caching
allocator, a fixed arena), or a loop that must not take the device
synchronisation an allocation can imply. The caller passes device arrays it
already owns, here torch tensors, and the solve runs in the library's static
scratch. Its answer must match the handle-based spg_solve on the same matrix
and right-hand side within the tolerance of the PCG parity test (1e-9
relative), on two calls in a row, and the oracle's CPU solve of the same
system within the same tolerance. The second call checks that nothing left in
the shared scratch by the first call leaks into it. Small hand-made systems
check the documented refusals: a zero right-hand side, a row without its
diagonal, and a matrix that is not positive definite.

This file sorts last so that a run stopping at the first failure has run
every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

EPS0 = 8.8541878128e-12


def _problem():
    import oracle
    from start_gb300.workloads import workload0

    w = workload0(n_particles=20000, collisions=False)
    w.params["cg_rtol"] = 1e-12
    o = oracle.Oracle(w.mesh, w.params)
    o.set_particles(w.pos, w.vel)
    rho = o.gather()
    rp, ci, av, lift = o.matrix()
    dv = o.dual_volumes()
    isd = np.zeros(o.n_nodes, bool)
    isd[w.mesh.dirichlet_nodes] = True
    g = np.zeros(o.n_nodes)
    g[w.mesh.dirichlet_nodes] = w.mesh.dirichlet_values
    return w, rho, (rp, ci, av), lift, dv, isd, g


def _rhs(rho, lift, dv, isd, g):
    return np.where(isd, g, rho * dv / EPS0 - lift)


def test_noalloc_solve_matches_spg_solve_twice(built):
    import torch

    from start_gb300 import StartPIC
    from start_gb300 import _native as N

    lib = N.load()
    w, rho, (rp, ci, av), lift, dv, isd, g = _problem()
    dev = torch.device("cuda", 0)
    t_rp = torch.from_numpy(rp.astype(np.int32)).to(dev)
    t_ci = torch.from_numpy(ci.astype(np.int32)).to(dev)
    t_av = torch.from_numpy(av).to(dev)
    n = len(rho)
    import oracle

    for scale in (1.0, -3.0):  # two calls in a row with different charge
        r = rho * scale
        # existing entry point: spg_solve on a fresh handle, which starts from
        # the Dirichlet values like the call below; the oracle likewise
        eng = StartPIC(w.mesh, w.params)
        ref, _, _ = eng.solve(r)
        eng.close()
        o = oracle.Oracle(w.mesh, w.params)
        cpu, _, cpu_rr = o.solve(r)
        o.close()
        assert cpu_rr <= 1e-12
        t_b = torch.from_numpy(_rhs(r, lift, dv, isd, g)).to(dev)
        t_x = torch.from_numpy(g.copy()).to(dev)  # same initial guess as a fresh handle
        torch.cuda.synchronize()
        it, rr = C.c_int32(), C.c_double()
        rc = lib.spg_pcg_solve_noalloc(n, t_rp.data_ptr(), t_ci.data_ptr(), t_av.data_ptr(), t_b.data_ptr(),
                                       t_x.data_ptr(), 1e-12, 20000, None, C.byref(it), C.byref(rr))
        assert rc == 0, lib.spg_last_error(None).decode()
        x = t_x.cpu().numpy()
        assert rr.value <= 1e-12 and it.value > 0
        assert np.max(np.abs(x - ref) / np.maximum(np.abs(ref), 1.0)) <= 1e-9
        assert np.max(np.abs(x - cpu) / np.maximum(np.abs(cpu), 1.0)) <= 1e-9


def _solve_small(lib, rp, ci, av, b, x0):
    import torch

    dev = torch.device("cuda", 0)
    t = [torch.from_numpy(np.asarray(a)).to(dev) for a in (np.int32(rp), np.int32(ci), av, b, x0)]
    torch.cuda.synchronize()
    it, rr = C.c_int32(), C.c_double()
    rc = lib.spg_pcg_solve_noalloc(len(b), *[a.data_ptr() for a in t], 1e-12, 100, None, C.byref(it), C.byref(rr))
    return rc, t[4].cpu().numpy(), it.value, rr.value


def test_noalloc_small_systems(built):
    from start_gb300 import _native as N

    lib = N.load()
    # 1-D Laplacian, 5 rows: SPD, solved to the stop rule
    n = 5
    A = 2.0 * np.eye(n) - np.eye(n, k=1) - np.eye(n, k=-1)
    rp = np.concatenate([[0], np.cumsum((A != 0).sum(1))])
    ci = np.nonzero(A)[1]
    av = A[A != 0]
    b = np.arange(1.0, n + 1)
    rc, x, it, rr = _solve_small(lib, rp, ci, av, b, np.zeros(n))
    assert rc == 0 and rr <= 1e-12
    assert np.allclose(x, np.linalg.solve(A, b), rtol=1e-10, atol=0)
    # b = 0: x becomes 0 whatever the initial guess
    rc, x, it, rr = _solve_small(lib, rp, ci, av, np.zeros(n), np.full(n, 7.0))
    assert rc == 0 and it == 0 and rr == 0.0 and not x.any()
    # a row without its diagonal entry is refused
    rc, *_ = _solve_small(lib, [0, 1, 2], [1, 0], np.array([1.0, 1.0]), np.ones(2), np.zeros(2))
    assert rc == N.SPG_E_INVALID and "diagonal" in lib.spg_last_error(None).decode()
    # -I is not positive definite: CG breaks down at the first step
    rc, *_ = _solve_small(lib, [0, 1, 2], [0, 1], np.array([-1.0, -1.0]), np.ones(2), np.zeros(2))
    assert rc == N.SPG_E_NOT_CONVERGED and "breakdown" in lib.spg_last_error(None).decode()


def test_noalloc_rejects_sizes_beyond_its_scratch(built):
    from start_gb300 import _native as N

    lib = N.load()
    dummy = C.c_void_p(1)  # never dereferenced: the size check comes first
    rc = lib.spg_pcg_solve_noalloc((1 << 17) + 1, dummy, dummy, dummy, dummy, dummy, 1e-10, 10, None, None, None)
    assert rc == N.SPG_E_INVALID
    assert "131072" in lib.spg_last_error(None).decode()

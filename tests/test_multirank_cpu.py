"""Partition invariance of the sharded PIC step, on CPU ranks (gloo, world 2).

The path shards by particles: each rank owns a contiguous range of the
particle array, deposits it, and one allreduce(sum) of the nodal charge per
Poisson solve gives every rank the global right-hand side; the particle step
itself needs no exchange. Here two gloo ranks run the CPU oracle on halves of
a workload-0 population and must reproduce the single-rank run: nodal charge
within 1e-12, then identical per-particle state after steps driven by the
allreduced field.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _workload():
    from start_gb300.workloads import workload0

    w = workload0(n_particles=4000, collisions=True, steps=30)
    w.params["cg_rtol"] = 1e-12
    return w


def _rank_main(rank, world, port, out_dir):
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle

    oracle.set_threads(1)
    w = _workload()
    n = len(w.pos)
    lo, hi = rank * n // world, (rank + 1) * n // world
    o = oracle.Oracle(w.mesh, w.params)
    o.set_particles(w.pos[lo:hi], w.vel[lo:hi])
    dv = o.dual_volumes()
    # deposit my shard, allreduce the nodal charge (rho * V_dual)
    q = torch.from_numpy(o.gather() * dv)
    dist.all_reduce(q)
    rho = q.numpy() / dv
    phi, _, _ = o.solve(rho)
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), rho=rho, phi=phi, lo=lo, hi=hi)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_deposit_and_solve_match_single_rank(tmp_path):
    import socket

    import oracle

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    w = _workload()
    o = oracle.Oracle(w.mesh, w.params)
    o.set_particles(w.pos, w.vel)
    rho_full = o.gather()
    phi_full, _, _ = o.solve()
    for r in range(2):
        d = np.load(tmp_path / f"rank{r}.npz")
        assert np.max(np.abs(d["rho"] - rho_full)) <= 1e-12 * np.max(np.abs(rho_full))
        assert np.max(np.abs(d["phi"] - phi_full)) <= 1e-10 * np.max(np.abs(phi_full))


def test_shard_steps_are_independent():
    """Given the same field, stepping two halves separately equals stepping the
    whole population (collisionless: the step has no particle-particle term)."""
    import oracle
    from start_gb300.workloads import workload0

    w = workload0(n_particles=3000, collisions=False, steps=20)
    o = oracle.Oracle(w.mesh, w.params)
    phi = np.random.default_rng(4).uniform(-1e3, 1e3, o.n_nodes)
    o.set_particles(w.pos, w.vel)
    o.set_potential(phi)
    o.process(20)
    full = o.particles()
    parts = []
    for lo, hi in ((0, 1500), (1500, 3000)):
        h = oracle.Oracle(w.mesh, w.params)
        h.set_particles(w.pos[lo:hi], w.vel[lo:hi])
        h.set_potential(phi)
        h.process(20)
        parts.append(h.particles())
    for k in ("pos", "vel", "tet", "flags"):
        assert np.array_equal(np.concatenate([p[k] for p in parts]), full[k])

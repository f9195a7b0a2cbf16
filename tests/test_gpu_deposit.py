"""The deposit's block tables under load: particles spread over many tets.

3e6 particles drawn uniformly over the 162,000 tets of the workload-0 box at
h = 3.3 mm, in input order (re-sort off), so each block's range of particles
touches thousands of tets: its table of tets fills past half, the tets it
does not hold go to the node accumulators directly, and the table is flushed
and cleared in the middle of the range. The fixed-point sums do not depend on
order, so the deposit must equal, bit for bit, the one made after the step-0
re-sort (long runs of equal tets, per-warp running sums) in both forms; the
FP64 form must also match the oracle (1e-12 relative, as the small-case
parity test) and both must conserve charge.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 3_000_000


def _spread(resort_every, precision):
    from start_gb300.workloads import workload0

    w = workload0(n_particles=10, collisions=False, steps=1, cells=30)
    w.params.update(resort_every=resort_every, precision=precision)
    rng = np.random.default_rng(11)
    pos = rng.uniform(1e-4, 0.1 - 1e-4, size=(N, 3))
    return w, pos, np.zeros_like(pos)


def _gpu_rho(resort_every, precision):
    from start_gb300 import StartPIC

    w, pos, vel = _spread(resort_every, precision)
    g = StartPIC(w.mesh, w.params)
    g.set_particles(pos, vel)
    rho = g.gather()
    g.close()
    return w, pos, vel, rho


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "mixed"])
def test_deposit_spread_unsorted_equals_sorted(built, precision):
    import oracle

    w, pos, vel, unsorted = _gpu_rho(0, precision)
    _, _, _, ordered = _gpu_rho(20, precision)
    assert np.array_equal(unsorted, ordered)
    o = oracle.Oracle(w.mesh, dict(w.params, precision=0))
    o.set_particles(pos, vel)
    ro = o.gather()
    dv = o.dual_volumes()
    total = w.params["weight"] * w.params["charge"] * N
    assert abs(np.dot(unsorted, dv) - total) <= 1e-12 * total
    if precision == 0:
        assert np.max(np.abs(unsorted - ro)) <= 1e-12 * np.max(np.abs(ro))
    else:
        # FP32 barycentrics of the tet-local position: ~1e-7 of a particle's share
        assert np.max(np.abs(unsorted - ro)) <= 1e-5 * np.max(np.abs(ro))

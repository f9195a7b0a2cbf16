"""The reference-named C++ path, run: tests/native/pic_loop_driver.cpp is the
time loop of ModelingMainDriver::startModeling (src/ModelingMainDriver.cpp:
146-184) written against include/start_pic.hpp (NodeChargeDensityProcessor::
gather -> ChargeDensityEquationSolver::solve -> ParticleDynamicsProcessor::
process). It is compiled with g++, linked to libstart_gpu.so and run on
workload 0 without gas; the oracle runs the same loop (oracle run: deposit and
solve every 10 steps, then the step).

Bars (the collisionless parity bars): every tet id and flag identical,
positions within 1e-9 relative, triangle counters identical; the nodal
density the shim reads lazily after the loop within 1e-12 of the oracle's
deposit at the same state; the potential within 1e-9; the density stayed on
the GPU until it was read, and solving it from the device copy or from its
uploaded host values gives the same potential within 1e-9.
"""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


def _compile(lib, out):
    src = ROOT / "tests" / "native" / "pic_loop_driver.cpp"
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-I", str(ROOT / "include"), str(src), "-L",
                    str(lib.parent), "-lstart_gpu", f"-Wl,-rpath,{lib.parent}", "-o", str(out)], check=True)


def _write_input(path, w, steps, every):
    from start_gb300.engine import _params_struct

    prm = _params_struct(w.params)
    m = w.mesh
    dn = np.ascontiguousarray(m.dirichlet_nodes, np.int32)
    with open(path, "wb") as f:
        f.write(b"SPGLOOP1")
        f.write(np.int64(C.sizeof(prm)).tobytes())
        f.write(bytes(prm))
        for arr, dt in ((m.nodes, np.float64), (m.tets, np.int32), (m.triangles, np.int32)):
            a = np.ascontiguousarray(arr, dt)
            f.write(np.int64(len(a)).tobytes())
            f.write(a.tobytes())
        f.write(np.int64(len(dn)).tobytes())
        f.write(dn.tobytes())
        f.write(np.ascontiguousarray(m.dirichlet_values, np.float64).tobytes())
        f.write(np.int64(len(w.pos)).tobytes())
        f.write(np.ascontiguousarray(w.pos, np.float64).tobytes())
        f.write(np.ascontiguousarray(w.vel, np.float64).tobytes())
        f.write(np.int64(steps).tobytes())
        f.write(np.int64(every).tobytes())


def _read_output(path, n, nn, ntri):
    b = open(path, "rb").read()
    o = 0

    def take(dt, count):
        nonlocal o
        a = np.frombuffer(b, dt, count, o)
        o += a.nbytes
        return a

    steps_run, n_alive, iters = take(np.int64, 3)
    r = dict(steps_run=int(steps_run), n_alive=int(n_alive), iters=int(iters))
    r["pos"] = take(np.float64, 3 * n).reshape(n, 3)
    r["vel"] = take(np.float64, 3 * n).reshape(n, 3)
    r["tet"] = take(np.int32, n)
    r["flags"] = take(np.uint32, n)
    r["counts"] = take(np.uint64, ntri)
    for k in ("rho", "phi", "phi_res", "phi_up"):
        r[k] = take(np.float64, nn)
    r["resident"] = int(take(np.int64, 1)[0])
    assert o == len(b)
    return r


def test_reference_loop_through_cpp_shim(built, tmp_path):
    import oracle
    from start_gb300.workloads import workload0

    lib, _ = built
    exe = tmp_path / "pic_loop_driver"
    _compile(lib, exe)
    steps, every = 200, 10
    w = workload0(n_particles=10000, collisions=False, steps=steps)
    w.params.update(cg_rtol=1e-12, poisson_every=every)
    _write_input(tmp_path / "in.bin", w, steps, every)
    run = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True,
                         text=True)
    assert run.returncode == 0, run.stderr
    n, nn, ntri = len(w.pos), w.mesh.n_nodes, w.mesh.n_triangles
    g = _read_output(tmp_path / "out.bin", n, nn, ntri)

    o = oracle.Oracle(w.mesh, w.params)
    o.set_particles(w.pos, w.vel)
    # the loop stops once every ion has settled (StopSubject); the oracle
    # runs the same number of steps and deposits where the loop last did
    ran = g["steps_run"]
    assert 0 < ran <= steps
    last = (ran - 1) // every * every
    o.run(last)
    rho_o = o.gather()
    so = o.run(ran - last)
    po = o.particles()
    assert ran == steps or so["n_alive"] == 0
    assert np.array_equal(g["tet"], po["tet"])
    assert np.array_equal(g["flags"], po["flags"])
    rel = np.abs(g["pos"] - po["pos"]) / np.maximum(np.abs(po["pos"]), 1e-3)
    assert rel.max() <= 1e-9
    assert np.array_equal(g["counts"], o.triangle_counts())
    assert g["n_alive"] == so["n_alive"]
    assert np.max(np.abs(g["rho"] - rho_o)) <= 1e-12 * np.max(np.abs(rho_o))
    pho = o.potential()
    scale = np.max(np.abs(pho))
    assert np.max(np.abs(g["phi"] - pho)) <= 1e-9 * scale
    assert g["resident"] == 1
    assert np.max(np.abs(g["phi_res"] - g["phi"])) <= 1e-9 * scale
    assert np.max(np.abs(g["phi_up"] - g["phi"])) <= 1e-9 * scale

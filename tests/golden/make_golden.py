"""Generates the committed golden fixtures under tests/golden/.

1. ref_meshes.npz: the reference's own Gmsh test meshes
   (tests/meshes/TetrahedronTestMesh.msh.gtest and BoxMeshTest.msh.gtest in
   ViNN280801/Start), read with start_gb300.mesh.read_msh41 and stored as
   arrays (millimetres), so the tests need no access to the reference tree.
2. oracle_w0_*.npz: inputs and outputs of the CPU oracle on reduced
   workload-0 runs (2,000 particles, 200 steps), collisionless and with HS
   collisions. Inputs are stored with the outputs so that the fixtures do not
   depend on the platform's numpy transcendental functions.

Run from the repository root:
    python tests/golden/make_golden.py REFERENCE_ROOT
or with REFERENCE_ROOT in the environment variable START_REFERENCE_ROOT. The
reference tree is needed only for ref_meshes.npz; without one, only the
oracle fixtures are rewritten.
"""
from __future__ import annotations

import platform
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))


def ref_meshes(ref_root: Path):
    from start_gb300.mesh import read_msh41

    out = {}
    for name in ("TetrahedronTestMesh", "BoxMeshTest"):
        m = read_msh41(ref_root / "tests" / "meshes" / f"{name}.msh.gtest", scale=1.0)
        out[f"{name}_nodes"] = m.nodes
        out[f"{name}_tets"] = m.tets
        out[f"{name}_triangles"] = m.triangles
        out[f"{name}_tri_tag"] = m.tri_tag
    np.savez_compressed(HERE / "ref_meshes.npz", **out)


def oracle_case(name, collisions):
    import oracle
    from start_gb300.workloads import workload0

    w = workload0(n_particles=2000, collisions=collisions, steps=200)
    w.params["cg_rtol"] = 1e-12
    if collisions:
        w.params["gas_concentration"] *= 200.0
    o = oracle.Oracle(w.mesh, w.params)
    o.set_particles(w.pos, w.vel)
    st = o.run(w.steps)
    p = o.particles()
    np.savez_compressed(
        HERE / f"oracle_w0_{name}.npz",
        pos0=w.pos, vel0=w.vel, pos=p["pos"], vel=p["vel"], tet=p["tet"], flags=p["flags"],
        tri_count=o.triangle_counts(), phi=o.potential(), steps=w.steps,
        gas_concentration=w.params["gas_concentration"], collision_model=w.params["collision_model"],
        particle_steps=st["particle_steps"], collisions=st["collisions"], crossings=st["crossings"],
        machine=platform.machine())


if __name__ == "__main__":
    import os

    arg = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("START_REFERENCE_ROOT")
    if arg:
        ref = Path(arg)
        if not (ref / "tests" / "meshes").is_dir():
            sys.exit(f"{ref} is not a reference tree (no tests/meshes)")
        ref_meshes(ref)
    else:
        print("no reference tree given: ref_meshes.npz left as it is")
    oracle_case("collisionless", False)
    oracle_case("hs", True)
    print("written:", sorted(p.name for p in HERE.glob("*.npz")))

"""Run outputs in the layout of the reference's HDF5 writers, as NPZ.

libhdf5 is not part of this build, so the data the reference writes with
HDF5 is written as NumPy NPZ with the same fields:

* surface deposition per triangle, TriangleMeshHdf5Manager::saveMeshToHDF5
  (src/DataHandling/TriangleMeshHdf5Manager.cpp:97-140): for each triangle id
  a group Triangle_<id> with Coordinates (9 doubles, the three vertices),
  Area (double) and Counter (size_t);
* settled particle positions, SettledParticleHDF5Writer
  (src/DataHandling/SettledParticleHDF5Writer.cpp:7-60): one N x 3 double
  dataset.

`to_hdf5` converts either file to HDF5 where h5py is installed.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np


def triangle_areas(nodes: np.ndarray, triangles: np.ndarray) -> np.ndarray:
    a, b, c = (nodes[triangles[:, k]] for k in range(3))
    return 0.5 * np.linalg.norm(np.cross(b - a, c - a), axis=1)


def write_triangle_counts(path, nodes, triangles, counts, ids=None, length_scale=1.0):
    """Writes the per-triangle deposition counters.

    nodes [Nn, 3] (metres), triangles [Ntri, 3] node indices, counts [Ntri]
    (spg_get_triangle_counts). ids: the triangle ids of the reference's
    TriangleCellMap (default 0..Ntri-1). length_scale multiplies coordinates
    and area (1e3: millimetres as in the reference's mesh files).
    """
    nodes = np.asarray(nodes, np.float64)
    triangles = np.asarray(triangles, np.int64).reshape(-1, 3)
    counts = np.asarray(counts)
    if counts.shape != (len(triangles),):
        raise ValueError("counts must have one entry per triangle")
    ids = np.arange(len(triangles), dtype=np.uint64) if ids is None else np.asarray(ids, np.uint64)
    coords = (nodes[triangles] * length_scale).reshape(-1, 9)
    area = triangle_areas(nodes, triangles) * length_scale**2
    np.savez(path, kind="TriangleMesh", id=ids, Coordinates=coords, Area=area,
             Counter=counts.astype(np.uint64))


def write_settled_particles(path, positions, flags, settled_bit=1, length_scale=1.0):
    """Writes the positions of the settled particles (flags & settled_bit)."""
    positions = np.asarray(positions, np.float64).reshape(-1, 3)
    sel = (np.asarray(flags) & settled_bit) != 0
    np.savez(path, kind="SettledParticles", positions=positions[sel] * length_scale)


def write_movements_json(path, tracks: dict):
    """Tracks in the layout of ParticleMovementTracker::saveMovementsToJson
    (ParticleMovementTracker.cpp:18-46): {"<id>": [{"x":..,"y":..,"z":..}, ...]}
    for every particle with more than one recorded position."""
    import json

    out = {str(k): [{"x": float(p[0]), "y": float(p[1]), "z": float(p[2])} for p in v]
           for k, v in tracks.items() if len(v) > 1}
    Path(path).write_text(json.dumps(out, indent=4))


def read(path) -> dict:
    with np.load(path, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def to_hdf5(npz_path, h5_path):
    """Converts an NPZ written here into the reference's HDF5 layout."""
    try:
        import h5py
    except ImportError as e:
        raise RuntimeError("to_hdf5 needs h5py, which is not installed") from e
    d = read(npz_path)
    with h5py.File(Path(h5_path), "w") as f:
        if str(d["kind"]) == "TriangleMesh":
            for k, tid in enumerate(d["id"]):
                g = f.create_group(f"Triangle_{int(tid)}")
                g.create_dataset("Coordinates", data=d["Coordinates"][k])
                g.create_dataset("Area", data=np.array([d["Area"][k]]))
                g.create_dataset("Counter", data=np.array([d["Counter"][k]], np.uint64))
        else:
            f.create_dataset("settled", data=d["positions"])

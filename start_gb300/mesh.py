"""Tet meshes for the PIC step: synthetic Kuhn boxes and a Gmsh 4.1 reader.

The reference reads Gmsh meshes (VolumetricMesh::_readMesh,
src/Geometry/Mesh/Volumetric/VolumetricMesh.cpp:35-121) and takes its surface
triangles from Gmsh type-2 elements (GmshUtils::getTriangleCellsMap,
src/Utilities/GmshUtilities/GmshUtils.cpp:96-153). Gmsh itself is not
available, so the workloads use a generated Kuhn (Freudenthal) split of a box
lattice: every cell is cut into the six tets that share its main diagonal,
which is conforming across cells. Tets are numbered in Morton order of their
cell so that tet-sorted particles walk memory in space-filling-curve order.
Coordinates are metres; the reference's meshes are in millimetres.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from itertools import permutations
from pathlib import Path

import numpy as np

# Box faces in triangle-tag order: (axis, side).
BOX_FACES = [(0, 0), (0, 1), (1, 0), (1, 1), (2, 0), (2, 1)]


@dataclass
class TetMesh:
    nodes: np.ndarray  # (Nn, 3) float64, metres
    tets: np.ndarray  # (Nt, 4) int32, positively oriented
    triangles: np.ndarray  # (Ntri, 3) int32; triangle id = row
    tri_tag: np.ndarray  # (Ntri,) int32 surface group (box face 1..6, plates 7..)
    dirichlet_nodes: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    dirichlet_values: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    meta: dict = field(default_factory=dict)

    @property
    def n_nodes(self):
        return len(self.nodes)

    @property
    def n_tets(self):
        return len(self.tets)

    @property
    def n_triangles(self):
        return len(self.triangles)

    def volumes(self) -> np.ndarray:
        p = self.nodes[self.tets]
        a, b, c = p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]
        return np.einsum("ij,ij->i", a, np.cross(b, c)) / 6.0

    def triangle_areas(self) -> np.ndarray:
        p = self.nodes[self.triangles]
        return 0.5 * np.linalg.norm(np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), axis=1)

    def triangle_centroids(self) -> np.ndarray:
        return self.nodes[self.triangles].mean(axis=1)

    def with_dirichlet(self, nodes, values) -> "TetMesh":
        self.dirichlet_nodes = np.ascontiguousarray(nodes, dtype=np.int32)
        self.dirichlet_values = np.ascontiguousarray(values, dtype=np.float64)
        return self


def _morton3(i, j, k):
    def spread(v):
        v = v.astype(np.uint64) & np.uint64(0x1FFFFF)
        v = (v | (v << np.uint64(32))) & np.uint64(0x1F00000000FFFF)
        v = (v | (v << np.uint64(16))) & np.uint64(0x1F0000FF0000FF)
        v = (v | (v << np.uint64(8))) & np.uint64(0x100F00F00F00F00F)
        v = (v | (v << np.uint64(4))) & np.uint64(0x10C30C30C30C30C3)
        v = (v | (v << np.uint64(2))) & np.uint64(0x1249249249249249)
        return v

    return spread(i) | (spread(j) << np.uint64(1)) | (spread(k) << np.uint64(2))


def _kuhn_local():
    """Six tets of the unit cube as corner indices (corner c = x + 2y + 4z),
    each positively oriented."""
    unit = [np.array([1, 0, 0]), np.array([0, 1, 0]), np.array([0, 0, 1])]
    out = []
    for perm in permutations(range(3)):
        v = [np.zeros(3, int)]
        for a in perm:
            v.append(v[-1] + unit[a])
        idx = [int(p[0] + 2 * p[1] + 4 * p[2]) for p in v]
        P = np.array(v, float)
        det = np.dot(P[1] - P[0], np.cross(P[2] - P[0], P[3] - P[0]))
        if det < 0:
            idx[2], idx[3] = idx[3], idx[2]
        out.append(idx)
    return np.array(out, np.int64)


def kuhn_box(cells, lengths, origin=(0.0, 0.0, 0.0)) -> TetMesh:
    """Kuhn 6-tet split of an nx*ny*nz lattice over a box (metres).

    Boundary triangles: two per lattice square on each box face, tagged 1..6
    in the order x=0, x=L, y=0, y=L, z=0, z=L."""
    nx, ny, nz = (int(c) for c in cells)
    L = np.asarray(lengths, float)
    o = np.asarray(origin, float)
    NX, NY = nx + 1, ny + 1
    gi, gj, gk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    nodes = np.empty(((nx + 1) * (ny + 1) * (nz + 1), 3))
    nid = (gi + NX * (gj + NY * gk)).ravel()
    nodes[nid, 0] = o[0] + gi.ravel() * (L[0] / nx)
    nodes[nid, 1] = o[1] + gj.ravel() * (L[1] / ny)
    nodes[nid, 2] = o[2] + gk.ravel() * (L[2] / nz)
    # exact end planes
    nodes[nid[gi.ravel() == nx], 0] = o[0] + L[0]
    nodes[nid[gj.ravel() == ny], 1] = o[1] + L[1]
    nodes[nid[gk.ravel() == nz], 2] = o[2] + L[2]

    ci, cj, ck = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    order = np.argsort(_morton3(ci, cj, ck), kind="stable")
    ci, cj, ck = ci[order], cj[order], ck[order]
    base = ci + NX * (cj + NY * ck)
    corner_off = np.array([dx + NX * (dy + NY * dz) for dz in (0, 1) for dy in (0, 1) for dx in (0, 1)])
    loc = _kuhn_local()  # (6, 4) corner ids
    tets = (base[:, None, None] + corner_off[loc][None, :, :]).reshape(-1, 4).astype(np.int32)

    tris, tags = [], []
    for f, (axis, side) in enumerate(BOX_FACES):
        a, b = [d for d in range(3) if d != axis]
        na, nb = (nx, ny, nz)[a], (nx, ny, nz)[b]
        ia, ib = np.meshgrid(np.arange(na), np.arange(nb), indexing="ij")
        ia, ib = ia.ravel(), ib.ravel()
        fixed = 0 if side == 0 else (nx, ny, nz)[axis]

        def nid_of(da, db):
            idx = [None, None, None]
            idx[axis] = np.full_like(ia, fixed)
            idx[a] = ia + da
            idx[b] = ib + db
            return idx[0] + NX * (idx[1] + NY * idx[2])

        c00, c10, c01, c11 = nid_of(0, 0), nid_of(1, 0), nid_of(0, 1), nid_of(1, 1)
        t1 = np.stack([c00, c10, c11], axis=1)
        t2 = np.stack([c00, c01, c11], axis=1)
        tt = np.stack([t1, t2], axis=1).reshape(-1, 3)
        tris.append(tt)
        tags.append(np.full(len(tt), f + 1, np.int32))
    m = TetMesh(nodes=nodes, tets=tets, triangles=np.concatenate(tris).astype(np.int32),
                tri_tag=np.concatenate(tags))
    m.meta.update(kind="kuhn_box", cells=(nx, ny, nz), lengths=tuple(L), origin=tuple(o),
                  h=tuple(L / np.array([nx, ny, nz])))
    return m


def box_face_nodes(m: TetMesh, axis: int, side: int, tol: float = 1e-12) -> np.ndarray:
    lo = m.nodes[:, axis].min()
    hi = m.nodes[:, axis].max()
    target = lo if side == 0 else hi
    return np.nonzero(np.abs(m.nodes[:, axis] - target) <= tol * max(1.0, abs(target)) + 1e-15)[0].astype(np.int32)


def add_plate(m: TetMesh, z: float, xlim, ylim, tag: int, tol=1e-12):
    """Mark an internal plate z = const over xlim x ylim: its lattice squares
    become surface triangles (one per tet face pair) and its nodes are
    returned for Dirichlet conditions. z and the limits must be lattice planes."""
    nx, ny, nz = m.meta["cells"]
    NX, NY = nx + 1, ny + 1
    hx, hy, hz = m.meta["h"]
    ox, oy, oz = m.meta["origin"]
    k = int(round((z - oz) / hz))
    i0, i1 = int(round((xlim[0] - ox) / hx)), int(round((xlim[1] - ox) / hx))
    j0, j1 = int(round((ylim[0] - oy) / hy)), int(round((ylim[1] - oy) / hy))
    if abs(oz + k * hz - z) > 1e-9 or abs(ox + i0 * hx - xlim[0]) > 1e-9 or abs(ox + i1 * hx - xlim[1]) > 1e-9:
        raise ValueError("plate must lie on lattice planes")
    ia, ib = np.meshgrid(np.arange(i0, i1), np.arange(j0, j1), indexing="ij")
    ia, ib = ia.ravel(), ib.ravel()

    def nid(da, db):
        return (ia + da) + NX * ((ib + db) + NY * k)

    c00, c10, c01, c11 = nid(0, 0), nid(1, 0), nid(0, 1), nid(1, 1)
    t = np.stack([np.stack([c00, c10, c11], 1), np.stack([c00, c01, c11], 1)], 1).reshape(-1, 3)
    m.triangles = np.concatenate([m.triangles, t.astype(np.int32)])
    m.tri_tag = np.concatenate([m.tri_tag, np.full(len(t), tag, np.int32)])
    gi, gj = np.meshgrid(np.arange(i0, i1 + 1), np.arange(j0, j1 + 1), indexing="ij")
    return (gi.ravel() + NX * (gj.ravel() + NY * k)).astype(np.int32)


def jitter(m: TetMesh, frac: float, seed: int, frozen: np.ndarray | None = None, min_ratio: float = 0.05):
    """Move nodes by U(-frac*h, frac*h) per axis, keeping box-boundary nodes on
    their planes and `frozen` nodes fixed; tets whose volume would fall below
    min_ratio of the original have their nodes' moves undone until none is left."""
    rng = np.random.default_rng(seed)
    h = np.asarray(m.meta["h"])
    d = rng.uniform(-frac, frac, size=m.nodes.shape) * h
    lo, hi = m.nodes.min(0), m.nodes.max(0)
    for ax in range(3):
        on = (m.nodes[:, ax] <= lo[ax] + 1e-12) | (m.nodes[:, ax] >= hi[ax] - 1e-12)
        d[on, ax] = 0.0
    if frozen is not None and len(frozen):
        d[frozen] = 0.0
    v0 = m.volumes()
    base = m.nodes.copy()
    for _ in range(50):
        m.nodes = base + d
        v = m.volumes()
        bad = v < min_ratio * v0
        if not bad.any():
            break
        d[np.unique(m.tets[bad].ravel())] = 0.0
    else:
        m.nodes = base
    m.meta["jitter"] = frac
    return m


# ---------------------------------------------------------------- Gmsh 4.1

def read_msh41(path: str | Path, scale: float = 1.0) -> TetMesh:
    """Read an ASCII Gmsh 4.1 mesh: nodes, type-4 tets and type-2 triangles.

    Node index = node tag - 1 (GSMAssembler.cpp:10-72); triangle ids follow
    element order; tri_tag is the triangle's entity tag. `scale` converts
    coordinates (0.001 for millimetre meshes)."""
    lines = Path(path).read_text().splitlines()
    pos = 0

    def seek(tag):
        nonlocal pos
        while lines[pos].strip() != tag:
            pos += 1
        pos += 1

    seek("$MeshFormat")
    ver = lines[pos].split()[0]
    if not ver.startswith("4"):
        raise ValueError(f"unsupported msh version {ver}")
    seek("$Nodes")
    n_blocks, n_nodes, _min_tag, max_tag = map(int, lines[pos].split())
    pos += 1
    coords = np.zeros((max_tag, 3))
    for _ in range(n_blocks):
        _dim, _ent, parametric, count = map(int, lines[pos].split())
        pos += 1
        tags = [int(lines[pos + k]) for k in range(count)]
        pos += count
        for k in range(count):
            vals = lines[pos + k].split()
            coords[tags[k] - 1] = [float(v) for v in vals[:3]]
        pos += count
        del parametric
    seek("$Elements")
    n_blocks, _n_el, _a, _b = map(int, lines[pos].split())
    pos += 1
    tets, tris, ttag = [], [], []
    for _ in range(n_blocks):
        _dim, ent, etype, count = map(int, lines[pos].split())
        pos += 1
        for k in range(count):
            v = list(map(int, lines[pos + k].split()))
            if etype == 4:
                tets.append([x - 1 for x in v[1:5]])
            elif etype == 2:
                tris.append([x - 1 for x in v[1:4]])
                ttag.append(ent)
        pos += count
    tets = np.asarray(tets, np.int32).reshape(-1, 4)
    nodes = coords * scale
    # orient positively
    p = nodes[tets]
    det = np.einsum("ij,ij->i", p[:, 1] - p[:, 0], np.cross(p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]))
    neg = det < 0
    tets[neg, 2], tets[neg, 3] = tets[neg, 3].copy(), tets[neg, 2].copy()
    m = TetMesh(nodes=nodes, tets=tets, triangles=np.asarray(tris, np.int32).reshape(-1, 3),
                tri_tag=np.asarray(ttag, np.int32))
    m.meta.update(kind="msh41", source=str(path), n_node_tags=n_nodes)
    return m

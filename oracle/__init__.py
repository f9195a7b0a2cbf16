"""CPU oracle of the PIC/DSMC step -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package, as the checker of the GPU library; the product never does.
`Oracle` has the same methods as start_gb300.StartPIC so tests can run both
on the same inputs.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import OUT, build_oracle

_pd = C.POINTER(C.c_double)
_pi32 = C.POINTER(C.c_int32)
_pu32 = C.POINTER(C.c_uint32)
_pu64 = C.POINTER(C.c_uint64)
_H = C.c_void_p

_lib = None


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def load(path: str | Path | None = None):
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else OUT
    if not p.exists():
        build_oracle()
    from start_gb300 import _native as N

    lib = C.CDLL(str(p))
    sig = {
        "spo_last_error": (C.c_char_p, []),
        "spo_set_threads": (C.c_int, [C.c_int]),
        "spo_get_threads": (C.c_int, []),
        "spo_create": (C.c_int, [C.POINTER(N.MeshDesc), C.POINTER(N.Params), C.POINTER(_H)]),
        "spo_destroy": (None, [_H]),
        "spo_mesh_info": (C.c_int, [_H, C.POINTER(C.c_int64)]),
        "spo_set_particles": (C.c_int, [_H, C.c_int64, _pd, _pd, _pi32]),
        "spo_get_particles": (C.c_int, [_H, C.c_int64, _pd, _pd, _pi32, _pu32]),
        "spo_gather": (C.c_int, [_H, _pd]),
        "spo_solve": (C.c_int, [_H, _pd, _pd, _pi32, _pd]),
        "spo_process": (C.c_int, [_H, C.c_int32]),
        "spo_process_range": (C.c_int, [_H, C.c_int64, C.c_int64]),
        "spo_run": (C.c_int, [_H, C.c_int32]),
        "spo_get_stats": (C.c_int, [_H, C.POINTER(N.Stats)]),
        "spo_get_triangle_counts": (C.c_int, [_H, _pu64]),
        "spo_get_potential": (C.c_int, [_H, _pd]),
        "spo_set_potential": (C.c_int, [_H, _pd]),
        "spo_get_efield": (C.c_int, [_H, _pd]),
        "spo_locate": (C.c_int, [_H, C.c_int64, _pd, _pi32]),
        "spo_get_matrix": (C.c_int, [_H, _pi32, _pi32, _pd, _pd]),
        "spo_get_dual_volumes": (C.c_int, [_H, _pd]),
        "spo_set_dirichlet": (C.c_int, [_H, _pd]),
        "spo_grad": (C.c_int, [_H, C.c_int32, _pd, C.c_double, _pd, C.POINTER(C.c_int64), _pd, _pd, _pd]),
        "spo_grad_freeze": (C.c_int, [_H, C.c_int]),
        "spo_grad_field_gradient": (C.c_int, [_H, C.c_int]),
        "spo_update_position": (None, [_pd, _pd, C.c_double]),
        "spo_segment_triangle": (C.c_int, [_pd, _pd, _pd, _pd, _pd, _pd]),
        "spo_gas_concentration": (C.c_double, [C.c_double, C.c_double]),
        "spo_collide_with": (C.c_int, [C.POINTER(N.Params), _pd, C.c_double, C.c_double, C.c_double]),
        "spo_collision_probability": (C.c_double, [C.POINTER(N.Params), _pd]),
        "spo_tet_map": (C.c_double, [_pd, _pd, _pd, _pd, _pd]),
        "spo_philox": (None, [_pu32, _pu32, _pu32]),
        "spo_collides": (None, [C.POINTER(C.c_uint64), _pu32, C.c_int64, C.c_uint64, C.c_double,
                                C.POINTER(C.c_uint8)]),
        "spo_set_ref_compat": (C.c_int, [_H, C.c_uint32, C.c_double]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def set_threads(n: int):
    load().spo_set_threads(int(n))


def get_threads() -> int:
    return int(load().spo_get_threads())


def params_struct(params):
    from start_gb300 import _native as N

    if isinstance(params, N.Params):
        return params
    p = N.Params()
    # defaults identical to spg_default_params, without loading the GPU library
    defaults = dict(dt=1e-8, charge=1.602176565e-19, mass=7.9485017e-26, weight=1.0, collision_model=0, precision=0,
                    gas_mass=6.6335209e-26, gas_concentration=0.0, hs_diameter=3.6e-10, vhs_dref=4.17e-10,
                    omega=0.81, alpha=1.40, kT_ref=297.0 * 1.380658e-23, epsilon0=8.8541878128e-12,
                    min_velocity=10.0, bbox_expansion=1.01, seed=0, poisson_every=10, resort_every=20,
                    max_crossings=4096, cg_max_iter=20000, cg_rtol=1e-10, device=0, preconditioner=0)
    defaults.update(dict(params))
    for k, v in defaults.items():
        setattr(p, k, v)
    return p


# Reference-behaviour switches of the oracle (pic_oracle.h, SPO_COMPAT_*): each
# reproduces one behaviour of the reference's own loop that the build changes.
PUSH_NEVER = 1          # src/Particle/Particle.cpp:113-155, src/Geometry/Mesh/Cubic/CubicGrid.cpp:149-158
E_SIGN_SCALE = 2        # src/Geometry/Mesh/Volumetric/VolumetricMesh.cpp:371-375,398
RHS_RAW_RHO = 4         # src/ParticleInCellEngine/ChargeDensityEquationSolver.cpp:17-29
DEPOSIT_VOLAVG = 8      # src/ParticleInCellEngine/NodeChargeDensityProcessor.cpp:25-113
CLOSED_TETS = 16        # src/Geometry/Mesh/Volumetric/VolumetricMesh.cpp:23-33
SOLVE_EVERY_STEP = 32   # src/ModelingMainDriver.cpp:146-161
MIXED_UNITS = 64        # src/Particle/Particle.cpp:157-165
REFERENCE_LOOP = 127    # all of them: the reference's own time loop


class Oracle:
    """CPU counterpart of start_gb300.StartPIC."""

    def __init__(self, mesh, params):
        from start_gb300 import _native as N

        self.lib = load()
        self.mesh = mesh
        self.params = params_struct(params)
        self._nodes = np.ascontiguousarray(mesh.nodes, np.float64)
        self._tets = np.ascontiguousarray(mesh.tets, np.int32)
        self._tris = np.ascontiguousarray(mesh.triangles, np.int32).reshape(-1, 3)
        self._dn = np.ascontiguousarray(mesh.dirichlet_nodes, np.int32)
        self._dv = np.ascontiguousarray(mesh.dirichlet_values, np.float64)
        d = N.MeshDesc()
        d.n_nodes = len(self._nodes)
        d.node_xyz = _ptr(self._nodes, C.c_double)
        d.n_tets = len(self._tets)
        d.tet_nodes = _ptr(self._tets, C.c_int32)
        d.n_triangles = len(self._tris)
        d.tri_nodes = _ptr(self._tris, C.c_int32)
        d.n_dirichlet = len(self._dn)
        d.dirichlet_nodes = _ptr(self._dn, C.c_int32)
        d.dirichlet_values = _ptr(self._dv, C.c_double)
        h = C.c_void_p()
        rc = self.lib.spo_create(C.byref(d), C.byref(self.params), C.byref(h))
        if rc != 0:
            raise RuntimeError(f"oracle create failed [{rc}]: {self.lib.spo_last_error().decode()}")
        self.h = h
        info = (C.c_int64 * 6)()
        self.lib.spo_mesh_info(self.h, info)
        self.n_nodes, self.n_tets, self.n_triangles, self.n_boundary_faces, self.nnz, self.n_dirichlet = list(info)
        self.n_particles = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.spo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_particles(self, pos, vel, tet=None):
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        vel = np.ascontiguousarray(vel, np.float64).reshape(-1, 3)
        tet = None if tet is None else np.ascontiguousarray(tet, np.int32)
        rc = self.lib.spo_set_particles(self.h, len(pos), _ptr(pos, C.c_double), _ptr(vel, C.c_double),
                                        _ptr(tet, C.c_int32))
        if rc:
            raise RuntimeError(self.lib.spo_last_error().decode())
        self.n_particles = len(pos)

    def particles(self):
        n = self.n_particles
        pos, vel = np.empty((n, 3)), np.empty((n, 3))
        tet, flags = np.empty(n, np.int32), np.empty(n, np.uint32)
        self.lib.spo_get_particles(self.h, n, _ptr(pos, C.c_double), _ptr(vel, C.c_double), _ptr(tet, C.c_int32),
                                   _ptr(flags, C.c_uint32))
        return dict(pos=pos, vel=vel, tet=tet, flags=flags)

    def locate(self, pos):
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        out = np.empty(len(pos), np.int32)
        self.lib.spo_locate(self.h, len(pos), _ptr(pos, C.c_double), _ptr(out, C.c_int32))
        return out

    def gather(self, want_rho=True):
        rho = np.empty(self.n_nodes) if want_rho else None
        self.lib.spo_gather(self.h, _ptr(rho, C.c_double))
        return rho

    def solve(self, rho=None, want_phi=True, raise_on_nonconvergence=True):
        phi = np.empty(self.n_nodes) if want_phi else None
        it, rr = C.c_int32(), C.c_double()
        rho = None if rho is None else np.ascontiguousarray(rho, np.float64)
        rc = self.lib.spo_solve(self.h, _ptr(rho, C.c_double), _ptr(phi, C.c_double), C.byref(it), C.byref(rr))
        if rc and raise_on_nonconvergence:
            raise RuntimeError(self.lib.spo_last_error().decode())
        return phi, it.value, rr.value

    def process(self, nsteps=1):
        self.lib.spo_process(self.h, int(nsteps))
        return self.stats()

    def process_range(self, first, count):
        rc = self.lib.spo_process_range(self.h, int(first), int(count))
        if rc:
            raise RuntimeError(self.lib.spo_last_error().decode())

    def run(self, nsteps, raise_on_nonconvergence=True):
        rc = self.lib.spo_run(self.h, int(nsteps))
        if rc and raise_on_nonconvergence:
            raise RuntimeError("oracle PCG did not converge")
        return self.stats()

    def stats(self):
        from start_gb300 import _native as N

        st = N.Stats()
        self.lib.spo_get_stats(self.h, C.byref(st))
        return st.as_dict()

    def triangle_counts(self):
        c = np.zeros(self.n_triangles, np.uint64)
        self.lib.spo_get_triangle_counts(self.h, _ptr(c, C.c_uint64))
        return c

    def potential(self):
        phi = np.empty(self.n_nodes)
        self.lib.spo_get_potential(self.h, _ptr(phi, C.c_double))
        return phi

    def set_ref_compat(self, flags, cubature_w0=1.0 / 6.0):
        """Turns on reference-behaviour switches (PUSH_NEVER, ...); cubature_w0
        is the weight of cubature point 0 that E_SIGN_SCALE multiplies in
        (1/6 for the one-point rule on the unit tet)."""
        rc = self.lib.spo_set_ref_compat(self.h, int(flags), float(cubature_w0))
        if rc != 0:
            raise ValueError(self.lib.spo_last_error().decode())

    def set_potential(self, phi):
        phi = np.ascontiguousarray(phi, np.float64)
        self.lib.spo_set_potential(self.h, _ptr(phi, C.c_double))

    def efield(self):
        E = np.empty((self.n_tets, 3))
        self.lib.spo_get_efield(self.h, _ptr(E, C.c_double))
        return E

    def matrix(self):
        rp = np.empty(self.n_nodes + 1, np.int32)
        self.lib.spo_get_matrix(self.h, _ptr(rp, C.c_int32), None, None, None)
        ci = np.empty(rp[-1], np.int32)
        av = np.empty(rp[-1])
        lift = np.empty(self.n_nodes)
        self.lib.spo_get_matrix(self.h, _ptr(rp, C.c_int32), _ptr(ci, C.c_int32), _ptr(av, C.c_double),
                                _ptr(lift, C.c_double))
        return rp, ci, av, lift

    def set_dirichlet(self, g):
        g = np.ascontiguousarray(g, np.float64)
        self.lib.spo_set_dirichlet(self.h, _ptr(g, C.c_double))

    def grad(self, nsteps, target, sigma):
        """FP64 reference gradient: (J, n_landed, dJ/dg, dJ/dx0, dJ/dv0)."""
        t = np.ascontiguousarray(target, np.float64)
        J, nl = C.c_double(), C.c_int64()
        dg = np.zeros(self.n_nodes)
        dx = np.zeros((self.n_particles, 3))
        dv = np.zeros((self.n_particles, 3))
        rc = self.lib.spo_grad(self.h, int(nsteps), _ptr(t, C.c_double), float(sigma), C.byref(J), C.byref(nl),
                               _ptr(dg, C.c_double), _ptr(dx, C.c_double), _ptr(dv, C.c_double))
        if rc:
            raise RuntimeError(self.lib.spo_last_error().decode())
        return J.value, nl.value, dg, dx, dv

    def grad_field_gradient(self, on=True):
        self.lib.spo_grad_field_gradient(self.h, 1 if on else 0)

    def grad_freeze(self, mode):
        """0 off, 1 record the field cells of the next grad(), 2 replay them."""
        self.lib.spo_grad_freeze(self.h, int(mode))

    def dual_volumes(self):
        dv = np.empty(self.n_nodes)
        self.lib.spo_get_dual_volumes(self.h, _ptr(dv, C.c_double))
        return dv


# ---- primitives pinned by the reference's unit tests

def update_position(pos, vel, dt):
    p = np.ascontiguousarray(pos, np.float64).copy()
    v = np.ascontiguousarray(vel, np.float64)
    load().spo_update_position(_ptr(p, C.c_double), _ptr(v, C.c_double), float(dt))
    return p


def segment_triangle(s0, s1, a, b, c):
    arr = [np.ascontiguousarray(x, np.float64) for x in (s0, s1, a, b, c)]
    out = np.zeros(3)
    hit = load().spo_segment_triangle(*[_ptr(x, C.c_double) for x in arr], _ptr(out, C.c_double))
    return out if hit else None


def gas_concentration(pressure, temperature):
    return float(load().spo_gas_concentration(float(pressure), float(temperature)))


def collide_with(params, vel, u0, u1, u2):
    p = params_struct(params)
    v = np.ascontiguousarray(vel, np.float64).copy()
    hit = load().spo_collide_with(C.byref(p), _ptr(v, C.c_double), float(u0), float(u1), float(u2))
    return bool(hit), v


def collision_probability(params, vel):
    p = params_struct(params)
    v = np.ascontiguousarray(vel, np.float64)
    return float(load().spo_collision_probability(C.byref(p), _ptr(v, C.c_double)))


def tet_map(x0, x1, x2, x3):
    arr = [np.ascontiguousarray(x, np.float64) for x in (x0, x1, x2, x3)]
    M = np.zeros(9)
    det = load().spo_tet_map(*[_ptr(x, C.c_double) for x in arr], _ptr(M, C.c_double))
    return det, M.reshape(3, 3)


def collides(steps, ids, seed, P):
    """Collision decisions (bool array) of the (step, id) pairs at probability P."""
    st = np.ascontiguousarray(steps, np.uint64)
    idv = np.ascontiguousarray(ids, np.uint32)
    out = np.zeros(len(st), np.uint8)
    load().spo_collides(st.ctypes.data_as(C.POINTER(C.c_uint64)), _ptr(idv, C.c_uint32), len(st), int(seed),
                        float(P), out.ctypes.data_as(C.POINTER(C.c_uint8)))
    return out.astype(bool)


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    load().spo_philox(_ptr(c, C.c_uint32), _ptr(k, C.c_uint32), _ptr(o, C.c_uint32))
    return o

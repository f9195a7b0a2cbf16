"""Python host layer over libstart_gpu.so.

`StartPIC` owns one library handle (mesh + particles + stream). The classes
`NodeChargeDensityProcessor`, `ChargeDensityEquationSolver` and
`ParticleDynamicsProcessor` keep the reference's static-method names
(include/ParticleInCellEngine/*.hpp) so a caller of the reference's engine
finds the same three calls, and failures surface as the reference's
exception types (include/ParticleInCellEngine/PICExceptions.hpp).
There is no CPU fallback: without the library or an sm_103 GPU, construction
raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .mesh import TetMesh


class PICBaseException(RuntimeError):
    """Base of the PIC errors (PICExceptions.hpp)."""

    def __init__(self, msg, code=None):
        super().__init__(msg)
        self.code = code


class PICUnknownException(PICBaseException):
    pass


class PICNodeChargeDensityProcessorOmpVersionHelperException(PICBaseException):
    pass


class PICChargeDensityEquationSolverSolvingException(PICBaseException):
    pass


class PICParticleDynamicsProcessorProcessingException(PICBaseException):
    pass


class MeshError(PICBaseException):
    pass


class DeviceError(PICBaseException):
    pass


def _params_struct(params) -> N.Params:
    if isinstance(params, N.Params):
        return params
    p = N.default_params()
    for k, v in dict(params).items():
        if not hasattr(p, k):
            raise KeyError(f"unknown parameter {k}")
        setattr(p, k, v)
    return p


class StartPIC:
    """One GPU handle: mesh, fields, particles, counters."""

    def __init__(self, mesh: TetMesh, params):
        self.lib = N.load()
        self.mesh = mesh
        self.params = _params_struct(params)
        self._nodes = np.ascontiguousarray(mesh.nodes, np.float64)
        self._tets = np.ascontiguousarray(mesh.tets, np.int32)
        self._tris = np.ascontiguousarray(mesh.triangles, np.int32).reshape(-1, 3)
        self._dn = np.ascontiguousarray(mesh.dirichlet_nodes, np.int32)
        self._dv = np.ascontiguousarray(mesh.dirichlet_values, np.float64)
        d = N.MeshDesc()
        d.n_nodes = len(self._nodes)
        d.node_xyz = N.as_ptr(self._nodes, C.c_double)
        d.n_tets = len(self._tets)
        d.tet_nodes = N.as_ptr(self._tets, C.c_int32)
        d.n_triangles = len(self._tris)
        d.tri_nodes = N.as_ptr(self._tris, C.c_int32)
        d.n_dirichlet = len(self._dn)
        d.dirichlet_nodes = N.as_ptr(self._dn, C.c_int32)
        d.dirichlet_values = N.as_ptr(self._dv, C.c_double)
        h = C.c_void_p()
        rc = self.lib.spg_create(C.byref(d), C.byref(self.params), C.byref(h))
        if rc != N.SPG_OK:
            msg = self.lib.spg_last_error(None).decode()
            if rc == N.SPG_E_BAD_MESH:
                raise MeshError(msg, rc)
            if rc == N.SPG_E_NO_DEVICE:
                raise DeviceError(msg, rc)
            raise PICBaseException(msg, rc)
        self.h = h
        info = (C.c_int64 * 6)()
        self.lib.spg_mesh_info(self.h, info)
        self.n_nodes, self.n_tets, self.n_triangles, self.n_boundary_faces, self.nnz, self.n_dirichlet = list(info)
        self.n_particles = 0

    # -- lifetime
    def close(self):
        if getattr(self, "h", None):
            self.lib.spg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc, exc=PICBaseException, allow=()):
        if rc != N.SPG_OK and rc not in allow:
            raise exc(self.lib.spg_last_error(self.h).decode(), rc)
        return rc

    # -- particles
    def set_particles(self, pos, vel, tet=None):
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        vel = np.ascontiguousarray(vel, np.float64).reshape(-1, 3)
        if pos.shape != vel.shape:
            raise ValueError("pos and vel must have the same shape")
        tp = None
        if tet is not None:
            tet = np.ascontiguousarray(tet, np.int32)
            tp = N.as_ptr(tet, C.c_int32)
        self._check(self.lib.spg_set_particles(self.h, len(pos), N.as_ptr(pos, C.c_double),
                                               N.as_ptr(vel, C.c_double), tp))
        self.n_particles = len(pos)

    def _source(self, shape="disk", directions="cone", energy="mono", centre=(0.0, 0.0, 0.0),
                normal=(0.0, 0.0, 1.0), radius=0.02, xlim=(0.0, 0.0), ylim=(0.0, 0.0), z=0.0, half_angle=None,
                energy_ev=1.0, binding_ev=4.9, emax_ev=50.0, displacement=0.05e-3, seed=0, cells=None,
                expansion=0.0):
        src = N.Source()
        self.lib.spg_default_source(C.byref(src))
        src.shape = {"disk": N.SPG_SRC_DISK, "rect": N.SPG_SRC_RECT, "plate": N.SPG_SRC_RECT,
                     "point": N.SPG_SRC_POINT, "cells": N.SPG_SRC_CELLS, "surface": N.SPG_SRC_CELLS}[shape]
        src.directions = {"cone": N.SPG_DIR_CONE, "cosine": N.SPG_DIR_COSINE, "fan": N.SPG_DIR_FAN}[directions]
        src.energy = {"mono": N.SPG_ENERGY_MONO, "thompson": N.SPG_ENERGY_THOMPSON}[energy]
        src.centre[:] = [float(v) for v in centre]
        src.normal[:] = [float(v) for v in normal]
        src.radius = radius
        src.xlim[:] = [float(v) for v in xlim]
        src.ylim[:] = [float(v) for v in ylim]
        src.z = z
        if half_angle is not None:
            src.half_angle = half_angle
        src.energy_ev, src.binding_ev, src.emax_ev = energy_ev, binding_ev, emax_ev
        src.displacement = displacement
        src.seed = int(seed)
        src.expansion = float(expansion)
        keep = None
        if cells is not None:
            keep = np.ascontiguousarray(cells, np.float64).reshape(-1, 6)
            src.n_cells = len(keep)
            src.cells = N.as_ptr(keep, C.c_double)
        return src, keep

    def generate_particles(self, n, **kw):
        """Samples n particles on the device (spg_generate_particles): disk,
        rectangle, point or surface-cell sources (cells: rows of centre xyz and
        normal xyz), cone, cosine or the reference's fan directions
        (expansion), monoenergetic or Thompson energies, and the reference's
        0.05 mm displacement."""
        src, keep = self._source(**kw)
        self._check(self.lib.spg_generate_particles(self.h, int(n), C.byref(src)))
        del keep
        self.n_particles = int(n)

    def inject_particles(self, n, **kw):
        """Appends n device-sampled particles (the same source options) to the
        current set mid-run, with the next ids (spg_inject_particles)."""
        src, keep = self._source(**kw)
        self._check(self.lib.spg_inject_particles(self.h, int(n), C.byref(src)))
        del keep
        self.n_particles += int(n)

    def track(self, ids, capacity=10000):
        """Samples the positions of particles `ids` before every step they are
        alive in (ParticleMovementTracker)."""
        ids = np.ascontiguousarray(ids, np.int64)
        self._check(self.lib.spg_track_particles(self.h, len(ids), N.as_ptr(ids, C.c_int64), int(capacity)))
        self._track = (ids, int(capacity))

    def tracks(self):
        """{id: (m, 3) positions}; a settled particle ends with its hit point."""
        ids, cap = self._track
        k = len(ids)
        counts = np.zeros(k, np.int32)
        xyz = np.zeros((k, cap, 3))
        last = np.zeros((k, 3))
        flags = np.zeros(k, np.uint32)
        self._check(self.lib.spg_get_tracks(self.h, N.as_ptr(counts, C.c_int32), N.as_ptr(xyz, C.c_double),
                                            N.as_ptr(last, C.c_double), N.as_ptr(flags, C.c_uint32)))
        out = {}
        for t, pid in enumerate(ids):
            path = xyz[t, :counts[t]]
            if flags[t] & N.SPG_FLAG_SETTLED:
                path = np.vstack([path, last[t]])
            out[int(pid)] = path
        return out

    def particles(self, out=None):
        """Positions, velocities, tets and flags by particle id. `out` may hold
        any of the four arrays (e.g. pinned host memory, so that the copy
        needs no staging); they must be C-contiguous with the dtypes and shapes
        returned here."""
        n = self.n_particles
        out = out or {}

        def take(key, shape, dtype):
            a = out.get(key)
            if a is None:
                return np.empty(shape, dtype)
            if a.dtype != dtype or a.shape != shape or not a.flags.c_contiguous:
                raise ValueError(f"particles: out[{key!r}] must be a C-contiguous {np.dtype(dtype)} array of "
                                 f"shape {shape}")
            return a

        pos = take("pos", (n, 3), np.float64)
        vel = take("vel", (n, 3), np.float64)
        tet = take("tet", (n,), np.int32)
        flags = take("flags", (n,), np.uint32)
        self._check(self.lib.spg_get_particles(self.h, n, N.as_ptr(pos, C.c_double), N.as_ptr(vel, C.c_double),
                                               N.as_ptr(tet, C.c_int32), N.as_ptr(flags, C.c_uint32)))
        return dict(pos=pos, vel=vel, tet=tet, flags=flags)

    def locate(self, pos):
        pos = np.ascontiguousarray(pos, np.float64).reshape(-1, 3)
        out = np.empty(len(pos), np.int32)
        self._check(self.lib.spg_locate(self.h, len(pos), N.as_ptr(pos, C.c_double), N.as_ptr(out, C.c_int32)))
        return out

    # -- the three reference calls
    def gather(self, want_rho=True):
        rho = np.empty(self.n_nodes) if want_rho else None
        self._check(self.lib.spg_gather(self.h, N.as_ptr(rho, C.c_double) if want_rho else None),
                    PICNodeChargeDensityProcessorOmpVersionHelperException)
        return rho

    def solve(self, rho=None, want_phi=True, raise_on_nonconvergence=True):
        phi = np.empty(self.n_nodes) if want_phi else None
        it = C.c_int32()
        rr = C.c_double()
        rp = None
        if rho is not None:
            rho = np.ascontiguousarray(rho, np.float64)
            rp = N.as_ptr(rho, C.c_double)
        rc = self.lib.spg_solve(self.h, rp, N.as_ptr(phi, C.c_double) if want_phi else None, C.byref(it),
                                C.byref(rr))
        allow = () if raise_on_nonconvergence else (N.SPG_E_NOT_CONVERGED,)
        self._check(rc, PICChargeDensityEquationSolverSolvingException, allow)
        return phi, it.value, rr.value

    def process(self, nsteps=1):
        st = N.Stats()
        self._check(self.lib.spg_process(self.h, int(nsteps), C.byref(st)),
                    PICParticleDynamicsProcessorProcessingException)
        return st.as_dict()

    def run(self, nsteps, raise_on_nonconvergence=True):
        st = N.Stats()
        allow = () if raise_on_nonconvergence else (N.SPG_E_NOT_CONVERGED,)
        self._check(self.lib.spg_run(self.h, int(nsteps), C.byref(st)), PICBaseException, allow)
        return st.as_dict()

    def resort(self):
        self._check(self.lib.spg_resort(self.h))

    # -- outputs
    def stats(self):
        st = N.Stats()
        self._check(self.lib.spg_get_stats(self.h, C.byref(st)))
        return st.as_dict()

    def triangle_counts(self):
        c = np.zeros(self.n_triangles, np.uint64)
        self._check(self.lib.spg_get_triangle_counts(self.h, N.as_ptr(c, C.c_uint64)))
        return c

    def potential(self):
        phi = np.empty(self.n_nodes)
        self._check(self.lib.spg_get_potential(self.h, N.as_ptr(phi, C.c_double)))
        return phi

    def set_potential(self, phi):
        phi = np.ascontiguousarray(phi, np.float64)
        self._check(self.lib.spg_set_potential(self.h, N.as_ptr(phi, C.c_double)))

    def setup_times(self):
        """Wall times of the set-up in ms (spg_setup_times)."""
        t = (C.c_double * 6)()
        self._check(self.lib.spg_setup_times(self.h, t))
        keys = ("create", "fem_elements_gpu", "fem_stiffness_gpu", "mesh_host", "amg", "upload_other")
        return dict(zip(keys, list(t)))

    def matrix(self):
        """The assembled FEM system: CSR (row_ptr, col, val), the lifting and
        the dual volumes (spg_get_matrix)."""
        rp = np.empty(self.n_nodes + 1, np.int32)
        self._check(self.lib.spg_get_matrix(self.h, rp.ctypes.data, None, None, None, None))
        col = np.empty(int(rp[-1]), np.int32)
        val = np.empty(int(rp[-1]))
        lift = np.empty(self.n_nodes)
        dual = np.empty(self.n_nodes)
        self._check(self.lib.spg_get_matrix(self.h, rp.ctypes.data, col.ctypes.data, val.ctypes.data,
                                            lift.ctypes.data, dual.ctypes.data))
        return rp, col, val, lift, dual

    def efield(self):
        E = np.empty((self.n_tets, 3))
        self._check(self.lib.spg_get_efield(self.h, N.as_ptr(E, C.c_double)))
        return E

    def checkpoint(self) -> bytes:
        n = C.c_size_t()
        self._check(self.lib.spg_checkpoint_size(self.h, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        self._check(self.lib.spg_checkpoint(self.h, buf, n.value))
        return buf.raw

    def restore(self, blob: bytes):
        buf = C.create_string_buffer(blob, len(blob))
        self._check(self.lib.spg_restore(self.h, buf, len(blob)))

    def set_dirichlet(self, g):
        """Dirichlet values g [n_nodes] (read at the Dirichlet nodes)."""
        g = np.ascontiguousarray(g, np.float64)
        self._check(self.lib.spg_set_dirichlet(self.h, N.as_ptr(g, C.c_double)))

    def grad_forward(self, nsteps, target, sigma, checkpoint_every=32):
        """Particle steps with landing records and checkpoints; returns (J, n_landed)."""
        t = np.ascontiguousarray(target, np.float64)
        J, nl = C.c_double(), C.c_int64()
        self._check(self.lib.spg_grad_forward(self.h, int(nsteps), int(checkpoint_every), N.as_ptr(t, C.c_double),
                                              float(sigma), C.byref(J), C.byref(nl)))
        return J.value, nl.value

    def grad_backward(self, particles=True):
        """Adjoint pass; returns dJ/dg [n_nodes], dJ/dx0 [n,3], dJ/dv0 [n,3], adjoint CG iterations."""
        g = np.zeros(self.n_nodes)
        dx = np.zeros((self.n_particles, 3)) if particles else None
        dv = np.zeros((self.n_particles, 3)) if particles else None
        it = C.c_int32()
        self._check(self.lib.spg_grad_backward(self.h, N.as_ptr(g, C.c_double),
                                               N.as_ptr(dx, C.c_double) if particles else None,
                                               N.as_ptr(dv, C.c_double) if particles else None, C.byref(it)))
        return g, dx, dv, it.value

    def grad_field_gradient(self, on=True):
        """Whether grad_backward also carries the push's dependence on the
        position through the recovered field's gradient (spg_grad_field_gradient)."""
        self._check(self.lib.spg_grad_field_gradient(self.h, 1 if on else 0))

    def set_step_segments(self, max_steps):
        """Steps of the mixed form between two events of the loop run as
        segments of up to max_steps steps (1: one launch per step); the
        results do not depend on it (spg_set_step_segments)."""
        self._check(self.lib.spg_set_step_segments(self.h, int(max_steps)))

    def synchronize(self):
        self._check(self.lib.spg_synchronize(self.h))

    def stream_ptr(self) -> int:
        return int(self.lib.spg_stream(self.h) or 0)

    def profile_enable(self, on=True):
        self._check(self.lib.spg_profile_enable(self.h, 1 if on else 0))

    def profile_reset(self):
        self._check(self.lib.spg_profile_reset(self.h))

    def profile(self):
        p = N.Profile()
        self._check(self.lib.spg_get_profile(self.h, C.byref(p)))
        return p.as_dict()


# ---- reference-named facades (static methods, same argument meaning)

class NodeChargeDensityProcessor:
    """NodeChargeDensityProcessor::gather (NodeChargeDensityProcessor.hpp:39-46):
    deposits all non-settled particles and returns nodal charge density."""

    @staticmethod
    def gather(engine: StartPIC):
        return engine.gather(want_rho=True)


class ChargeDensityEquationSolver:
    """ChargeDensityEquationSolver::solve (ChargeDensityEquationSolver.hpp:38-42):
    Poisson solve from nodal charge density, then E per tet."""

    @staticmethod
    def solve(engine: StartPIC, node_charge_density=None):
        return engine.solve(rho=node_charge_density)


class ParticleDynamicsProcessor:
    """ParticleDynamicsProcessor::process (ParticleDynamicsProcessor.hpp:154-170):
    one time step of push, move, gas collision and surface settle."""

    @staticmethod
    def process(engine: StartPIC, nsteps: int = 1):
        return engine.process(nsteps)

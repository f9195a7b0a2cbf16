"""ctypes binding of libstart_gpu.so (include/start_gpu.h).

The library is the product: there is no CPU fallback. If it is missing, or
no sm_103 device is present, loading or creating a handle raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .build import LIBDIR, LIBNAME

SPG_OK = 0
SPG_E_INVALID = -1
SPG_E_CUDA = -2
SPG_E_BAD_MESH = -3
SPG_E_NOT_CONVERGED = -4
SPG_E_LOST_PARTICLES = -5
SPG_E_NO_DEVICE = -6
SPG_E_OOM = -7
SPG_E_STATE = -8

SPG_COLL_NONE, SPG_COLL_HS, SPG_COLL_VHS, SPG_COLL_VSS = 0, 1, 2, 3
SPG_FP64, SPG_MIXED = 0, 1
SPG_PRECOND_JACOBI, SPG_PRECOND_AMG, SPG_PRECOND_AMG_F32 = 0, 1, 2
SPG_FLAG_SETTLED, SPG_FLAG_LOST = 1, 2

_pd = C.POINTER(C.c_double)
_pi32 = C.POINTER(C.c_int32)


class MeshDesc(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_int64), ("node_xyz", _pd),
        ("n_tets", C.c_int64), ("tet_nodes", _pi32),
        ("n_triangles", C.c_int64), ("tri_nodes", _pi32),
        ("n_dirichlet", C.c_int64), ("dirichlet_nodes", _pi32), ("dirichlet_values", _pd),
    ]


class Params(C.Structure):
    _fields_ = [
        ("dt", C.c_double), ("charge", C.c_double), ("mass", C.c_double), ("weight", C.c_double),
        ("collision_model", C.c_int32), ("precision", C.c_int32),
        ("gas_mass", C.c_double), ("gas_concentration", C.c_double),
        ("hs_diameter", C.c_double), ("vhs_dref", C.c_double), ("omega", C.c_double), ("alpha", C.c_double),
        ("kT_ref", C.c_double), ("epsilon0", C.c_double), ("min_velocity", C.c_double),
        ("bbox_expansion", C.c_double), ("seed", C.c_uint64),
        ("poisson_every", C.c_int32), ("resort_every", C.c_int32),
        ("max_crossings", C.c_int32), ("cg_max_iter", C.c_int32), ("cg_rtol", C.c_double),
        ("device", C.c_int32), ("preconditioner", C.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Source(C.Structure):
    _fields_ = [
        ("shape", C.c_int32), ("directions", C.c_int32), ("energy", C.c_int32), ("reserved0", C.c_int32),
        ("centre", C.c_double * 3), ("normal", C.c_double * 3), ("radius", C.c_double),
        ("xlim", C.c_double * 2), ("ylim", C.c_double * 2), ("z", C.c_double),
        ("half_angle", C.c_double), ("energy_ev", C.c_double), ("binding_ev", C.c_double),
        ("emax_ev", C.c_double), ("displacement", C.c_double), ("seed", C.c_uint64),
        ("n_cells", C.c_int32), ("reserved1", C.c_int32), ("cells", C.POINTER(C.c_double)),
        ("expansion", C.c_double),
    ]


SPG_SRC_DISK, SPG_SRC_RECT, SPG_SRC_POINT, SPG_SRC_CELLS = 0, 1, 2, 3
SPG_DIR_CONE, SPG_DIR_COSINE, SPG_DIR_FAN = 0, 1, 2
SPG_ENERGY_MONO, SPG_ENERGY_THOMPSON = 0, 1


class Stats(C.Structure):
    _fields_ = [
        ("step", C.c_int64), ("n_particles", C.c_int64), ("n_alive", C.c_int64), ("n_settled", C.c_int64),
        ("n_lost", C.c_int64), ("particle_steps", C.c_int64), ("collisions", C.c_int64),
        ("crossings", C.c_int64), ("cg_iters_total", C.c_int64), ("cg_iters_last", C.c_int32),
        ("cg_solves", C.c_int32), ("cg_relres_last", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Profile(C.Structure):
    _fields_ = [
        ("step_ms", C.c_double), ("step_launches", C.c_int64), ("step_bytes", C.c_double),
        ("deposit_ms", C.c_double), ("deposit_launches", C.c_int64), ("deposit_bytes", C.c_double),
        ("pcg_ms", C.c_double), ("pcg_solves", C.c_int64), ("pcg_bytes", C.c_double), ("pcg_iters", C.c_int64),
        ("efield_ms", C.c_double), ("efield_launches", C.c_int64),
        ("sort_ms", C.c_double), ("sort_launches", C.c_int64), ("sort_bytes", C.c_double),
        ("kernel_launches", C.c_int64), ("occupied_tets", C.c_int64),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# Every function the header declares, with its C signature.
_H = C.c_void_p
SIGNATURES = {
    "spg_version": (C.c_char_p, []),
    "spg_default_params": (None, [C.POINTER(Params)]),
    "spg_last_error": (C.c_char_p, [_H]),
    "spg_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(Params), C.POINTER(_H)]),
    "spg_destroy": (C.c_int, [_H]),
    "spg_mesh_info": (C.c_int, [_H, C.POINTER(C.c_int64)]),
    "spg_setup_times": (C.c_int, [_H, C.POINTER(C.c_double)]),
    "spg_set_particles": (C.c_int, [_H, C.c_int64, _pd, _pd, _pi32]),
    "spg_default_source": (None, [C.POINTER(Source)]),
    "spg_generate_particles": (C.c_int, [_H, C.c_int64, C.POINTER(Source)]),
    "spg_inject_particles": (C.c_int, [_H, C.c_int64, C.POINTER(Source)]),
    "spg_get_matrix": (C.c_int, [_H, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "spg_track_particles": (C.c_int, [_H, C.c_int32, C.POINTER(C.c_int64), C.c_int32]),
    "spg_get_tracks": (C.c_int, [_H, _pi32, _pd, _pd, C.POINTER(C.c_uint32)]),
    "spg_get_particles": (C.c_int, [_H, C.c_int64, _pd, _pd, _pi32, C.POINTER(C.c_uint32)]),
    "spg_gather": (C.c_int, [_H, _pd]),
    "spg_grad_field_gradient": (C.c_int, [_H, C.c_int32]),
    "spg_set_step_segments": (C.c_int, [_H, C.c_int32]),
    "spg_get_charge_density": (C.c_int, [_H, _pd]),
    "spg_solve": (C.c_int, [_H, _pd, _pd, _pi32, _pd]),
    "spg_process": (C.c_int, [_H, C.c_int32, C.POINTER(Stats)]),
    "spg_run": (C.c_int, [_H, C.c_int32, C.POINTER(Stats)]),
    "spg_resort": (C.c_int, [_H]),
    "spg_get_stats": (C.c_int, [_H, C.POINTER(Stats)]),
    "spg_get_triangle_counts": (C.c_int, [_H, C.POINTER(C.c_uint64)]),
    "spg_get_potential": (C.c_int, [_H, _pd]),
    "spg_set_potential": (C.c_int, [_H, _pd]),
    "spg_get_efield": (C.c_int, [_H, _pd]),
    "spg_locate": (C.c_int, [_H, C.c_int64, _pd, _pi32]),
    "spg_checkpoint_size": (C.c_int, [_H, C.POINTER(C.c_size_t)]),
    "spg_checkpoint": (C.c_int, [_H, C.c_void_p, C.c_size_t]),
    "spg_restore": (C.c_int, [_H, C.c_void_p, C.c_size_t]),
    "spg_synchronize": (C.c_int, [_H]),
    "spg_stream": (C.c_void_p, [_H]),
    "spg_profile_enable": (C.c_int, [_H, C.c_int32]),
    "spg_get_profile": (C.c_int, [_H, C.POINTER(Profile)]),
    "spg_profile_reset": (C.c_int, [_H]),
    "spg_set_dirichlet": (C.c_int, [_H, _pd]),
    "spg_grad_forward": (C.c_int, [_H, C.c_int32, C.c_int32, _pd, C.c_double, _pd, C.POINTER(C.c_int64)]),
    "spg_grad_backward": (C.c_int, [_H, _pd, _pd, _pd, _pi32]),
    "spg_pcg_solve_noalloc":(C.c_int, [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_double, C.c_int32, C.c_void_p, _pi32, _pd]),
}

_lib = None


def library_path() -> Path:
    return LIBDIR / LIBNAME


def load(path: str | Path | None = None):
    """Load libstart_gpu.so and declare every entry point. Raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else library_path()
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with start_gb300.build.build_library()")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class SpgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def default_params() -> Params:
    p = Params()
    load().spg_default_params(C.byref(p))
    return p


def as_ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))

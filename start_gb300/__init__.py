"""start_gb300: GB300-native particle-in-cell / DSMC time step of Start.

The compute path is libstart_gpu.so (hand-written sm_103a kernels behind the
C ABI in include/start_gpu.h); this package is its host-side layer: mesh and
source generation, the ctypes binding and the reference-named engine calls.
"""
from .build import build_library
from .engine import (ChargeDensityEquationSolver, NodeChargeDensityProcessor, ParticleDynamicsProcessor,
                     PICBaseException, StartPIC)
from .mesh import TetMesh, kuhn_box, read_msh41
from .workloads import WORKLOADS, Workload

__all__ = [
    "build_library", "StartPIC", "NodeChargeDensityProcessor", "ChargeDensityEquationSolver",
    "ParticleDynamicsProcessor", "PICBaseException", "TetMesh", "kuhn_box", "read_msh41", "WORKLOADS", "Workload",
]

"""Compile libstart_gpu.so (sm_103a) in-tree with nvcc and g++.

No cmake and no torch extension machinery: four translation units compiled in
parallel, one link. The FP64 particle kernels are built with --fmad=false so
that their arithmetic matches the CPU oracle, which is built with
-ffp-contract=off; the host-side mesh preparation is built the same way.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIBNAME = "libstart_gpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _sources():
    CUDA = cuda_home()
    inc = f"-I{CUDA / 'include'}"
    nvcc = str(CUDA / "bin" / "nvcc")
    common_nv = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                 f"-I{CSRC}"]
    common_cc = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", inc, f"-I{CSRC}"]
    return [
        ("kernels_particles.cu", common_nv + ["--fmad=false"]),
        ("kernels_pcg.cu", common_nv),
        ("kernels_mixed.cu", common_nv),
        ("noalloc.cu", common_nv),
        ("kernels_adjoint.cu", common_nv + ["--fmad=false"]),
        ("kernels_amg.cu", common_nv),
        ("kernels_sources.cu", common_nv),
        ("kernels_track.cu", common_nv),
        ("kernels_fem.cu", common_nv + ["--fmad=false"]),
        ("mesh_prep.cpp", common_cc + ["-fopenmp"]),
        ("amg_setup.cpp", common_cc + ["-O3", "-fopenmp"]),
        ("capi.cpp", common_cc),
    ]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}")
    return r.stdout


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Build (if needed) and return the path of libstart_gpu.so."""
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "start_gpu.h"]
    jobs, objs = [], []
    for src, flags in _sources():
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src, *headers, Path(__file__)]):
            jobs.append(flags + ["-c", str(CSRC / src), "-o", str(obj)])
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            for out in ex.map(_run, jobs):
                if verbose and out.strip():
                    print(out)
    lib = LIBDIR / LIBNAME
    if force or jobs or _stale(lib, objs):
        nvcc = str(cuda_home() / "bin" / "nvcc")
        _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-Xcompiler", "-fopenmp", "-lgomp"])
    return lib


if __name__ == "__main__":
    print(build_library(force=True, verbose=True))

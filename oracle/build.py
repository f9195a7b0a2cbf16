"""Build the CPU oracle (test infrastructure) into oracle/_build/liboracle.so.

Plain g++, no cmake: -O2 -fopenmp -ffp-contract=off so that unfused FP64
arithmetic matches the GPU kernels built with --fmad=false.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build" / "liboracle.so"


def build_oracle(force: bool = False) -> Path:
    srcs = [HERE / "pic_oracle.cpp"]
    deps = srcs + [HERE / "pic_oracle.h", HERE.parent / "include" / "start_gpu.h", Path(__file__)]
    if not force and OUT.exists() and all(d.stat().st_mtime <= OUT.stat().st_mtime for d in deps):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           *map(str, srcs), "-o", str(OUT)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}")
    return OUT


if __name__ == "__main__":
    print(build_oracle(force=True))

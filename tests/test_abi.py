"""The C ABI library loads and exports every symbol its headers declare
(CPU only: no compute call needs a GPU here), and the product path fails
loudly without a GPU instead of falling back to the CPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared(header: Path, prefix: str):
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(" + prefix + r"[a-z0-9_]+)\s*\(", text)))


def test_gpu_library_exports_header(built):
    from start_gb300 import _native as N

    lib = C.CDLL(str(N.library_path()))
    names = _declared(ROOT / "include" / "start_gpu.h", "spg_")
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes table covers the header exactly
    assert sorted(N.SIGNATURES) == names


def test_oracle_exports_header(built):
    import oracle

    lib = oracle.load()
    names = _declared(ROOT / "oracle" / "pic_oracle.h", "spo_")
    assert not [n for n in names if not hasattr(lib, n)]


def test_default_params_without_device(built):
    from start_gb300 import _native as N

    p = N.default_params()
    assert p.dt == 1e-8 and p.min_velocity == 10.0 and p.bbox_expansion == 1.01
    assert p.kT_ref == 297.0 * 1.380658e-23
    assert N.load().spg_version().decode().startswith("start_gb300")


def test_create_fails_loudly_without_gpu(built):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from start_gb300 import StartPIC
    from start_gb300.engine import DeviceError
    from start_gb300.mesh import kuhn_box

    m = kuhn_box((2, 2, 2), (0.1, 0.1, 0.1))
    with pytest.raises(DeviceError, match="device"):
        StartPIC(m, {"dt": 1e-8})


def test_invalid_params_rejected_before_device(built):
    from start_gb300 import StartPIC
    from start_gb300.engine import PICBaseException
    from start_gb300.mesh import kuhn_box

    m = kuhn_box((2, 2, 2), (0.1, 0.1, 0.1))
    with pytest.raises(PICBaseException, match="dt"):
        StartPIC(m, {"dt": -1.0})
    with pytest.raises(PICBaseException, match="collision_model"):
        StartPIC(m, {"collision_model": 9})


def test_struct_layouts_match_header(built):
    """ctypes struct sizes equal the C sizes (compiled probe)."""
    import subprocess
    import tempfile

    from start_gb300 import _native as N

    src = r'''
    #include <stdio.h>
    #include "start_gpu.h"
    int main(void) {
      printf("%zu %zu %zu %zu %zu\n", sizeof(spg_mesh_desc), sizeof(spg_params), sizeof(spg_stats),
             sizeof(spg_profile), sizeof(spg_source));
      return 0; }
    '''
    with tempfile.TemporaryDirectory() as d:
        c = Path(d) / "probe.c"
        c.write_text(src)
        exe = Path(d) / "probe"
        subprocess.run(["gcc", "-I", str(ROOT / "include"), str(c), "-o", str(exe)], check=True)
        sizes = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()))
    assert sizes == [C.sizeof(N.MeshDesc), C.sizeof(N.Params), C.sizeof(N.Stats), C.sizeof(N.Profile),
                     C.sizeof(N.Source)]


def test_cpp_shim_compiles(built):
    """The reference-named C++ shim (include/start_pic.hpp) and the time-loop
    driver written against it compile and link against libstart_gpu.so (the
    GPU test test_gpu_cpp_shim.py runs the same driver)."""
    import subprocess
    import tempfile

    lib, _ = built
    src = ROOT / "tests" / "native" / "pic_loop_driver.cpp"
    with tempfile.TemporaryDirectory() as d:
        exe = Path(d) / "pic_loop_driver"
        subprocess.run(["g++", "-std=c++17", "-O0", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"), str(src),
                        "-L", str(lib.parent), "-lstart_gpu", f"-Wl,-rpath,{lib.parent}", "-o", str(exe)], check=True)
        assert exe.exists()

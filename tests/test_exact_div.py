"""The FP64 field kernel's division by the particle mass (exact_div.h) must
round exactly like IEEE division, so the push increment stays bit-identical
to the oracle's (q E) / m. The header is compiled for the host with g++ and
checked on 14 million dividends, a sixth of them next to midpoints of the
quotient grid."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_division_by_known_divisor_is_correctly_rounded(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = tmp_path / "exact_div_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{ROOT / 'start_gb300' / 'csrc'}",
                    str(ROOT / "tests" / "native" / "exact_div_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "2000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout
    assert "mismatches 0" in out.stdout

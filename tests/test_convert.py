"""Integer-pipe FP64 <-> FP32 conversions and floor comparison used by the
FP32 + FP64-u path (guacho_gb300/csrc/gch_convert.h), the integer-pipe FP64
division of the FP64 Riemann solvers (gch_ddiv.h) and the integer-pipe FP64
square root of the FP64 CFL pass (gch_dsqrt.h): bit-identical to the C casts,
the C comparison and the IEEE division and square root on random bit
patterns, values around the FP32 range, exact rounding ties, quotients and
roots next to a rounding boundary and the special values, compiled for the
host with g++."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_conversions_and_division_match_ieee(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    exe = tmp_path / "convert_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", f"-I{ROOT / 'guacho_gb300' / 'csrc'}",
                    str(ROOT / "tests" / "convert_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "2000000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout


def test_conversions_and_division_free_of_undefined_behaviour(tmp_path):
    """The same check built with the undefined-behaviour sanitizer (signed
    overflow, shifts out of range), where the host toolchain has it."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    exe = tmp_path / "convert_check_ubsan"
    r = subprocess.run([cxx, "-O1", "-std=c++17", "-ffp-contract=off", "-fsanitize=undefined",
                        "-fno-sanitize-recover=all", f"-I{ROOT / 'guacho_gb300' / 'csrc'}",
                        str(ROOT / "tests" / "convert_check.cpp"), "-o", str(exe)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("no undefined-behaviour sanitizer in this toolchain")
    r = subprocess.run([str(exe), "200000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout

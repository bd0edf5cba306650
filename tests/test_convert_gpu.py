"""Integer-pipe FP64 <-> FP32 conversions and floor comparison
(guacho_gb300/csrc/gch_convert.h), the integer-pipe FP64 division (gch_ddiv.h)
and square root (gch_dsqrt.h) on the device: a kernel runs them on the host
check's cases (random bit patterns, exact rounding ties and their
neighbours, quotients and roots next to a rounding boundary, range edges,
special values) and compares them bitwise with the device's own IEEE
division, square root, conversions and comparisons,
under both flag sets the library compiles them with (the FP64 units'
-fmad=false and the FP32 units' -use_fast_math)."""
import subprocess
from pathlib import Path

import pytest

from guacho_gb300 import build

ROOT = Path(__file__).resolve().parent.parent


@pytest.mark.gpu
@pytest.mark.parametrize("flags", [["-fmad=false"], ["-use_fast_math"]], ids=["fp64_units", "fp32_units"])
def test_device_conversions_and_division_match_ieee(tmp_path, flags):
    exe = tmp_path / "convert_check_gpu"
    subprocess.run([build.nvcc(), *build.ARCH, "-O3", "-std=c++17", *flags,
                    f"-I{ROOT / 'guacho_gb300' / 'csrc'}", f"-I{ROOT / 'tests'}",
                    str(ROOT / "tests" / "convert_check_gpu.cu"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "200000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout

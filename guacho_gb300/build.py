"""Build the GB300 library in-tree: guacho_gb300/lib/libguacho_gb300.so.

Compiles every CUDA translation unit for sm_103a only (one -gencode), in
parallel, and links them with nvcc into a shared library exporting the C ABI
of include/guacho_gb300.h.  The FP64 unit is compiled with -fmad=false so
that the plain FP64 path rounds like the reference's x86-64 FP64 build.

    python -m guacho_gb300.build [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIBNAME = "libguacho_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", f"-I{INCLUDE}", f"-I{CSRC}"]
# unit -> extra flags
UNITS = {
    "gch_fp64.cu": ["-fmad=false"],
    # FP32 units: x/y as the hardware reciprocal times x (__fdividef, 2 ulp;
    # the full-range FP32 divide costs several times more and changes only
    # denominators beyond 2^126, which no physical state reaches), sqrt
    # through the hardware approximation, subnormals flushed.  The kernels
    # call no FP32 transcendental function; FP64 operations are unaffected.
    "gch_fp32.cu": ["-use_fast_math"],
    "gch_kahan.cu": ["-use_fast_math"],
    # grouped many-box kernels of the two FP32 policies (same flags)
    "gch_fp32_grp.cu": ["-use_fast_math"],
    "gch_kahan_grp.cu": ["-use_fast_math"],
    # the passive-scalar stage kernels of each policy (same flags)
    "gch_fp64_pas.cu": ["-fmad=false"],
    "gch_fp32_pas.cu": ["-use_fast_math"],
    "gch_kahan_pas.cu": ["-use_fast_math"],
    "gch_api.cu": [],
    "gch_batch.cu": [],
    # FP64 arithmetic in the reference's order, as gch_fp64.cu
    "gch_noalloc.cu": ["-fmad=false"],
    # thermal conduction: FP64 device arithmetic and host-side super-step
    # scalars, neither contracted into multiply-adds
    "gch_tc.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "gch_tc32.cu": ["-use_fast_math"],
    "gch_split.cu": ["-fmad=false"],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the GB300 library needs the CUDA toolkit")


def _sources_newer(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def _compile(unit: str, extra: list[str]) -> Path:
    obj = BUILD / (Path(unit).stem + ".o")
    cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", str(CSRC / unit), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {unit}:\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = True) -> Path:
    lib = LIBDIR / LIBNAME
    if not force and not _sources_newer(lib):
        return lib
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(*kv), UNITS.items()))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv)

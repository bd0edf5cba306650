"""The C-ABI library: builds, loads, exports every declared symbol, validates
parameters like the reference's configuration checks, and its ctypes mirror
matches the C struct layout.  No GPU needed."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from guacho_gb300 import _abi
from guacho_gb300 import params as P
from guacho_gb300 import problems

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "guacho_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:int|void)\s+(gch_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(gpu_lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(gpu_lib, n), f"{n} declared in the header but not exported"
    assert sorted(_abi.exported_symbols()) == names


def test_library_is_sm103a_only(gpu_lib):
    out = subprocess.run(["cuobjdump", "--list-elf", str(_abi.LIB_PATH)], capture_output=True,
                         text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    arches = set(re.findall(r"sm_\d+a?", out.stdout))
    assert arches == {"sm_103a"}, arches


def _check(p: P.Params) -> int:
    s = _abi.to_struct(p)
    return _abi.lib().gch_params_check(C.byref(s))


@pytest.mark.parametrize("make", [
    lambda: problems.orszag_tang(16, 16, 4)[0],
    lambda: problems.blast(8)[0],
    lambda: problems.wind_cooling(16)[0],
    lambda: problems.turbulence(8)[0],
    lambda: problems.orszag_tang(16, 16, 4, precision=P.FP32_MIXED)[0],
])
def test_params_check_accepts_configs(gpu_lib, make):
    assert _check(make()) == 0


@pytest.mark.parametrize("bad", [
    dict(riemann_solver=P.SOLVER_HLLC),            # HLLC with full MHD
    dict(mhd=False, riemann_solver=P.SOLVER_HLLD),  # HLLD without B
    dict(slope_limiter=9),
    dict(bc_left=P.BC_OUTFLOW),                    # unpaired periodic wall
    dict(bc_in=7),
    dict(nx=0),
    dict(cfl=0.0),
    dict(eta=-1.0),
    dict(cooling=P.COOL_DMC),                      # no table
    dict(bc_user=True),                            # no spheres
    dict(user_source_terms=True),                  # no point masses
    dict(precision=7),
    dict(cooling=2),                               # COOL_BBC is not on this path
    dict(th_cond=3),
    dict(th_cond=P.TC_ISOTROPIC, rsc=0.0),          # conduction needs the cgs scalings
    # the split solver: FP64 MHD without sources, cooling or spheres
    dict(riemann_solver=P.SOLVER_HLLE_SPLIT_ALL, precision=P.FP32_KAHAN),
    dict(riemann_solver=P.SOLVER_HLLE_SPLIT_ALL, eight_wave=True),
    dict(riemann_solver=P.SOLVER_HLLE_SPLIT_ALL, mhd=False, pmhd=True),
])
def test_params_check_rejects(gpu_lib, bad):
    p = problems.orszag_tang(16, 16, 4)[0].replace(**bad)
    assert _check(p) == _abi.ERR_PARAM


def test_split_all_params(gpu_lib):
    p = problems.orszag_tang(16, 16, 4, riemann_solver=P.SOLVER_HLLE_SPLIT_ALL)[0]
    assert _check(p) == 0


def test_conduction_params(gpu_lib):
    assert _check(problems.conduction_blob(8)[0]) == 0
    assert _check(problems.conduction_blob(8, th_cond=P.TC_ANISOTROPIC, mhd=True)[0]) == 0
    # anisotropic conduction needs B; conduction with table cooling is rejected
    assert _check(problems.conduction_blob(8, th_cond=P.TC_ANISOTROPIC)[0]) == _abi.ERR_PARAM
    p = problems.wind_cooling(16)[0].replace(th_cond=P.TC_ISOTROPIC)
    assert _check(p) == _abi.ERR_PARAM


def test_passive_scalar_params(gpu_lib):
    p, _ = problems.h_cooling_blob(8)
    assert p.npas == 2 and p.neq == 7 and _check(p) == 0
    assert _check(problems.h_cooling_blob(8, mhd=True)[0]) == 0
    base = problems.orszag_tang(8, 8, 4)[0]
    assert _check(base.replace(npas=2)) == 0
    for bad in (dict(npas=1), dict(npas=3),                  # 0 or 2 passives
                dict(eq_of_state=P.EOS_H_RATE),              # needs n_HI
                dict(cooling=P.COOL_H)):                     # needs n_HI
        assert _check(base.replace(**bad)) == _abi.ERR_PARAM, bad
    p = problems.wind_cooling(16)[0].replace(npas=2)          # user spheres + passives
    assert _check(p) == _abi.ERR_PARAM


def test_hydro_with_flux_cd_rejected(gpu_lib):
    p = problems.wind_cooling(16)[0].replace(enable_flux_cd=True)
    assert _check(p) == _abi.ERR_PARAM


def test_params_default_matches_ot_parameters(gpu_lib):
    s = _abi.Params_t()
    _abi.lib().gch_params_default(C.byref(s), 64, 64, 2)
    # OT/parameters.f90:58,63,94-99,111,157-158,176-177
    assert s.riemann_solver == P.SOLVER_HLLD and s.enable_flux_cd == 1
    assert s.slope_limiter == P.LIMITER_MINMOD
    assert s.bc_left == s.bc_in == P.BC_PERIODIC
    assert s.cv == 1.5 and s.gamma == (1.5 + 1.0) / 1.5
    assert s.cfl == 0.2 and s.eta == 0.0
    assert _abi.lib().gch_params_check(C.byref(s)) == 0


def test_struct_layout_matches_c(tmp_path):
    """offsetof/sizeof from the C compiler == the ctypes mirror."""
    fields = [f for f, _ in _abi.Params_t._fields_]
    prog = ["#include <stdio.h>", "#include <stddef.h>", '#include "guacho_gb300.h"',
            "int main(void){", 'printf("%zu\\n", sizeof(gch_params_t));',
            'printf("%zu\\n", sizeof(gch_sphere_t));']
    prog += [f'printf("%zu\\n", offsetof(gch_params_t, {f}));' for f in fields]
    prog += ["return 0;}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(prog))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", f"-I{ROOT / 'include'}", str(src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                           check=True).stdout.split()]
    assert vals[0] == C.sizeof(_abi.Params_t)
    assert vals[1] == C.sizeof(_abi.Sphere_t)
    for f, off in zip(fields, vals[2:]):
        assert getattr(_abi.Params_t, f).offset == off, f


def test_switch_ids_match_reference_constants():
    """src/constants.f90:56-98."""
    text = HEADER.read_text()
    want = {"SOLVER_HLL": 1, "SOLVER_HLLC": 2, "SOLVER_HLLE": 3, "SOLVER_HLLD": 4,
            "EOS_ADIABATIC": 1, "EOS_SINGLE_SPECIE": 2, "COOL_NONE": 0, "COOL_DMC": 3,
            "COOL_CHI": 4, "BC_OUTFLOW": 1, "BC_CLOSED": 2, "BC_PERIODIC": 3, "BC_OTHER": 4,
            "LIMITER_NO_AVERAGE": -1, "LIMITER_NO_LIMIT": 0, "LIMITER_MINMOD": 1,
            "LIMITER_VAN_LEER": 2, "LIMITER_VAN_ALBADA": 3, "LIMITER_UMIST": 4,
            "LIMITER_WOODWARD": 5, "LIMITER_SUPERBEE": 6,
            "TC_OFF": 0, "TC_ISOTROPIC": 1, "TC_ANISOTROPIC": 2,
            "EOS_H_RATE": 3, "COOL_H": 1}
    for k, v in want.items():
        m = re.search(rf"#define GCH_{k} \(?(-?\d+)\)?", text)
        assert m and int(m.group(1)) == v, k
        assert getattr(P, k) == v, k


def test_create_without_device_fails_loudly(gpu_lib):
    """No CPU fallback: without a GPU, gch_create refuses."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    p = problems.orszag_tang(16, 16, 4)[0]
    s = _abi.to_struct(p)
    h = C.c_void_p()
    st = gpu_lib.gch_create(C.byref(s), None, C.byref(h))
    assert st == _abi.ERR_NO_DEVICE and not h.value

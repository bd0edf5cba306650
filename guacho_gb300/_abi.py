"""ctypes binding of the C ABI in include/guacho_gb300.h.

Loads the in-tree guacho_gb300/lib/libguacho_gb300.so.  There is no CPU
fallback: if the library is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .params import Params

ABI_VERSION = 3
MAX_SPHERES, MAX_GRAV, MAX_TABLE = 8, 4, 512

ERR_PARAM, ERR_CUDA, ERR_HLLD, ERR_HLLC = 0x1, 0x2, 0x4, 0x8
ERR_DT, ERR_TIMEOUT, ERR_NO_DEVICE, ERR_STATE = 0x10, 0x20, 0x40, 0x80
ERR_TOO_LARGE = 0x100
ERR_NAMES = {ERR_PARAM: "PARAM", ERR_CUDA: "CUDA", ERR_HLLD: "HLLD", ERR_HLLC: "HLLC",
             ERR_DT: "DT", ERR_TIMEOUT: "TIMEOUT", ERR_NO_DEVICE: "NO_DEVICE",
             ERR_STATE: "STATE", ERR_TOO_LARGE: "TOO_LARGE"}

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libguacho_gb300.so"


class Sphere_t(C.Structure):
    _fields_ = [("xc", C.c_double), ("yc", C.c_double), ("zc", C.c_double),
                ("radius", C.c_double), ("dens", C.c_double), ("vwind", C.c_double),
                ("vorb", C.c_double * 3), ("tfac", C.c_double), ("bdip", C.c_double),
                ("orbit_r", C.c_double), ("orbit_omega", C.c_double), ("orbit_phase", C.c_double)]


class Params_t(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("precision", C.c_int32),
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("neq", C.c_int32),
        ("mhd", C.c_int32), ("pmhd", C.c_int32),
        ("riemann_solver", C.c_int32), ("slope_limiter", C.c_int32),
        ("eq_of_state", C.c_int32), ("cooling", C.c_int32),
        ("enable_flux_cd", C.c_int32), ("eight_wave", C.c_int32),
        ("user_source_terms", C.c_int32),
        ("bc_left", C.c_int32), ("bc_right", C.c_int32), ("bc_bottom", C.c_int32),
        ("bc_top", C.c_int32), ("bc_out", C.c_int32), ("bc_in", C.c_int32),
        ("bc_user", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("cv", C.c_double), ("gamma", C.c_double), ("cfl", C.c_double), ("eta", C.c_double),
        ("Tempsc", C.c_double), ("Psc", C.c_double), ("tsc", C.c_double),
        ("ntab", C.c_int32), ("tab_i0", C.c_int32),
        ("tab_inv_dlog", C.c_double), ("tab_tail", C.c_double), ("tab_Tmin", C.c_double),
        ("tab_T", C.c_double * MAX_TABLE), ("tab_L", C.c_double * MAX_TABLE),
        ("nsph", C.c_int32), ("ngrav", C.c_int32),
        ("sph", Sphere_t * MAX_SPHERES),
        ("grav_GM", C.c_double * MAX_GRAV), ("grav_x", C.c_double * MAX_GRAV),
        ("grav_y", C.c_double * MAX_GRAV), ("grav_z", C.c_double * MAX_GRAV),
        ("th_cond", C.c_int32), ("tc_saturation", C.c_int32),
        ("rsc", C.c_double), ("rhosc", C.c_double), ("vsc2", C.c_double), ("bsc", C.c_double),
        ("mu", C.c_double),
        ("npas", C.c_int32),
    ]


def to_struct(p: Params) -> Params_t:
    s = Params_t()
    s.abi_version = ABI_VERSION
    s.precision = p.precision
    s.nx, s.ny, s.nz, s.neq = p.nx, p.ny, p.nz, p.neq
    s.mhd, s.pmhd = int(p.mhd), int(p.pmhd)
    s.riemann_solver, s.slope_limiter = p.riemann_solver, p.slope_limiter
    s.eq_of_state, s.cooling = p.eq_of_state, p.cooling
    s.enable_flux_cd, s.eight_wave = int(p.enable_flux_cd), int(p.eight_wave)
    s.user_source_terms = int(p.user_source_terms)
    s.bc_left, s.bc_right, s.bc_bottom = p.bc_left, p.bc_right, p.bc_bottom
    s.bc_top, s.bc_out, s.bc_in = p.bc_top, p.bc_out, p.bc_in
    s.bc_user = int(p.bc_user)
    s.dx, s.dy, s.dz = p.dx, p.dy, p.dz
    s.cv, s.gamma, s.cfl, s.eta = p.cv, p.gamma, p.cfl, p.eta
    s.Tempsc, s.Psc, s.tsc = p.Tempsc, p.Psc, p.tsc
    s.ntab = len(p.tab_T)
    s.tab_i0, s.tab_inv_dlog = p.tab_i0, p.tab_inv_dlog
    s.tab_tail, s.tab_Tmin = p.tab_tail, p.tab_Tmin
    for i, (t, l) in enumerate(zip(p.tab_T, p.tab_L)):
        s.tab_T[i], s.tab_L[i] = t, l
    s.nsph = len(p.spheres)
    for i, sp in enumerate(p.spheres):
        d = s.sph[i]
        d.xc, d.yc, d.zc, d.radius = sp.xc, sp.yc, sp.zc, sp.radius
        d.dens, d.vwind, d.tfac, d.bdip = sp.dens, sp.vwind, sp.tfac, sp.bdip
        d.orbit_r, d.orbit_omega, d.orbit_phase = sp.orbit_r, sp.orbit_omega, sp.orbit_phase
        for a in range(3):
            d.vorb[a] = sp.vorb[a]
    s.ngrav = len(p.grav)
    for i, (gm, x, y, z) in enumerate(p.grav):
        s.grav_GM[i], s.grav_x[i], s.grav_y[i], s.grav_z[i] = gm, x, y, z
    s.th_cond, s.tc_saturation = p.th_cond, int(p.tc_saturation)
    s.rsc, s.rhosc, s.vsc2, s.bsc, s.mu = p.rsc, p.rhosc, p.vsc2, p.bsc, p.mu
    s.npas = p.npas
    return s


_lib = None


def lib() -> C.CDLL:
    """The loaded library (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                           "`python -m guacho_gb300.build` (no CPU fallback exists)")
    L = C.CDLL(str(LIB_PATH))
    P, D, I, DP, IP = C.c_void_p, C.c_double, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_int)
    VPP = C.POINTER(C.c_void_p)
    sig = {
        "gch_params_default": (None, [C.POINTER(Params_t), I, I, I]),
        "gch_params_check": (I, [C.POINTER(Params_t)]),
        "gch_create": (I, [C.POINTER(Params_t), P, VPP]),
        "gch_destroy": (I, [P]),
        "gch_upload": (I, [P, P]),
        "gch_download": (I, [P, P, P]),
        "gch_set_background": (I, [P, P]),
        "gch_boundaryI": (I, [P]),
        "gch_calcprim": (I, [P]),
        "gch_get_timestep": (I, [P, I, I, D, D, DP, IP]),
        "gch_tstep": (I, [P, D]),
        "gch_tc_info": (I, [P, IP, DP]),
        "gch_step_host": (I, [P, P, I, I, D, D, DP, IP]),
        "gch_step_host_overlaps": (I, [P]),
        "gch_advance": (I, [P, I, D, D, I, DP, IP, DP, IP]),
        "gch_last_step_info": (I, [P, C.POINTER(C.c_longlong), IP]),
        "gch_launches_per_step": (I, [P]),
        "gch_advance_timed": (I, [P, I, I, C.POINTER(C.c_float)]),
        "gch_profile_step": (I, [P, I, C.POINTER(C.c_float), C.c_char_p, I, IP]),
        "gch_get_kz": (I, [P]),
        "gch_set_kz": (I, [P, I]),
        "gch_autotune": (I, [P, I, IP, C.POINTER(C.c_float), IP]),
        "gch_batch_create": (I, [I, C.POINTER(Params_t), P, VPP]),
        "gch_batch_destroy": (I, [P]),
        "gch_batch_upload": (I, [P, I, P]),
        "gch_batch_download": (I, [P, I, P]),
        "gch_batch_advance": (I, [P, I, I]),
        "gch_batch_time": (I, [P, DP, IP]),
        "gch_batch_tuning": (I, [P, IP, IP, I, IP, C.POINTER(C.c_float), IP]),
        "gch_batch_tuning_grid": (I, [P, IP, IP, IP, I, IP, IP, C.POINTER(C.c_float), IP]),
        "gch_get_timestep_noalloc": (I, [C.POINTER(Params_t), P, I, I, D, D, P, P, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def exported_symbols() -> list[str]:
    return ["gch_params_default", "gch_params_check", "gch_create", "gch_destroy",
            "gch_upload", "gch_download", "gch_set_background", "gch_boundaryI", "gch_calcprim",
            "gch_get_timestep", "gch_tstep", "gch_tc_info", "gch_step_host",
            "gch_step_host_overlaps", "gch_advance",
            "gch_last_step_info", "gch_launches_per_step", "gch_advance_timed",
            "gch_profile_step", "gch_get_kz", "gch_set_kz", "gch_autotune",
            "gch_batch_create",
            "gch_batch_destroy", "gch_batch_upload", "gch_batch_download",
            "gch_batch_advance", "gch_batch_time", "gch_batch_tuning", "gch_batch_tuning_grid",
            "gch_get_timestep_noalloc"]


class GuachoError(RuntimeError):
    def __init__(self, where: str, status: int):
        names = [n for b, n in ERR_NAMES.items() if status & b]
        super().__init__(f"{where} failed with status 0x{status:x} ({'|'.join(names)})")
        self.status = status


def check(where: str, status: int) -> None:
    if status:
        raise GuachoError(where, status)


def ptr(a: np.ndarray) -> int:
    assert a.flags.c_contiguous
    return a.ctypes.data

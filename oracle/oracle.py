"""ctypes wrapper of the CPU oracle (oracle/guacho_oracle.c).

TEST INFRASTRUCTURE ONLY: the FP64 CPU restatement of the reference's
timestep, used by the tests, the smoke check and the benchmark's CPU
baseline as the checker.  The product (guacho_gb300) never imports it.

Parity status: see the header of guacho_oracle.c.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SRC = HERE / "guacho_oracle.c"
MAXSPH, MAXGRAV, MAXTAB, MAXNEQ = 8, 4, 512, 10


def build(force: bool = False) -> Path:
    """gcc -O2 -ffp-contract=off (no FMA contraction, IEEE semantics)."""
    if not force and LIB.exists() and LIB.stat().st_mtime >= max(
            SRC.stat().st_mtime, (HERE / "guacho_oracle.h").stat().st_mtime):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
           "-o", str(tmp), str(SRC), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


class Sph(C.Structure):
    _fields_ = [("xc", C.c_double), ("yc", C.c_double), ("zc", C.c_double),
                ("radius", C.c_double), ("dens", C.c_double), ("vwind", C.c_double),
                ("vorb", C.c_double * 3), ("tfac", C.c_double), ("bdip", C.c_double),
                ("orbit_r", C.c_double), ("orbit_omega", C.c_double), ("orbit_phase", C.c_double)]


class GorParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("neq", C.c_int),
        ("mhd", C.c_int), ("pmhd", C.c_int),
        ("riemann_solver", C.c_int), ("slope_limiter", C.c_int), ("eq_of_state", C.c_int),
        ("cooling", C.c_int),
        ("enable_flux_cd", C.c_int), ("eight_wave", C.c_int), ("user_source_terms", C.c_int),
        ("bc_left", C.c_int), ("bc_right", C.c_int), ("bc_bottom", C.c_int), ("bc_top", C.c_int),
        ("bc_out", C.c_int), ("bc_in", C.c_int), ("bc_user", C.c_int),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("cv", C.c_double), ("gamma", C.c_double), ("cfl", C.c_double), ("eta", C.c_double),
        ("Tempsc", C.c_double), ("Psc", C.c_double), ("tsc", C.c_double),
        ("ntab", C.c_int), ("tab_T", C.c_double * MAXTAB), ("tab_L", C.c_double * MAXTAB),
        ("tab_inv_dlog", C.c_double), ("tab_i0", C.c_int), ("tab_tail", C.c_double),
        ("tab_Tmin", C.c_double),
        ("nsph", C.c_int), ("sph", Sph * MAXSPH),
        ("ngrav", C.c_int), ("grav_GM", C.c_double * MAXGRAV), ("grav_x", C.c_double * MAXGRAV),
        ("grav_y", C.c_double * MAXGRAV), ("grav_z", C.c_double * MAXGRAV),
        ("th_cond", C.c_int), ("tc_saturation", C.c_int),
        ("rsc", C.c_double), ("rhosc", C.c_double), ("vsc2", C.c_double), ("bsc", C.c_double),
        ("mu", C.c_double),
        ("npas", C.c_int),
    ]


def params_struct(p) -> GorParams:
    """From a guacho_gb300.params.Params (same field names)."""
    s = GorParams()
    s.nx, s.ny, s.nz, s.neq = p.nx, p.ny, p.nz, p.neq
    s.mhd, s.pmhd = int(p.mhd), int(p.pmhd)
    s.riemann_solver, s.slope_limiter = p.riemann_solver, p.slope_limiter
    s.eq_of_state, s.cooling = p.eq_of_state, p.cooling
    s.enable_flux_cd, s.eight_wave = int(p.enable_flux_cd), int(p.eight_wave)
    s.user_source_terms = int(p.user_source_terms)
    s.bc_left, s.bc_right, s.bc_bottom = p.bc_left, p.bc_right, p.bc_bottom
    s.bc_top, s.bc_out, s.bc_in, s.bc_user = p.bc_top, p.bc_out, p.bc_in, int(p.bc_user)
    s.dx, s.dy, s.dz = p.dx, p.dy, p.dz
    s.cv, s.gamma, s.cfl, s.eta = p.cv, p.gamma, p.cfl, p.eta
    s.Tempsc, s.Psc, s.tsc = p.Tempsc, p.Psc, p.tsc
    s.ntab = len(p.tab_T)
    for i, (t, l) in enumerate(zip(p.tab_T, p.tab_L)):
        s.tab_T[i], s.tab_L[i] = t, l
    s.tab_inv_dlog, s.tab_i0, s.tab_tail, s.tab_Tmin = (p.tab_inv_dlog, p.tab_i0, p.tab_tail,
                                                         p.tab_Tmin)
    s.nsph = len(p.spheres)
    for i, sp in enumerate(p.spheres):
        d = s.sph[i]
        d.xc, d.yc, d.zc, d.radius, d.dens, d.vwind = (sp.xc, sp.yc, sp.zc, sp.radius, sp.dens,
                                                       sp.vwind)
        d.tfac, d.bdip = sp.tfac, sp.bdip
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
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P, D, I = C.c_void_p, C.c_double, C.c_int
        DP, IP = C.POINTER(C.c_double), C.POINTER(C.c_int)
        GP = C.POINTER(GorParams)
        sigs = {
            "gor_create": (P, [GP]), "gor_destroy": (None, [P]), "gor_nthreads": (I, [I]),
            "gor_set_u": (None, [P, P]), "gor_get_u": (None, [P, P]),
            "gor_get_primit": (None, [P, P]), "gor_set_primit": (None, [P, P]),
            "gor_set_background": (None, [P, P]),
            "gor_riemann_split": (None, [GP, P, P, P, P, P]),
            "gor_boundaryI": (None, [P]), "gor_calcprim": (None, [P, I]),
            "gor_get_timestep": (None, [P, I, I, D, D, DP, IP]),
            "gor_tstep": (None, [P, D]), "gor_time": (D, [P]), "gor_set_time": (None, [P, D]),
            "gor_error": (I, [P]),
            "gor_riemann": (None, [GP, P, P, P, IP]), "gor_prim2f": (None, [GP, P, P]),
            "gor_u2prim": (None, [GP, P, P, DP]), "gor_prim2u": (None, [GP, P, P]),
            "gor_limiter": (None, [GP, P, P, P, P]), "gor_cooltab": (D, [GP, D]),
            "gor_divb": (None, [P, P]),
            "gor_run": (I, [P, D, D, I, I, IP, DP]),
            "gor_thermal_conduction": (None, [P, D, IP, DP]),
            "gor_get_temp": (None, [P, P]),
            "gor_superstep": (D, [I, D]), "gor_substep": (D, [I, I, D]),
            "gor_st_steps": (None, [D, IP, DP]),
        }
        for name, (res, args) in sigs.items():
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        _lib = L
    return _lib


def _p(a: np.ndarray) -> int:
    assert a.flags.c_contiguous and a.dtype == np.float64
    return a.ctypes.data


class Oracle:
    """One domain of the CPU restatement, same host layout as the GPU API."""

    def __init__(self, params, threads: int = 0):
        self.params = params
        self.ps = params_struct(params)
        self.L = lib()
        if threads:
            self.L.gor_nthreads(threads)
        self.h = self.L.gor_create(C.byref(self.ps))
        if not self.h:
            raise RuntimeError("gor_create rejected the parameters")
        self.iter = 1
        self.tprint = None

    def close(self):
        if self.h:
            self.L.gor_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def time(self) -> float:
        return self.L.gor_time(self.h)

    @time.setter
    def time(self, t: float):
        self.L.gor_set_time(self.h, t)

    def upload(self, u: np.ndarray):
        u = np.ascontiguousarray(u, dtype=np.float64)
        assert u.shape == self.params.shape
        self.L.gor_set_u(self.h, _p(u))

    def set_background(self, prim0: np.ndarray):
        """The split solver's background primit0 (same layout as u)."""
        prim0 = np.ascontiguousarray(prim0, dtype=np.float64)
        assert prim0.shape == self.params.shape
        self.L.gor_set_background(self.h, _p(prim0))

    def download(self, with_primit: bool = False):
        u = np.empty(self.params.shape)
        self.L.gor_get_u(self.h, _p(u))
        if not with_primit:
            return u
        pr = np.empty(self.params.shape)
        self.L.gor_get_primit(self.h, _p(pr))
        return u, pr

    def init(self, u0: np.ndarray):
        """src/main.f90:73-79."""
        self.upload(u0)
        self.L.gor_boundaryI(self.h)
        self.L.gor_calcprim(self.h, 0)

    def boundaryI(self):
        """src/boundaries.f90 boundaryI on u (user spheres at the state's time)."""
        self.L.gor_boundaryI(self.h)

    def get_timestep(self, it, n_iter, t, tprint):
        dt = C.c_double()
        dump = C.c_int(0)
        self.L.gor_get_timestep(self.h, it, n_iter, t, tprint, C.byref(dt), C.byref(dump))
        return dt.value, bool(dump.value)

    def tstep(self, dt: float):
        self.L.gor_tstep(self.h, dt)

    def run(self, tmax: float, dtprint: float, max_steps: int = 1 << 30, n_iter: int = 10) -> int:
        if self.tprint is None:
            self.tprint = dtprint
        it = C.c_int(self.iter)
        tp = C.c_double(self.tprint)
        n = self.L.gor_run(self.h, tmax, dtprint, max_steps, n_iter, C.byref(it), C.byref(tp))
        self.iter, self.tprint = it.value, tp.value
        return n

    @property
    def error(self) -> int:
        return self.L.gor_error(self.h)

    def divb(self) -> np.ndarray:
        p = self.params
        out = np.empty((p.nz, p.ny, p.nx))
        self.L.gor_divb(self.h, _p(out))
        return out

    def thermal_conduction(self, dt_cfl: float) -> tuple[int, float]:
        """src/thermal_cond.f90:690-768 on the current state; returns the
        substep count and the conduction timescale (seconds)."""
        n = C.c_int()
        dtc = C.c_double()
        self.L.gor_thermal_conduction(self.h, dt_cfl, C.byref(n), C.byref(dtc))
        return n.value, dtc.value

    def temp(self) -> np.ndarray:
        """Temp of every cell, (z, y, x) with ghosts."""
        p = self.params
        out = np.empty(p.shape[:3])
        self.L.gor_get_temp(self.h, _p(out))
        return out


def riemann(params, pl, pr):
    ps = params_struct(params)
    pl = np.ascontiguousarray(pl, dtype=np.float64)
    pr = np.ascontiguousarray(pr, dtype=np.float64)
    ff = np.zeros(MAXNEQ)
    err = C.c_int(0)
    lib().gor_riemann(C.byref(ps), _p(pl), _p(pr), _p(ff), C.byref(err))
    return ff[:params.neq], err.value


def riemann_split(params, pl, pr, p0l, p0r):
    """src/hlle_split_all.f90:51-84 for one x-interface."""
    ps = params_struct(params)
    a = [np.ascontiguousarray(np.pad(np.asarray(v, dtype=np.float64),
                                     (0, MAXNEQ - len(v))), dtype=np.float64)
         for v in (pl, pr, p0l, p0r)]
    ff = np.zeros(MAXNEQ)
    lib().gor_riemann_split(C.byref(ps), *[_p(v) for v in a], _p(ff))
    return ff[:params.neq]


def prim2f(params, prim):
    ps = params_struct(params)
    prim = np.ascontiguousarray(prim, dtype=np.float64)
    ff = np.zeros(MAXNEQ)
    lib().gor_prim2f(C.byref(ps), _p(prim), _p(ff))
    return ff[:params.neq]


def u2prim(params, uu):
    ps = params_struct(params)
    uu = np.ascontiguousarray(uu, dtype=np.float64)
    pr = np.zeros(MAXNEQ)
    T = C.c_double()
    lib().gor_u2prim(C.byref(ps), _p(uu), _p(pr), C.byref(T))
    return pr[:params.neq], T.value


def prim2u(params, prim):
    ps = params_struct(params)
    prim = np.ascontiguousarray(prim, dtype=np.float64)
    uu = np.zeros(MAXNEQ)
    lib().gor_prim2u(C.byref(ps), _p(prim), _p(uu))
    return uu[:params.neq]


def limiter(params, pll, pl, pr, prr):
    ps = params_struct(params)
    a = [np.ascontiguousarray(x, dtype=np.float64).copy() for x in (pll, pl, pr, prr)]
    lib().gor_limiter(C.byref(ps), *[_p(x) for x in a])
    return a[1], a[2]


def cooltab(params, T: float) -> float:
    ps = params_struct(params)
    return lib().gor_cooltab(C.byref(ps), T)


def superstep(n: int, snu: float) -> float:
    return lib().gor_superstep(n, snu)


def substep(j: int, n: int, nu: float) -> float:
    return lib().gor_substep(j, n, nu)


def st_steps(fs: float) -> tuple[int, float]:
    ns = C.c_int()
    fstep = C.c_double()
    lib().gor_st_steps(fs, C.byref(ns), C.byref(fstep))
    return ns.value, fstep.value

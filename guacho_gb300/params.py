"""The parameter surface of Guacho's parameters.f90 as a Python object.

Field names follow OT/parameters.f90:48-177 (riemann_solver, slope_limiter,
bc_left, cfl, eta, ...).  `Params` is converted to the C-ABI struct
`gch_params_t` (include/guacho_gb300.h) by `guacho_gb300._abi`.
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass, field

# src/constants.f90:56-98
SOLVER_HLL, SOLVER_HLLC, SOLVER_HLLE, SOLVER_HLLD = 1, 2, 3, 4
SOLVER_HLLE_SPLIT_ALL = 7  # src/constants.f90:62, fluctuations over a background
EOS_ADIABATIC, EOS_SINGLE_SPECIE, EOS_H_RATE = 1, 2, 3
COOL_NONE, COOL_H, COOL_DMC, COOL_CHI = 0, 1, 3, 4
TC_OFF, TC_ISOTROPIC, TC_ANISOTROPIC = 0, 1, 2
BC_OUTFLOW, BC_CLOSED, BC_PERIODIC, BC_OTHER = 1, 2, 3, 4
(LIMITER_NO_AVERAGE, LIMITER_NO_LIMIT, LIMITER_MINMOD, LIMITER_VAN_LEER,
 LIMITER_VAN_ALBADA, LIMITER_UMIST, LIMITER_WOODWARD, LIMITER_SUPERBEE) = range(-1, 7)

# precision modes (include/guacho_gb300.h)
FP64, FP32_MIXED, FP32_KAHAN = 0, 1, 2
NGHOST = 2


@dataclass
class Sphere:
    """A wind sphere re-imposed by the user boundary hook (EXO pattern).
    With orbit_omega != 0 it moves on a circular orbit in the x-z plane
    (EXO/exoplanet.f90:143-148): centre (orbit_r cos th, yc, orbit_r sin th)
    and velocity orbit_omega*orbit_r*(-sin th, 0, cos th) at
    th = orbit_omega*t + orbit_phase, t the step's start time."""
    xc: float = 0.0
    yc: float = 0.0
    zc: float = 0.0
    radius: float = 0.1
    dens: float = 1.0
    vwind: float = 0.0
    vorb: tuple = (0.0, 0.0, 0.0)
    tfac: float = 1.0
    bdip: float = 0.0
    orbit_r: float = 0.0
    orbit_omega: float = 0.0
    orbit_phase: float = 0.0


@dataclass
class Params:
    nx: int = 128
    ny: int = 128
    nz: int = 4
    precision: int = FP64
    mhd: bool = True
    pmhd: bool = False
    riemann_solver: int = SOLVER_HLLD
    slope_limiter: int = LIMITER_MINMOD
    eq_of_state: int = EOS_ADIABATIC
    cooling: int = COOL_NONE
    enable_flux_cd: bool = True
    eight_wave: bool = False
    user_source_terms: bool = False
    bc_left: int = BC_PERIODIC
    bc_right: int = BC_PERIODIC
    bc_bottom: int = BC_PERIODIC
    bc_top: int = BC_PERIODIC
    bc_out: int = BC_PERIODIC
    bc_in: int = BC_PERIODIC
    bc_user: bool = False
    xmax: float = 1.0
    ymax: float = 1.0
    zmax: float = 1.0
    cv: float = 1.5
    cfl: float = 0.2
    eta: float = 0.0
    Tempsc: float = 1.0
    Psc: float = 1.0
    tsc: float = 1.0
    # tabulated cooling
    tab_T: list = field(default_factory=list)
    tab_L: list = field(default_factory=list)
    tab_inv_dlog: float = 10.0
    tab_i0: int = 40
    tab_tail: float = 0.27e-26
    tab_Tmin: float = 1e4
    spheres: list = field(default_factory=list)
    # point masses: (GM, x, y, z)
    grav: list = field(default_factory=list)
    # thermal conduction (src/thermal_cond.f90) and the cgs scalings it
    # converts with (parameters.f90:159-170: rsc = xphys/xmax, rhosc,
    # vsc2, bsc = sqrt(4 pi Psc), mu)
    th_cond: int = TC_OFF
    tc_saturation: bool = False
    rsc: float = 1.0
    rhosc: float = 1.0
    vsc2: float = 1.0
    bsc: float = math.sqrt(4.0 * math.pi)
    mu: float = 1.0
    # passive scalars (parameters.f90:131-135): the last npas equations;
    # with EOS_H_RATE / COOL_H the first is the neutral hydrogen density
    npas: int = 0

    @property
    def bfield(self) -> bool:
        return self.mhd or self.pmhd

    @property
    def neqdyn(self) -> int:
        return 8 if self.bfield else 5

    @property
    def neq(self) -> int:
        return self.neqdyn + self.npas

    @property
    def gamma(self) -> float:
        return (self.cv + 1.0) / self.cv  # OT/parameters.f90:158

    # dx = xmax/nxtot (src/init.f90:120-122)
    @property
    def dx(self) -> float:
        return self.xmax / self.nx if self.nx else float("nan")

    @property
    def dy(self) -> float:
        return self.ymax / self.ny if self.ny else float("nan")

    @property
    def dz(self) -> float:
        return self.zmax / self.nz if self.nz else float("nan")

    @property
    def shape(self) -> tuple:
        """Host array shape in C order (z, y, x, neq) of the Fortran
        u(neq, nxmin:nxmax, nymin:nymax, nzmin:nzmax)."""
        g = NGHOST
        return (self.nz + 2 * g, self.ny + 2 * g, self.nx + 2 * g, self.neq)

    def replace(self, **kw) -> "Params":
        return dataclasses.replace(self, **kw)


def table_from_log(logT: list, logL: list, tail: float) -> dict:
    """Cooling-table fields from rows equally spaced in log10 T."""
    n = len(logT)
    dlog = (logT[-1] - logT[0]) / (n - 1)
    inv = 1.0 / dlog
    return dict(tab_T=[10.0 ** a for a in logT], tab_L=[10.0 ** b for b in logL],
                tab_inv_dlog=round(inv, 9), tab_i0=int(round(logT[0] * inv)), tab_tail=tail)


# The reference's two shipped cooling curves: 41 rows at 0.1 dex from
# 10^4 K, read by src/cooling_dmc.f90:57-82 and src/cooling_chi.f90:56-80,
# with their own tails above 10^8 K (cooling_dmc.f90:96, cooling_chi.f90:95).
COOL_TABLE_ROWS = 41
COOL_TABLE_TAIL = {COOL_DMC: 0.27e-26, COOL_CHI: 0.21e-26}


def parse_cooling_rows(text: str, kind: int) -> tuple:
    """Rows of a cooling table file in the reference's own format (list
    directed `read(10,*) a, b`, Fortran exponents such as 4.0d0 allowed):
    COOL_DMC rows are (log10 T, -log10 Lambda) and decode to
    (10**a, 10**(-b)) (src/cooling_dmc.f90:71-75); COOL_CHI rows are raw
    (T, Lambda) (src/cooling_chi.f90:69-73).  Returns (T, Lambda) lists."""
    if kind not in COOL_TABLE_TAIL:
        raise ValueError(f"cooling kind {kind} has no table")
    T, L = [], []
    for line in text.splitlines():
        tok = line.replace("d", "e").replace("D", "e").split()
        if len(tok) < 2:
            continue
        a, b = float(tok[0]), float(tok[1])
        if kind == COOL_DMC:
            T.append(10.0 ** a)
            L.append(10.0 ** (-b))
        else:
            T.append(a)
            L.append(b)
        if len(T) == COOL_TABLE_ROWS:
            break
    if len(T) != COOL_TABLE_ROWS:
        raise ValueError(f"a cooling table has {COOL_TABLE_ROWS} rows, found {len(T)}")
    return T, L


def cooling_table(T: list, L: list, kind: int) -> dict:
    """Params fields for one of the reference's 41-row tables: row index
    int(log10(T)*10) - 39 (1-based, src/cooling_dmc.f90:98), the tail of the
    kind above 10^8 K, cooling above Tmin = 10^4 K."""
    return dict(cooling=kind, tab_T=list(T), tab_L=list(L), tab_inv_dlog=10.0, tab_i0=40,
                tab_tail=COOL_TABLE_TAIL[kind], tab_Tmin=1.0e4)


def read_cooling_table(path, kind: int) -> dict:
    """The reference's table file at `path` (src/DMClib/coolingDMC.tab for
    COOL_DMC, src/CHIANTIlib/coolingCHIANTI.tab for COOL_CHI) as Params
    fields, decoded the way the reference's reader decodes it."""
    with open(path) as f:
        T, L = parse_cooling_rows(f.read(), kind)
    return cooling_table(T, L, kind)

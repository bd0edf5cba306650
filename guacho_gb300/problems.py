"""Initial conditions of the benchmark problems (the user_mod
`initial_conditions` hook of the reference, restated on the host).

Every generator returns (Params, u0) with u0 in the reference's host layout
(C-ordered (nz+4, ny+4, nx+4, neq) float64, ghost cells included).  Seeded
inputs are deterministic for a given seed.

  orszag_tang   OT/orzag_tang.f90:14-70 (ideal MHD, periodic)
  turbulence    decaying MHD turbulence, random-phase solenoidal velocity
  blast         low-beta MHD blast wave (outflow)
  wind_cooling  hydro wind interaction with tabulated cooling (outflow,
                spheres re-imposed by the user boundary hook)
  batch_boxes   the mixed set of OT / blast boxes of uneven size
"""
from __future__ import annotations

import math
from dataclasses import replace

import numpy as np

from .params import (BC_OUTFLOW, BC_PERIODIC, COOL_DMC, COOL_H, EOS_H_RATE, FP64,
                     LIMITER_MINMOD, LIMITER_VAN_LEER, NGHOST, SOLVER_HLLC, SOLVER_HLLD,
                     Params, Sphere, table_from_log)

G = NGHOST


def _cell_index(n: int) -> np.ndarray:
    """Fortran cell indices 1-nghost .. n+nghost."""
    return np.arange(1 - G, n + G + 1)


def conserved(p: Params, rho, vx, vy, vz, pr, bx=None, by=None, bz=None) -> np.ndarray:
    """u from primitives on the full array, src/hydro_core.f90:331-383 order."""
    u = np.zeros(p.shape)
    rho = np.broadcast_to(rho, p.shape[:3])
    u[..., 0] = rho
    u[..., 1] = rho * vx
    u[..., 2] = rho * vy
    u[..., 3] = rho * vz
    e = 0.5 * rho * (vx * vx + vy * vy + vz * vz) + p.cv * pr
    if p.bfield:
        u[..., 5] = bx
        u[..., 6] = by
        u[..., 7] = bz
        if p.mhd:
            e = e + 0.5 * (bx * bx + by * by + bz * bz)
    u[..., 4] = e
    return u


# ---------------------------------------------------------------------------
def orszag_tang(nx=128, ny=128, nz=4, precision=FP64, cfl=0.4, b0_scale=1.0, **kw) -> tuple:
    """Orszag-Tang vortex, OT/orzag_tang.f90:14-70 and OT/parameters.f90
    (HLLD, minmod, flux-CD, periodic), with dz = dx (zmax = nz/nx)."""
    opts = dict(riemann_solver=SOLVER_HLLD, slope_limiter=LIMITER_MINMOD)
    opts.update(kw)
    p = Params(nx=nx, ny=ny, nz=nz, precision=precision, mhd=True,
               xmax=1.0, ymax=ny / nx, zmax=nz / nx, cfl=cfl, **opts)
    pi = math.acos(-1.0)
    rho = 25.0 / (36.0 * pi)
    pr = 5.0 / (12.0 * pi)
    twopi = 2.0 * pi
    s4 = math.sqrt(4 * pi)
    # position measured from the bottom corner: x = (float(i)+0.5)*dx (i 1-based)
    x = (_cell_index(nx).astype(np.float64) + 0.5) * p.dx
    y = (_cell_index(ny).astype(np.float64) + 0.5) * p.dy
    vx1 = np.array([-math.sin(v * twopi) for v in y])
    vy1 = np.array([math.sin(v * twopi) for v in x])
    bx1 = np.array([-math.sin(v * twopi) / s4 for v in y]) * b0_scale
    by1 = np.array([math.sin(2.0 * v * twopi) / s4 for v in x]) * b0_scale
    sh = p.shape[:3]
    vx = np.broadcast_to(vx1[None, :, None], sh)
    vy = np.broadcast_to(vy1[None, None, :], sh)
    bx = np.broadcast_to(bx1[None, :, None], sh)
    by = np.broadcast_to(by1[None, None, :], sh)
    z = np.zeros(sh)
    return p, conserved(p, rho, vx, vy, z, pr, bx, by, z)


# ---------------------------------------------------------------------------
def _solenoidal_field(n: int, rng: np.random.Generator, kmin: float, kmax: float,
                      slope: float) -> np.ndarray:
    """Random-phase divergence-free field on an n^3 periodic grid whose shell
    spectrum follows E(k) ~ k^slope for kmin <= |k| <= kmax.  Returns
    (3, n, n, n) in (z, y, x) order, unnormalised."""
    k1 = np.fft.fftfreq(n, d=1.0 / n)
    kr = np.fft.rfftfreq(n, d=1.0 / n)
    KZ, KY, KX = np.meshgrid(k1, k1, kr, indexing="ij")
    K = np.sqrt(KX ** 2 + KY ** 2 + KZ ** 2)
    mask = (K >= kmin) & (K <= kmax)
    Ks = np.where(K > 0, K, 1.0)
    # per-mode amplitude: E(k) dk ~ |v_k|^2 4 pi k^2 dk  ->  |v_k| ~ k^((slope-2)/2)
    amp = np.where(mask, Ks ** ((slope - 2.0) / 2.0), 0.0)
    comps = []
    for _ in range(3):
        ph = rng.uniform(0.0, 2.0 * np.pi, size=K.shape)
        g = rng.standard_normal(size=K.shape)
        comps.append(amp * g * np.exp(1j * ph))
    vx, vy, vz = comps
    # Helmholtz projection onto k-perpendicular modes
    kdotv = (KX * vx + KY * vy + KZ * vz) / (Ks * Ks)
    vx = vx - KX * kdotv
    vy = vy - KY * kdotv
    vz = vz - KZ * kdotv
    out = np.stack([np.fft.irfftn(c, s=(n, n, n), axes=(0, 1, 2)) for c in (vx, vy, vz)])
    return out


def _pad_periodic(a: np.ndarray) -> np.ndarray:
    return np.pad(a, G, mode="wrap")


def turbulence(n=256, precision=FP64, seed=20260001, mach=1.0, b0=0.1, brms=0.05,
               cfl=0.4, **kw) -> tuple:
    """Decaying MHD turbulence: periodic unit cube, rho = 1, p = 1,
    gamma = 5/3; random-phase solenoidal velocity with E(k) ~ k^-2 on
    2 <= |k| <= 8 scaled to RMS Mach `mach`; B = (b0,0,0) + a solenoidal
    perturbation of RMS `brms` built as the centred-difference curl of a
    random vector potential (so its centred div B is round-off).  HLLD,
    van Leer, flux-CD."""
    opts = dict(riemann_solver=SOLVER_HLLD, slope_limiter=LIMITER_VAN_LEER)
    opts.update(kw)
    p = Params(nx=n, ny=n, nz=n, precision=precision, mhd=True, cfl=cfl, **opts)
    rng = np.random.default_rng(seed)
    v = _solenoidal_field(n, rng, 2.0, 8.0, -2.0)
    cs = math.sqrt(p.gamma * 1.0 / 1.0)
    vrms = math.sqrt(np.mean(v[0] ** 2 + v[1] ** 2 + v[2] ** 2))
    v *= mach * cs / vrms
    a = _solenoidal_field(n, rng, 2.0, 8.0, -2.0)
    ax, ay, az = a[0], a[1], a[2]   # (z, y, x) arrays

    def dcen(f, axis, d):
        return (np.roll(f, -1, axis=axis) - np.roll(f, 1, axis=axis)) / (2.0 * d)

    # arrays are (z, y, x): axis 2 = x, axis 1 = y, axis 0 = z
    bx = dcen(az, 1, p.dy) - dcen(ay, 0, p.dz)
    by = dcen(ax, 0, p.dz) - dcen(az, 2, p.dx)
    bz = dcen(ay, 2, p.dx) - dcen(ax, 1, p.dy)
    bpr = math.sqrt(np.mean(bx ** 2 + by ** 2 + bz ** 2))
    bx, by, bz = (c * (brms / bpr) for c in (bx, by, bz))
    bx = bx + b0
    fields = [_pad_periodic(f) for f in (v[0], v[1], v[2], bx, by, bz)]
    u = conserved(p, 1.0, fields[0], fields[1], fields[2], 1.0, fields[3], fields[4], fields[5])
    return p, u


# ---------------------------------------------------------------------------
def _centered_coords(p: Params):
    """Cell centres measured from the box centre, (z, y, x) broadcastable."""
    x = (_cell_index(p.nx) - p.nx / 2.0 - 0.5) * p.dx
    y = (_cell_index(p.ny) - p.ny / 2.0 - 0.5) * p.dy
    z = (_cell_index(p.nz) - p.nz / 2.0 - 0.5) * p.dz
    return x[None, None, :], y[None, :, None], z[:, None, None]


def blast(n=192, precision=FP64, p_in=10.0, p_out=0.1, radius=0.1, cfl=0.4, b_scale=1.0,
          **kw) -> tuple:
    """Low-beta MHD blast wave: unit cube, outflow, rho = 1, p = p_out,
    B = (10/sqrt2, 10/sqrt2, 0)/sqrt(4 pi); p = p_in inside r < radius
    (cell-centre test).  HLLD, minmod, flux-CD."""
    bc = dict(bc_left=BC_OUTFLOW, bc_right=BC_OUTFLOW, bc_bottom=BC_OUTFLOW,
              bc_top=BC_OUTFLOW, bc_out=BC_OUTFLOW, bc_in=BC_OUTFLOW)
    bc.update(riemann_solver=SOLVER_HLLD, slope_limiter=LIMITER_MINMOD)
    bc.update(kw)
    p = Params(nx=n, ny=n, nz=n, precision=precision, mhd=True, cfl=cfl, **bc)
    x, y, z = _centered_coords(p)
    r = np.sqrt(x * x + y * y + z * z)
    pr = np.where(r < radius, p_in, p_out)
    b = 10.0 / math.sqrt(2.0) / math.sqrt(4.0 * math.pi) * b_scale
    sh = p.shape[:3]
    zero = np.zeros(sh)
    return p, conserved(p, 1.0, zero, zero, zero, pr, np.full(sh, b), np.full(sh, b), zero)


# ---------------------------------------------------------------------------
AMH, RG, KB = 1.66e-24, 8.3145e7, 1.38e-16   # src/constants.f90:33-35
GGRAV, MSUN = 6.67259e-8, 1.99e33             # src/constants.f90:36,39


def synthetic_cooling_table(n=101, peak=5.3):
    """Smooth synthetic log Lambda(log T): n rows on [4, 8] dex with a bump
    peaking near log T = peak (a stand-in with the shape of coronal curves)."""
    logT = [4.0 + 4.0 * i / (n - 1) for i in range(n)]
    logL = [-23.0 + 1.8 * math.exp(-((t - peak) / 0.45) ** 2) + 0.35 * (t - 4.0) / 4.0
            - 0.9 * math.exp(-((t - 4.0) / 0.12) ** 2) for t in logT]
    return logT, logL


def wind_cooling(n=256, precision=FP64, xphys=3.0e13, nsc=1.0e5, cfl=0.4, orbit=True,
                 **kw) -> tuple:
    """Hydro wind interaction with optically-thin cooling (EXO pattern).
    Star sphere r = 0.1 at the centre (rho = 1, T = 1e6 K, v_r = 200 km/s),
    planet sphere r = 0.02 at distance 0.3 (rho = 100, T = 1e4 K,
    v_r = 10 km/s), both re-imposed in every boundary call; HLLC, outflow;
    tabulated cooling (101 rows, COOL_DMC-style implicit update).
    With `orbit` the planet moves on its circular Keplerian orbit about a
    1.1 solar-mass star in the x-z plane, starting 25 degrees below the x
    axis (EXO/exoplanet.f90:83-84,106-111,143-148); otherwise it stays at
    x = 0.3.  Scalings as EXO/parameters.f90:162-170 with T0 = 1e4 K,
    density scale nsc * amh (code rho = 1 is nsc particles per cm^3)."""
    cv = 1.5
    gamma = (cv + 1.0) / cv
    T0 = 1.0e4
    rsc = xphys
    rhosc = AMH * nsc
    Tempsc = T0 * gamma
    vsc2 = gamma * RG * T0
    Psc = rhosc * vsc2
    tsc = rsc / math.sqrt(vsc2)
    vsc = math.sqrt(vsc2)
    logT, logL = synthetic_cooling_table()
    tab = table_from_log(logT, logL, tail=0.27e-26)
    star = Sphere(xc=0.0, yc=0.0, zc=0.0, radius=0.1, dens=1.0, vwind=2.0e7 / vsc,
                  tfac=1.0e6 / Tempsc)
    planet = Sphere(xc=0.3, yc=0.0, zc=0.0, radius=0.02, dens=100.0, vwind=1.0e6 / vsc,
                    tfac=1.0e4 / Tempsc)
    if orbit:
        # omega = sqrt(G M / r^3) at r = 0.3 xphys, in units of 1/tsc
        rorb = 0.3
        omega = math.sqrt(GGRAV * 1.1 * MSUN / (rorb * xphys) ** 3) * tsc
        planet = replace(planet, orbit_r=rorb, orbit_omega=omega,
                         orbit_phase=-25.0 * math.pi / 180.0)
    bc = dict(bc_left=BC_OUTFLOW, bc_right=BC_OUTFLOW, bc_bottom=BC_OUTFLOW,
              bc_top=BC_OUTFLOW, bc_out=BC_OUTFLOW, bc_in=BC_OUTFLOW)
    p = Params(nx=n, ny=n, nz=n, precision=precision, mhd=False, pmhd=False,
               riemann_solver=SOLVER_HLLC, slope_limiter=LIMITER_MINMOD, enable_flux_cd=False,
               cooling=COOL_DMC, cfl=cfl, cv=cv, Tempsc=Tempsc, Psc=Psc, tsc=tsc,
               bc_user=True, spheres=[star, planet], tab_Tmin=1.0e4, **bc, **tab, **kw)
    # ambient: the star's wind filled in as if the planet were absent
    # (EXO/user_mod.f90:71-116), density ~ r^-2 outside the star
    x = (_cell_index(n) - n // 2 + 0.5) * p.dx
    X, Y, Z = x[None, None, :], x[None, :, None], x[:, None, None]
    r = np.sqrt(X * X + Y * Y + Z * Z)
    r = np.maximum(r, 0.5 * p.dx)
    dens = star.dens * (star.radius / np.maximum(r, star.radius)) ** 2
    vx, vy, vz = (star.vwind * c / r for c in (X, Y, Z))
    pr = dens * star.tfac
    u = conserved(p, dens, np.broadcast_to(vx, p.shape[:3]), np.broadcast_to(vy, p.shape[:3]),
                  np.broadcast_to(vz, p.shape[:3]), pr)
    return p, u


def conduction_blob(n=32, precision=FP64, th_cond=1, saturation=False, mhd=False, b0=0.5,
                    xphys=3.0e17, nsc=1.0, T_hot=1.0e6, T_amb=1.0e4, radius=0.3, cfl=0.4,
                    bc=BC_OUTFLOW, ny=None, nz=None, **kw) -> tuple:
    """A hot sphere in a cool medium at rest with thermal conduction
    (src/thermal_cond.f90): T = T_amb + (T_hot - T_amb)(1 - (r/radius)^2)^2
    inside `radius` and exactly T_amb outside (so no heat crosses the walls
    while the blob is small), rho = 1.  Guacho's cgs scalings with T0 = 1e4 K
    and mu = 1 (parameters.f90:159-170); xphys is the box size in cm.  Hydro
    HLLC, or MHD HLLD + flux-CD with B = (b0, 0, 0) in code units
    (anisotropic conduction, th_cond = 2, needs mhd=True).  The ambient
    sound speed is 1 in code units: b0 = 1 would make it equal the Alfven
    speed along a purely normal field, the degenerate HLLD state in which
    the reference's star denominators vanish only approximately."""
    cv = 1.5
    gamma = (cv + 1.0) / cv
    T0, mu = 1.0e4, 1.0
    rsc = xphys
    rhosc = AMH * mu * nsc
    Tempsc = T0 * gamma
    vsc2 = gamma * RG * T0 / mu
    Psc = rhosc * vsc2
    tsc = rsc / math.sqrt(vsc2)
    bsc = math.sqrt(4.0 * math.pi * Psc)
    walls = dict(bc_left=bc, bc_right=bc, bc_bottom=bc, bc_top=bc, bc_out=bc, bc_in=bc)
    if mhd:
        phys = dict(mhd=True, riemann_solver=SOLVER_HLLD, enable_flux_cd=True)
    else:
        phys = dict(mhd=False, pmhd=False, riemann_solver=SOLVER_HLLC, enable_flux_cd=False)
    phys.update(walls)
    phys.update(kw)
    p = Params(nx=n, ny=ny or n, nz=nz or n, precision=precision, slope_limiter=LIMITER_MINMOD,
               cfl=cfl, cv=cv, Tempsc=Tempsc, Psc=Psc, tsc=tsc, th_cond=th_cond,
               tc_saturation=saturation, rsc=rsc, rhosc=rhosc, vsc2=vsc2, bsc=bsc, mu=mu, **phys)
    x, y, z = _centered_coords(p)
    r = np.sqrt(x * x + y * y + z * z)
    prof = np.clip(1.0 - (r / radius) ** 2, 0.0, None) ** 2
    T = T_amb + (T_hot - T_amb) * prof
    sh = p.shape[:3]
    rho = np.ones(sh)
    pr = rho * T / Tempsc
    zero = np.zeros(sh)
    if mhd:
        return p, conserved(p, rho, zero, zero, zero, pr, np.full(sh, b0), zero, zero)
    return p, conserved(p, rho, zero, zero, zero, pr)


def with_passives(p: Params, u: np.ndarray, *fields) -> tuple:
    """Append passive scalars (conserved values, e.g. a species density) to
    a state: npas = len(fields) extra equations after the dynamical ones."""
    sh = p.shape[:3]
    cols = [np.broadcast_to(np.asarray(f, dtype=np.float64), sh)[..., None] for f in fields]
    return p.replace(npas=p.npas + len(fields)), np.ascontiguousarray(
        np.concatenate([u] + cols, axis=-1))


def h_cooling_blob(n=24, precision=FP64, T_hot=1.0e6, T_amb=8.0e3, radius=0.3, nsc=1.0,
                   xphys=3.0e18, cfl=0.4, mhd=False, b0=0.2, **kw) -> tuple:
    """Hot ionised gas cooling into a warm neutral medium with the
    hydrogen-rate EOS and COOL_H (src/hydro_core.f90:106-111,
    src/cooling_h.f90): two passive scalars, the neutral hydrogen density
    n_HI (neutral fraction 0.999 in the warm gas, 1e-4 in the hot blob) and
    a tracer equal to the blob's density.  T = T_amb + (T_hot - T_amb)
    (1 - (r/radius)^2)^2 inside the blob, rho = 1 (nsc cm^-3), outflow
    walls, HLLC hydro or HLLD MHD with B = (b0, 0, 0); Guacho's cgs scalings
    with T0 = 1e4 K (parameters.f90:159-170)."""
    cv = 1.5
    gamma = (cv + 1.0) / cv
    T0, mu = 1.0e4, 1.0
    rhosc = AMH * mu * nsc
    Tempsc = T0 * gamma
    vsc2 = gamma * RG * T0 / mu
    Psc = rhosc * vsc2
    tsc = xphys / math.sqrt(vsc2)
    walls = dict(bc_left=BC_OUTFLOW, bc_right=BC_OUTFLOW, bc_bottom=BC_OUTFLOW,
                 bc_top=BC_OUTFLOW, bc_out=BC_OUTFLOW, bc_in=BC_OUTFLOW)
    if mhd:
        phys = dict(mhd=True, riemann_solver=SOLVER_HLLD, enable_flux_cd=True)
    else:
        phys = dict(mhd=False, pmhd=False, riemann_solver=SOLVER_HLLC, enable_flux_cd=False)
    phys.update(walls)
    phys.update(kw)
    p = Params(nx=n, ny=n, nz=n, precision=precision, slope_limiter=LIMITER_MINMOD, cfl=cfl,
               cv=cv, Tempsc=Tempsc, Psc=Psc, tsc=tsc, rsc=xphys, rhosc=rhosc, vsc2=vsc2,
               bsc=math.sqrt(4.0 * math.pi * Psc), mu=mu, eq_of_state=EOS_H_RATE,
               cooling=COOL_H, **phys)
    x, y, z = _centered_coords(p)
    r = np.sqrt(x * x + y * y + z * z)
    prof = np.clip(1.0 - (r / radius) ** 2, 0.0, None) ** 2
    T = T_amb + (T_hot - T_amb) * prof
    sh = p.shape[:3]
    rho = np.ones(sh)
    xn = np.where(prof > 0.5, 1e-4, 0.999) * np.ones(sh)
    nhi = xn * rho
    pr = (2.0 * rho - nhi) * T / Tempsc  # the H-rate EOS: n = 2 rho - n_HI
    zero = np.zeros(sh)
    if mhd:
        u = conserved(p, rho, zero, zero, zero, pr, np.full(sh, b0), zero, zero)
    else:
        u = conserved(p, rho, zero, zero, zero, pr)
    return with_passives(p, u, nhi, rho * (prof > 0))


# ---------------------------------------------------------------------------
def batch_boxes(nbox=64, seed=20260004, sizes=(32, 48, 64, 96), precision=FP64, cfl=0.4):
    """The batched set: `nbox` boxes with sizes drawn from `sizes`, each an
    Orszag-Tang box (B0 scaled by U[0.5, 2]) or a blast wave (pressure ratio
    log-uniform in [10, 1000])."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nbox):
        n = int(rng.choice(sizes))
        if rng.uniform() < 0.5:
            p, u = orszag_tang(n, n, n, precision=precision, cfl=cfl,
                               b0_scale=float(rng.uniform(0.5, 2.0)))
        else:
            ratio = 10.0 ** rng.uniform(1.0, 3.0)
            p, u = blast(n, precision=precision, p_in=0.1 * ratio, p_out=0.1, cfl=cfl)
        out.append((p, u))
    return out

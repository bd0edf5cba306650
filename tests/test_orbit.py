"""The orbiting planet of the EXO problem (EXO/exoplanet.f90:125-266): a user
boundary sphere whose centre moves on a circular orbit in the x-z plane,
XP = Rorb cos(omegap t + phi), ZP = Rorb sin(omegap t + phi), and whose cells
carry the orbital velocity (:143-148), at the time of the boundary call.

CPU: the oracle's boundary fill at several times puts the planet's cells
where the analytic orbit says, with the orbital velocity added to the wind.
GPU: the device fill at the same times matches the oracle's, and a 6-step
MHD run with dipole fields on a fast orbit matches it too (FP64 within the
last bits of sin/cos, FP32 paths in L1)."""
import math

import numpy as np
import pytest

from conftest import interior
from guacho_gb300 import params as P
from guacho_gb300 import problems

N = 64


def _centres(p):
    g = P.NGHOST
    x = (np.arange(p.nx + 2 * g) - g + 1 - p.nx // 2 + 0.5) * p.dx
    return x[None, None, :], x[None, :, None], x[:, None, None]


def _expected_planet(p, t):
    """Cells of the planet at time t and their density and momenta."""
    star, pl = p.spheres
    th = pl.orbit_omega * t + pl.orbit_phase
    xp, zp = pl.orbit_r * math.cos(th), pl.orbit_r * math.sin(th)
    vo = (-pl.orbit_omega * pl.orbit_r * math.sin(th), 0.0, pl.orbit_omega * pl.orbit_r * math.cos(th))
    X, Y, Z = _centres(p)
    xs, ys, zs = X - xp, Y - pl.yc + 0 * Z, Z - zp + 0 * X
    r = np.sqrt(xs ** 2 + ys ** 2 + zs ** 2)
    rstar = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    inside = (r <= pl.radius) & ~(rstar <= star.radius)
    mom = [pl.dens * (vo[a] + pl.vwind * c / np.where(r == 0, p.dx * 0.1, r))
           for a, c in enumerate((xs, ys, zs))]
    return inside, mom


def test_oracle_planet_follows_orbit():
    from oracle.oracle import Oracle
    p, u0 = problems.wind_cooling(N)
    assert p.spheres[1].orbit_omega > 0
    o = Oracle(p)
    o.init(u0)
    for t in (0.0, 0.05, 0.2):
        o.time = t
        o.boundaryI()
        u = o.download()
        inside, mom = _expected_planet(p, t)
        assert inside.sum() >= 4, inside.sum()
        assert np.all(u[..., 0][inside] == 100.0)
        for a in range(3):
            np.testing.assert_allclose(u[..., 1 + a][inside], mom[a][inside], rtol=1e-9, atol=1e-9)
    # the planet has moved: the cells at t = 0.2 are not those at t = 0
    assert not np.array_equal(_expected_planet(p, 0.0)[0], _expected_planet(p, 0.2)[0])


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [P.FP64, P.FP32_KAHAN, P.FP32_MIXED])
def test_gpu_boundary_fill_follows_orbit(gpu_lib, prec):
    from guacho_gb300.domain import Domain
    from oracle.oracle import Oracle
    p, u0 = problems.wind_cooling(N)
    o = Oracle(p)
    o.init(u0)
    with Domain(p.replace(precision=prec)) as d:
        d.init(u0)
        for t in (0.05, 0.2):
            o.time = t
            o.boundaryI()
            d.get_timestep(1, 10, t, 1e30)  # sets the device's time
            d.boundaryI()
            ur, ug = o.download(), d.download()
            inside, _ = _expected_planet(p, t)
            assert np.all(ug[..., 0][inside] == 100.0)
            tol = 1e-13 if prec == P.FP64 else 1e-6
            np.testing.assert_allclose(ug[inside], ur[inside], rtol=tol, atol=tol)


def _mhd_orbit():
    """The wind problem as MHD with dipole fields (HLLD, flux-CD, no cooling)
    on an orbit fast enough to cross cells within a few steps."""
    p, u0 = problems.wind_cooling(24)
    star, pl = p.spheres
    from dataclasses import replace
    sph = [replace(star, bdip=0.5), replace(pl, bdip=0.2, orbit_omega=1.0e4)]
    p8 = p.replace(mhd=True, riemann_solver=P.SOLVER_HLLD, enable_flux_cd=True,
                   cooling=P.COOL_NONE, spheres=sph)
    u8 = np.zeros(p8.shape)
    u8[..., :5] = u0
    return p8, u8


@pytest.mark.gpu
def test_gpu_mhd_orbit_run(gpu_lib):
    from test_parity_gpu import _gpu_run, _oracle_run
    p, u0 = _mhd_orbit()
    ur, dr = _oracle_run(p, u0, 6)
    assert sum(dr) * p.spheres[1].orbit_omega * p.spheres[1].orbit_r > 1.5 * p.dx
    ug, dg = _gpu_run(p, u0, 6)
    np.testing.assert_allclose(dg, dr, rtol=1e-12)
    np.testing.assert_allclose(interior(ug), interior(ur), rtol=1e-10, atol=1e-12)
    for prec in (P.FP32_KAHAN, P.FP32_MIXED):
        uf, _ = _gpu_run(p.replace(precision=prec), u0, 6)
        a, b = interior(uf), interior(ur)
        for q in (0, 4, 5, 6, 7):
            err = np.abs(a[..., q] - b[..., q]).mean() / np.abs(b[..., q]).mean()
            assert err < 1e-4, (prec, q, err)

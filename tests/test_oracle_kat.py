"""Known-answer tests that pin the CPU oracle (the reference ships no tests or
golden vectors; its own check is the min/max of div B, OT/plots.py:23-24).

  - Riemann consistency F(U, U) = prim2f(U) for every solver, both regimes
  - mirror symmetry of the interface flux
  - limiter values from the formulas of src/hydro_core.f90:735-796
  - u2prim / prim2u round trip, pressure and density floors
  - conservation of mass, momentum, energy and B with periodic walls
  - centred div B preserved to round-off by flux-CD, grows without it
  - x <-> y transposition symmetry of a whole step
  - cooling-table lookup against the reference's row-index formula
"""
import math

import numpy as np
import pytest

from conftest import interior
from guacho_gb300 import params as P
from guacho_gb300 import problems
from oracle import oracle as O

rng = np.random.default_rng(1234)


def _mhd():
    return problems.orszag_tang(8, 8, 4)[0]


def _hydro(**kw):
    kw.setdefault("riemann_solver", P.SOLVER_HLLC)
    return P.Params(nx=8, ny=8, nz=8, mhd=False, enable_flux_cd=False, **kw)


def _rand_prim(neq, mach=0.5, bmag=1.0):
    pr = np.empty(neq)
    pr[0] = rng.uniform(0.5, 2.0)
    pr[1:4] = rng.uniform(-mach, mach, 3)
    pr[4] = rng.uniform(0.5, 2.0)
    if neq == 8:
        pr[5:8] = rng.uniform(-bmag, bmag, 3)
    return pr


SOLVERS = [
    ("hlld", lambda: _mhd(), 8),
    ("hlle", lambda: _mhd().replace(riemann_solver=P.SOLVER_HLLE), 8),
    ("hllc", lambda: _hydro(), 5),
    ("hll", lambda: _hydro(riemann_solver=P.SOLVER_HLL), 5),
    ("hllc_pmhd", lambda: _hydro(pmhd=True), 8),
]


@pytest.mark.parametrize("name,make,neq", SOLVERS)
@pytest.mark.parametrize("mach", [0.3, 3.0])
def test_riemann_consistency(name, make, neq, mach):
    p = make()
    for _ in range(50):
        u = _rand_prim(neq, mach=mach)
        f, err = O.riemann(p, u, u)
        assert err == 0
        np.testing.assert_allclose(f, O.prim2f(p, u), rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("name,make,neq", SOLVERS)
def test_riemann_mirror_symmetry(name, make, neq):
    """Reflecting x (v_x, B_x -> -v_x, -B_x) and swapping L/R negates every
    flux component but the x-momentum one."""
    p = make()
    sign = np.array([-1, 1, -1, -1, -1, 1, -1, -1])[:neq]
    flip = np.array([1, -1, 1, 1, 1, -1, 1, 1])[:neq]
    for _ in range(50):
        l, r = _rand_prim(neq), _rand_prim(neq)
        f, _ = O.riemann(p, l, r)
        g, _ = O.riemann(p, r * flip, l * flip)
        if neq == 8:
            f[5] = g[5] = 0.0  # normal-field flux (zero, or unused with flux-CD)
        np.testing.assert_allclose(g, sign * f, rtol=1e-10, atol=1e-12)


def test_hlld_star_regions_reached():
    """Strong B jumps hit UL*/UR*/UL**/UR** branches and stay finite."""
    p = _mhd()
    seen = set()
    for _ in range(400):
        l = _rand_prim(8, mach=1.0, bmag=2.0)
        r = _rand_prim(8, mach=1.0, bmag=2.0)
        f, err = O.riemann(p, l, r)
        assert err == 0 and np.all(np.isfinite(f))
        seen.add(tuple(np.sign(f[:1])))
    assert len(seen) == 2


@pytest.mark.parametrize("lim,a,b,want", [
    (P.LIMITER_NO_AVERAGE, 1.0, 2.0, 0.0),
    (P.LIMITER_NO_LIMIT, 1.0, 2.0, 1.5),
    (P.LIMITER_MINMOD, 1.0, 2.0, 1.0),
    (P.LIMITER_MINMOD, -1.0, -3.0, -1.0),
    (P.LIMITER_MINMOD, 1.0, -2.0, 0.0),
    (P.LIMITER_VAN_LEER, 1.0, 3.0, 1.2),
    (P.LIMITER_VAN_LEER, 1.0, -3.0, 0.0),
    (P.LIMITER_VAN_ALBADA, 1.0, 1.0, (1 * (1 + 1e-7) + 1 * (1 + 1e-7)) / (2 + 1e-7)),
    (P.LIMITER_UMIST, 1.0, 2.0, 1.25),
    (P.LIMITER_WOODWARD, 1.0, 2.0, 1.5),
    (P.LIMITER_WOODWARD, 1.0, 5.0, 2.0),
    (P.LIMITER_SUPERBEE, 1.0, 2.0, 2.0),
    (P.LIMITER_SUPERBEE, 1.0, 0.25, 0.5),
])
def test_limiter_values(lim, a, b, want):
    """pl = pl + 0.5*average(pl-pll, pr-pl): with pll=0, pl=a, pr=a+b."""
    p = _mhd().replace(slope_limiter=lim)
    pll = np.zeros(8)
    pl = np.full(8, a)
    pr = np.full(8, a + b)
    prr = np.full(8, a + b + b)
    l2, _ = O.limiter(p, pll, pl, pr, prr)
    assert l2[0] == pytest.approx(a + 0.5 * want, rel=1e-14, abs=1e-15)


def test_u2prim_roundtrip_and_floors():
    p = _mhd()
    for _ in range(50):
        pr = _rand_prim(8)
        u = O.prim2u(p, pr)
        back, T = O.u2prim(p, u)
        np.testing.assert_allclose(back, pr, rtol=1e-12)
        assert T == pytest.approx(pr[4] / pr[0] * p.Tempsc, rel=1e-12)
    # floors of src/hydro_core.f90:62,78
    u = np.array([0.0, 0, 0, 0, -1.0, 0, 0, 0])
    back, _ = O.u2prim(p, u)
    assert back[0] == 1e-15 and back[4] == 1e-16


def _run_oracle(p, u0, steps):
    o = O.Oracle(p)
    o.init(u0)
    t = 0.0
    for it in range(1, steps + 1):
        dt, _ = o.get_timestep(it, 10, t, 1e30)
        o.tstep(dt)
        t += dt
    assert o.error == 0
    return o


def test_conservation_periodic():
    p, u0 = problems.turbulence(16, seed=3)
    o = _run_oracle(p, u0, 10)
    s0 = interior(u0).sum(axis=(0, 1, 2))
    s1 = interior(o.download()).sum(axis=(0, 1, 2))
    scale = np.abs(interior(u0)).sum(axis=(0, 1, 2))
    assert np.all(np.abs(s1 - s0) <= 1e-13 * scale + 1e-13)


def _divb(p, u):
    bx, by, bz = u[..., 5], u[..., 6], u[..., 7]
    return ((bx[2:-2, 2:-2, 3:-1] - bx[2:-2, 2:-2, 1:-3]) / (2 * p.dx)
            + (by[2:-2, 3:-1, 2:-2] - by[2:-2, 1:-3, 2:-2]) / (2 * p.dy)
            + (bz[3:-1, 2:-2, 2:-2] - bz[1:-3, 2:-2, 2:-2]) / (2 * p.dz))


def test_flux_cd_keeps_divb_roundoff():
    p, u0 = problems.turbulence(16, seed=4)
    d0 = np.abs(_divb(p, u0)).max()
    o = _run_oracle(p, u0, 10)
    d1 = np.abs(o.divb()).max()
    np.testing.assert_allclose(o.divb(), _divb(p, o.download()), rtol=0, atol=1e-12)
    assert d0 < 1e-11 and d1 < 1e-11
    o2 = _run_oracle(p.replace(enable_flux_cd=False), u0, 10)
    assert np.abs(o2.divb()).max() > 1e3 * max(d1, 1e-15)


def test_transpose_symmetry():
    """Evolving the x<->y transposed state gives the transposed result."""
    p, u0 = problems.turbulence(12, seed=6)
    ut = np.ascontiguousarray(np.swapaxes(u0, 1, 2))[..., [0, 2, 1, 3, 4, 6, 5, 7]]
    a = _run_oracle(p, u0, 4).download()
    b = _run_oracle(p, ut, 4).download()
    bt = np.swapaxes(b, 1, 2)[..., [0, 2, 1, 3, 4, 6, 5, 7]]
    np.testing.assert_allclose(interior(bt), interior(a), rtol=1e-11, atol=1e-13)


def test_cooling_row_index_matches_reference_formula():
    """Row index int(log10(T)*10)-39 (src/cooling_dmc.f90:98) for the 0.1-dex
    table, and linear interpolation between its rows."""
    logT = [4.0 + 0.1 * i for i in range(41)]
    logL = [-21.0 - 0.01 * i for i in range(41)]
    p = _hydro(cooling=P.COOL_DMC, **P.table_from_log(logT, logL, tail=0.27e-26))
    assert p.tab_inv_dlog == 10.0 and p.tab_i0 == 40
    for T in np.logspace(4.0, 7.99, 997):
        if1 = int(math.log10(T) * 10) - 39          # 1-based, reference formula
        T0, T1 = 10.0 ** logT[if1 - 1], 10.0 ** logT[if1]
        c0, c1 = 10.0 ** logL[if1 - 1], 10.0 ** logL[if1]
        want = (c1 - c0) * (T - T0) / (T1 - T0) + c0
        assert O.cooltab(p, T) == want
    assert O.cooltab(p, 4e8) == 0.27e-26 * math.sqrt(4e8)

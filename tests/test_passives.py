"""Passive scalars, the hydrogen-rate EOS and COOL_H (src/hydro_core.f90:86-125,
src/hlld.f90:149-153, src/hllc.f90:95-126, src/flux_cd_module.f90:304-308,
src/cooling_h.f90): known answers of the oracle (CPU), then the GB300 path
against the oracle (GPU).

The reference ships no test for these.  The oracle is pinned by:
  - passives do not act on the dynamics: a run with two passive scalars has
    bitwise the dynamical fields of the same run without them;
  - a passive scalar proportional to the density stays proportional to it
    (its fluxes are the mass fluxes times the constant in every solver and
    star region, and both limiters are homogeneous);
  - the H-rate EOS temperature T = max(1, p/(2 rho - n_HI) Tempsc) and its
    pressure floor;
  - COOL_H leaves gas at or below 1e4 K at its temperature (ALOSS = 0 there),
    keeps the neutral fraction in [0, 0.9999], conserves mass and cools the
    hot gas."""
import numpy as np
import pytest

from guacho_gb300 import params as P
from guacho_gb300 import problems
from oracle import oracle as O

INT = (slice(2, -2),) * 3


def _ot_passives(n=16, nz=4, **kw):
    p, u = problems.orszag_tang(n, n, nz, **kw)
    rho = u[..., 0]
    x = np.linspace(0.0, 1.0, u.shape[2])[None, None, :]
    return problems.with_passives(p, u, 0.3 * rho, 1.0 + 0.5 * np.sin(2 * np.pi * x) * rho / rho)


def _hydro_passives(n=16):
    p, u = problems.conduction_blob(n, th_cond=P.TC_OFF)  # HLLC hydro, hot blob
    return problems.with_passives(p, u, 0.7 * u[..., 0], np.ones(u.shape[:3]))


@pytest.mark.parametrize("make", [_ot_passives, _hydro_passives])
def test_passives_leave_dynamics_bitwise(make):
    pp, up = make()
    p = pp.replace(npas=0)
    u = np.ascontiguousarray(up[..., :p.neq])
    a, b = O.Oracle(p), O.Oracle(pp)
    a.init(u)
    b.init(up)
    a.run(0.02, 1e30)
    b.run(0.02, 1e30)
    assert a.iter == b.iter > 3
    assert np.array_equal(a.download(), b.download()[..., :p.neq])


@pytest.mark.parametrize("make", [_ot_passives, _hydro_passives])
def test_passive_proportional_to_density_stays(make):
    pp, up = make()
    o = O.Oracle(pp)
    o.init(up)
    o.run(0.02, 1e30)
    u = o.download()[INT]
    c0 = up[INT][..., pp.neqdyn] / up[INT][..., 0]
    c1 = u[..., pp.neqdyn] / u[..., 0]
    assert np.abs(c1 - c0).max() < 1e-12


def test_h_rate_eos_temperature():
    p, u = problems.h_cooling_blob(8)
    nd = p.neqdyn
    for i in range(4):
        cell = u[2 + i, 3, 4].copy()
        prim, T = O.u2prim(p, cell)
        dentot = 2.0 * cell[0] - cell[nd]
        pth = (cell[4] - 0.5 * (cell[1] ** 2 + cell[2] ** 2 + cell[3] ** 2) / cell[0]) / p.cv
        assert T == pytest.approx(max(1.0, pth / dentot * p.Tempsc), rel=1e-14)
        assert prim[4] == pytest.approx(dentot * T / p.Tempsc, rel=1e-14)
        assert np.array_equal(prim[nd:], cell[nd:])
    # the floor: a cold cell's pressure is raised to T = 1 K
    cold = u[2, 2, 2].copy()
    cold[4] = 1e-30
    prim, T = O.u2prim(p, cold)
    assert T == 1.0 and prim[4] == (2.0 * cold[0] - cold[nd]) * 1.0 / p.Tempsc


def test_cool_h_known_answers():
    p, u = problems.h_cooling_blob(24)
    nd = p.neqdyn
    o = O.Oracle(p)
    o.init(u)
    T0 = o.temp()[INT].copy()
    dt, _ = o.get_timestep(20, 10, 0.0, 1e30)
    o.tstep(dt)
    u1 = o.download()[INT]
    T1 = o.temp()[INT]
    xn = u1[..., nd] / u1[..., 0]
    assert np.all(xn >= 0.0) and np.all(xn <= 0.9999 + 1e-15)
    assert abs(u1[..., 0].sum() - u[INT][..., 0].sum()) <= 1e-12 * u[INT][..., 0].sum()
    hot = T0 > 5e5
    assert T1[hot].max() < T0[hot].max()          # the hot gas cools
    # no loss below 1e4 K: the corners, out of the blob's reach in one step,
    # keep their temperature while their neutral fraction relaxes
    x = (np.arange(p.nx) - p.nx / 2 + 0.5) * p.dx
    r = np.sqrt(x[None, None, :] ** 2 + x[None, :, None] ** 2 + x[:, None, None] ** 2)
    far = r > 0.65
    assert far.sum() > 100
    assert np.allclose(T1[far], T0[far], rtol=1e-12, atol=0.0)
    assert not np.allclose(u1[far][..., nd], u[INT][far][..., nd], rtol=1e-12, atol=0.0)


# ---------------------------------------------------------------------------
def _gpu_vs_oracle(p, u, steps, it0=1):
    from guacho_gb300.domain import Domain
    o = O.Oracle(p.replace(precision=P.FP64))
    o.init(u)
    with Domain(p) as d:
        d.init(u)
        t = 0.0
        for it in range(it0, it0 + steps):
            dto, _ = o.get_timestep(it, 10, t, 1e30)
            dtg, _ = d.get_timestep(it, 10, t, 1e30)
            o.tstep(dto)
            d.tstep(dtg)
            t += dto
        ug = d.download()
    return ug, o.download(), dtg / dto - 1.0


@pytest.mark.gpu
@pytest.mark.parametrize("make", [_ot_passives, _hydro_passives])
def test_gpu_fp64_passives_bitwise(gpu_lib, make):
    p, u = make()
    ug, uo, ddt = _gpu_vs_oracle(p, u, 4)
    assert ddt == 0.0
    assert np.array_equal(ug[INT], uo[INT])


@pytest.mark.gpu
@pytest.mark.parametrize("mhd", [False, True])
def test_gpu_fp64_h_rate_cool_h(gpu_lib, mhd):
    """exp/log/pow of COOL_H come from CUDA's libm on the device and glibc
    in the oracle: agreement to ~1e-12 of each field's scale."""
    p, u = problems.h_cooling_blob(16, mhd=mhd)
    ug, uo, ddt = _gpu_vs_oracle(p, u, 3, it0=11)
    assert abs(ddt) < 1e-11
    a, b = ug[INT].reshape(-1, p.neq), uo[INT].reshape(-1, p.neq)
    scale = np.maximum(np.abs(b).max(axis=0), 1e-300)
    assert np.all(np.abs(a - b).max(axis=0) <= 1e-10 * scale)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [P.FP32_MIXED, P.FP32_KAHAN])
@pytest.mark.parametrize("case", ["ot", "hydro", "h_cool"])
def test_gpu_fp32_passives(gpu_lib, prec, case):
    """FP32 paths with passive scalars (and COOL_H): relative L1 of every
    field within 1e-4 of the FP64 oracle after 4 steps."""
    if case == "ot":
        p, u = _ot_passives()
        it0 = 1
    elif case == "hydro":
        p, u = _hydro_passives()
        it0 = 1
    else:
        p, u = problems.h_cooling_blob(16)
        it0 = 11
    ug, uo, _ = _gpu_vs_oracle(p.replace(precision=prec), u, 4, it0=it0)
    a, b = ug[INT].reshape(-1, p.neq), uo[INT].reshape(-1, p.neq)
    l1 = np.abs(a - b).mean(axis=0) / np.maximum(np.abs(b).mean(axis=0), 1e-300)
    for q in range(p.neq):
        if np.abs(b[:, q]).max() > 1e-8:   # skip fields that stay at zero
            assert l1[q] < 1e-4, (q, l1)

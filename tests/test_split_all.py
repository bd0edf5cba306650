"""The split solver SOLVER_HLLE_SPLIT_ALL (src/hlle_split_all.f90, the split
branches of src/hydro_core.f90): the state is a fluctuation over a background
primit0 (src/globals.f90:42) that the caller supplies.  The reference
allocates primit0 but never sets it; here it is zero until set.

The reference ships no test for it.  The oracle's restatement is pinned by:
  - with a zero background the split expressions reduce to the plain ones,
    so a run with SPLIT_ALL equals the same run with HLLE bit for bit (the
    plain u2prim's floors are not reached);
  - a uniform background with no fluctuation stays at rest exactly;
  - a uniform fluctuation over a uniform background stays uniform, and the
    interface flux is independent of how the total state is split between
    background and fluctuation for the mass flux.
The GB300 FP64 path then matches the oracle bitwise with a non-uniform
background (GPU)."""
import numpy as np
import pytest

from guacho_gb300 import params as P
from guacho_gb300 import problems
from oracle import oracle as O

INT = (slice(2, -2),) * 3


def _ot(n=16, nz=4, **kw):
    return problems.orszag_tang(n, n, nz, riemann_solver=P.SOLVER_HLLE,
                                slope_limiter=P.LIMITER_VAN_LEER, **kw)


def _run(p, u, steps, prim0=None):
    o = O.Oracle(p)
    if prim0 is not None:
        o.set_background(prim0)
    o.init(u)
    t = 0.0
    dts = []
    for it in range(1, steps + 1):
        dt, _ = o.get_timestep(it, 10, t, 1e30)
        o.tstep(dt)
        t += dt
        dts.append(dt)
    return o.download(), dts


def test_zero_background_equals_hlle_bitwise():
    p, u = _ot()
    a, da = _run(p, u, 6)
    b, db = _run(p.replace(riemann_solver=P.SOLVER_HLLE_SPLIT_ALL), u, 6)
    assert da == db
    assert np.array_equal(a[INT], b[INT])


def test_interface_zero_background_equals_hlle():
    p = _ot()[0]
    rng = np.random.default_rng(3)
    zero = np.zeros(8)
    for _ in range(20):
        pl = np.r_[rng.uniform(0.5, 2), rng.normal(0, 1, 3), rng.uniform(0.2, 2), rng.normal(0, 1, 3)]
        pr = np.r_[rng.uniform(0.5, 2), rng.normal(0, 1, 3), rng.uniform(0.2, 2), rng.normal(0, 1, 3)]
        a, _ = O.riemann(p, pl, pr)
        b = O.riemann_split(p.replace(riemann_solver=P.SOLVER_HLLE_SPLIT_ALL), pl, pr, zero, zero)
        assert np.array_equal(a, b)


def _background(p, rho0=1.0, p0=0.5, b0=(0.3, 0.1, 0.0), vary=0.0):
    sh = p.shape
    prim0 = np.zeros(sh)
    z, y, x = np.meshgrid(*[np.linspace(0, 2 * np.pi, s) for s in sh[:3]], indexing="ij")
    prim0[..., 0] = rho0 * (1 + vary * np.sin(x) * np.cos(y))
    prim0[..., 4] = p0 * (1 + vary * np.cos(x + z))
    prim0[..., 5] = b0[0]
    prim0[..., 6] = b0[1] * (1 + vary * np.sin(y))
    prim0[..., 7] = b0[2]
    return prim0


def test_background_alone_stays_at_rest():
    p, _ = _ot()
    ps = p.replace(riemann_solver=P.SOLVER_HLLE_SPLIT_ALL)
    u0 = np.zeros(p.shape)
    got, _ = _run(ps, u0, 4, _background(p))
    assert np.array_equal(got[INT], u0[INT])


def test_uniform_fluctuation_stays_uniform():
    p, _ = _ot()
    ps = p.replace(riemann_solver=P.SOLVER_HLLE_SPLIT_ALL)
    u0 = np.zeros(p.shape)
    u0[..., 0] = 0.2      # density fluctuation
    u0[..., 1] = 0.3      # momentum
    u0[..., 4] = 0.4      # energy fluctuation
    u0[..., 6] = 0.05     # B_y fluctuation
    got, _ = _run(ps, u0, 4, _background(p))
    g = got[INT].reshape(-1, p.neq)
    assert np.all(np.abs(g - g[0]).max(axis=0) <= 1e-14 * np.maximum(np.abs(g[0]), 1.0))


def test_mass_flux_depends_on_the_total_density_only():
    """F_rho = (rho + rho0) v in every region of the split solver."""
    p = _ot()[0].replace(riemann_solver=P.SOLVER_HLLE_SPLIT_ALL)
    pl = np.array([0.3, 0.4, 0.1, -0.2, 0.2, 0.5, 0.1, 0.0])
    pr = np.array([0.1, 0.4, 0.1, -0.2, 0.2, 0.5, 0.1, 0.0])
    bg = np.array([1.0, 0.0, 0.0, 0.0, 0.5, 0.0, 0.0, 0.0])
    f = O.riemann_split(p, pl, pr, bg, bg)
    # the same total densities split differently: rho 1.3 | 1.1 as 0.8 + 0.5
    bg2 = bg.copy(); bg2[0] = 0.5
    pl2, pr2 = pl.copy(), pr.copy(); pl2[0] += 0.5; pr2[0] += 0.5
    f2 = O.riemann_split(p, pl2, pr2, bg2, bg2)
    assert f[0] == pytest.approx(f2[0], rel=1e-14)


# ---------------------------------------------------------------------------
@pytest.mark.gpu
@pytest.mark.parametrize("flux_cd", [True, False])
def test_gpu_fp64_split_all_bitwise(gpu_lib, flux_cd):
    from guacho_gb300.domain import Domain
    p, u = _ot(20, 6, enable_flux_cd=flux_cd)
    p = p.replace(riemann_solver=P.SOLVER_HLLE_SPLIT_ALL)
    prim0 = _background(p, vary=0.2)
    uo, do = _run(p, u, 6, prim0)
    with Domain(p) as d:
        d.set_background(prim0)
        d.init(u)
        t = 0.0
        dg = []
        for it in range(1, 7):
            dt, _ = d.get_timestep(it, 10, t, 1e30)
            d.tstep(dt)
            t += dt
            dg.append(dt)
        ug = d.download()
    assert dg == do
    assert np.array_equal(ug[INT], uo[INT])


def test_bin_output_writes_the_total_state(tmp_path):
    """src/Out_BIN_Module.f90:144-158: rho + rho0, momenta, E + cv p0 +
    B0^2/2 and B + B0 for the split solver."""
    from guacho_gb300 import binio
    p, u = _ot(8, 4)
    p = p.replace(riemann_solver=P.SOLVER_HLLE_SPLIT_ALL)
    prim0 = _background(p, vary=0.1)
    path = tmp_path / "points000.000.bin"
    binio.write_bin(path, u, p, prim0=prim0)
    _, got = binio.read_bin(path)
    q = prim0
    want = u.copy()
    want[..., 0] += q[..., 0]
    want[..., 4] = u[..., 4] + p.cv * q[..., 4] + 0.5 * (q[..., 5] ** 2 + q[..., 6] ** 2 + q[..., 7] ** 2)
    want[..., 5:8] += q[..., 5:8]
    assert np.array_equal(got[..., 1:4], u[..., 1:4])
    np.testing.assert_allclose(got, want, rtol=1e-15, atol=0)

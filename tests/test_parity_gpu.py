"""Parity of the CUDA path against the CPU oracle, through the C ABI.

FP64 (plain drop-in): bitwise equal to the oracle wherever every operation is
IEEE-exact (no exp/log10/pow on the path), step after step; otherwise within
1e-12 relative.  FP32-mixed: per-field relative L1 within 1e-4 of the FP64
oracle (the bar set for the mixed path), div B at round-off.
"""
import numpy as np
import pytest

from conftest import interior
from guacho_gb300 import params as P
from guacho_gb300 import problems

pytestmark = pytest.mark.gpu


def _oracle_run(p, u0, steps, n_iter=10, dtprint=1e30):
    from oracle.oracle import Oracle
    o = Oracle(p)
    o.init(u0)
    dts = []
    t, tprint = 0.0, dtprint
    for it in range(1, steps + 1):
        dt, dump = o.get_timestep(it, n_iter, t, tprint)
        o.tstep(dt)
        t = t + dt
        dts.append(dt)
    assert o.error == 0
    return o.download(), dts


def _gpu_run(p, u0, steps, n_iter=10, dtprint=1e30):
    from guacho_gb300.domain import Domain
    with Domain(p) as d:
        d.init(u0)
        dts = []
        t, tprint = 0.0, dtprint
        for it in range(1, steps + 1):
            dt, dump = d.get_timestep(it, n_iter, t, tprint)
            d.tstep(dt)
            t = t + dt
            dts.append(dt)
        return d.download(), dts


def _hydro_state(n, seed=7, closed=False, **kw):
    """A smooth random hydro state (neq = 5) on an n^3 box."""
    kw.setdefault("riemann_solver", P.SOLVER_HLLC)
    p = P.Params(nx=n, ny=n, nz=n, mhd=False, enable_flux_cd=False, cfl=0.3, **kw)
    if closed:
        p = p.replace(**{k: P.BC_CLOSED for k in
                         ("bc_left", "bc_right", "bc_bottom", "bc_top", "bc_out", "bc_in")})
    rng = np.random.default_rng(seed)
    sh = p.shape[:3]
    z, y, x = np.meshgrid(*[np.linspace(0, 2 * np.pi, s) for s in sh], indexing="ij")
    rho = 1.0 + 0.3 * np.sin(x + rng.uniform()) * np.cos(y)
    vx = 0.5 * np.sin(y + z)
    vy = 0.4 * np.cos(x)
    vz = 0.3 * np.sin(x + y)
    pr = 1.0 + 0.2 * np.cos(z + rng.uniform())
    return p, problems.conserved(p, rho, vx, vy, vz, pr)


def _pmhd_state(n):
    p, u = _hydro_state(n, seed=3)
    p = p.replace(pmhd=True)
    sh = p.shape[:3]
    u8 = np.zeros(p.shape)
    u8[..., :5] = u
    z, y, x = np.meshgrid(*[np.linspace(0, 2 * np.pi, s) for s in sh], indexing="ij")
    u8[..., 5] = 0.1 * np.sin(y)
    u8[..., 6] = 0.2 * np.cos(z)
    u8[..., 7] = 0.05 * np.sin(x)
    return p, u8


CASES = {
    "ot_hlld_minmod": lambda: problems.orszag_tang(32, 32, 4),
    "ot_hlld_nonsquare": lambda: problems.orszag_tang(40, 24, 6),
    "blast_hlld_outflow": lambda: problems.blast(16, p_in=1.0),
    "blast_hlld_closed": lambda: problems.blast(
        16, p_in=1.0, bc_left=P.BC_CLOSED, bc_right=P.BC_CLOSED, bc_bottom=P.BC_CLOSED,
        bc_top=P.BC_CLOSED, bc_out=P.BC_CLOSED, bc_in=P.BC_CLOSED),
    "ot_hlle_vanleer": lambda: problems.orszag_tang(
        24, 24, 4, riemann_solver=P.SOLVER_HLLE, slope_limiter=P.LIMITER_VAN_LEER),
    "ot_no_flux_cd": lambda: problems.orszag_tang(24, 24, 4, enable_flux_cd=False),
    "ot_eight_wave": lambda: problems.orszag_tang(24, 24, 4, enable_flux_cd=False,
                                                  eight_wave=True),
    "ot_eta": lambda: problems.orszag_tang(24, 24, 4, eta=0.01),
    "ot_eight_wave_cd": lambda: problems.orszag_tang(24, 24, 4, eight_wave=True),
    "turbulence_16": lambda: problems.turbulence(16, seed=5),
    "hydro_hllc_periodic": lambda: _hydro_state(12),
    "hydro_hllc_closed": lambda: _hydro_state(12, closed=True),
    "hydro_hll_outflow": lambda: _hydro_state(
        12, riemann_solver=P.SOLVER_HLL, bc_left=P.BC_OUTFLOW, bc_right=P.BC_OUTFLOW),
    "pmhd_hllc": lambda: _pmhd_state(12),
    "wind_cooling_24": lambda: problems.wind_cooling(24),
    # partial 32 x 8 tiles in x and y and a partial z chunk; walls on every
    # side of partial tiles; the smallest box whose second ghost layer still
    # maps to interior cells
    "ot_ragged": lambda: problems.orszag_tang(37, 19, 11),
    "ot_ragged_closed": lambda: problems.orszag_tang(
        37, 19, 11, bc_left=P.BC_CLOSED, bc_right=P.BC_OUTFLOW, bc_bottom=P.BC_OUTFLOW,
        bc_top=P.BC_CLOSED, bc_out=P.BC_CLOSED, bc_in=P.BC_OUTFLOW),
    "ot_tiny": lambda: problems.orszag_tang(2, 3, 2),
    # one-cell-thick boxes: the second ghost layer of that axis is filled
    # axis by axis, as the reference's array copies leave it
    "ot_2d_nz1": lambda: problems.orszag_tang(16, 16, 1),
    "ot_thin_y": lambda: problems.orszag_tang(16, 1, 8),
    "ot_thin_x": lambda: problems.orszag_tang(1, 12, 6),
}
for lim in range(-1, 7):
    CASES[f"ot_limiter_{lim}"] = (lambda l=lim: problems.orszag_tang(16, 16, 4,
                                                                       slope_limiter=l))


@pytest.mark.parametrize("name", sorted(k for k in CASES if not k.startswith("wind")))
def test_fp64_bitwise(gpu_lib, name):
    p, u0 = CASES[name]()
    steps = 6
    ur, dr = _oracle_run(p, u0, steps)
    ug, dg = _gpu_run(p, u0, steps)
    assert dr == dg, f"dt sequences differ: {dr} vs {dg}"
    a, b = interior(ug), interior(ur)
    bad = np.argwhere(a != b)
    assert bad.size == 0, (f"{len(bad)} interior values differ, first at {bad[0]}: "
                           f"{a[tuple(bad[0])]!r} vs {b[tuple(bad[0])]!r}")


def test_c1_orszag_tang_to_t05(gpu_lib):
    """The CPU-runnable configuration: Orszag-Tang 128x128x4, HLLD, minmod,
    flux-CD, CFL 0.4, run to t = 0.5 with outputs every 0.1 through the loop
    of src/main.f90:94-125 (one step past tmax included).  FP64 device loop
    against the oracle: same step count, same time, bitwise equal state."""
    from guacho_gb300.domain import Domain
    from oracle.oracle import Oracle
    p, u0 = problems.orszag_tang(128, 128, 4, cfl=0.4)
    o = Oracle(p)
    o.init(u0)
    no = o.run(0.5, 0.1)
    with Domain(p) as d:
        d.init(u0)
        nd = d.run(0.5, 0.1)
        assert nd == no and d.time == o.time and d.iter == o.iter
        ug = d.download()
    uo = o.download()
    assert np.array_equal(interior(ug), interior(uo))
    assert np.abs(o.divb()).max() < 1e-10


@pytest.mark.parametrize("prec", [P.FP32_MIXED, P.FP32_KAHAN])
def test_low_beta_blast_pressure_floor(gpu_lib, prec):
    """Low-beta blast (beta ~ 0.025, pressure ratio 100): the FP32 paths
    keep the pressure recovery clear of the floor and within 1e-4 of FP64."""
    from guacho_gb300.domain import Domain
    p, u0 = problems.blast(32, p_in=10.0, p_out=0.1)
    ur, _ = _oracle_run(p, u0, 15)
    with Domain(p.replace(precision=prec)) as d:
        d.init(u0)
        d.run(1e30, 1e30, max_steps=15)
        floors, err = d.step_info()
        ug = d.download()
    assert err == 0 and floors == 0
    fr, fg = _prims(p, ur), _prims(p, ug)
    for k in ("rho", "p"):
        assert np.abs(fg[k] - fr[k]).mean() / np.abs(fr[k]).mean() < 1e-4


def test_fp64_long_run_ot(gpu_lib):
    """OT 64x64x4 over 60 steps: still bitwise."""
    p, u0 = problems.orszag_tang(64, 64, 4)
    ur, dr = _oracle_run(p, u0, 60)
    ug, dg = _gpu_run(p, u0, 60)
    assert dr == dg
    assert np.array_equal(interior(ug), interior(ur))


def test_fp64_gravity_sources(gpu_lib):
    """User point-mass sources go through pow(): equal within 1e-12."""
    p, u0 = _hydro_state(12, seed=11)
    p = p.replace(user_source_terms=True, grav=[(0.01, 0.0, 0.0, 0.0), (0.002, 0.3, 0.0, 0.1)])
    ur, _ = _oracle_run(p, u0, 5)
    ug, _ = _gpu_run(p, u0, 5)
    np.testing.assert_allclose(interior(ug), interior(ur), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("prec", [P.FP32_MIXED, P.FP32_KAHAN])
def test_fp32_gravity_sources(gpu_lib, prec):
    """User point masses on the FP32 paths (FP32 positions and masses, r^3 as
    r^2 sqrt(r^2), dt*s added in FP32 to the pairs): relative L1 of rho, p
    and the momenta within 1e-4 of the FP64 oracle after 20 steps."""
    p, u0 = _hydro_state(12, seed=11)
    p = p.replace(user_source_terms=True, grav=[(0.01, 0.0, 0.0, 0.0), (0.002, 0.3, 0.0, 0.1)])
    ur, dr = _oracle_run(p, u0, 20)
    ug, dg = _gpu_run(p.replace(precision=prec), u0, 20)
    np.testing.assert_allclose(dg, dr, rtol=1e-5)
    a, b = interior(ug), interior(ur)
    for q in range(5):
        err = np.abs(a[..., q] - b[..., q]).mean() / np.abs(b[..., q]).mean()
        assert err < 1e-4, (q, err)


def test_fp64_wind_cooling(gpu_lib):
    """Spheres + tabulated cooling (exp/log10 on the path): within 1e-12."""
    p, u0 = problems.wind_cooling(24)
    ur, dr = _oracle_run(p, u0, 5)
    ug, dg = _gpu_run(p, u0, 5)
    np.testing.assert_allclose(dg, dr, rtol=1e-12)
    np.testing.assert_allclose(interior(ug), interior(ur), rtol=1e-11, atol=1e-14)


def _rel_l1(a, b):
    return np.abs(a - b).mean() / np.abs(b).mean()


def _prims(p, u):
    """rho, p, vx, vy, vz, Bx, By, Bz of the interior (FP64)."""
    ui = interior(u)
    rho = ui[..., 0]
    v = ui[..., 1:4] / rho[..., None]
    e = ui[..., 4] - 0.5 * rho * (v ** 2).sum(-1)
    if p.mhd:
        e = e - 0.5 * (ui[..., 5:8] ** 2).sum(-1)
    out = {"rho": rho, "p": e / p.cv, "vx": v[..., 0], "vy": v[..., 1], "vz": v[..., 2]}
    if p.bfield:
        out.update(Bx=ui[..., 5], By=ui[..., 6], Bz=ui[..., 7])
    return out


@pytest.mark.parametrize("prec", [P.FP32_MIXED, P.FP32_KAHAN])
@pytest.mark.parametrize("name", ["ot_hlld_minmod", "blast_hlld_outflow", "turbulence_16",
                                  "hydro_hllc_periodic", "ot_hlle_vanleer", "ot_limiter_4",
                                  "hydro_hllc_closed", "ot_eta", "ot_eight_wave",
                                  "wind_cooling_24", "ot_ragged", "ot_ragged_closed",
                                  "ot_eight_wave_cd"])
def test_fp32_l1(gpu_lib, name, prec):
    """FP32-mixed (FP64 u) and FP32 + Kahan pairs against the FP64 oracle."""
    p, u0 = CASES[name]()
    steps = 20
    ur, dr = _oracle_run(p, u0, steps)
    ug, dg = _gpu_run(p.replace(precision=prec), u0, steps)
    np.testing.assert_allclose(dg, dr, rtol=1e-5)
    fr, fg = _prims(p, ur), _prims(p, ug)
    # relative L1 per field; B components are normalised by the mean |B| so
    # that a component that is round-off noise in the FP64 run (Bz of a
    # z-independent vortex) does not divide by ~0
    bmag = (np.sqrt(fr["Bx"] ** 2 + fr["By"] ** 2 + fr["Bz"] ** 2).mean()
            if "Bx" in fr else None)
    for k in ("rho", "p", "Bx", "By", "Bz"):
        if k not in fr:
            continue
        den = bmag if k.startswith("B") else np.abs(fr[k]).mean()
        err = np.abs(fg[k] - fr[k]).mean() / den
        assert err < 1e-4, (k, err)


def test_device_loop_matches_host_loop(gpu_lib):
    """gch_advance (dt kept on the device, CUDA graph) == host-driven loop."""
    from guacho_gb300.domain import Domain
    p, u0 = problems.orszag_tang(32, 32, 4)
    with Domain(p) as a, Domain(p) as b:
        a.init(u0)
        b.init(u0)
        na = a.run(0.05, 0.02, device_loop=True)
        nb = b.run(0.05, 0.02, device_loop=False)
        assert na == nb and a.iter == b.iter
        assert a.time == b.time and a.tprint == b.tprint
        assert np.array_equal(a.download(), b.download())


def test_device_loop_matches_oracle_main_loop(gpu_lib):
    """The src/main.f90:94-125 loop to t = 0.1 with output clipping."""
    from guacho_gb300.domain import Domain
    from oracle.oracle import Oracle
    p, u0 = problems.orszag_tang(32, 32, 4)
    o = Oracle(p)
    o.init(u0)
    no = o.run(0.1, 0.03)
    with Domain(p) as d:
        d.init(u0)
        nd = d.run(0.1, 0.03)
        assert nd == no and d.time == o.time
        assert np.array_equal(interior(d.download()), interior(o.download()))


@pytest.mark.parametrize("prec", [P.FP64, P.FP32_KAHAN])
def test_host_round_trip_keeps_dt(gpu_lib, prec):
    """A download -> upload round trip of u between steps (the host view of
    the Kahan pairs is their FP64 sum) gives back the same CFL dt."""
    from guacho_gb300.domain import Domain
    p, u0 = problems.turbulence(24, seed=8)
    p = p.replace(precision=prec)
    with Domain(p) as a, Domain(p) as b:
        a.init(u0)
        b.init(u0)
        t = 0.0
        for it in range(1, 5):
            dta, _ = a.get_timestep(it, 10, t, 1e30)
            b.upload(b.download())
            dtb, _ = b.get_timestep(it, 10, t, 1e30)
            assert dta == dtb
            a.tstep(dta)
            b.tstep(dtb)
            t += dta


def test_step_host_matches_device(gpu_lib):
    from guacho_gb300.domain import Domain
    p, u0 = problems.blast(16, p_in=1.0)
    with Domain(p) as a, Domain(p) as b:
        a.init(u0)
        b.init(u0)
        uh = a.download()
        t = 0.0
        for it in range(1, 4):
            dt, _ = a.step_host(uh, it, 10, t, 1e30)
            dtb, _ = b.get_timestep(it, 10, t, 1e30)
            b.tstep(dtb)
            assert dt == dtb
            t += dt
        assert np.array_equal(interior(uh), interior(b.download()))


@pytest.mark.parametrize("prec", [P.FP64, P.FP32_KAHAN])
def test_pinned_and_pageable_host_arrays_agree(gpu_lib, prec):
    """Page-locked host arrays are read and written by the layout kernels
    over the host link; pageable ones go through the staging buffer: both
    routes move the same bytes (upload, download with primit, step_host)."""
    torch = pytest.importorskip("torch")
    from guacho_gb300.domain import Domain
    p, u0 = problems.turbulence(20, seed=6)
    p = p.replace(precision=prec)

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
        t[...] = a
        return t

    with Domain(p) as a, Domain(p) as b:
        a.upload(u0)
        b.upload(pinned(u0))
        ua, pa = a.download(with_primit=True)
        ub = pinned(np.zeros(p.shape))
        pb = pinned(np.zeros(p.shape))
        assert b._lib.gch_download(b._h, ub.ctypes.data, pb.ctypes.data) == 0
        assert np.array_equal(ua, ub) and np.array_equal(pa, pb)
        a.init(u0)
        b.init(u0)
        ha, hb = a.download(), pinned(b.download())
        t = 0.0
        for it in range(1, 3):
            dta, _ = a.step_host(ha, it, 10, t, 1e30)
            dtb, _ = b.step_host(hb, it, 10, t, 1e30)
            assert dta == dtb
            t += dta
        assert np.array_equal(ha, hb)


@pytest.mark.parametrize("prec", [P.FP64, P.FP32_MIXED, P.FP32_KAHAN])
def test_deterministic(gpu_lib, prec):
    p, u0 = problems.turbulence(16, seed=9)
    pm = p.replace(precision=prec)
    a, _ = _gpu_run(pm, u0, 5)
    b, _ = _gpu_run(pm, u0, 5)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("prec", [P.FP32_MIXED, P.FP32_KAHAN])
def test_divb_roundoff_mixed(gpu_lib, prec):
    from guacho_gb300.domain import Domain
    p, u0 = problems.turbulence(32, seed=2)
    with Domain(p.replace(precision=prec)) as d:
        d.init(u0)
        d.run(1e30, 1e30, max_steps=20)
        u = d.download()
    bx, by, bz = u[..., 5], u[..., 6], u[..., 7]
    div = ((bx[2:-2, 2:-2, 3:-1] - bx[2:-2, 2:-2, 1:-3]) / (2 * p.dx)
           + (by[2:-2, 3:-1, 2:-2] - by[2:-2, 1:-3, 2:-2]) / (2 * p.dy)
           + (bz[3:-1, 2:-2, 2:-2] - bz[1:-3, 2:-2, 2:-2]) / (2 * p.dz))
    bmag = np.sqrt(bx ** 2 + by ** 2 + bz ** 2).max()
    assert np.abs(div).max() * p.dx / bmag < 1e-6


def test_batch_matches_single_domains(gpu_lib):
    """A grouped FP32 batch runs the one-box kernel bodies in other kernel
    instantiations, where the compiler may contract a*b+c differently: each
    box matches its single-domain run to a few FP32 roundings per field."""
    from guacho_gb300.domain import Batch, Domain
    boxes = problems.batch_boxes(nbox=4, sizes=(16, 24), precision=P.FP32_MIXED)
    b = Batch([p for p, _ in boxes])
    for i, (_, u) in enumerate(boxes):
        b.upload(i, u)
    b.advance(5)
    for i, (p, u) in enumerate(boxes):
        with Domain(p) as d:
            d.init(u)
            d.run(1e300, 1e300, max_steps=5)
            ref = d.download()
        got = b.download(i)
        scale = np.abs(ref).reshape(-1, p.neq).max(axis=0)
        err = np.abs(got - ref).reshape(-1, p.neq).max(axis=0)
        assert np.all(err <= 1e-5 * np.maximum(scale, 1e-30)), (i, err / scale)
    b.close()

"""gch_step_host with its copies of a pageable host array overlapped with the
step: u goes up slab by slab of z chunks while the CFL pass and the first
stage's fluxes (deferred: their flux differences, the update once dt is
known) start on the slabs that have landed; the second stage, its CT and the
x/y ghost ring run slab by slab and each finished slab is copied to the host
while the next ones compute.  Page-locked arrays take the serial order
(kernel-driven transfers).  Either way the host array must end bit for bit
as the serial order leaves it (upload, get_timestep, tstep, download), ghost
cells included, for every precision, wall type, and boxes whose z extent is
not a multiple of the chunk depth."""
import numpy as np
import pytest

from guacho_gb300 import params as P
from guacho_gb300 import problems

pytestmark = pytest.mark.gpu

WALLS = dict(bc_left=P.BC_CLOSED, bc_right=P.BC_OUTFLOW, bc_bottom=P.BC_OUTFLOW,
             bc_top=P.BC_CLOSED, bc_out=P.BC_CLOSED, bc_in=P.BC_OUTFLOW)
CASES = {
    "turbulence_48": lambda: problems.turbulence(48, seed=4),
    "ot_ragged_walls": lambda: problems.orszag_tang(37, 19, 45, **WALLS),
    "blast_outflow": lambda: problems.blast(24, p_in=1.0),
    "ot_no_flux_cd": lambda: problems.orszag_tang(24, 24, 30, enable_flux_cd=False),
    # hydro (5 equations, HLLC): the deferred first stage without B
    "hydro_hllc": lambda: __import__("test_parity_gpu")._hydro_state(24),
}


def _pinned(a):
    torch = pytest.importorskip("torch")
    t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
    t[...] = a
    return t


@pytest.mark.parametrize("prec", [P.FP64, P.FP32_KAHAN, P.FP32_MIXED])
@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("host", ["pinned", "pageable"])
def test_overlapped_step_host_equals_serial(gpu_lib, name, prec, host):
    from guacho_gb300.domain import Domain
    p, u0 = CASES[name]()
    p = p.replace(precision=prec)
    with Domain(p) as a, Domain(p) as b:
        a.init(u0)
        b.init(u0)
        if a.kz * 3 > p.nz:  # at least three z chunks
            a.kz = b.kz = max(1, p.nz // 4)
        # the FP64 step keeps the serial order (bound by its arithmetic)
        assert a.step_host_overlaps() == (prec != P.FP64)
        h = a.download()
        if host == "pinned":
            h = _pinned(h)
        hb = b.download()
        t = 0.0
        for it in range(1, 4):
            dt, _ = a.step_host(h, it, 10, t, 1e30)
            # the serial order, with the state carried through the host
            # array as step_host carries it (the FP32 pair paths re-split
            # each FP64 value on upload)
            b.upload(hb)
            dtb, _ = b.get_timestep(it, 10, t, 1e30)
            b.tstep(dtb)
            hb = b.download()
            assert dt == dtb
            bad = np.argwhere(h != hb)
            assert bad.size == 0, (it, len(bad), bad[:3])
            t += dt


def test_serial_order_kept_where_it_cannot_overlap(gpu_lib):
    """User spheres are re-imposed after the whole-shell fill: no overlap,
    and the result is that of the serial order."""
    from guacho_gb300.domain import Domain
    p, u0 = problems.wind_cooling(24)
    with Domain(p) as a, Domain(p) as b:
        a.init(u0)
        b.init(u0)
        assert not a.step_host_overlaps()
        h = a.download()
        dt, _ = a.step_host(h, 1, 10, 0.0, 1e30)
        b.upload(b.download())
        b.calcprim()
        dtb, _ = b.get_timestep(1, 10, 0.0, 1e30)
        b.tstep(dtb)
        assert dt == dtb and np.array_equal(h, b.download())

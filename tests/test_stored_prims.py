"""The primitives get_timestep stores for the first stage (FP32 with FP64 u).

get_timestep's CFL pass recovers every interior cell's primitives from u;
on the FP32 path with FP64 u it also stores them (and those of the one-cell
ghost shell), and the first stage of the following tstep reads them instead
of recovering them again in FP64.  When u has changed since -- a tstep without a
get_timestep before it, an upload, a boundary fill -- tstep recovers them
itself, with the same arithmetic.  Either way a step computes the same bits."""
import numpy as np
import pytest

from guacho_gb300 import params as P
from guacho_gb300 import problems

pytestmark = pytest.mark.gpu


def _steps(p, u0, dts, with_get=True, reupload=False):
    from guacho_gb300.domain import Domain
    with Domain(p) as d:
        d.init(u0)
        t = 0.0
        for it, dt in enumerate(dts, start=1):
            if with_get:
                d.get_timestep(it, 10, t, 1e30)
            if reupload:  # a new u through the C ABI: the stored primitives are stale
                d.upload(d.download())
                d.boundaryI()
            d.tstep(dt)
            t += dt
        return d.download()


@pytest.mark.parametrize("case", ["turbulence", "blast", "hydro"])
def test_stored_and_recomputed_primitives_agree(gpu_lib, case):
    # (FP64 u: the download/upload round trip of the third run is exact)
    prec = P.FP32_MIXED
    if case == "turbulence":
        p, u0 = problems.turbulence(20, seed=4)
    elif case == "blast":
        p, u0 = problems.blast(18, p_in=20.0)
    else:
        p, u0 = problems.orszag_tang(20, 12, 6)
        p = p.replace(mhd=False, riemann_solver=P.SOLVER_HLLC, enable_flux_cd=False)
        u0 = np.ascontiguousarray(u0[..., :5])
    p = p.replace(precision=prec)
    dts = [2e-4, 3e-4, 2.5e-4, 1e-4]
    a = _steps(p, u0, dts)                       # primitives stored by get_timestep
    b = _steps(p, u0, dts, with_get=False)       # tstep recovers them itself
    c = _steps(p, u0, dts, reupload=True)        # stale after an upload: recovered
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(a, c)

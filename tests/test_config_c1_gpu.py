"""The Orszag-Tang configuration at its full size and length: 128 x 128 x 4
(dz = dx), HLLD, minmod, flux-CD, periodic, CFL 0.4, run by the time loop of
src/main.f90:94-125 to t = 0.5 with an output every 0.1 (OT/parameters.f90:
173-175), so get_timestep's clip to tprint shapes the dt sequence.

The plain FP64 path (the device loop, dt never leaving the GPU) must end
bit for bit on the oracle's state, after the same number of steps at the
same time; the FP32 paths within the relative L1 bar of 1e-4 per field."""
import numpy as np
import pytest

from conftest import interior
from guacho_gb300 import params as P
from guacho_gb300 import problems

pytestmark = pytest.mark.gpu

TMAX, DTPRINT = 0.5, 0.1


@pytest.fixture(scope="module")
def oracle_run():
    from oracle.oracle import Oracle
    p, u0 = problems.orszag_tang(128, 128, 4)
    o = Oracle(p)
    o.init(u0)
    steps = o.run(TMAX, DTPRINT)
    assert o.error == 0
    return p, u0, o.download(), steps, o.time


def test_fp64_device_loop_bitwise_to_t05(gpu_lib, oracle_run):
    from guacho_gb300.domain import Domain
    p, u0, ur, steps, t = oracle_run
    assert steps > 200 and t > TMAX
    with Domain(p) as d:
        d.init(u0)
        done = d.run(TMAX, DTPRINT)
        ug = d.download()
        assert done == steps
        assert d.time == t
    a, b = interior(ug), interior(ur)
    bad = np.argwhere(a != b)
    assert bad.size == 0, (len(bad), bad[:3])


@pytest.mark.parametrize("prec", [P.FP32_KAHAN, P.FP32_MIXED])
def test_fp32_paths_l1_to_t05(gpu_lib, oracle_run, prec):
    from guacho_gb300.domain import Domain
    p, u0, ur, steps, _ = oracle_run
    with Domain(p.replace(precision=prec)) as d:
        d.init(u0)
        d.run(TMAX, DTPRINT, max_steps=steps)  # the FP32 dt may differ: equal step count
        ug = d.download()
    a, b = interior(ug), interior(ur)
    for q in range(8):
        scale = np.abs(b[..., q]).mean()
        if scale == 0.0:  # rho vz and Bz: zero throughout the 2.5-D vortex
            assert np.abs(a[..., q]).max() <= 1e-12, q
            continue
        err = np.abs(a[..., q] - b[..., q]).mean() / scale
        assert err < 1e-4, (q, err)

"""The configurations at their full sizes, a few steps each, on the plain FP64
path against the oracle through the C ABI (get_timestep + tstep, dt read
back every step):

- decaying MHD turbulence 256^3 (HLLD, van Leer, flux-CD, periodic): bit for bit;
- the low-beta blast 192^3 (HLLD, minmod, flux-CD, outflow): bit for bit;
- the wind with table cooling 256^3 (hydro HLLC, outflow, two spheres, the
  planet on its orbit): within 1e-11 (exp and log10 on the cooling path).

The small-box cases of test_parity_gpu cover the branches; these show the
same arithmetic at the benchmark's sizes (array extents beyond 2^24 cells,
every tile and z chunk of the bench launches)."""
import numpy as np
import pytest

from conftest import interior
from guacho_gb300 import problems
from test_parity_gpu import _gpu_run, _oracle_run

pytestmark = pytest.mark.gpu

STEPS = 3


@pytest.mark.parametrize("name", ["turbulence_256", "blast_192"])
def test_fp64_full_size_bitwise(gpu_lib, name):
    p, u0 = {"turbulence_256": lambda: problems.turbulence(256),
             "blast_192": lambda: problems.blast(192)}[name]()
    ur, dr = _oracle_run(p, u0, STEPS)
    ug, dg = _gpu_run(p, u0, STEPS)
    assert dr == dg, (dr, dg)
    a, b = interior(ug), interior(ur)
    bad = np.argwhere(a != b)
    assert bad.size == 0, (len(bad), bad[:3])


def test_fp64_wind_cooling_full_size(gpu_lib):
    p, u0 = problems.wind_cooling(256)
    ur, dr = _oracle_run(p, u0, STEPS)
    ug, dg = _gpu_run(p, u0, STEPS)
    np.testing.assert_allclose(dg, dr, rtol=1e-12)
    np.testing.assert_allclose(interior(ug), interior(ur), rtol=1e-11, atol=1e-14)

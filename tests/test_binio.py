"""BIN output / warm-start format (src/Out_BIN_Module.f90:40-248,
src/init.f90:437-467), pinned by the reference's own Python reader: the
golden file tests/golden/bin_ot8.npz holds a file written by binio and the
arrays that py/guacho_utils.py read back from it (tests/golden/
make_bin_golden.py made it)."""
from pathlib import Path

import numpy as np
import pytest

from guacho_gb300 import binio, problems

GOLD = Path(__file__).resolve().parent / "golden" / "bin_ot8.npz"


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _params():
    return problems.orszag_tang(8, 8, 4)[0]


def test_writer_bytes_stable(gold, tmp_path):
    p = _params()
    f = tmp_path / "points000.000.bin"
    binio.write_bin(f, gold["u"], p)
    assert f.read_bytes() == gold["raw"].tobytes()
    d = tmp_path / "divB-000.000.bin"
    binio.write_divb(d, gold["u"], p)
    assert d.read_bytes() == gold["divb_raw"].tobytes()


def test_reference_reader_sees_our_header(gold):
    p = _params()
    assert gold["hdr_kind"].tobytes() == b"d"
    assert tuple(gold["hdr_n"]) == (p.nx, p.ny, p.nz)
    assert np.allclose(gold["hdr_d"], (p.dx, p.dy, p.dz), rtol=0, atol=0)
    assert tuple(gold["hdr_origin"]) == (0, 0, 0) and tuple(gold["hdr_mpi"]) == (1, 1, 1)
    assert tuple(gold["hdr_neq"]) == (8, 8, 2)
    assert float(np.ravel(gold["hdr_cv"])[0]) == p.cv


def test_reference_reader_sees_our_data(gold):
    u = gold["u"]
    for eq in range(8):
        # reference arrays are Fortran-ordered (x, y, z) interiors
        np.testing.assert_array_equal(gold[f"cons{eq}"], u[2:-2, 2:-2, 2:-2, eq].T)
    np.testing.assert_array_equal(gold["rho"], u[2:-2, 2:-2, 2:-2, 0].T)
    # the reference reader's pressure equals the u2prim pressure (rounding aside)
    ui = u[2:-2, 2:-2, 2:-2]
    rho = ui[..., 0]
    v = ui[..., 1:4] / rho[..., None]
    pr = (ui[..., 4] - 0.5 * rho * (v ** 2).sum(-1) - 0.5 * (ui[..., 5:8] ** 2).sum(-1)) / 1.5
    np.testing.assert_allclose(gold["p"], pr.T, rtol=1e-12)


def test_read_bin_roundtrip(gold, tmp_path):
    p = _params()
    f = binio.bin_path(tmp_path, 7)
    assert f.name == "points000.007.bin"
    binio.write_bin(f, gold["u"], p)
    hdr, arr = binio.read_bin(f)
    assert hdr["nx"] == 8 and hdr["nghost"] == 2 and hdr["neq"] == 8
    np.testing.assert_array_equal(arr, gold["u"])


@pytest.mark.gpu
def test_checkpoint_restart_bitwise(gpu_lib, tmp_path):
    """Warm start (src/init.f90:437-467): 6 steps straight equal 3 steps,
    a BIN checkpoint, a fresh domain read from it, and 3 more steps."""
    from guacho_gb300.domain import Domain
    p, u0 = problems.orszag_tang(32, 32, 4)
    with Domain(p) as a:
        a.init(u0)
        a.run(1e30, 1e30, max_steps=6)
        straight = a.download()
    with Domain(p) as b:
        b.init(u0)
        b.run(1e30, 1e30, max_steps=3)
        f = binio.bin_path(tmp_path, 1)
        binio.write_bin(f, b.download(), p)
        state = (b.time, b.iter, b.tprint)
    _, uc = binio.read_bin(f)
    with Domain(p) as c:
        c.upload(uc)
        c.calcprim()
        c.time, c.iter, c.tprint = state
        c.run(1e30, 1e30, max_steps=3)
        restarted = c.download()
    np.testing.assert_array_equal(restarted[2:-2, 2:-2, 2:-2], straight[2:-2, 2:-2, 2:-2])

"""Generate tests/golden/u2prim_ref.npz: conserved MHD states and the
primitives that the reference's own Python reader computes from them
(py/guacho_utils.py:39-69 u2prim, through readbin3d_block with mhd=True and
scale=False, i.e. code units).  The states are written to a BIN file with
guacho_gb300.binio (the format is pinned by tests/golden/bin_ot8.npz) and
read back by the reference's reader.

States: a 16 x 8 x 4 box of random cells -- density log-uniform over
1e-3..1e3, velocities up to Mach ~10, |B| chosen so that the plasma beta is
log-uniform over 1e-4..1e2 (the low-beta cells are the catastrophic
cancellation E - rho v^2/2 - B^2/2 of the pressure recovery), pressures
log-uniform over 1e-6..1e2, all above the reference's floors.

Run where the reference sources are present, giving the root of the
reference checkout:
    python tests/golden/make_u2prim_golden.py <reference-root>
The tests read only the stored arrays; they never import the reference."""
import importlib.util
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from guacho_gb300 import binio  # noqa: E402
from guacho_gb300.params import Params  # noqa: E402


def states(seed=20260002, nx=16, ny=8, nz=4):
    p = Params(nx=nx, ny=ny, nz=nz, mhd=True)
    rng = np.random.default_rng(seed)
    sh = p.shape[:3]
    rho = 10.0 ** rng.uniform(-3.0, 3.0, sh)
    pr = 10.0 ** rng.uniform(-6.0, 2.0, sh)
    cs = np.sqrt(p.gamma * pr / rho)
    v = rng.standard_normal(sh + (3,))
    v *= (cs * 10.0 ** rng.uniform(-2.0, 1.0, sh) / np.linalg.norm(v, axis=-1))[..., None]
    beta = 10.0 ** rng.uniform(-4.0, 2.0, sh)
    b = rng.standard_normal(sh + (3,))
    b *= (np.sqrt(2.0 * pr / beta) / np.linalg.norm(b, axis=-1))[..., None]
    u = np.zeros(p.shape)
    u[..., 0] = rho
    u[..., 1:4] = rho[..., None] * v
    u[..., 4] = 0.5 * rho * (v ** 2).sum(-1) + p.cv * pr + 0.5 * (b ** 2).sum(-1)
    u[..., 5:8] = b
    return p, u


def main(ref_root: str) -> None:
    spec = importlib.util.spec_from_file_location("guacho_utils",
                                                  Path(ref_root) / "py" / "guacho_utils.py")
    gu = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gu)
    p, u = states()
    out = {"u": u}
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "points000.000.bin"
        binio.write_bin(path, u, p, scal=(1.0, 1.0, 1.0))
        for eq, name in enumerate(("rho", "vx", "vy", "vz", "p", "Bx", "By", "Bz")):
            # (nx, ny, nz) Fortran order -> (nz, ny, nx) like the host arrays
            a = gu.readbin3d_block(str(path), eq, mhd=True, scale=False)
            out[name] = np.ascontiguousarray(np.transpose(a, (2, 1, 0)))
    dst = Path(__file__).with_name("u2prim_ref.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_u2prim_golden.py <reference-root>")
    main(sys.argv[1])

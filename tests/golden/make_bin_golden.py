"""Generate tests/golden/bin_ot8.npz: a BIN file written by
guacho_gb300.binio, and what the reference's own Python reader
(py/guacho_utils.py: read_header, readbin3d_block, u2prim) reads back from it.

Run where the reference sources are present, giving the root of the
reference checkout (the directory that holds py/guacho_utils.py):
    python tests/golden/make_bin_golden.py <reference-root>
The GPU-free test tests/test_binio.py compares against the stored arrays; it
never imports the reference."""
import importlib.util
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from guacho_gb300 import binio, problems  # noqa: E402


def main(ref_root: str) -> None:
    spec = importlib.util.spec_from_file_location("guacho_utils",
                                                  Path(ref_root) / "py" / "guacho_utils.py")
    gu = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gu)
    p, u = problems.orszag_tang(8, 8, 4)
    rng = np.random.default_rng(3)
    u = u + 0.01 * rng.standard_normal(u.shape) * np.abs(u).max(axis=(0, 1, 2))
    with tempfile.TemporaryDirectory() as td:
        path = Path(td) / "points000.000.bin"
        binio.write_bin(path, u, p, scal=(1.0, 1.0, 1.0))
        raw = path.read_bytes()
        hdr = gu.read_header(str(path), verbose=False)
        hdr[0].close()
        fields = {}
        for eq in range(8):
            fields[f"cons{eq}"] = gu.readbin3d_block(str(path), eq, conserved=True)
        fields["rho"] = gu.readbin3d_block(str(path), 0, mhd=True, scale=False)
        fields["p"] = gu.readbin3d_block(str(path), 4, mhd=True, scale=False)
        dpath = Path(td) / "divB-000.000.bin"
        binio.write_divb(dpath, u, p)
        draw = dpath.read_bytes()
    np.savez_compressed(
        Path(__file__).with_name("bin_ot8.npz"), u=u, raw=np.frombuffer(raw, dtype=np.uint8),
        divb_raw=np.frombuffer(draw, dtype=np.uint8),
        hdr_kind=np.frombuffer(hdr[1], dtype=np.uint8), hdr_n=np.array(hdr[2]),
        hdr_d=np.array(hdr[3]), hdr_origin=np.array(hdr[4]), hdr_mpi=np.array(hdr[5]),
        hdr_neq=np.array([hdr[6], hdr[7], hdr[8]]), hdr_scal=np.array(hdr[9]),
        hdr_cv=np.array(hdr[10]), **fields)
    print("wrote", Path(__file__).with_name("bin_ot8.npz"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_bin_golden.py <reference-root>")
    main(sys.argv[1])

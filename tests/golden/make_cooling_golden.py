"""Generate tests/golden/cooling_tables.npz: the reference's two shipped
cooling curves (src/DMClib/coolingDMC.tab, src/CHIANTIlib/coolingCHIANTI.tab),
decoded by guacho_gb300.params.read_cooling_table the way the reference's
readers decode them (src/cooling_dmc.f90:57-82, src/cooling_chi.f90:56-80),
together with the raw columns of each file.

Run where the reference sources are present, giving the root of the
reference checkout:
    python tests/golden/make_cooling_golden.py <reference-root>
The tests read only the stored arrays; they never open the reference."""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from guacho_gb300 import params as P  # noqa: E402

FILES = {P.COOL_DMC: ("dmc", "src/DMClib/coolingDMC.tab"),
         P.COOL_CHI: ("chi", "src/CHIANTIlib/coolingCHIANTI.tab")}


def raw_columns(text: str) -> np.ndarray:
    rows = []
    for line in text.splitlines():
        tok = line.replace("d", "e").replace("D", "e").split()
        if len(tok) >= 2:
            rows.append((float(tok[0]), float(tok[1])))
    return np.array(rows[:P.COOL_TABLE_ROWS])


def main(ref_root: str) -> None:
    out = {}
    for kind, (name, rel) in FILES.items():
        path = Path(ref_root) / rel
        tab = P.read_cooling_table(path, kind)
        out[f"{name}_raw"] = raw_columns(path.read_text())
        out[f"{name}_T"] = np.array(tab["tab_T"])
        out[f"{name}_L"] = np.array(tab["tab_L"])
        out[f"{name}_tail"] = np.array(tab["tab_tail"])
    dst = Path(__file__).with_name("cooling_tables.npz")
    np.savez_compressed(dst, **out)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_cooling_golden.py <reference-root>")
    main(sys.argv[1])

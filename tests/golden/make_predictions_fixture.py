"""Build tests/golden/predictions_fit03_fit08.npz from two of MILADY's regression fits.

Each fit directory of the reference's tests (tests/train_tests/fitNN) holds the parameter file
its run wrote (bso4_*_params.pot) next to the predictions of that run (train_energy.out,
train_force.out, train_stress.out: es20.10 predicted value, reference value, class, file).  With
the same weights, design rows x weights must reproduce those predictions.  This script packs a
few structures of each fit with their predicted E, F (atom-major x,y,z) and S:

* fit03: W, quadratic QNML (mld_order 2), j_max=2, r_cut=4.7, 211 weights; 47-atom vacancy cells
  (E, F), 128-atom strained cells (E, F, S, large box) and 1-atom deformed cells (small box, S);
* fit08: Ta-Ti-V-W, linear, weighted + weighted_3ch + weighted_auto, j_max=4, r_cut=5.0,
  166 weights; 128- and 100-atom cells (E, F, S).

Usage:  python tests/golden/make_predictions_fixture.py [/path/to/MILADY]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from mld_gb300 import potfile  # noqa: E402
from mld_gb300.poscar import read_poscar  # noqa: E402

CASES = {
    "fit03": dict(pot="bso4_qnml1_params.pot", elements=["W"], j_max=2.0, r_cut=4.7, order=2,
                  names=["01_111_000001", "01_111_000002", "09_111_000001", "12_111_000001", "12_111_000002",
                         "12_111_000003"]),
    "fit08": dict(pot="bso4_snap1_params.pot", elements=["Ta", "Ti", "V", "W"], j_max=4.0, r_cut=5.0, order=1,
                  names=["00_001_000001", "28_001_000001", "29_001_000001"]),
}


def _by_name(path):
    out = {}
    for line in open(path):
        t = line.split()
        out.setdefault(os.path.basename(t[3]).replace(".poscar", ""), []).append(float(t[0]))
    return out


def main(root: str) -> None:
    out = {}
    for fit, c in CASES.items():
        d = os.path.join(root, "tests", "train_tests", fit)
        E, F, S = (_by_name(os.path.join(d, f"train_{k}.out")) for k in ("energy", "force", "stress"))
        out[f"{fit}_w"] = potfile.read_milady_pot(os.path.join(d, c["pot"]))
        out[f"{fit}_names"] = np.array(c["names"])
        out[f"{fit}_params"] = np.array([c["j_max"], c["r_cut"], c["order"]])
        out[f"{fit}_elements"] = np.array(c["elements"])
        for i, n in enumerate(c["names"]):
            s = read_poscar(os.path.join(d, "DB", n + ".poscar"), want_forces=False)
            m = np.array([c["elements"].index(e) for e in s.elements], np.int32)
            out[f"{fit}_cell_{i}"] = s.cell
            out[f"{fit}_pos_{i}"] = s.positions
            out[f"{fit}_types_{i}"] = m[s.types]
            out[f"{fit}_E_{i}"] = np.array(E.get(n, [np.nan]))
            out[f"{fit}_F_{i}"] = np.array(F.get(n, []))
            out[f"{fit}_S_{i}"] = np.array(S.get(n, []))
            assert out[f"{fit}_F_{i}"].size in (0, 3 * s.nat) and out[f"{fit}_S_{i}"].size in (0, 6), n
    np.savez_compressed(os.path.join(HERE, "predictions_fit03_fit08.npz"), **out)
    print("wrote", sum(len(c["names"]) for c in CASES.values()), "structures")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {os.path.basename(__file__)} <path of the MILADY source tree>")
    main(sys.argv[1])
